import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and libgbns.so")
    # temporary files of the tests stay inside the repository, in the git-ignored build folder
    if not config.option.basetemp:
        os.makedirs(os.path.join(ROOT, "_build"), exist_ok=True)   # pytest creates only the last level
        config.option.basetemp = os.path.join(ROOT, "_build", "pytest-tmp")


def corr_gauss(D, seed):
    """mu ~ N(0,1)^D, Sigma = A A^T / D + 0.1 I with A ~ N(0,1)^{DxD} (numpy default_rng(seed))."""
    rng = np.random.default_rng(seed)
    mu = rng.standard_normal(D)
    A = rng.standard_normal((D, D))
    return mu, A @ A.T / D + 0.1 * np.eye(D)


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu_lib():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from jaxns_gb300.build import build_library
    build_library()
    from jaxns_gb300 import _ffi
    return _ffi.load()


def model32_of_spec(oracle_mod, spec, warp_min_D=17):
    """The fp32 kernel-arithmetic model of a run (the device's fp32 tables; the reduction order
    of the kernel that runs it in a batch with this warp_min_D)."""
    return oracle_mod.model32(spec.family, spec.D, np.asarray(spec.params, np.float32), spec.prior_kind,
                              np.asarray(spec.prior_a, np.float32), np.asarray(spec.prior_b, np.float32),
                              warp_min_D=warp_min_D)


def assert_shell_exact(oracle_mod, b, r, Lstar_raw, key, num_chains=None):
    """The shell just run on the device for run r (contour Lstar_raw relative to the run's
    log-likelihood offset, sample key `key`) equals the fp32 kernel-arithmetic oracle bit for
    bit in every chain: evaluation count, accepted point, its log-likelihood and the phantoms.
    Returns the oracle's outputs (U, L relative, E)."""
    spec = b.specs[r]
    s = num_chains or spec.shell_size
    live = b.live_view(r)
    m32 = model32_of_spec(oracle_mod, spec, b.warp_min_D)
    U3, L3, E3, pU3, pL3 = oracle_mod.slice_shell32(
        m32, key, np.float32(Lstar_raw), live["U"].cpu().numpy(), live["log_L_raw"].cpu().numpy(), s,
        spec.num_slices, num_phantom=spec.num_phantom, midpoint_shrink=spec.midpoint_shrink,
        gradient_guided=spec.gradient_guided, gradient_slice=spec.gradient_slice)
    so = int(b.offsets["shell"][r])
    E_g = b.new_E[so:so + s].cpu().numpy()
    U_g = b.new_U_view(r).cpu().numpy()[:s]
    L_g = b.new_L[so:so + s].cpu().numpy()
    bad = np.nonzero((E_g != E3) | np.any(U_g.view(np.uint32) != U3.view(np.uint32), axis=1)
                     | (L_g.view(np.uint32) != L3.view(np.uint32)))[0]
    assert len(bad) == 0, (f"{len(bad)} of {s} chains differ from the fp32 oracle; first {bad[:5]}: "
                           f"E {E_g[bad[:5]]} vs {E3[bad[:5]]}, L {L_g[bad[:5]]} vs {L3[bad[:5]]}")
    K = spec.num_phantom
    if K > 0:
        D = spec.D
        po, pu = int(b.offsets["phL"][r]), int(b.offsets["phU"][r])  # run r's [s, K] and [s, K, D] blocks
        pL_g = b.ph_L[po:po + s * K].view(s, K).cpu().numpy()
        np.testing.assert_array_equal(pL_g.view(np.uint32), pL3.view(np.uint32))
        pU_g = b.ph_U[pu:pu + s * K * D].view(s, K, D).cpu().numpy()
        np.testing.assert_array_equal(pU_g.view(np.uint32), pU3.view(np.uint32))
    return U3, L3, E3
