"""Launch-shape autotuning: the sampler's results do not depend on the launch shape (every
chain's random stream is fixed by its index), and the tuner returns the fastest candidate."""
import numpy as np
import pytest

from tests.test_gpu_parity import _spec

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _mixed_specs(oracle_mod):
    from jaxns_gb300.engine import FAMILY_SHELLS, shells_offset, shells_params
    specs = []
    for i, (D, n) in enumerate([(4, 64), (12, 96), (20, 64), (40, 64)]):
        spec, _ = _spec(D, n, 2 * D, oracle_mod.PRNGKey(300 + i), seed=30 + i)
        specs.append(spec)
    c1 = np.zeros(6)
    c1[0] = 1.0
    sh, _ = _spec(6, 80, 12, oracle_mod.PRNGKey(399), family=FAMILY_SHELLS,
                  params=shells_params(c1, -c1, 0.8, 0.2), offset=shells_offset(0.2), low=-3.0, high=3.0)
    specs.append(sh)
    return specs


def test_results_independent_of_launch_shape(gpu_lib, oracle_mod):
    from jaxns_gb300.engine import NSBatch
    specs = _mixed_specs(oracle_mod)
    out = []
    for cpi, cpl, wide in ((32, 1, 128), (128, 4, 512), (64, 2, 256)):
        b = NSBatch(specs, chains_per_item=cpi, chains_per_lane=cpl, wide_chains_per_item=wide)
        b.init()
        b.iterate(3)
        torch.cuda.synchronize()
        out.append((b.store_L.cpu().numpy().copy(), b.store_S.cpu().numpy().copy(), b.store_E.cpu().numpy().copy(),
                    b.state()))
    L1, S1, E1, st1 = out[0]
    for L2, S2, E2, st2 in out[1:]:
        np.testing.assert_array_equal(L1.view(np.uint32), L2.view(np.uint32))
        np.testing.assert_array_equal(S1, S2)
        np.testing.assert_array_equal(E1, E2)
        np.testing.assert_array_equal(st1["key"], st2["key"])
        np.testing.assert_array_equal(st1["num_likelihood_evaluations"], st2["num_likelihood_evaluations"])


def test_kernel_choice_exact_against_its_oracle_model(gpu_lib, oracle_mod):
    """A correlated Gaussian with 8 < D <= 16 on either sampler kernel (warp_min_D 17: one
    thread per chain; 9: warp-cooperative): each shell equals the fp32 oracle of that kernel's
    reduction order bit for bit."""
    from jaxns_gb300.engine import NSBatch
    from tests.conftest import assert_shell_exact
    spec, _ = _spec(12, 256, 24, oracle_mod.PRNGKey(12), seed=12)
    for wmin in (17, 9):
        b = NSBatch([spec], warp_min_D=wmin)
        b.init()
        live = b.live_view(0)
        Ls = float(live["log_L_raw"][127].item())
        key = oracle_mod.PRNGKey(4242)
        b.slice_shell(torch.tensor([Ls]), torch.tensor(key.view(np.int32)).view(1, 2))
        torch.cuda.synchronize()
        assert_shell_exact(oracle_mod, b, 0, Ls, key)


def test_autotune_picks_the_fastest(gpu_lib, oracle_mod):
    from jaxns_gb300.autotune import CHAINS_PER_LANE, THREAD_WIDTHS, WIDE_ITEMS, autotune_launch
    res = autotune_launch(_mixed_specs(oracle_mod), iterations=1)
    nt = len(THREAD_WIDTHS) * len(CHAINS_PER_LANE)
    assert len(res["table"]) == nt + len(WIDE_ITEMS) + 2
    assert all(t["sampler_ms"] > 0 for t in res["table"])
    stage1 = res["table"][:nt]
    pick = min(stage1, key=lambda t: t["sampler_ms"])
    assert (res["chains_per_item"], res["chains_per_lane"]) == (pick["chains_per_item"], pick["chains_per_lane"])
    last = res["table"][-2:]
    assert res["warp_min_D"] == min(last, key=lambda t: t["sampler_ms"])["warp_min_D"]
    assert res["sampler_ms"] == min(t["sampler_ms"] for t in last)
