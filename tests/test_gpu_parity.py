"""GPU parity: libgbns.so (through its C ABI) against the FP64 oracle on seeded inputs."""
import ctypes

import numpy as np
import pytest

from tests.conftest import assert_shell_exact, corr_gauss, model32_of_spec

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def _s():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _spec(D, n, S, seed_key, family=0, params=None, cap=None, tc=None, K=0, store_U=True, seed=0, low=-10., high=10.,
          offset=None):
    from jaxns_gb300.engine import RunSpec, mvn_offset, mvn_params
    mu, cov = corr_gauss(D, seed)
    if params is None:
        params = mvn_params(mu, cov)
        offset = mvn_offset(cov)
    s = n // 2
    cap = cap or 100 * n
    cap = int(np.ceil(cap / (s * (1 + K))) * s * (1 + K))
    return RunSpec(D=D, num_live_points=n, shell_size=s, num_slices=S, family=family, params=params,
                   prior_kind=np.zeros(D, np.int32), prior_a=np.full(D, low), prior_b=np.full(D, high - low),
                   max_samples=cap, term_cond=dict(tc or {"dlogZ": 1e-4, "max_samples": float(cap)}),
                   key=np.asarray(seed_key, np.uint32), num_phantom=K, store_U=store_U,
                   log_L_offset=float(offset or 0.0)), (mu, cov)


def test_rng_words_exact(gpu_lib, oracle_mod):
    from jaxns_gb300 import _ffi
    key = torch.tensor(np.array([0x13198a2e, 0x03707344], np.uint32).view(np.int32), device="cuda")
    ctr = torch.tensor(np.array([0x243f6a88, 0x85a308d3, 0, 0, 0xffffffff, 0xffffffff], np.uint32).view(np.int32),
                       device="cuda")
    out = torch.zeros(6, dtype=torch.int32, device="cuda")
    _ffi.call("gbns_threefry2x32", _p(key), _p(ctr), _p(out), ctypes.c_longlong(3), _s())
    got = out.cpu().numpy().view(np.uint32)
    assert (got[0], got[1]) == (0xc4923a9c, 0x483df7a0)
    for seed in (0, 1, 12345):
        k = oracle_mod.PRNGKey(seed)
        kt = torch.tensor(k.view(np.int32), device="cuda")
        n = 4099
        sp = torch.zeros(2 * n, dtype=torch.int32, device="cuda")
        _ffi.call("gbns_threefry_split", _p(kt), _p(sp), ctypes.c_longlong(n), _s())
        np.testing.assert_array_equal(sp.cpu().numpy().view(np.uint32).reshape(n, 2), oracle_mod.split(k, n))
        bits = torch.zeros(n, dtype=torch.int64, device="cuda")
        _ffi.call("gbns_random_bits64", _p(kt), _p(bits), ctypes.c_longlong(n), _s())
        np.testing.assert_array_equal(bits.cpu().numpy().view(np.uint64), oracle_mod.random_bits64(k, n))


def test_uniform_normal_values(gpu_lib, oracle_mod):
    from jaxns_gb300 import _ffi
    n = 20000
    k = oracle_mod.PRNGKey(99)
    kt = torch.tensor(k.view(np.int32), device="cuda")
    u = torch.zeros(n, device="cuda")
    z = torch.zeros(n, device="cuda")
    _ffi.call("gbns_uniform", _p(kt), _p(u), ctypes.c_longlong(n), _s())
    _ffi.call("gbns_normal", _p(kt), _p(z), ctypes.c_longlong(n), _s())
    uo = oracle_mod.uniform(k, n)
    zo = oracle_mod.normal(k, n)
    # fp32 rounding of the f64 variates (tolerance: 1 ulp of fp32 for uniform, 4e-7 rel for normal)
    np.testing.assert_allclose(u.cpu().numpy(), uo, rtol=6e-8, atol=0)
    np.testing.assert_allclose(z.cpu().numpy(), zo, rtol=4e-6, atol=1e-7)


def test_forward_matches_oracle(gpu_lib, oracle_mod):
    """Model.forward on the device: bit for bit the fp32 kernel-arithmetic oracle, and within
    fp32 rounding of the FP64 oracle (correlated Gaussian with Uniform and with Normal priors,
    Gaussian shells)."""
    from jaxns_gb300.engine import NSBatch, shells_offset, shells_params
    for D in (2, 8, 13, 37, 64):
        for normal_prior in (False, True):
            spec, (mu, cov) = _spec(D, 64, D, oracle_mod.PRNGKey(0), seed=D)
            if normal_prior:
                spec.prior_kind = np.ones(D, np.int32)
                spec.prior_a, spec.prior_b = mu + 0.3, np.full(D, 1.5)
            b = NSBatch([spec])
            U = np.random.default_rng(D).uniform(0.3, 0.7, size=(257, D))
            U[:3, 0] = [1e-7, 0.999999, 0.5]
            got = b.forward(0, torch.tensor(U, dtype=torch.float32)).cpu().numpy()
            m32 = model32_of_spec(oracle_mod, spec)
            m32.variant = 0  # Model.forward sums sequentially whatever the sampler kernel
            ref32 = oracle_mod.forward32(m32, U.astype(np.float32)).astype(np.float64) + spec.log_L_offset
            np.testing.assert_array_equal(got.view(np.uint32), ref32.astype(np.float32).view(np.uint32))
            if normal_prior:
                om = oracle_mod.OracleModel(D, 0, np.ones(D, np.int32), np.asarray(spec.prior_a, np.float64),
                                            np.asarray(spec.prior_b, np.float64),
                                            np.concatenate([mu, np.linalg.cholesky(cov).ravel()]))
            else:
                om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
            ref = oracle_mod.forward(om, U.astype(np.float32).astype(np.float64))
            np.testing.assert_allclose(got, ref, rtol=2e-4, atol=2e-3)
    D = 10
    c1 = np.zeros(D); c1[0] = 3.5
    c2 = -c1
    spec, _ = _spec(D, 64, D, oracle_mod.PRNGKey(0), family=1, params=shells_params(c1, c2, 2.0, 0.1), low=-6., high=6.,
                    offset=shells_offset(0.1))
    b = NSBatch([spec])
    U = np.random.default_rng(0).uniform(0, 1, size=(300, D))
    U[:100] = (np.concatenate([[3.5 + 2.0], np.zeros(D - 1)]) + 6) / 12 + 0.01 * np.random.default_rng(1).standard_normal((100, D))
    got = b.forward(0, torch.tensor(U, dtype=torch.float32)).cpu().numpy()
    ref32 = oracle_mod.forward32(model32_of_spec(oracle_mod, spec), U.astype(np.float32)).astype(np.float64)
    np.testing.assert_array_equal(got.view(np.uint32), (ref32 + spec.log_L_offset).astype(np.float32).view(np.uint32))
    om = oracle_mod.shells_model(-6, 6, c1, c2, 2.0, 0.1)
    ref = oracle_mod.forward(om, U.astype(np.float32).astype(np.float64))
    np.testing.assert_allclose(got, ref, rtol=2e-4, atol=5e-3)


def test_init_live_points_match_oracle(gpu_lib, oracle_mod):
    from jaxns_gb300.engine import NSBatch
    for D, n in ((2, 64), (8, 512), (33, 200)):
        key = oracle_mod.PRNGKey(D * 7 + 1)
        spec, (mu, cov) = _spec(D, n, D, key, seed=D)
        b = NSBatch([spec])
        b.init()
        live = b.live_view(0)
        om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
        orun = oracle_mod.ns_run(om, key, n, D, init_only=True)
        # U: the 52-bit jax uniform rounded once to fp32, exactly
        np.testing.assert_array_equal(live["U"].cpu().numpy(), orun.register["live_U"].astype(np.float32))
        np.testing.assert_allclose(live["log_L"].cpu().numpy(), orun.register["live_log_L"], rtol=2e-4, atol=2e-3)
        # log L: bit for bit the fp32 kernel-arithmetic oracle of the same points
        m32 = model32_of_spec(oracle_mod, spec)
        m32.variant = 0
        np.testing.assert_array_equal(live["log_L_raw"].cpu().numpy().view(np.uint32),
                                      oracle_mod.forward32(m32, live["U"].cpu().numpy()).view(np.uint32))
        st = b.state()[0]
        np.testing.assert_array_equal(np.array(st["key"], np.uint32), orun.register["key"])


@pytest.mark.parametrize("D,n,S,K,normal", [(2, 64, 8, 0, False), (8, 512, 32, 0, False), (10, 200, 50, 0, False),
                                             (24, 128, 24, 0, False), (64, 96, 64, 0, False), (5, 128, 20, 3, False),
                                             (12, 256, 24, 0, True), (40, 96, 40, 2, True), (7, 256, 16, 0, "mixed"),
                                             (13, 128, 13, 2, "mixed"), (30, 96, 30, 0, "mixed")])
def test_slice_shell_chain_parity(gpu_lib, oracle_mod, D, n, S, K, normal):
    """One shell from the same live set, contour and key.  Every chain equals the fp32
    kernel-arithmetic oracle bit for bit (evaluation count, accepted point, log L, phantoms):
    the same RNG stream, seed choice, shrink rule and accept test in the same fp32 operation
    order.  Priors: all Uniform, all Normal, or mixed (Normal in the odd dimensions), each
    through the thread-per-chain kernel (D <= 16) and the warp-cooperative one.  Against the
    FP64 restatement the chains agree where no likelihood comparison sits within fp32 rounding
    of the contour (reported, not a pass criterion of the fp32 path)."""
    from jaxns_gb300.engine import NSBatch
    key = oracle_mod.PRNGKey(D)
    spec, (mu, cov) = _spec(D, n, S, key, seed=D, K=K)
    if normal:
        kind = np.ones(D, np.int32) if normal is True else (np.arange(D) % 2).astype(np.int32)
        spec.prior_kind = kind
        spec.prior_a = np.where(kind == 1, mu + 0.2, -10.0)
        spec.prior_b = np.where(kind == 1, 2.0, 20.0)
    b = NSBatch([spec])
    b.init()
    live = b.live_view(0)
    s = n // 2
    Lstar_dev = float(live["log_L_raw"][s - 1].item())  # relative to the run's offset, as on the device
    skey = oracle_mod.PRNGKey(1000 + D)
    b.slice_shell(torch.tensor([Lstar_dev]), torch.tensor(skey.view(np.int32)).view(1, 2))
    torch.cuda.synchronize()
    U3, L3, E3 = assert_shell_exact(oracle_mod, b, 0, Lstar_dev, skey)
    assert np.all(L3 > np.float32(Lstar_dev))
    if not normal:
        Lstar = float(live["log_L"][s - 1].item())
        om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
        U_o, L_o, E_o = oracle_mod.slice_shell(om, skey, Lstar, live["U"].cpu().double().numpy(),
                                               live["log_L"].cpu().double().numpy(), s, S, num_phantom=K)
        same = (E3 == E_o) & np.all(np.abs(U3 - U_o) < 2e-4, axis=1)
        print(f"D={D}: fp32 chains equal to the FP64 restatement: {same.mean():.3f} ({np.count_nonzero(~same)} differ)")
        assert same.mean() >= 0.9


def test_count_crossed_edges_exact(gpu_lib, oracle_mod):
    from jaxns_gb300 import _ffi
    rng = np.random.default_rng(5)
    cases = [([0, 0, 0, 1, 2, 3], [1, 2, 3, 4, 5, 6]), ([0, 0, 0, 1, 3, 2], [1, 2, 3, 4, 6, 5])]
    # a random tree (unsorted store, ties, -0/+0) and a big sorted one
    N = 5000
    sender = rng.integers(0, N // 2, size=N)
    L = np.round(rng.standard_normal(N), 2).astype(np.float32)
    L[:10] = 0.0
    L[10:20] = -0.0
    cases.append((sender, L))
    N2 = 200000  # beyond 65536 samples the count runs over many CTAs: sorted, then unsorted with ties
    L2 = np.sort(rng.standard_normal(N2)).astype(np.float32)
    cases.append((np.minimum(np.arange(N2), rng.integers(0, N2, size=N2)), L2))
    N3 = 300001
    L3 = np.round(rng.standard_normal(N3), 3).astype(np.float32)
    cases.append((rng.integers(-3, N3 + 5, size=N3), L3))
    for sender, L in cases:
        sender = np.asarray(sender, np.int32)
        L = np.asarray(L, np.float32)
        N = len(L)
        ts, tL = torch.tensor(sender, device="cuda"), torch.tensor(L, device="cuda")
        si = torch.zeros(N, dtype=torch.int32, device="cuda")
        nl = torch.zeros(N, dtype=torch.int32, device="cuda")
        sll = torch.zeros(2 * (N + 1), dtype=torch.int64, device="cuda")
        si_ = torch.zeros(N + 1, dtype=torch.int32, device="cuda")
        _ffi.call("gbns_count_crossed_edges", _p(ts), _p(tL), ctypes.c_longlong(N), _p(si), _p(nl), _p(sll), _p(si_),
                  _s())
        osi, onl = oracle_mod.count_crossed_edges(sender, L.astype(np.float64))
        np.testing.assert_array_equal(si.cpu().numpy(), osi)
        np.testing.assert_array_equal(nl.cpu().numpy(), onl)


def test_evidence_stats_fp64(gpu_lib, oracle_mod):
    from jaxns_gb300 import _ffi
    from jaxns_gb300.engine import ncoef_table
    rng = np.random.default_rng(3)
    for N, n in ((37, 10), (20000, 500), (70001, 3200)):
        L = np.sort(rng.standard_normal(N) * 30).astype(np.float32)
        nl = np.full(N, n, np.int32)
        nl[-n:] = np.arange(n, 0, -1)
        tab = torch.tensor(ncoef_table(4096), device="cuda")
        tL, tn = torch.tensor(L, device="cuda"), torch.tensor(nl, device="cuda")
        fin = torch.zeros(8, dtype=torch.float64, device="cuda")
        lX = torch.zeros(N, dtype=torch.float64, device="cuda")
        ldZ = torch.zeros(N, dtype=torch.float64, device="cuda")
        lZ = torch.zeros(N, dtype=torch.float64, device="cuda")
        _ffi.call("gbns_evidence_stats", _p(tL), _p(tn), ctypes.c_longlong(N), _p(tab), ctypes.c_int(4096), _p(fin),
                  _p(lX), _p(ldZ), _p(lZ), _s())
        ofin, oper = oracle_mod.compute_evidence_stats(L.astype(np.float64), nl.astype(np.float64))
        f = fin.cpu().numpy()
        names = ("log_L", "log_X_mean", "log_X2_mean", "log_Z_mean", "log_ZX_mean", "log_Z2_mean", "log_dZ_mean",
                 "log_dZ2_mean")
        for i, nm in enumerate(names):
            np.testing.assert_allclose(f[i], ofin[nm], rtol=1e-6, atol=1e-6, err_msg=nm)
        np.testing.assert_allclose(lX.cpu().numpy(), oper["log_X_mean"], rtol=1e-12, atol=1e-9)
        np.testing.assert_allclose(ldZ.cpu().numpy(), oper["log_dZ_mean"], rtol=1e-6, atol=1e-5)
        np.testing.assert_allclose(lZ.cpu().numpy(), oper["log_Z_mean"], rtol=1e-6, atol=1e-5)


@pytest.mark.parametrize("D,n,S,guided,climb", [(4, 128, 3, True, False), (12, 256, 24, True, False),
                                                 (4, 128, 16, False, True), (12, 256, 24, False, True),
                                                 (6, 128, 12, True, True), (24, 128, 3, True, False),
                                                 (40, 96, 3, True, False), (24, 128, 6, False, True)])
def test_gradient_options_chain_parity(gpu_lib, oracle_mod, D, n, S, guided, climb):
    """UniDimSliceSampler's gradient options: gradient_guided (the direction of the next slice
    is the reflection about the U-space gradient at the accepted point, uni_slice_sampler.py:
    255-269) and gradient_slice (each slice runs along the normalised gradient at its seed,
    t >= 0, :202-214), one extra evaluation per gradient.  Every chain bit for bit the fp32
    kernel-arithmetic oracle, for the thread-per-chain kernel (D <= 16) and the
    warp-cooperative one (D > 16, whose gradient norm and reflection sums run over lanes).
    Against the FP64 restatement each direction depends on the previous accepted point, so
    fp32-vs-FP64 differences carry from slice to slice: reported for the warp kernel, not a
    pass criterion."""
    from jaxns_gb300.engine import NSBatch
    key = oracle_mod.PRNGKey(50 + D)
    spec, (mu, cov) = _spec(D, n, S, key, seed=D)
    spec.gradient_guided, spec.gradient_slice = guided, climb
    b = NSBatch([spec])
    b.init()
    live = b.live_view(0)
    s = n // 2
    Lstar = float(live["log_L"][s - 1].item())
    Ls_raw = float(live["log_L_raw"][s - 1].item())
    skey = oracle_mod.PRNGKey(2000 + D)
    b.slice_shell(torch.tensor([Ls_raw]), torch.tensor(skey.view(np.int32)).view(1, 2))
    torch.cuda.synchronize()
    E_g = b.new_E[:s].cpu().numpy()
    assert np.all(E_g >= S * (1 + int(guided) + int(climb)))  # a proposal and each gradient per slice
    assert_shell_exact(oracle_mod, b, 0, Ls_raw, skey)
    if D <= 16:
        return
    om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    U_o, L_o, E_o = oracle_mod.slice_shell(om, skey, Lstar, live["U"].cpu().double().numpy(),
                                           live["log_L"].cpu().double().numpy(), s, S, gradient_guided=guided,
                                           gradient_slice=climb)
    U_g = b.new_U[:s * D].view(s, D).cpu().numpy()
    same = (E_g == E_o) & np.all(np.abs(U_g - U_o) < 2e-4, axis=1)
    print(f"D={D}: warp-kernel chains equal to the FP64 restatement: {same.mean():.3f}")


def test_gradient_slice_shells_exact(gpu_lib, oracle_mod):
    """gradient_slice on the Gaussian-shells family (thread per chain, softmax-weighted radial
    gradient): bit for bit the fp32 oracle."""
    from jaxns_gb300.engine import NSBatch, shells_offset, shells_params
    D = 6
    c1 = np.zeros(D)
    c1[0] = 1.0
    spec, _ = _spec(D, 128, 12, oracle_mod.PRNGKey(61), family=1, params=shells_params(c1, -c1, 0.8, 0.2),
                    offset=shells_offset(0.2), low=-3.0, high=3.0)
    spec.gradient_slice = True
    b = NSBatch([spec])
    b.init()
    b.iterate(3)
    torch.cuda.synchronize()
    live = b.live_view(0)
    Ls = float(live["log_L_raw"][63].item())
    key = oracle_mod.PRNGKey(62)
    b.slice_shell(torch.tensor([Ls]), torch.tensor(key.view(np.int32)).view(1, 2))
    torch.cuda.synchronize()
    assert_shell_exact(oracle_mod, b, 0, Ls, key)


def test_gradient_slice_run_matches_oracle(gpu_lib, oracle_mod):
    """ShardedStaticNestedSampler with UniDimSliceSampler(gradient_slice=True) end to end on a
    correlated Gaussian (D = 5).  The reference offers gradient_slice for global optimisation
    (experimental/public.py:44-77): every slice starts from its seed along the normalised
    gradient with the left end at the seed, a climb that does not leave the constrained prior
    invariant.  Its evidence is therefore biased (about +8 nats here, in the FP64 oracle as on
    the device), so the run is checked against the FP64 oracle's run of the same algorithm and
    for what the option is for: the maximum likelihood it reaches."""
    import jaxns_gb300 as gb
    from jaxns_gb300.public import ShardedStaticNestedSampler, UniDimSliceSampler
    D = 5
    mu, cov = corr_gauss(D, 8)

    def prior_model():
        x = yield gb.Prior(gb.Uniform(-10.0 * np.ones(D), 10.0 * np.ones(D)), name="x")
        return x

    model = gb.Model(prior_model, gb.MultivariateNormalLikelihood(mu, cov))
    ns = ShardedStaticNestedSampler(model=model, max_samples=100000, init_efficiency_threshold=0.1,
                                    sampler=UniDimSliceSampler(model=model, num_slices=5 * D, num_phantom_save=0,
                                                               midpoint_shrink=True, perfect=True,
                                                               gradient_slice=True),
                                    num_live_points=300)
    reason, batch = ns._run(gb.random.PRNGKey(9), gb.TerminationCondition(dlogZ=1e-4))
    sc = batch.results(with_U=False)["scalars"].cpu().numpy()[0]
    om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    r = oracle_mod.ns_run(om, oracle_mod.PRNGKey(9), 300, 5 * D, max_samples=100000,
                          term_cond={"dlogZ": 1e-4}, gradient_slice=True)
    ref, ref_unc = r.results["log_Z_mean"], r.results["log_Z_uncert"]
    assert abs(sc[0] - ref) < 4 * np.hypot(sc[1], ref_unc) + 0.05, (sc[0], sc[1], ref, ref_unc)
    # the climb reaches the likelihood's peak: log L_max = -0.5 log det(2 pi cov)
    peak = -0.5 * np.linalg.slogdet(2 * np.pi * cov)[1]
    top = float(batch.live_view(0)["log_L"].max().item())
    assert top > peak - 1e-3, (top, peak)


def test_gradient_guided_log_Z(gpu_lib):
    """NestedSampler(gradient_guided=True) end to end: correlated Gaussian D=6 (analytic) and
    Gaussian shells D=4 (the oracle's own run as the reference value)."""
    import jaxns_gb300 as gb
    D = 6
    mu, cov = corr_gauss(D, 3)

    def prior_model():
        x = yield gb.Prior(gb.Uniform(-10.0 * np.ones(D), 10.0 * np.ones(D)), name="x")
        return x

    ns = gb.NestedSampler(gb.Model(prior_model, gb.MultivariateNormalLikelihood(mu, cov)), num_live_points=300,
                          gradient_guided=True)
    reason, state = ns(gb.random.PRNGKey(4), gb.TerminationCondition(dlogZ=1e-4))
    res = ns.to_results(reason, state)
    assert abs(res.log_Z_mean + D * np.log(20.0)) < 4 * res.log_Z_uncert + 0.02, (res.log_Z_mean, res.log_Z_uncert)
    assert res.total_num_likelihood_evaluations > 0


def test_empty_and_single_sample_sets(gpu_lib, oracle_mod):
    """The empty and one-sample edge cases the reference's own tests exercise: tree count,
    FP64 evidence statistics and sample_evidence with N = 0 and N = 1 against the oracle
    (device buffers keep one element so that no pointer is NULL)."""
    from jaxns_gb300 import _ffi, sample_evidence
    from jaxns_gb300.engine import ncoef_table
    tab = torch.tensor(ncoef_table(64), device="cuda")
    for N in (0, 1):
        n1 = max(N, 1)
        ts = torch.zeros(n1, dtype=torch.int32, device="cuda")          # the one sample hangs off the root
        tL = torch.full((n1,), -2.0, dtype=torch.float32, device="cuda")
        si = torch.full((n1,), -7, dtype=torch.int32, device="cuda")
        nl = torch.full((n1,), -7, dtype=torch.int32, device="cuda")
        sll = torch.zeros(2 * (N + 1), dtype=torch.int64, device="cuda")
        si_ = torch.zeros(N + 1, dtype=torch.int32, device="cuda")
        _ffi.call("gbns_count_crossed_edges", _p(ts), _p(tL), ctypes.c_longlong(N), _p(si), _p(nl), _p(sll), _p(si_),
                  _s())
        osi, onl = oracle_mod.count_crossed_edges(np.zeros(N, np.int64), np.full(N, -2.0))
        np.testing.assert_array_equal(si.cpu().numpy()[:N], osi)
        np.testing.assert_array_equal(nl.cpu().numpy()[:N], onl)

        tn = torch.full((n1,), 3, dtype=torch.int32, device="cuda")
        fin = torch.zeros(8, dtype=torch.float64, device="cuda")
        lX, ldZ, lZ = (torch.zeros(n1, dtype=torch.float64, device="cuda") for _ in range(3))
        _ffi.call("gbns_evidence_stats", _p(tL), _p(tn), ctypes.c_longlong(N), _p(tab), ctypes.c_int(64), _p(fin),
                  _p(lX), _p(ldZ), _p(lZ), _s())
        ofin, _ = oracle_mod.compute_evidence_stats(np.full(N, -2.0), np.full(N, 3.0))
        names = ("log_L", "log_X_mean", "log_X2_mean", "log_Z_mean", "log_ZX_mean", "log_Z2_mean", "log_dZ_mean",
                 "log_dZ2_mean")
        np.testing.assert_allclose(fin.cpu().numpy(), [ofin[k] for k in names], rtol=1e-6, atol=1e-6)

        key = oracle_mod.PRNGKey(1)
        got = sample_evidence(key, np.full(N, 5, np.int64), np.full(N, -1.0), S=3).cpu().numpy()
        ref = oracle_mod.sample_evidence(key, np.full(N, 5, np.int64), np.full(N, -1.0), S=3)
        np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9)
        if N == 0:
            assert np.all(np.isneginf(got))
