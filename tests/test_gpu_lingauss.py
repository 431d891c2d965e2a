"""Linear-Gaussian (Phi w) family on the GPU: likelihood, chain parity of one lock-step
shell, end-to-end evidence against the analytic Bayesian-linear-regression value, and the
reweighted-evidence adjoint against the FP64 oracle and finite differences."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def blr(N, P, seed=0, sigma=0.5):
    rng = np.random.default_rng(seed)
    Phi = rng.standard_normal((N, P))
    w = rng.standard_normal(P)
    return Phi, Phi @ w + sigma * rng.standard_normal(N)


def blr_model(gb, Phi, y, sigma=0.5, tau=1.0):
    P = Phi.shape[1]

    def prior_model():
        w = yield gb.Prior(gb.Normal(np.zeros(P), tau * np.ones(P)), name="w")
        return w

    return gb.Model(prior_model, gb.LinearGaussianLikelihood(Phi, y, sigma))


def test_lingauss_forward(gpu_lib, oracle_mod):
    import jaxns_gb300 as gb
    from jaxns_gb300.engine import NSBatch
    Phi, y = blr(700, 12, seed=3)
    model = blr_model(gb, Phi, y)
    ns = gb.NestedSampler(model, num_live_points=64, num_slices=12)
    b = NSBatch([ns.nested_sampler.run_spec(gb.random.PRNGKey(0), ns.normalise_term_cond(None))])
    U = np.random.default_rng(0).uniform(0.05, 0.95, size=(100, 12))
    U[:4, 0] = [1e-12, 1 - 1e-12, 3e-9, 1 - 3e-9]   # tails beyond fp32 resolution of u
    got = b.forward(0, torch.tensor(U, dtype=torch.float64)).cpu().numpy()
    om = oracle_mod.lingauss_model(Phi, y, 0.5, 1.0)
    ref = oracle_mod.forward(om, U)
    np.testing.assert_allclose(got, ref, rtol=1e-4, atol=5e-2)


@pytest.mark.parametrize("fused", [False, True])
def test_lingauss_shell_chain_parity(gpu_lib, oracle_mod, fused):
    """One shell from the initial live set (same keys as the reference's _collect_shell), chain by
    chain against the FP64 oracle, through the two-launch lock step and through the fused shell.
    Its residual sums come from 3xTF32 tensor-core products whose accumulation order is the
    hardware's, so no model reproduces them bit for bit; instead the oracle reports for every
    chain how close its likelihoods came to the contour, and every chain that never came within
    the device's rounding band (1e-3 + 1e-5 |L*|: fp32 directions, pair arithmetic and fp32
    residual tiles) makes the same decisions: the same evaluation count and the same point."""
    import jaxns_gb300 as gb
    from jaxns_gb300 import _ffi
    from jaxns_gb300.engine import NSBatch
    import ctypes
    Phi, y = blr(500, 6, seed=4)
    model = blr_model(gb, Phi, y)
    n, S = 100, 30
    ns = gb.NestedSampler(model, num_live_points=n, num_slices=S)
    spec = ns.nested_sampler.run_spec(gb.random.PRNGKey(9), ns.normalise_term_cond(None))
    b = NSBatch([spec], lg_fused=fused)
    assert b.lg_fused == fused
    b.init()
    live = b.live_view(0)
    K0 = np.array(b.state()[0]["key"], np.uint32)
    sample_key = gb.random.split(gb.random.split(K0)[0])[1]
    s = n // 2
    Lstar = float(live["log_L"][s - 1].item())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if fused:
        _ffi.call("gbns_lg_shell_fused", ctypes.byref(b._b), ctypes.byref(b._lgb), stream)
    else:
        _ffi.call("gbns_lg_shell_begin", ctypes.byref(b._b), ctypes.byref(b._lgb), stream)
        for _ in range(400):
            _ffi.call("gbns_lg_steps", ctypes.byref(b._b), ctypes.byref(b._lgb), 16, stream)
            if int(b.lg_t["chains_left"][0].item()) == 0:
                break
    torch.cuda.synchronize()
    assert int(b.state()[0]["status"]) == 0
    om = oracle_mod.lingauss_model(Phi, y, 0.5, 1.0)
    U_o, L_o, E_o, M_o = oracle_mod.slice_shell_margin(om, sample_key, Lstar, live["U"].cpu().double().numpy(),
                                                       live["log_L"].cpu().double().numpy(), s, S)
    E_g = b.new_E[:s].cpu().numpy()
    U_g = b.new_U_view(0).cpu().numpy()
    same = (E_g == E_o) & np.all(np.abs(U_g - U_o) < 2e-4, axis=1)
    band = 1e-3 + 1e-5 * abs(Lstar)
    clear = M_o > band
    bad = np.nonzero(clear & ~same)[0]
    assert len(bad) == 0, (f"chains {bad[:5]} differ although their FP64 likelihoods stayed farther than {band:.2e} "
                           f"from the contour (margins {M_o[bad[:5]]})")
    print(f"linear-Gaussian shell ({'fused' if fused else 'lock step'}): {np.count_nonzero(same)} of {s} chains "
          f"equal to the FP64 oracle; {np.count_nonzero(~clear)} came within {band:.1e} of a tie")


def test_lingauss_evidence_small(gpu_lib):
    import jaxns_gb300 as gb
    from jaxns_gb300.adjoint import blr_log_evidence
    Phi, y = blr(1024, 8, seed=5)
    model = blr_model(gb, Phi, y)
    ns = gb.NestedSampler(model, num_live_points=200, num_slices=40)
    reason, state = ns(gb.random.PRNGKey(1), gb.TerminationCondition(dlogZ=1e-4))
    res = ns.to_results(reason, state)
    truth, _ = blr_log_evidence(Phi, y, 0.0, np.log(0.5))
    assert abs(res.log_Z_mean - truth) < 4 * res.log_Z_uncert + 0.05, (res.log_Z_mean, res.log_Z_uncert, truth)


def test_adjoint_against_oracle_and_fd(gpu_lib, oracle_mod):
    """On the GPU run's own dead set: log Z(theta) and its gradient against the FP64 oracle of
    the reweighted estimator and against central differences of that FP64 estimator; the
    device's log Z at displaced hyperparameters against the oracle's; the autograd.Function
    returns the same gradient."""
    import jaxns_gb300 as gb
    from jaxns_gb300.adjoint import DeadSet, EvidenceFn, evidence_and_grad
    Phi, y = blr(1024, 8, seed=6)
    model = blr_model(gb, Phi, y)
    ns = gb.NestedSampler(model, num_live_points=200, num_slices=40)
    reason, state = ns(gb.random.PRNGKey(2), gb.TerminationCondition(dlogZ=1e-4))
    res = ns.to_results(reason, state)
    ds = DeadSet.from_results(res, Phi, y)
    lt, ls = 0.05, np.log(0.55)
    out = evidence_and_grad(ds, lt, ls).cpu().numpy()
    lz_o, g_o = oracle_mod.blr_reweighted(Phi, y, ds.U.cpu().double().numpy(), ds.log_w.cpu().numpy(), lt, ls)
    assert abs(out[0] - lz_o) < 2e-4 * max(1.0, abs(lz_o))
    np.testing.assert_allclose(out[1:], g_o, rtol=2e-3, atol=2e-2)
    # the reweighted estimator is strongly curved in log tau (every dead point's w scales with
    # tau, and log L moves by ~|Phi w|^2 / sigma^2), so a central difference with h = 1e-3 is off
    # by its third-derivative term; in FP64 a step of 1e-5 leaves only rounding: the adjoint is
    # the derivative of the estimator to 2e-3
    U64, lw = ds.U.cpu().double().numpy(), ds.log_w.cpu().numpy()
    f = lambda a, b: oracle_mod.blr_reweighted(Phi, y, U64, lw, a, b)[0]
    fd_of = lambda fn, h: [(fn(lt + h, ls) - fn(lt - h, ls)) / (2 * h), (fn(lt, ls + h) - fn(lt, ls - h)) / (2 * h)]
    np.testing.assert_allclose(out[1:], fd_of(f, 1e-5), rtol=2e-3, atol=2e-2)
    # the device's log Z at the displaced hyperparameters: its central differences (h = 1e-3,
    # the bench's step) equal the FP64 estimator's, truncation term included
    fdev = lambda a, b: evidence_and_grad(ds, a, b)[0].item()
    np.testing.assert_allclose(fd_of(fdev, 1e-3), fd_of(f, 1e-3), rtol=2e-3, atol=2e-2)
    theta = torch.tensor([lt, ls], dtype=torch.float64, requires_grad=True)
    lz = EvidenceFn.apply(theta, ds)
    lz.backward()
    np.testing.assert_allclose(theta.grad.numpy(), out[1:], rtol=1e-12)


def _gradient_standard_error(ds, log_tau, log_sigma):
    """Standard error of the reweighted gradient estimate sum_i p_i g_i of one run: the
    weighted spread of the per-point gradients g_i = d log L(U_i) / d theta over the Kish
    effective sample size of p (FP64 on the device; test-side only)."""
    M, P = ds.U.shape
    N = ds.Phi.shape[0]
    tau, s2 = np.exp(log_tau), np.exp(2 * log_sigma)
    Phi, y = ds.Phi.double(), ds.y.double()
    ss, rp = [], []
    for i0 in range(0, M, 8192):                    # [8192, N] FP64 blocks
        w = tau * np.sqrt(2.0) * torch.erfinv(2.0 * ds.U[i0:i0 + 8192].double() - 1.0)
        Pw = w @ Phi.T
        r = y[None, :] - Pw
        ss.append((r * r).sum(1))
        rp.append((r * Pw).sum(1))
    ss, rp = torch.cat(ss), torch.cat(rp)
    g = torch.stack([rp / s2, ss / s2 - N], 1)
    a = -0.5 * ss / s2 + ds.log_w
    p = torch.softmax(a, 0)
    mean = (p[:, None] * g).sum(0)
    var = (p[:, None] * (g - mean) ** 2).sum(0)
    ess = 1.0 / (p * p).sum()
    return (torch.sqrt(var / ess)).cpu().numpy(), float(ess)


def test_config4_blr_evidence_and_gradient(gpu_lib):
    """Config 4: Phi in R^{4096x32} ~ N(0,1), w_true ~ N(0, I), y = Phi w + eps (sigma = 0.5),
    prior w ~ N(0, tau^2 I), (log tau, log sigma) = (0, log 0.5), 1024 live points, default
    termination (dlogZ < log(1 + 1e-3)): log Z against the analytic evidence; the
    reweighted-evidence gradient against the analytic gradient within the run's own Monte
    Carlo error.  The per-point d log L / d log tau has a posterior spread of ~|Phi w| / sigma
    (~700 here) around a mean of ~-5, so one run's tau gradient carries an error of order 10;
    the sigma gradient is far less noisy."""
    import jaxns_gb300 as gb
    from jaxns_gb300.adjoint import DeadSet, blr_log_evidence, evidence_and_grad
    Phi, y = blr(4096, 32, seed=2024)
    model = blr_model(gb, Phi, y)
    # H ~ 32 log(prior / posterior width) ~ 150 nats needs ~1.7e5 samples at n = 1024: above
    # the default max_samples = 100 c, so the store is sized explicitly
    ns = gb.NestedSampler(model, num_live_points=1024, max_samples=600000)
    reason, state = ns(gb.random.PRNGKey(0))
    res = ns.to_results(reason, state)
    assert reason & 4, reason  # terminated by dlogZ
    lz_true, g_true = blr_log_evidence(Phi, y, 0.0, np.log(0.5))
    assert abs(res.log_Z_mean - lz_true) < 4 * res.log_Z_uncert + 0.05, (res.log_Z_mean, res.log_Z_uncert, lz_true)
    ds = DeadSet.from_results(res, Phi, y)
    out = evidence_and_grad(ds, 0.0, np.log(0.5)).cpu().numpy()
    se, ess = _gradient_standard_error(ds, 0.0, np.log(0.5))
    rel = np.abs(out[1:] - g_true) / np.abs(g_true)
    print("config4 log Z", res.log_Z_mean, "+-", res.log_Z_uncert, "truth", lz_true, "grad", out[1:], "truth",
          g_true, "rel", rel, "standard error", se, "ESS", ess)
    assert np.all(np.abs(out[1:] - g_true) < 5 * se + 1e-3 * np.abs(g_true)), (out[1:], g_true, se)


def _adjoint_scratch(entry, U, log_w, Phi, y, log_tau, log_sigma):
    """Call one adjoint entry point and return (out, per-point sum r^2, per-point sum r y)."""
    import ctypes
    from jaxns_gb300 import _ffi
    dev = "cuda"
    t = lambda a, dt: torch.tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    Ud, lw, Pd, yd = t(U, torch.float64), t(log_w, torch.float64), t(Phi, torch.float32), t(y, torch.float32)
    M, P = U.shape
    N = Phi.shape[0]
    out = torch.zeros(3, dtype=torch.float64, device=dev)
    ss = torch.zeros(M, dtype=torch.float64, device=dev)
    ry = torch.zeros(M, dtype=torch.float64, device=dev)
    p = lambda a: ctypes.c_void_p(a.data_ptr())
    args = [p(Ud), p(lw), ctypes.c_longlong(M), ctypes.c_int(P), p(Pd), p(yd), ctypes.c_int(N),
            ctypes.c_double(log_tau), ctypes.c_double(log_sigma), p(out), p(ss), p(ry)]
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    if entry == "tc":
        ld = 32 if P <= 32 else 64
        ws = torch.empty(2 * M * ld, dtype=torch.float32, device=dev)
        ps = torch.empty(2 * N * ld, dtype=torch.float32, device=dev)
        status = torch.zeros(1, dtype=torch.int32, device=dev)
        _ffi.call("gbns_evidence_adjoint_tc", *args, p(ws), p(ps), p(status), stream)
        assert int(status.item()) == 0
    else:
        _ffi.call("gbns_evidence_adjoint", *args, stream)
    torch.cuda.synchronize()
    return out.cpu().numpy(), ss.cpu().numpy(), ry.cpu().numpy()


@pytest.mark.parametrize("P,N,M", [(8, 300, 100), (32, 4096, 1000), (48, 1000, 777), (64, 700, 3000),
                                   (5, 257, 129), (33, 256, 128)])
def test_tc_residuals_against_fp64(gpu_lib, P, N, M):
    """The 3xTF32 tcgen05 contraction: per-point sum (y - Phi w)^2 and sum (y - Phi w) y
    against FP64 numpy on the same fp32 inputs (w = tau ndtri(u) evaluated in FP64), on
    ragged point / row tiles and one or two K blocks; the CUDA-core path alongside."""
    from scipy.special import ndtri
    rng = np.random.default_rng(P * 100003 + N * 7 + M)
    Phi = rng.standard_normal((N, P)).astype(np.float32)
    y = (Phi.astype(np.float64) @ rng.standard_normal(P) + 0.5 * rng.standard_normal(N)).astype(np.float32)
    U = rng.uniform(0.02, 0.98, (M, P))
    U[0, 0], U[-1, -1] = 2e-10, 1 - 2e-10    # FP64 tails
    log_w = rng.standard_normal(M)
    lt = 0.2
    w = np.exp(lt) * ndtri(U)
    r = y.astype(np.float64)[None, :] - w @ Phi.astype(np.float64).T
    ss_ref = (r * r).sum(1)
    ry_ref = r @ y.astype(np.float64)
    for entry in ("tc", "cuda_core"):
        _, ss, ry = _adjoint_scratch(entry, U, log_w, Phi, y, lt, np.log(0.5))
        err = np.abs(ss - ss_ref) / ss_ref
        assert err.max() < 2e-5, (entry, err.max())
        assert np.max(np.abs(ry - ry_ref) / (np.abs(ry_ref) + np.sqrt(ss_ref * (y.astype(np.float64) ** 2).sum()))) < 2e-5


def test_tc_sampler_shell_matches_cuda_core(gpu_lib):
    """One lock-step shell of a batch of three uneven linear-Gaussian runs (P = 8, 40, 64;
    N = 300, 700, 257; several 128-chain and 256-row tiles, one and two K blocks) with the
    tensor-core residual and with the CUDA-core residual: chain by chain the same."""
    import ctypes
    import jaxns_gb300 as gb
    from jaxns_gb300 import _ffi
    from jaxns_gb300.engine import NSBatch
    specs = []
    for i, (P, N, n) in enumerate([(8, 300, 300), (40, 700, 400), (64, 257, 260)]):
        Phi, y = blr(N, P, seed=10 + i)
        ns = gb.NestedSampler(blr_model(gb, Phi, y), num_live_points=n, num_slices=2 * P)
        specs.append(ns.nested_sampler.run_spec(gb.random.PRNGKey(20 + i), ns.normalise_term_cond(None)))
    outs = []
    for tc in (True, False):
        b = NSBatch(specs, lg_tensor_cores=tc)
        b.init()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        _ffi.call("gbns_lg_shell_begin", ctypes.byref(b._b), ctypes.byref(b._lgb), stream)
        for _ in range(1000):
            _ffi.call("gbns_lg_steps", ctypes.byref(b._b), ctypes.byref(b._lgb), 16, stream)
            if int(b.lg_t["chains_left"].sum().item()) == 0:
                break
        torch.cuda.synchronize()
        assert int(b.lg_t["chains_left"].sum().item()) == 0
        st = b.state()
        assert np.all(st["status"] == 0), st["status"]
        outs.append((b.new_U.cpu().numpy().copy(), b.new_E.cpu().numpy().copy(), b.new_L.cpu().numpy().copy()))
    (U1, E1, L1), (U2, E2, L2) = outs
    nc = sum(s.shell_size for s in specs)
    same_E = E1[:nc] == E2[:nc]
    assert same_E.mean() >= 0.95, same_E.mean()
    np.testing.assert_allclose(L1[:nc][same_E], L2[:nc][same_E], rtol=1e-4, atol=2e-2)


def test_fused_shell_matches_lock_step(gpu_lib):
    """One shell of a batch of three uneven linear-Gaussian runs (P = 8, 40, 64; N = 300, 700,
    257; two K blocks for P > 32) through the fused cluster kernel (Phi slices resident in
    shared memory, partial sums exchanged in distributed shared memory) and through the
    two-launch lock step: the same chains chain by chain.  The two paths add the residual
    partial sums in different orders, so a chain may part ways only where a likelihood sits
    within rounding of the contour (at most one chain in 50 here); every chain finishes and no
    status bit is set."""
    import ctypes
    import jaxns_gb300 as gb
    from jaxns_gb300 import _ffi
    from jaxns_gb300.engine import NSBatch
    specs = []
    for i, (P, N, n) in enumerate([(8, 300, 300), (40, 700, 400), (64, 257, 260)]):
        Phi, y = blr(N, P, seed=10 + i)
        ns = gb.NestedSampler(blr_model(gb, Phi, y), num_live_points=n, num_slices=2 * P)
        specs.append(ns.nested_sampler.run_spec(gb.random.PRNGKey(20 + i), ns.normalise_term_cond(None)))
    stream = lambda: ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    fused = NSBatch(specs, lg_fused=True)
    assert fused.lg_fused and fused.fused_plan["cluster_size"] in (8, 16)
    fused.init()
    _ffi.call("gbns_lg_shell_fused", ctypes.byref(fused._b), ctypes.byref(fused._lgb), stream())
    ref = NSBatch(specs, lg_fused=False)
    ref.init()
    _ffi.call("gbns_lg_shell_begin", ctypes.byref(ref._b), ctypes.byref(ref._lgb), stream())
    for _ in range(1000):
        _ffi.call("gbns_lg_steps", ctypes.byref(ref._b), ctypes.byref(ref._lgb), 16, stream())
        if int(ref.lg_t["chains_left"].sum().item()) == 0:
            break
    torch.cuda.synchronize()
    assert np.all(fused.state()["status"] == 0), fused.state()["status"]
    assert np.all(ref.state()["status"] == 0)
    nc = sum(s.shell_size for s in specs)
    E1, E2 = fused.new_E[:nc].cpu().numpy(), ref.new_E[:nc].cpu().numpy()
    L1, L2 = fused.new_L[:nc].cpu().numpy(), ref.new_L[:nc].cpu().numpy()
    assert np.all(E1 > 0)
    same = E1 == E2
    assert same.mean() >= 0.98, same.mean()
    np.testing.assert_allclose(L1[same], L2[same], rtol=1e-4, atol=2e-2)
    for r in range(3):
        U1, U2 = fused.new_U_view(r).cpu().numpy(), ref.new_U_view(r).cpu().numpy()
        o = int(fused.offsets["shell"][r])
        ok = same[o:o + specs[r].shell_size]
        np.testing.assert_allclose(U1[ok], U2[ok], rtol=0, atol=1e-5)


@pytest.mark.parametrize("guided,climb,S", [(True, False, 3), (False, True, 3), (True, True, 2)])
def test_lingauss_gradient_options_chain_parity(gpu_lib, oracle_mod, guided, climb, S):
    """UniDimSliceSampler's gradient options on the linear-Gaussian lock step: gradient_guided
    (Householder reflection of the direction about the U-space gradient at each accepted point,
    uni_slice_sampler.py:255-272) and gradient_slice (each slice along the normalised gradient
    at its seed, t >= 0, :202-214), one evaluation per gradient.  The device gradient is
    Phi^T (y - Phi w) / sigma^2 times dw/du in fp32; each direction then carries fp32-vs-FP64
    differences into the next slice, so the comparison with the FP64 oracle covers a few slices:
    every chain that stayed clear of the contour by ten times the lock step's rounding band
    matches, and at least 90 % of all chains do."""
    import ctypes
    import jaxns_gb300 as gb
    from jaxns_gb300 import _ffi
    from jaxns_gb300.engine import NSBatch
    Phi, y = blr(500, 6, seed=4)
    model = blr_model(gb, Phi, y)
    n = 100
    ns = gb.NestedSampler(model, num_live_points=n, num_slices=S)
    spec = ns.nested_sampler.run_spec(gb.random.PRNGKey(9), ns.normalise_term_cond(None))
    spec.gradient_guided, spec.gradient_slice = guided, climb
    b = NSBatch([spec])
    assert not b.lg_fused
    b.init()
    live = b.live_view(0)
    K0 = np.array(b.state()[0]["key"], np.uint32)
    sample_key = gb.random.split(gb.random.split(K0)[0])[1]
    s = n // 2
    Lstar = float(live["log_L"][s - 1].item())
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _ffi.call("gbns_lg_shell_begin", ctypes.byref(b._b), ctypes.byref(b._lgb), stream)
    for _ in range(400):
        _ffi.call("gbns_lg_steps", ctypes.byref(b._b), ctypes.byref(b._lgb), 16, stream)
        if int(b.lg_t["chains_left"][0].item()) == 0:
            break
    torch.cuda.synchronize()
    assert int(b.state()[0]["status"]) == 0
    E_g = b.new_E[:s].cpu().numpy()
    assert np.all(E_g >= S * (1 + int(guided) + int(climb)))  # a proposal and each gradient per slice
    om = oracle_mod.lingauss_model(Phi, y, 0.5, 1.0)
    U_o, L_o, E_o, M_o = oracle_mod.slice_shell_margin(om, sample_key, Lstar, live["U"].cpu().double().numpy(),
                                                       live["log_L"].cpu().double().numpy(), s, S,
                                                       gradient_guided=guided, gradient_slice=climb)
    U_g = b.new_U_view(0).cpu().numpy()
    same = (E_g == E_o) & np.all(np.abs(U_g - U_o) < 2e-4, axis=1)
    band = 10 * (1e-3 + 1e-5 * abs(Lstar))
    bad = np.nonzero((M_o > band) & ~same)[0]
    assert len(bad) == 0, (bad[:5], M_o[bad[:5]], E_g[bad[:5]], E_o[bad[:5]])
    assert same.mean() >= 0.9, same.mean()


def test_lingauss_gradient_guided_evidence(gpu_lib):
    """NestedSampler(gradient_guided=True) on a Bayesian linear regression end to end (lock step
    with the gradient launch): log Z within 4 sigma of the analytic value."""
    import jaxns_gb300 as gb
    from jaxns_gb300.adjoint import blr_log_evidence
    Phi, y = blr(1024, 8, seed=5)
    model = blr_model(gb, Phi, y)
    ns = gb.NestedSampler(model, num_live_points=200, num_slices=40, gradient_guided=True)
    reason, state = ns(gb.random.PRNGKey(1), gb.TerminationCondition(dlogZ=1e-4))
    res = ns.to_results(reason, state)
    truth, _ = blr_log_evidence(Phi, y, 0.0, np.log(0.5))
    assert abs(res.log_Z_mean - truth) < 4 * res.log_Z_uncert + 0.05, (res.log_Z_mean, res.log_Z_uncert, truth)


def test_lingauss_gradient_options_refuse_fused_shell(gpu_lib):
    """The fused shell does not take the slice sampler's gradient options: the engine refuses
    lg_fused=True with them and otherwise picks the lock step, and the fused C entry point
    refuses a batch that has them set."""
    import ctypes
    import jaxns_gb300 as gb
    from jaxns_gb300 import _ffi
    from jaxns_gb300.engine import NSBatch
    Phi, y = blr(500, 6, seed=4)
    ns = gb.NestedSampler(blr_model(gb, Phi, y), num_live_points=100, num_slices=6)
    spec = ns.nested_sampler.run_spec(gb.random.PRNGKey(9), ns.normalise_term_cond(None))
    fused = NSBatch([spec], lg_fused=True)
    assert fused.lg_fused
    spec.gradient_guided = True
    with pytest.raises(ValueError, match="lock step"):
        NSBatch([spec], lg_fused=True)
    assert not NSBatch([spec]).lg_fused
    fused._b.gradient_guided = 1
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    with pytest.raises(_ffi.GBNSError, match="gradient"):
        _ffi.call("gbns_lg_shell_fused", ctypes.byref(fused._b), ctypes.byref(fused._lgb), stream)
