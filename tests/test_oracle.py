"""CPU tests of the FP64 oracle against the reference's own known answers and against
independent implementations (Random123 KAT vectors, scipy, analytic evidences)."""
import numpy as np
import pytest

from tests.conftest import corr_gauss


# Random123 known-answer vectors for threefry2x32_20 (also used by JAX's own threefry test)
KAT = [((0x00000000, 0x00000000), (0x00000000, 0x00000000), (0x6b200159, 0x99ba4efe)),
       ((0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff), (0x1cb996fc, 0xbb002be7)),
       ((0x13198a2e, 0x03707344), (0x243f6a88, 0x85a308d3), (0xc4923a9c, 0x483df7a0))]


@pytest.mark.parametrize("key,ctr,expected", KAT)
def test_threefry_kat(oracle_mod, key, ctr, expected):
    assert tuple(int(x) for x in oracle_mod.threefry2x32(key, ctr)) == expected


@pytest.mark.parametrize("key,ctr,expected", KAT)
def test_host_threefry_kat(key, ctr, expected):
    from jaxns_gb300 import random as grandom
    a, b = grandom.threefry2x32(key, np.uint32([ctr[0]]), np.uint32([ctr[1]]))
    assert (int(a[0]), int(b[0])) == expected


def test_host_split_matches_oracle(oracle_mod):
    from jaxns_gb300 import random as grandom
    for seed in (0, 1, 42, 2**33 + 5):
        k = grandom.PRNGKey(seed)
        np.testing.assert_array_equal(grandom.split(k, 7), oracle_mod.split(k, 7))


def test_prngkey_layout():
    from jaxns_gb300 import random as grandom
    np.testing.assert_array_equal(grandom.PRNGKey(42), [0, 42])
    np.testing.assert_array_equal(grandom.PRNGKey(2**32 + 3), [1, 3])


def test_erfinv_against_scipy(oracle_mod):
    sp = pytest.importorskip("scipy.special")
    u = np.concatenate([np.linspace(-0.999999, 0.999999, 2001), [1e-300, -1e-17, 1 - 2**-53, -1 + 2**-53]])
    ref = sp.erfinv(u)
    got = oracle_mod.erfinv(u)
    np.testing.assert_allclose(got, ref, rtol=4e-15, atol=0)


def test_uniform_and_normal_moments(oracle_mod):
    k = oracle_mod.PRNGKey(3)
    u = oracle_mod.uniform(k, 20000)
    assert 0 <= u.min() and u.max() < 1
    assert abs(u.mean() - 0.5) < 0.01
    z = oracle_mod.normal(k, 20000)
    assert abs(z.mean()) < 0.03 and abs(z.std() - 1) < 0.03


def test_count_crossed_edges_reference_goldens(oracle_mod):
    # internals/tests/test_tree_structure.py:19-30 (test_naive)
    si, nl = oracle_mod.count_crossed_edges([0, 0, 0, 1, 2, 3], [1, 2, 3, 4, 5, 6])
    np.testing.assert_array_equal(si, [0, 1, 2, 3, 4, 5])
    np.testing.assert_array_equal(nl, [3, 3, 3, 3, 2, 1])
    # second tree of test_basic (:33-49): samples 4,5 swapped in log L
    si, nl = oracle_mod.count_crossed_edges([0, 0, 0, 1, 3, 2], [1, 2, 3, 4, 6, 5])
    np.testing.assert_array_equal(si, [0, 1, 2, 3, 5, 4])
    np.testing.assert_array_equal(nl, [3, 3, 3, 3, 2, 1])


def test_count_crossed_edges_num_samples(oracle_mod):
    # test_with_num_samples (:52-70): +inf padding rows get count 0 and the rest equals the trimmed tree
    s1 = [0, 0, 0, 1, 2, 3, 4, 5, 0, 0]
    l1 = [1, 2, 3, 4, 5, 6, 7, 8, np.inf, np.inf]
    si1, nl1 = oracle_mod.count_crossed_edges(s1, l1, num_samples=8)
    si2, nl2 = oracle_mod.count_crossed_edges(s1[:8], l1[:8])
    np.testing.assert_array_equal(si1[:8], si2)
    np.testing.assert_array_equal(nl1[:8], nl2)
    np.testing.assert_array_equal(nl1[8:], 0)


def _naive_counts(sender, log_L):
    # count_intervals_naive (tree_structure.py:136-206): live points = samples whose
    # constraint interval contains each sample's log L
    log_L = np.asarray(log_L, float)
    nodes = np.concatenate([[-np.inf], log_L])
    cons = nodes[np.asarray(sender)]
    order = np.argsort(log_L, kind="stable")
    counts = []
    for i in order:
        counts.append(int(np.sum((cons < log_L[i]) & (log_L >= log_L[i]))))
    return order, np.array(counts)


def test_count_crossed_edges_random_tree(oracle_mod):
    # the seeded random tree of test_random_tree (:73-103), against the naive count
    np.random.seed(42)
    log_L = [0.0]
    parent = []
    for idx in range(10):
        log_L.append(log_L[idx] + np.random.uniform(low=0, high=1 - log_L[idx]) ** 4)
        parent.append(idx)
    for idx in range(10):
        for _ in range(5):
            log_L.append(np.random.uniform(low=log_L[idx], high=1.))
            parent.append(idx)
    si, nl = oracle_mod.count_crossed_edges(parent, log_L[1:])
    order, counts = _naive_counts(parent, log_L[1:])
    np.testing.assert_array_equal(si, order)
    np.testing.assert_array_equal(nl, counts)


def test_stable_argsort_total_order(oracle_mod):
    keys = np.array([3.0, -0.0, np.nan, 0.0, -np.inf, np.inf, 3.0, np.nan, -1.0])
    # jnp.argsort: -0 == +0 (stable), NaN after +inf (stable)
    np.testing.assert_array_equal(oracle_mod.stable_argsort(keys), [4, 8, 1, 3, 0, 6, 5, 2, 7])


def test_evidence_constant_n(oracle_mod):
    # with n fixed, log X_i = i log(n/(n+1)) exactly in expectation (shrinkage_statistics.py:62)
    n = 50
    L = np.linspace(-10, 0, 400)
    fin, per = oracle_mod.compute_evidence_stats(L, np.full(400, n))
    i = np.arange(1, 401)
    np.testing.assert_allclose(per["log_X_mean"], i * np.log(n / (n + 1)), rtol=1e-12)
    # Z mean = sum X_{i-1} / (n+1) * midL
    X = np.exp(np.concatenate([[0], per["log_X_mean"][:-1]]))
    mid = 0.5 * (np.exp(L) + np.exp(np.concatenate([[-np.inf], L[:-1]])))
    np.testing.assert_allclose(fin["log_Z_mean"], np.log(np.sum(X / (n + 1) * mid)), rtol=1e-12)


def test_linear_to_log_stats(oracle_mod):
    # internals/tests/test_stats.py:7-19 restated: log-normal moments
    mu, var = oracle_mod.linear_to_log_stats(np.log(2.0), np.log(5.0))
    assert np.isclose(mu, 2 * np.log(2.0) - 0.5 * np.log(5.0))
    assert np.isclose(var, np.log(5.0) - 2 * np.log(2.0))


def test_seed_index_integer_formula(oracle_mod):
    """The device picks the seed as the k-th satisfying live point, k = ceil(m (1 - U)), with
    exact 64-bit integer arithmetic; check it equals the reference's cumulative-logsumexp +
    searchsorted (internals/random.py:34-84) on many keys."""
    import ctypes
    lib = oracle_mod.lib()
    f = lib.orc_seed_index_export if hasattr(lib, "orc_seed_index_export") else None
    assert f is not None
    f.restype = ctypes.c_long
    rng = np.random.default_rng(0)
    for trial in range(300):
        n = int(rng.integers(2, 700))
        L = np.sort(rng.standard_normal(n))
        s = int(rng.integers(1, n))
        Lstar = L[s - 1]
        key = oracle_mod.split(oracle_mod.PRNGKey(trial), 2)[1]
        idx = f(ctypes.c_uint32(int(key[0])), ctypes.c_uint32(int(key[1])), L.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                ctypes.c_long(n), ctypes.c_double(Lstar))
        m = int(np.sum(L > Lstar))
        b = int(oracle_mod.random_bits64(key, 1)[0])
        M = b >> 12
        if m == 0:
            expect = 0
        else:
            k = -((-m * ((1 << 52) - M)) >> 52)
            expect = (n - m) + k - 1
        assert idx == expect, (trial, n, m, idx, expect)


def test_config1_oracle_log_Z_unbiased(oracle_mod):
    """Config 1 (D=8 correlated Gaussian, U[-10,10]^8, 512 live points, 32 slices,
    dlogZ<1e-4): the ensemble of oracle runs is centred on the analytic -8 log 20."""
    D = 8
    mu, cov = corr_gauss(D, 0)
    m = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    R = 8
    lz, nev, reasons = oracle_mod.ns_run_batch([m] * R, [dict(num_live_points=512, num_slices=32,
                                                                max_samples=51200)] * R,
                                               np.array([oracle_mod.PRNGKey(i) for i in range(R)]),
                                               [{"dlogZ": 1e-4}] * R, 8)
    truth = -D * np.log(20.0)
    assert np.all(reasons == 4)
    assert abs(lz.mean() - truth) < 3 * 0.25 / np.sqrt(R)


def _blr(N=300, P=5, seed=0, sigma=0.5):
    rng = np.random.default_rng(seed)
    Phi = rng.standard_normal((N, P))
    w = rng.standard_normal(P)
    return Phi, Phi @ w + sigma * rng.standard_normal(N)


def test_blr_analytic_evidence_and_gradient():
    """log N(y; 0, s^2 I + t^2 Phi Phi^T) via Woodbury against a dense FP64 evaluation, and
    its gradient against central differences."""
    from jaxns_gb300.adjoint import blr_log_evidence
    Phi, y = _blr()
    lt, ls = 0.1, np.log(0.5)
    lz, g = blr_log_evidence(Phi, y, lt, ls)
    C = np.exp(2 * ls) * np.eye(len(y)) + np.exp(2 * lt) * Phi @ Phi.T
    sign, logdet = np.linalg.slogdet(C)
    dense = -0.5 * (len(y) * np.log(2 * np.pi) + logdet + y @ np.linalg.solve(C, y))
    assert abs(lz - dense) < 1e-8 * abs(dense)
    h = 1e-5
    fd = [(blr_log_evidence(Phi, y, lt + h, ls)[0] - blr_log_evidence(Phi, y, lt - h, ls)[0]) / (2 * h),
          (blr_log_evidence(Phi, y, lt, ls + h)[0] - blr_log_evidence(Phi, y, lt, ls - h)[0]) / (2 * h)]
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-6)


def test_oracle_reweighted_gradient_matches_fd(oracle_mod):
    """The oracle's reweighted evidence gradient (evidence_maximisation.py:151-160) against
    central differences of its own log Z on a fixed point set."""
    Phi, y = _blr(N=200, P=4, seed=1)
    rng = np.random.default_rng(2)
    U = rng.uniform(0.05, 0.95, size=(300, 4))
    log_w = rng.standard_normal(300) - 5.0
    lt, ls = -0.2, np.log(0.7)
    lz, g = oracle_mod.blr_reweighted(Phi, y, U, log_w, lt, ls)
    h = 1e-5
    fd = [(oracle_mod.blr_reweighted(Phi, y, U, log_w, lt + h, ls)[0] -
           oracle_mod.blr_reweighted(Phi, y, U, log_w, lt - h, ls)[0]) / (2 * h),
          (oracle_mod.blr_reweighted(Phi, y, U, log_w, lt, ls + h)[0] -
           oracle_mod.blr_reweighted(Phi, y, U, log_w, lt, ls - h)[0]) / (2 * h)]
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-6)


def test_grad_U_matches_finite_differences(oracle_mod):
    """The oracle's analytic U-space gradients (used by the gradient-guided slice) against
    central differences of its own forward, for MVN, shells and the linear-Gaussian family,
    Uniform and Normal priors."""
    rng = np.random.default_rng(0)
    D = 4
    A = rng.standard_normal((D, D))
    models = [oracle_mod.mvn_model(-3 * np.ones(D), 3 * np.ones(D), rng.standard_normal(D), A @ A.T / D + 0.5 * np.eye(D)),
              oracle_mod.shells_model(-2, 2, 0.4 * np.ones(D), -0.4 * np.ones(D), 0.8, 0.3)]
    Phi = rng.standard_normal((30, D))
    models.append(oracle_mod.lingauss_model(Phi, Phi @ rng.standard_normal(D), 0.7, 1.3))
    for m in models:
        for _ in range(3):
            U = rng.uniform(0.2, 0.8, D)
            g = oracle_mod.grad_U(m, U)
            h = 1e-6
            fd = np.array([(oracle_mod.forward(m, (U + h * e)[None])[0] - oracle_mod.forward(m, (U - h * e)[None])[0])
                           / (2 * h) for e in np.eye(D)])
            np.testing.assert_allclose(g, fd, rtol=1e-5, atol=1e-6 * max(1.0, np.abs(fd).max()))


def test_slice_shell_margin_reports_closest_approach(oracle_mod):
    """The margin-reporting shell runs the same chains as slice_shell, and every margin is the
    smallest |log L - L*| over the chain's accept tests (non-negative, finite)."""
    from tests.conftest import corr_gauss
    D = 4
    mu, cov = corr_gauss(D, 1)
    om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    U = np.random.default_rng(0).uniform(size=(200, D))
    L = oracle_mod.forward(om, U)
    o = np.argsort(L)
    U, L = U[o], L[o]
    U1, L1, E1, M1 = oracle_mod.slice_shell_margin(om, oracle_mod.PRNGKey(3), L[99], U, L, 100, 8)
    U0, L0, E0 = oracle_mod.slice_shell(om, oracle_mod.PRNGKey(3), L[99], U, L, 100, 8)
    np.testing.assert_array_equal(E1, E0)
    np.testing.assert_array_equal(U1, U0)
    assert np.all(np.isfinite(M1)) and np.all(M1 >= 0)
    assert np.all(M1 <= np.abs(L1 - L[99]) + 1e-12)  # the accepted point itself is one of the tests


@pytest.mark.parametrize("guided,climb", [(True, False), (False, True)])
def test_fp32_mode_gradient_options_both_reduction_orders(oracle_mod, guided, climb):
    """The fp32 kernel-arithmetic mode's gradient options, in the thread kernel's sequential sums
    and in the warp kernel's lane-butterfly sums (gradient norm, reflection dot product and
    norm), against the FP64 restatement over a few slices at D = 40: the chains agree to fp32
    rounding, and the two reduction orders differ only where a comparison sits within rounding
    of the contour."""
    from jaxns_gb300.engine import mvn_offset, mvn_params
    D, n, S = 40, 96, 3
    mu, cov = corr_gauss(D, D)
    om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    U = np.random.default_rng(D).uniform(0.3, 0.7, (n, D))
    L = oracle_mod.forward(om, U)
    o = np.argsort(L)
    U, L = U[o], L[o]
    s = n // 2
    params = mvn_params(mu, cov)
    Uo, Lo, Eo = oracle_mod.slice_shell(om, oracle_mod.PRNGKey(5), L[s - 1], U, L, s, S, gradient_guided=guided,
                                        gradient_slice=climb)
    outs = []
    for warp_min_D in (17, 100):  # the warp kernel's order (variant 64), the thread kernel's (variant 0)
        m32 = oracle_mod.model32(0, D, params, np.zeros(D, np.int32), np.full(D, -10.0), np.full(D, 20.0),
                                 warp_min_D=warp_min_D)
        assert m32.variant == (64 if warp_min_D == 17 else 0)
        L32 = oracle_mod.forward32(m32, U.astype(np.float32))
        np.testing.assert_allclose(L32.astype(np.float64) + mvn_offset(cov), L, rtol=1e-4, atol=2e-3)
        U3, L3, E3, _, _ = oracle_mod.slice_shell32(m32, oracle_mod.PRNGKey(5), L32[s - 1], U.astype(np.float32), L32,
                                                    s, S, gradient_guided=guided, gradient_slice=climb)
        assert np.all(E3 >= S * 2)  # a proposal and a gradient per slice
        same = (E3 == Eo) & np.all(np.abs(U3 - Uo) < 2e-4, axis=1)
        assert same.mean() >= 0.9, (warp_min_D, same.mean())
        outs.append((U3, E3))
    (Uw, Ew), (Ut, Et) = outs
    assert np.any(Uw.view(np.uint32) != Ut.view(np.uint32))  # the two orders round differently
    assert np.mean((Ew == Et) & np.all(np.abs(Uw - Ut) < 2e-4, axis=1)) >= 0.9
