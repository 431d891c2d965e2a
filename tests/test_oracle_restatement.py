"""A second, independent restatement of the slice sampler's chain, the FP64 evidence
recurrence and the results pass (plain Python, written from the reference's source, small cases
only) against the C oracle on the same inputs.

The C oracle is the checker for every GPU parity test, and jax cannot run here to pin it, so
this test restates ``UniDimSliceSampler._get_sample`` once more, directly from
samplers/bases.py:63-75, samplers/uni_slice_sampler.py:23-441 and internals/random.py:34-84,
and requires bit-identical chains: seed index, every shrink step, the final point, its log L,
the evaluation count and the phantoms.  Shared with the oracle are only the pinned primitives
(threefry split and 64-bit words, checked against the Random123 known answers; the f64
normal, checked against scipy's erfinv) and the model's log-likelihood, which is the model,
not the sampler.

Reduction orders, stated because jnp leaves them to XLA: the direction norm is a sequential sum
of squares, and ``jnp.linspace(0.5, 1, S)[j]`` is ``0.5 (1 - j/(S-1)) + 1 (j/(S-1))`` with
the last element exactly 1.
"""
import math
import struct

import numpy as np
import pytest


def _uniform(o, key):
    """jax.random.uniform(key, (), float64): the top 52 of 64 random bits as the mantissa of a
    float in [1, 2), minus 1."""
    b = int(o.random_bits64(key, 1)[0])
    f = struct.unpack("<d", struct.pack("<Q", (b >> 12) | 0x3FF0000000000000))[0] - 1.0
    return max(0.0, f * (1.0 - 0.0) + 0.0)


def _direction(o, key, D):
    """_sample_direction (uni_slice_sampler.py:23-38)."""
    if D == 1:
        return np.ones(1)
    d = np.asarray(o.normal(key, D), np.float64)
    s = 0.0
    for x in d:
        s += x * x
    return d / math.sqrt(s)


def _bounds(U0, d):
    """_slice_bounds (uni_slice_sampler.py:41-64)."""
    t1 = (1.0 - U0) / d
    t0 = -U0 / d
    right = min(np.min(np.where(t0 >= 0, t0, np.inf)), np.min(np.where(t1 >= 0, t1, np.inf)))
    left = max(np.max(np.where(t0 <= 0, t0, -np.inf)), np.max(np.where(t1 <= 0, t1, -np.inf)))
    return float(left), float(right)


def _alpha(j, S):
    if S == 1:
        return 0.5
    if j == S - 1:
        return 1.0
    step = j / (S - 1)
    return 0.5 * (1.0 - step) + 1.0 * step


def _new_proposal(o, model, key, U0, logL0, d, midpoint, alpha, Lstar, trace):
    """_new_proposal (uni_slice_sampler.py:114-273), perfect=True, no gradient options."""
    run_key, _n_key, t_key, after_key = o.split(key, 4)
    left, right = _bounds(U0, d)
    t = left + _uniform(o, t_key) * (right - left)
    U = U0 + t * d
    logL = float(o.forward(model, U)[0])
    ne = 1
    k = run_key
    trace.append((left, right, t))
    while not ((logL > Lstar) or (logL0 == Lstar and logL == Lstar)):
        k, t_key, _shrink_key = o.split(k, 3)
        if t < 0:
            left = t
        if t > 0:
            right = t
        if midpoint:
            if t < 0:
                left = alpha * left
            if t > 0:
                right = alpha * right
        t = left + _uniform(o, t_key) * (right - left)
        U = U0 + t * d
        logL = float(o.forward(model, U)[0])
        ne += 1
        trace.append((left, right, t))
    return U, _direction(o, after_key, len(U0)), logL, ne


def _seed_index(o, seed_key, live_logL, Lstar):
    """get_seed_point -> sample_uniformly_masked -> resample_indicies(replace=True, S=1)
    (internals/random.py:34-84); jax clamps an out-of-range gather index to the last row."""
    log_w = np.where(live_logL > Lstar, 0.0, -np.inf)
    cum = np.empty(len(log_w))
    acc = -np.inf
    for i, w in enumerate(log_w):
        acc = np.logaddexp(acc, w)
        cum[i] = acc
    log_r = cum[-1] + math.log(1.0 - _uniform(o, seed_key))
    return min(int(np.searchsorted(cum, log_r, side="left")), len(cum) - 1)


def restated_get_sample(o, model, key, Lstar, live_U, live_logL, S, num_phantom, midpoint):
    """BaseAbstractMarkovSampler._get_sample (bases.py:63-75) + get_sample_from_seed
    (uni_slice_sampler.py:360-441)."""
    sample_key, seed_key = o.split(key, 2)
    idx = _seed_index(o, seed_key, live_logL, Lstar)
    U, logL = live_U[idx].copy(), float(live_logL[idx])
    direction_key, slices_key = o.split(sample_key, 2)
    d = _direction(o, direction_key, live_U.shape[1])
    keys = o.split(slices_key, S)
    total, hist, trace = 0, [], []
    for j in range(S):
        U, d, logL, ne = _new_proposal(o, model, keys[j], U, logL, d, midpoint, _alpha(j, S), Lstar, trace)
        total += ne
        hist.append((U, logL))
    phantoms = hist[-(num_phantom + 1):-1] if num_phantom else []
    return idx, U, logL, total, phantoms, trace


def _live_set(o, model, n, seed):
    g = np.random.default_rng(seed)
    U = g.random((n, model.D))
    L = o.forward(model, U)
    order = np.argsort(L, kind="stable")
    return U[order], L[order]


@pytest.mark.parametrize("family,D,S,k,midpoint", [("mvn", 2, 4, 0, True), ("mvn", 5, 10, 2, True),
                                                   ("mvn", 8, 6, 0, False), ("shells", 3, 9, 3, True),
                                                   ("shells", 1, 5, 1, True)])
def test_restated_chain_is_bit_identical(oracle_mod, family, D, S, k, midpoint):
    o = oracle_mod
    g = np.random.default_rng(D * 100 + S)
    if family == "mvn":
        A = g.standard_normal((D, D))
        model = o.mvn_model(np.full(D, -10.0), np.full(D, 10.0), g.standard_normal(D), A @ A.T / D + 0.1 * np.eye(D))
    else:
        c = np.zeros(D); c[0] = 3.5
        model = o.shells_model(-6.0, 6.0, c, -c, 2.0, 0.5)
    live_U, live_L = _live_set(o, model, 40, D)
    for trial in range(12):
        key = o.split(o.PRNGKey(1000 + trial), 2)[1]
        s = int(g.integers(1, 30))
        Lstar = float(live_L[s - 1])
        idx, U, logL, ne, ph, trace = restated_get_sample(o, model, key, Lstar, live_U, live_L, S, k, midpoint)
        U_o, L_o, ne_o, pU_o, pL_o = o.slice_get_sample(model, key, Lstar, live_U, live_L, S, num_phantom=k,
                                                        midpoint_shrink=midpoint)
        assert ne == ne_o and ne == len(trace), (trial, ne, ne_o)
        np.testing.assert_array_equal(U, U_o)
        assert logL == L_o and logL > Lstar
        assert len(ph) == len(pL_o)
        for (pu, pl), qu, ql in zip(ph, pU_o, pL_o):
            np.testing.assert_array_equal(pu, qu)
            assert pl == ql


def test_restated_uniform_and_seed_index_match_the_oracle(oracle_mod):
    o = oracle_mod
    for seed in range(50):
        key = o.PRNGKey(seed)
        assert _uniform(o, key) == float(o.uniform(key, 1)[0])
    g = np.random.default_rng(3)
    import ctypes
    f = o.lib().orc_seed_index_export
    f.restype = ctypes.c_long
    for trial in range(100):
        n = int(g.integers(2, 300))
        L = np.sort(g.standard_normal(n))
        Lstar = float(L[int(g.integers(0, n - 1))])
        key = o.split(o.PRNGKey(trial), 2)[1]
        want = f(ctypes.c_uint32(int(key[0])), ctypes.c_uint32(int(key[1])),
                 L.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_long(n), ctypes.c_double(Lstar))
        assert _seed_index(o, key, L, Lstar) == want


# ------------------------------------------------------------------ evidence statistics

def _jnp_logaddexp(x1, x2):
    """jnp.logaddexp for floats: max + log1p(exp(-|x1 - x2|)), x1 + x2 where the difference is
    NaN (both infinite of one sign)."""
    delta = x1 - x2
    if math.isnan(delta):
        return x1 + x2
    return max(x1, x2) + math.log1p(math.exp(-abs(delta)))


class _LS:
    """The positive ("naked") LogSpace of internals/log_semiring.py: + is logaddexp (:147),
    * adds logs (:181), ** n scales the log (:329)."""

    def __init__(self, v):
        self.v = float(v)

    def __add__(self, o):
        return _LS(_jnp_logaddexp(self.v, o.v))

    def __mul__(self, o):
        return _LS(self.v + o.v)

    def __pow__(self, n):
        return _LS(float(n) * self.v)


def _restated_update(c, n, log_L_next):
    """_update_evidence_calc_op (internals/shrinkage_statistics.py:43-94), its expressions as
    written there, evaluated with Python's own operator associativity."""
    LS = _LS
    next_L = LS(log_L_next)
    L_contour = LS(c["log_L"])
    midL = LS(math.log(0.5)) * (next_L + L_contour)
    X_mean, X2_mean, Z_mean = LS(c["log_X_mean"]), LS(c["log_X2_mean"]), LS(c["log_Z_mean"])
    ZX_mean, Z2_mean, dZ2_mean = LS(c["log_ZX_mean"]), LS(c["log_Z2_mean"]), LS(c["log_dZ2_mean"])
    n = float(n)
    log_n, log_n1, log_n2 = math.log(n), math.log(n + 1.0), math.log(n + 2.0)
    T_mean = LS(-_jnp_logaddexp(0.0, -log_n))
    t_mean = LS(-log_n1)
    T2_mean = LS(-_jnp_logaddexp(0.0, math.log(2.0) - log_n))
    t2_mean = LS(math.log(2.0) - log_n1 - log_n2)
    tT_mean = LS(-_jnp_logaddexp(0.0, -log_n) - log_n2)
    dZ_mean = X_mean * t_mean * midL
    next_X_mean = X_mean * T_mean
    next_X2_mean = X2_mean * T2_mean
    next_Z_mean = Z_mean + dZ_mean
    next_ZX_mean = ZX_mean * T_mean + X2_mean * tT_mean * midL
    next_Z2_mean = Z2_mean + LS(math.log(2.0)) * ZX_mean * t_mean * midL + (X2_mean * t2_mean * midL ** 2)
    next_dZ2_mean = dZ2_mean + (X2_mean * t2_mean * midL ** 2)
    return {"log_L": float(log_L_next), "log_X_mean": next_X_mean.v, "log_X2_mean": next_X2_mean.v,
            "log_Z_mean": next_Z_mean.v, "log_Z2_mean": next_Z2_mean.v, "log_ZX_mean": next_ZX_mean.v,
            "log_dZ_mean": dZ_mean.v, "log_dZ2_mean": next_dZ2_mean.v}


def _restated_init():
    """create_init_evidence_calc (shrinkage_statistics.py:112-128)."""
    inf = float("inf")
    return {"log_L": -inf, "log_X_mean": 0.0, "log_X2_mean": 0.0, "log_Z_mean": -inf, "log_ZX_mean": -inf,
            "log_Z2_mean": -inf, "log_dZ_mean": -inf, "log_dZ2_mean": -inf}


@pytest.mark.parametrize("seed", range(4))
def test_restated_evidence_recurrence_is_bit_identical(oracle_mod, seed):
    """Every per-sample field of compute_evidence_stats equals the restatement exactly, over
    sample sets with a varying live-point count, ties and a -inf first likelihood."""
    g = np.random.default_rng(seed)
    M = 400
    log_L = np.sort(np.round(g.standard_normal(M) * 5, 1))
    if seed % 2:
        log_L[0] = -np.inf
    n = np.maximum(1, np.round(50 + 30 * np.sin(np.arange(M) / 17.0) - np.arange(M) / 20)).astype(np.float64)
    fin, per = oracle_mod.compute_evidence_stats(log_L, n)
    c = _restated_init()
    for i in range(M):
        c = _restated_update(c, n[i], log_L[i])
        for f, v in c.items():
            w = per[f][i]
            assert (v == w) or (math.isnan(v) and math.isnan(w)), (i, f, v, w)
    for f, v in c.items():
        assert v == fin[f] or (math.isnan(v) and math.isnan(fin[f])), f


# ------------------------------------------------------------------ _to_results

def _logsumexp(a):
    m = np.max(a)
    if not np.isfinite(m):
        return float(m)
    return float(m + np.log(np.sum(np.exp(a - m))))


def restated_to_results(o, run):
    """ShardedStaticNestedSampler._to_results with trim=True (sharded_static.py:652-773) over
    the run's stored samples: live-point counts, the evidence recurrence (restated above),
    linear_to_log_stats (internals/stats.py:55-74), the phantom correction sqrt(1 + k), Kish's
    ESS (stats.py:77-86), the normalised dp and H (instable form, stable fallback)."""
    idx, nl = o.count_crossed_edges(run.sender, run.log_L)
    log_L = run.log_L[idx]
    c = _restated_init()
    log_dZ, log_X = [], []
    for i in range(len(log_L)):
        c = _restated_update(c, nl[i], log_L[i])
        log_dZ.append(c["log_dZ_mean"])
        log_X.append(c["log_X_mean"])
    log_dZ, log_X = np.array(log_dZ), np.array(log_X)
    N = len(log_L)
    log_Z_mean = 2.0 * c["log_Z_mean"] - 0.5 * c["log_Z2_mean"]
    log_Z_var = max(c["log_Z2_mean"] - 2.0 * c["log_Z_mean"], np.finfo(np.float64).eps)
    tp = int(np.sum(run.phantom != 0))
    pf = tp / N
    k = pf / (1.0 - pf)
    log_Z_uncert = math.sqrt(log_Z_var) * math.sqrt(1.0 + k)
    ESS = math.exp(2.0 * c["log_Z_mean"] - c["log_dZ2_mean"]) / (1.0 + k)
    norm = _logsumexp(log_dZ)
    log_dp = np.where(np.isneginf(norm), -np.inf, log_dZ - norm)
    p = np.exp(log_dp)
    H_instable = -(np.sum(p * np.where(np.isneginf(log_dp), 0.0, log_L)) - log_Z_mean)
    H_stable = -np.sum(p * np.log(-log_X))
    H = H_instable if np.isfinite(H_instable) else H_stable
    total_evals = int(np.sum(run.nevals[idx]))
    return {"log_Z_mean": log_Z_mean, "log_Z_uncert": log_Z_uncert, "ESS": ESS, "H_mean": H,
            "total_num_samples": N, "total_phantom_samples": tp, "total_num_likelihood_evaluations": total_evals,
            "log_efficiency": math.log(N) - math.log(total_evals), "log_dp_mean": log_dp, "log_X_mean": log_X,
            "num_live_points": nl, "samples_indices": idx}


@pytest.mark.parametrize("case", ["mvn", "shells_k2"])
def test_restated_to_results(oracle_mod, case):
    o = oracle_mod
    if case == "mvn":
        model = o.mvn_model(np.full(3, -10.0), np.full(3, 10.0), np.array([0.2, -0.1, 0.4]),
                            np.array([[1.0, 0.3, 0.0], [0.3, 0.8, 0.2], [0.0, 0.2, 0.5]]))
        run = o.ns_run(model, o.PRNGKey(21), num_live_points=60, num_slices=9, term_cond={"dlogZ": 1e-3})
    else:
        model = o.shells_model(-6.0, 6.0, [3.5, 0.0], [-3.5, 0.0], 2.0, 0.4)
        run = o.ns_run(model, o.PRNGKey(22), num_live_points=50, num_slices=8, num_phantom=2,
                       term_cond={"dlogZ": 1e-3})
    want = restated_to_results(o, run)
    got = run.results
    for f in ("total_num_samples", "total_phantom_samples", "total_num_likelihood_evaluations"):
        assert int(got[f]) == want[f], f
    for f in ("log_Z_mean", "log_Z_uncert", "ESS", "H_mean", "log_efficiency"):
        np.testing.assert_allclose(got[f], want[f], rtol=1e-10, atol=1e-12, err_msg=f)
    np.testing.assert_array_equal(run.samples_indices, want["samples_indices"])
    np.testing.assert_array_equal(run.num_live_points, want["num_live_points"])
    np.testing.assert_array_equal(run.log_X_mean, want["log_X_mean"])
    np.testing.assert_allclose(run.log_dp_mean, want["log_dp_mean"], rtol=1e-12, atol=1e-12)
    if case == "shells_k2":
        assert want["total_phantom_samples"] > 0
