"""ctypes front end of the FP64 CPU oracle (``oracle/ns_oracle.c``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py``, as the checker.  The product (``jaxns_gb300``) never
imports this module.

The C file restates jaxns v2.6.9's static nested sampler (see the citations there).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from typing import Optional

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "ns_oracle.c")
# the fp32 kernel-arithmetic mode evaluates the product's elementary functions (pure IEEE
# arithmetic, no device code): a change there rebuilds the oracle
_FMATH = os.path.join(os.path.dirname(_HERE), "jaxns_gb300", "csrc", "gbns_fmath.h")
_BUILD = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_BUILD, "libnsoracle.so")

PRIOR_UNIFORM = 0
PRIOR_NORMAL = 1
LIK_MVN = 0
LIK_SHELLS = 1
LIK_LINGAUSS = 2


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction, IEEE semantics)."""
    os.makedirs(_BUILD, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(_SRC), os.path.getmtime(_FMATH))):
        return _LIB_PATH
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math",
           "-std=c11", "-D_GNU_SOURCE", "-o", tmp, _SRC, "-lm", "-lpthread"]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


class _Model(ctypes.Structure):
    _fields_ = [("D", ctypes.c_int), ("family", ctypes.c_int),
                ("prior_kind", ctypes.POINTER(ctypes.c_int)),
                ("prior_a", ctypes.POINTER(ctypes.c_double)),
                ("prior_b", ctypes.POINTER(ctypes.c_double)),
                ("p", ctypes.POINTER(ctypes.c_double)), ("N", ctypes.c_int),
                ("prior_A", ctypes.POINTER(ctypes.c_double)), ("prior_c", ctypes.POINTER(ctypes.c_double))]


class _SliceCfg(ctypes.Structure):
    _fields_ = [("num_slices", ctypes.c_int), ("num_phantom", ctypes.c_int),
                ("midpoint_shrink", ctypes.c_int), ("gradient_guided", ctypes.c_int),
                ("gradient_slice", ctypes.c_int)]


class _NSCfg(ctypes.Structure):
    _fields_ = [("num_live_points", ctypes.c_int), ("shell_size", ctypes.c_int),
                ("max_samples", ctypes.c_long), ("init_efficiency_threshold", ctypes.c_double),
                ("slice", _SliceCfg), ("uniform_max_evals", ctypes.c_int)]


class _EvCalc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in
                ("log_L", "log_X_mean", "log_X2_mean", "log_Z_mean", "log_ZX_mean",
                 "log_Z2_mean", "log_dZ_mean", "log_dZ2_mean")]


_TC_FIELDS = ("ess", "evidence_uncert", "dlogZ", "max_samples", "max_nlik", "log_L_contour",
              "efficiency_threshold", "rtol", "atol", "peak_XL_frac")
_TC_FLAGS = ("has_ess", "has_evidence_uncert", "has_dlogZ", "has_max_samples", "has_max_nlik",
             "has_log_L_contour", "has_efficiency", "has_rtol", "has_atol", "has_peak_XL")


class _TermCond(ctypes.Structure):
    _fields_ = [x for f, v in zip(_TC_FLAGS, _TC_FIELDS)
                for x in ((f, ctypes.c_int), (v, ctypes.c_double))]


class _TermReg(ctypes.Structure):
    _fields_ = [("num_samples_used", ctypes.c_long), ("ev", _EvCalc), ("ev_rem", _EvCalc),
                ("num_likelihood_evaluations", ctypes.c_long), ("log_L_contour", ctypes.c_double),
                ("efficiency", ctypes.c_double), ("plateau", ctypes.c_int),
                ("no_seed_points", ctypes.c_int), ("relative_spread", ctypes.c_double),
                ("absolute_spread", ctypes.c_double), ("peak_log_XL", ctypes.c_double)]


class _NSState(ctypes.Structure):
    _fields_ = [("sender", ctypes.POINTER(ctypes.c_long)),
                ("log_L", ctypes.POINTER(ctypes.c_double)),
                ("U", ctypes.POINTER(ctypes.c_double)),
                ("nevals", ctypes.POINTER(ctypes.c_long)),
                ("phantom", ctypes.POINTER(ctypes.c_int)),
                ("next_sample_idx", ctypes.c_long), ("num_samples", ctypes.c_long),
                ("key0", ctypes.c_uint32), ("key1", ctypes.c_uint32),
                ("termination_reason", ctypes.c_long), ("reg", _TermReg),
                ("iterations", ctypes.c_long)]


class _Results(ctypes.Structure):
    _fields_ = [("log_Z_mean", ctypes.c_double), ("log_Z_uncert", ctypes.c_double),
                ("ESS", ctypes.c_double), ("H_mean", ctypes.c_double),
                ("total_num_samples", ctypes.c_long), ("total_phantom_samples", ctypes.c_long),
                ("total_num_likelihood_evaluations", ctypes.c_long),
                ("log_efficiency", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        _lib = ctypes.CDLL(path)
        _lib.orc_ns_run.restype = ctypes.c_long
        _lib.orc_erfinv.restype = ctypes.c_double
        for nm in ("orc32_fm_exp", "orc32_fm_log", "orc32_fm_log1p", "orc32_fm_ndtri"):
            getattr(_lib, nm).restype = ctypes.c_float
            getattr(_lib, nm).argtypes = [ctypes.c_float]
        _lib.orc32_fm_ndtri_d.restype = ctypes.c_float
        _lib.orc32_fm_ndtri_d.argtypes = [ctypes.c_double]
        _lib.orc32_fm_normal_from_bits.restype = ctypes.c_float
        _lib.orc32_fm_normal_from_bits.argtypes = [ctypes.c_uint64]
        _lib.orc32_forward.restype = ctypes.c_float
        for nm in ("orc_fm_log64", "orc_fm_ndtri64"):
            getattr(_lib, nm).restype = ctypes.c_double
            getattr(_lib, nm).argtypes = [ctypes.c_double]
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _lp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_long))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def _up(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))


# ----------------------------------------------------------------------------- RNG

def threefry2x32(key, count):
    out = np.zeros(2, np.uint32)
    lib().orc_threefry2x32(ctypes.c_uint32(int(key[0])), ctypes.c_uint32(int(key[1])),
                           ctypes.c_uint32(int(count[0])), ctypes.c_uint32(int(count[1])), _up(out))
    return out


def split(key, n=2):
    """jax.random.split under jax_threefry_partitionable=True."""
    return np.stack([threefry2x32(key, (i >> 32, i & 0xFFFFFFFF)) for i in range(n)])


def random_bits64(key, n):
    out = np.zeros(n, np.uint64)
    for i in range(n):
        x = threefry2x32(key, (i >> 32, i & 0xFFFFFFFF))
        out[i] = (np.uint64(x[0]) << np.uint64(32)) | np.uint64(x[1])
    return out


def uniform(key, n, minval=0.0, maxval=1.0):
    b = random_bits64(key, n)
    fb = (b >> np.uint64(12)) | np.uint64(0x3FF0000000000000)
    f = fb.view(np.float64) - 1.0
    return np.maximum(minval, f * (maxval - minval) + minval)


def erfinv(u):
    f = lib().orc_erfinv
    f.restype = ctypes.c_double
    return np.array([f(ctypes.c_double(float(x))) for x in np.ravel(u)]).reshape(np.shape(u))


def normal(key, n):
    lo = np.nextafter(-1.0, 0.0)
    return np.sqrt(2.0) * erfinv(uniform(key, n, lo, 1.0))


def PRNGKey(seed: int):
    seed = int(seed)
    return np.array([(seed >> 32) & 0xFFFFFFFF, seed & 0xFFFFFFFF], np.uint32)


# --------------------------------------------------------------------------- model

@dataclass
class OracleModel:
    """Flat description of a model the oracle can evaluate (prior per dimension + family)."""
    D: int
    family: int
    prior_kind: np.ndarray
    prior_a: np.ndarray
    prior_b: np.ndarray
    params: np.ndarray
    N: int = 0
    prior_A: Optional[np.ndarray] = None  # X = A q + c after the per-dimension quantiles q
    prior_c: Optional[np.ndarray] = None

    def _c(self):
        self._keep = [np.ascontiguousarray(self.prior_kind, np.int32),
                      np.ascontiguousarray(self.prior_a, np.float64),
                      np.ascontiguousarray(self.prior_b, np.float64),
                      np.ascontiguousarray(self.params, np.float64)]
        k, a, b, p = self._keep
        A = c = None
        if self.prior_A is not None:
            self._keep += [np.ascontiguousarray(self.prior_A, np.float64), np.ascontiguousarray(self.prior_c, np.float64)]
            A, c = _dp(self._keep[4]), _dp(self._keep[5])
        return _Model(self.D, self.family, _ip(k), _dp(a), _dp(b), _dp(p), self.N, A, c)


def mvn_model(low, high, mu, cov):
    D = len(mu)
    L = np.linalg.cholesky(np.asarray(cov, np.float64))
    params = np.concatenate([np.asarray(mu, np.float64), L.ravel()])
    return OracleModel(D, LIK_MVN, np.zeros(D, np.int32), np.asarray(low, np.float64) * np.ones(D),
                       (np.asarray(high, np.float64) - np.asarray(low, np.float64)) * np.ones(D), params)


def mvn_tril_prior_model(prior_loc, prior_L, mu, cov):
    """Correlated-Gaussian likelihood N(mu, cov) under a MultivariateNormalTriL(prior_loc,
    prior_L) prior: X = prior_loc + prior_L ndtri(U)."""
    D = len(mu)
    L = np.linalg.cholesky(np.asarray(cov, np.float64))
    params = np.concatenate([np.asarray(mu, np.float64), L.ravel()])
    return OracleModel(D, LIK_MVN, np.ones(D, np.int32), np.zeros(D), np.ones(D), params,
                       prior_A=np.tril(np.asarray(prior_L, np.float64)), prior_c=np.asarray(prior_loc, np.float64))


def shells_model(low, high, c1, c2, radius, width):
    D = len(c1)
    params = np.concatenate([np.asarray(c1, np.float64), np.asarray(c2, np.float64),
                             [float(radius), float(width)]])
    return OracleModel(D, LIK_SHELLS, np.zeros(D, np.int32), np.full(D, float(low)),
                       np.full(D, float(high) - float(low)), params)


def lingauss_model(Phi, y, sigma, tau):
    N, P = Phi.shape
    params = np.concatenate([np.asarray(Phi, np.float64).ravel(), np.asarray(y, np.float64),
                             [float(sigma)]])
    return OracleModel(P, LIK_LINGAUSS, np.ones(P, np.int32), np.zeros(P),
                       np.full(P, float(tau)), params, N)


def forward(model: OracleModel, U):
    U = np.ascontiguousarray(np.atleast_2d(U), np.float64)
    out = np.zeros(U.shape[0])
    m = model._c()
    lib().orc_forward_batch(ctypes.byref(m), _dp(U), ctypes.c_long(U.shape[0]), _dp(out))
    return out


# -------------------------------------------------------------------- samplers

def grad_U(model, U):
    """jax.grad of Model.forward w.r.t. U (analytic, FP64)."""
    U = np.ascontiguousarray(U, np.float64)
    g = np.zeros(model.D)
    m = model._c()
    lib().orc_grad_U(ctypes.byref(m), _dp(U), _dp(g))
    return g


def slice_get_sample(model, key, L_star, live_U, live_logL, num_slices, num_phantom=0,
                     midpoint_shrink=True, gradient_guided=False, gradient_slice=False):
    D = model.D
    live_U = np.ascontiguousarray(live_U, np.float64)
    live_logL = np.ascontiguousarray(live_logL, np.float64)
    cfg = _SliceCfg(num_slices, num_phantom, int(midpoint_shrink), int(gradient_guided), int(gradient_slice))
    U = np.zeros(D)
    logL = ctypes.c_double()
    ne = ctypes.c_long()
    pU = np.zeros((max(num_phantom, 1), D))
    pL = np.zeros(max(num_phantom, 1))
    m = model._c()
    lib().orc_slice_get_sample(ctypes.byref(m), ctypes.byref(cfg), ctypes.c_uint32(int(key[0])),
                               ctypes.c_uint32(int(key[1])), ctypes.c_double(L_star), _dp(live_U),
                               _dp(live_logL), ctypes.c_long(len(live_logL)), _dp(U), ctypes.byref(logL),
                               ctypes.byref(ne), _dp(pU), _dp(pL))
    return U, logL.value, ne.value, pU[:num_phantom], pL[:num_phantom]


def slice_shell(model, key, L_star, live_U, live_logL, num_chains, num_slices, num_phantom=0,
                midpoint_shrink=True, gradient_guided=False, gradient_slice=False):
    D = model.D
    live_U = np.ascontiguousarray(live_U, np.float64)
    live_logL = np.ascontiguousarray(live_logL, np.float64)
    cfg = _SliceCfg(num_slices, num_phantom, int(midpoint_shrink), int(gradient_guided), int(gradient_slice))
    U = np.zeros((num_chains, D))
    L = np.zeros(num_chains)
    E = np.zeros(num_chains, np.int64)
    m = model._c()
    lib().orc_slice_shell(ctypes.byref(m), ctypes.byref(cfg), ctypes.c_uint32(int(key[0])),
                          ctypes.c_uint32(int(key[1])), ctypes.c_double(L_star), _dp(live_U),
                          _dp(live_logL), ctypes.c_long(len(live_logL)), ctypes.c_long(num_chains),
                          _dp(U), _dp(L), _lp(E))
    return U, L, E


def slice_shell_margin(model, key, L_star, live_U, live_logL, num_chains, num_slices, num_phantom=0,
                       midpoint_shrink=True, gradient_guided=False, gradient_slice=False):
    """slice_shell with, per chain, the smallest |log L - L*| over its accept tests (FP64)."""
    D = model.D
    live_U = np.ascontiguousarray(live_U, np.float64)
    live_logL = np.ascontiguousarray(live_logL, np.float64)
    cfg = _SliceCfg(num_slices, num_phantom, int(midpoint_shrink), int(gradient_guided), int(gradient_slice))
    U = np.zeros((num_chains, D))
    L = np.zeros(num_chains)
    E = np.zeros(num_chains, np.int64)
    M = np.zeros(num_chains)
    m = model._c()
    lib().orc_slice_shell_margin(ctypes.byref(m), ctypes.byref(cfg), ctypes.c_uint32(int(key[0])),
                                 ctypes.c_uint32(int(key[1])), ctypes.c_double(L_star), _dp(live_U), _dp(live_logL),
                                 ctypes.c_long(len(live_logL)), ctypes.c_long(num_chains), _dp(U), _dp(L), _lp(E),
                                 _dp(M))
    return U, L, E, M


def uniform_get_sample(model, key, L_star, max_evals):
    U = np.zeros(model.D)
    logL = ctypes.c_double()
    ne = ctypes.c_long()
    m = model._c()
    lib().orc_uniform_get_sample(ctypes.byref(m), ctypes.c_uint32(int(key[0])), ctypes.c_uint32(int(key[1])),
                                 ctypes.c_double(L_star), ctypes.c_long(max_evals), _dp(U),
                                 ctypes.byref(logL), ctypes.byref(ne))
    return U, logL.value, ne.value


# --------------------------------------------------------------- bookkeeping

def stable_argsort(keys):
    keys = np.ascontiguousarray(keys, np.float64)
    perm = np.zeros(len(keys), np.int64)
    lib().orc_stable_argsort(_dp(keys), ctypes.c_long(len(keys)), _lp(perm))
    return perm


def count_crossed_edges(sender, log_L, num_samples: Optional[int] = None):
    sender = np.ascontiguousarray(sender, np.int64)
    log_L = np.ascontiguousarray(log_L, np.float64)
    N = len(log_L)
    si = np.zeros(N, np.int64)
    nl = np.zeros(N, np.int64)
    lib().orc_count_crossed_edges(_lp(sender), _dp(log_L), ctypes.c_long(N),
                                  ctypes.c_long(-1 if num_samples is None else int(num_samples)),
                                  _lp(si), _lp(nl))
    return si, nl


EV_FIELDS = ("log_L", "log_X_mean", "log_X2_mean", "log_Z_mean", "log_ZX_mean", "log_Z2_mean",
             "log_dZ_mean", "log_dZ2_mean")


def _ev_tuple(e):
    return {f: getattr(e, f) for f in EV_FIELDS}


def sample_evidence(key, num_live_points_per_sample, log_L_samples, S=100):
    """utils.py:433-484 (sample_evidence), FP64."""
    n = np.ascontiguousarray(num_live_points_per_sample, np.int64)
    L = np.ascontiguousarray(log_L_samples, np.float64)
    out = np.zeros(S, np.float64)
    key = np.asarray(key, np.uint32)
    lib().orc_sample_evidence(ctypes.c_uint32(int(key[0])), ctypes.c_uint32(int(key[1])),
                              n.ctypes.data_as(ctypes.c_void_p), _dp(L), ctypes.c_long(len(L)), ctypes.c_int(S),
                              _dp(out))
    return out


def compute_evidence_stats(log_L, num_live_points):
    log_L = np.ascontiguousarray(log_L, np.float64)
    nl = np.ascontiguousarray(num_live_points, np.float64)
    N = len(log_L)
    fin = _EvCalc()
    per = (_EvCalc * max(N, 1))()
    lib().orc_compute_evidence_stats(_dp(log_L), _dp(nl), ctypes.c_long(N), ctypes.byref(fin), per)
    per_arr = {f: np.array([getattr(per[i], f) for i in range(N)]) for f in EV_FIELDS}
    return _ev_tuple(fin), per_arr


def evidence_update(carry: dict, n: float, log_L_next: float) -> dict:
    c = _EvCalc(*[carry[f] for f in EV_FIELDS])
    lib().orc_evcalc_update(ctypes.byref(c), ctypes.c_double(n), ctypes.c_double(log_L_next))
    return _ev_tuple(c)


def evidence_init() -> dict:
    c = _EvCalc()
    lib().orc_evcalc_init(ctypes.byref(c))
    return _ev_tuple(c)


def linear_to_log_stats(log_f_mean, log_f2_mean):
    mu = ctypes.c_double()
    var = ctypes.c_double()
    lib().orc_linear_to_log_stats(ctypes.c_double(log_f_mean), ctypes.c_double(log_f2_mean),
                                  ctypes.byref(mu), ctypes.byref(var))
    return mu.value, var.value


def make_term_cond(**kw) -> _TermCond:
    tc = _TermCond()
    names = {"ess": "ess", "evidence_uncert": "evidence_uncert", "dlogZ": "dlogZ",
             "max_samples": "max_samples", "max_num_likelihood_evaluations": "max_nlik",
             "log_L_contour": "log_L_contour", "efficiency_threshold": "efficiency_threshold",
             "rtol": "rtol", "atol": "atol", "peak_XL_frac": "peak_XL_frac"}
    for k, v in kw.items():
        if v is None:
            continue
        field = names[k]
        idx = _TC_FIELDS.index(field)
        setattr(tc, _TC_FLAGS[idx], 1)
        setattr(tc, field, float(v))
    return tc


def determine_termination(term_cond: dict, register: dict):
    tc = make_term_cond(**term_cond)
    r = _TermReg()
    for k, v in register.items():
        if k in ("ev", "ev_rem"):
            setattr(r, k, _EvCalc(*[v[f] for f in EV_FIELDS]))
        else:
            setattr(r, k, v)
    reason = ctypes.c_long()
    done = lib().orc_determine_termination(ctypes.byref(tc), ctypes.byref(r), ctypes.byref(reason))
    return bool(done), reason.value


# -------------------------------------------------------------------- NS run

@dataclass
class OracleRun:
    termination_reason: int
    num_samples: int
    sender: np.ndarray
    log_L: np.ndarray
    U: np.ndarray
    nevals: np.ndarray
    phantom: np.ndarray
    iterations: int
    register: dict
    results: dict
    samples_indices: np.ndarray
    num_live_points: np.ndarray
    log_L_sorted: np.ndarray
    log_dp_mean: np.ndarray
    log_X_mean: np.ndarray
    U_sorted: np.ndarray


def round_up_num_live_points(n, shell_frac, num_devices=1):
    """sharded_static.py:577-584"""
    n = int(n)
    while int(n * shell_frac) % num_devices != 0:
        n += 1
    return n


def round_up_max_samples(max_samples, num_discard, num_phantom):
    """sharded_static.py:587-594"""
    m = int(max_samples)
    block = num_discard * (1 + num_phantom)
    while m % block != 0:
        m += 1
    return m


def ns_run(model: OracleModel, key, num_live_points, num_slices, max_samples=None, num_phantom=0,
           midpoint_shrink=True, shell_fraction=0.5, init_efficiency_threshold=0.1,
           term_cond: Optional[dict] = None, max_iterations=0, init_only=False,
           gradient_guided=False, gradient_slice=False) -> OracleRun:
    """NestedSampler(...)(key, term_cond) followed by to_results(trim=True)."""
    shell_fraction = max(shell_fraction, 1.0 / num_live_points)
    n = round_up_num_live_points(num_live_points, shell_fraction)
    s = int(n * shell_fraction)
    if max_samples is None:
        max_samples = n * 100
    cap = round_up_max_samples(max_samples, s, num_phantom)
    tc = dict(term_cond or {"dlogZ": float(np.log(1.0 + 1e-3))})
    big = float(np.iinfo(np.int64).max)
    tc["max_samples"] = min(float(tc.get("max_samples") or big), float(cap))
    cfg = _NSCfg(n, s, cap, float(init_efficiency_threshold), _SliceCfg(num_slices, num_phantom,
                                                                      int(midpoint_shrink),
                                                                      int(gradient_guided),
                                                                      int(gradient_slice)), 100)
    D = model.D
    sender = np.zeros(cap, np.int64)
    log_L = np.zeros(cap)
    U = np.zeros((cap, D))
    nevals = np.zeros(cap, np.int64)
    phantom = np.zeros(cap, np.int32)
    st = _NSState(_lp(sender), _dp(log_L), _dp(U), _lp(nevals), _ip(phantom))
    ctc = make_term_cond(**tc)
    m = model._c()
    liveU = np.zeros((n, D))
    liveL = np.zeros(n)
    reason = lib().orc_ns_run(ctypes.byref(m), ctypes.byref(cfg), ctypes.byref(ctc),
                              ctypes.c_uint32(int(key[0])), ctypes.c_uint32(int(key[1])), ctypes.byref(st),
                              ctypes.c_long(max_iterations), ctypes.c_int(int(init_only)), _dp(liveU),
                              _dp(liveL))
    N = min(st.num_samples, cap)
    reg = {"num_samples_used": st.reg.num_samples_used, "ev": _ev_tuple(st.reg.ev),
           "ev_rem": _ev_tuple(st.reg.ev_rem),
           "num_likelihood_evaluations": st.reg.num_likelihood_evaluations,
           "log_L_contour": st.reg.log_L_contour, "efficiency": st.reg.efficiency,
           "plateau": st.reg.plateau, "no_seed_points": st.reg.no_seed_points,
           "relative_spread": st.reg.relative_spread, "absolute_spread": st.reg.absolute_spread,
           "peak_log_XL": st.reg.peak_log_XL, "live_U": liveU, "live_log_L": liveL,
           "next_sample_idx": st.next_sample_idx, "key": np.array([st.key0, st.key1], np.uint32)}
    res = _Results()
    si = np.zeros(max(N, 1), np.int64)
    nl = np.zeros(max(N, 1), np.int64)
    ls = np.zeros(max(N, 1))
    dp = np.zeros(max(N, 1))
    lx = np.zeros(max(N, 1))
    Us = np.zeros((max(N, 1), D))
    if N > 0:
        lib().orc_to_results(ctypes.byref(m), ctypes.byref(st), ctypes.c_long(cap), ctypes.byref(res), _lp(si),
                             _lp(nl), _dp(ls), _dp(dp), _dp(lx), _dp(Us))
    results = {f: getattr(res, f) for f, _ in _Results._fields_}
    return OracleRun(int(reason), int(st.num_samples), sender[:N], log_L[:N], U[:N], nevals[:N],
                     phantom[:N], int(st.iterations), reg, results, si[:N], nl[:N], ls[:N], dp[:N],
                     lx[:N], Us[:N])


def ns_run_batch(models, cfg_list, keys, term_conds, num_threads, max_iterations=0, timed=False):
    """Independent runs on host threads: returns (log_Z, nevals, reasons) [+ (seconds,
    iterations) when timed].  cfg_list items are dicts with num_live_points, num_slices,
    max_samples, num_phantom."""
    R = len(models)
    ms = (_Model * R)()
    cs = (_NSCfg * R)()
    ts = (_TermCond * R)()
    for r in range(R):
        ms[r] = models[r]._c()
        c = cfg_list[r]
        n = c["num_live_points"]
        s = n // 2
        cap = round_up_max_samples(c["max_samples"], s, c.get("num_phantom", 0))
        cs[r] = _NSCfg(n, s, cap, 0.1, _SliceCfg(c["num_slices"], c.get("num_phantom", 0), 1, 0), 100)
        tc = dict(term_conds[r])
        tc["max_samples"] = min(float(tc.get("max_samples") or cap), float(cap))
        ts[r] = make_term_cond(**tc)
    k = np.ascontiguousarray(np.asarray(keys, np.uint32).reshape(R, 2))
    log_Z = np.zeros(R)
    nev = np.zeros(R, np.int64)
    reasons = np.zeros(R, np.int64)
    secs = np.zeros(R)
    its = np.zeros(R, np.int64)
    lib().orc_ns_run_batch(ms, cs, ts, _up(k), ctypes.c_int(R), ctypes.c_int(num_threads), _dp(log_Z), _lp(nev),
                           _lp(reasons), ctypes.c_long(max_iterations), _dp(secs), _lp(its))
    if timed:
        return log_Z, nev, reasons, secs, its
    return log_Z, nev, reasons


def ns_run_batch_timed(models, cfg_list, keys, term_conds, num_threads, max_iterations):
    """Per-run host seconds, likelihood evaluations and iterations of bounded oracle runs."""
    _, nev, _, secs, its = ns_run_batch(models, cfg_list, keys, term_conds, num_threads, max_iterations, timed=True)
    return secs, nev, its


def blr_reweighted(Phi, y, U, log_w, log_tau, log_sigma):
    Phi = np.ascontiguousarray(Phi, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    U = np.ascontiguousarray(U, np.float64)
    log_w = np.ascontiguousarray(log_w, np.float64)
    N, P = Phi.shape
    lz = ctypes.c_double()
    g = np.zeros(2)
    lib().orc_blr_reweighted(_dp(Phi), _dp(y), ctypes.c_int(N), ctypes.c_int(P), _dp(U), _dp(log_w),
                             ctypes.c_long(U.shape[0]), ctypes.c_double(log_tau), ctypes.c_double(log_sigma),
                             ctypes.byref(lz), _dp(g))
    return lz.value, g


# ------------------------------------------------------- fp32 kernel-arithmetic mode

class _Model32(ctypes.Structure):
    _fields_ = [("D", ctypes.c_int), ("family", ctypes.c_int),
                ("prior_kind", ctypes.POINTER(ctypes.c_int)),
                ("prior_a", ctypes.POINTER(ctypes.c_float)),
                ("prior_b", ctypes.POINTER(ctypes.c_float)),
                ("p", ctypes.POINTER(ctypes.c_float)), ("variant", ctypes.c_int)]


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


@dataclass
class Model32:
    """A model in the device's fp32 tables (prior a/b, the family's parameter vector in the
    device layout) and the reduction order of the kernel that runs it: variant 0 = one thread
    per chain, 32 / 64 = the warp-cooperative correlated-Gaussian kernel of that width."""
    D: int
    family: int
    prior_kind: np.ndarray
    prior_a: np.ndarray
    prior_b: np.ndarray
    params: np.ndarray
    variant: int = 0

    def _c(self):
        self._keep = [np.ascontiguousarray(self.prior_kind, np.int32),
                      np.ascontiguousarray(self.prior_a, np.float32),
                      np.ascontiguousarray(self.prior_b, np.float32),
                      np.ascontiguousarray(self.params, np.float32)]
        k, a, b, p = self._keep
        return _Model32(self.D, self.family, _ip(k), _fp(a), _fp(b), _fp(p), int(self.variant))


def kernel_variant(family: int, D: int, warp_min_D: int = 17) -> int:
    """Which sampler kernel runs a (family, D) run: the correlated-Gaussian family with
    warp_min_D <= D <= 32 (32) or 32 < D <= 64 (64) runs warp-cooperatively, everything else
    one thread per chain (0)."""
    if family == LIK_MVN and D >= warp_min_D:
        return 32 if D <= 32 else 64
    return 0


def model32(family, D, params, prior_kind, prior_a, prior_b, variant=None, warp_min_D=17):
    if variant is None:
        variant = kernel_variant(family, D, warp_min_D)
    return Model32(D, family, np.asarray(prior_kind, np.int32), np.asarray(prior_a, np.float32),
                   np.asarray(prior_b, np.float32), np.asarray(params, np.float32), variant)


def forward32(model: Model32, U):
    U = np.ascontiguousarray(np.atleast_2d(U), np.float32)
    out = np.zeros(U.shape[0], np.float32)
    m = model._c()
    lib().orc32_forward_batch(ctypes.byref(m), _fp(U), ctypes.c_long(U.shape[0]), _fp(out))
    return out


def slice_shell32(model: Model32, key, L_star, live_U, live_logL, num_chains, num_slices, num_phantom=0,
                  midpoint_shrink=True, max_evals_per_slice=100000, gradient_guided=False, gradient_slice=False):
    """One shell in the kernels' fp32 arithmetic; L_star and live_logL are the device's fp32
    values (relative to the run's log-likelihood offset)."""
    D = model.D
    live_U = np.ascontiguousarray(live_U, np.float32)
    live_logL = np.ascontiguousarray(live_logL, np.float32)
    cfg = _SliceCfg(num_slices, num_phantom, int(midpoint_shrink), int(gradient_guided), int(gradient_slice))
    U = np.zeros((num_chains, D), np.float32)
    L = np.zeros(num_chains, np.float32)
    E = np.zeros(num_chains, np.int64)
    K = max(num_phantom, 1)
    pU = np.zeros((num_chains, K, D), np.float32)
    pL = np.zeros((num_chains, K), np.float32)
    m = model._c()
    lib().orc32_slice_shell(ctypes.byref(m), ctypes.byref(cfg), ctypes.c_uint32(int(key[0])),
                            ctypes.c_uint32(int(key[1])), ctypes.c_float(float(np.float32(L_star))),
                            _fp(live_U), _fp(live_logL), ctypes.c_long(len(live_logL)), ctypes.c_long(num_chains),
                            ctypes.c_long(int(max_evals_per_slice)), _fp(U), _fp(L), _lp(E), _fp(pU), _fp(pL))
    return U, L, E, pU[:, :num_phantom], pL[:, :num_phantom]


def fm(name, x):
    """The product's fp32 elementary function `name` (exp, log, log1p, ndtri, ndtri_d,
    normal_from_bits) elementwise over x."""
    f = getattr(lib(), "orc32_fm_" + name)
    flat = np.ravel(x)
    if name == "normal_from_bits":
        vals = [f(ctypes.c_uint64(int(v))) for v in flat]
    elif name == "ndtri_d":
        vals = [f(float(v)) for v in flat]
    else:
        vals = [f(float(np.float32(v))) for v in flat]
    return np.array(vals, np.float32).reshape(np.shape(x))


# ----------------------------------------------------------------------------- prior transform

def fm_log64(x: float) -> float:
    return lib().orc_fm_log64(float(x))


def fm_ndtri64(p: float) -> float:
    return lib().orc_fm_ndtri64(float(p))


def prior_transform(kind, a, b, log_norm, U, A=None, row_start=None, c=None, log_det=0.0, log_L=None):
    """Model.transform / Model.log_prob_prior of the rows of U (framework/model.py:155-187) in
    the device transform's arithmetic: returns (X [M, D] float64, log density [M] float64)."""
    U = np.ascontiguousarray(U)
    M, D = U.shape
    kind = np.ascontiguousarray(kind, np.int32)
    a, b, log_norm = (np.ascontiguousarray(v, np.float64) for v in (a, b, log_norm))
    X = np.zeros((M, D), np.float64)
    out = np.zeros(M, np.float64)
    U32 = U if U.dtype == np.float32 else None
    U64 = np.ascontiguousarray(U, np.float64) if U32 is None else None
    fp = ctypes.POINTER(ctypes.c_float)
    Ak = np.ascontiguousarray(A, np.float64) if A is not None else None
    rs = np.ascontiguousarray(row_start, np.int32) if A is not None else None
    ck = np.ascontiguousarray(c, np.float64) if A is not None else None
    lL = np.ascontiguousarray(log_L, np.float64) if log_L is not None else None
    lib().orc_prior_transform(
        ctypes.c_int(D), _ip(kind), _dp(a), _dp(b), _dp(log_norm),
        _dp(Ak) if Ak is not None else None, _ip(rs) if rs is not None else None,
        _dp(ck) if ck is not None else None, ctypes.c_double(log_det),
        U32.ctypes.data_as(fp) if U32 is not None else None, _dp(U64) if U64 is not None else None,
        ctypes.c_long(M), _dp(lL) if lL is not None else None, _dp(X), _dp(out))
    return X, out


# ----------------------------------------------------------------------------- results of a store

def results_of_store(sender, log_L, nevals, phantom):
    """_to_results (sharded_static.py:652-773) of one sample store given as arrays (sender,
    FP64 log L, evaluation counts, phantom flags, in store order): returns (scalars dict,
    samples_indices, num_live_points, log_L sorted, log_dp_mean, log_X_mean)."""
    N = len(log_L)
    snd = np.ascontiguousarray(sender, np.int64)
    lL = np.ascontiguousarray(log_L, np.float64)
    nev = np.ascontiguousarray(nevals, np.int64)
    ph = np.ascontiguousarray(phantom, np.int32)
    st = _NSState()
    st.sender, st.log_L, st.nevals, st.phantom = _lp(snd), _dp(lL), _lp(nev), _ip(ph)
    st.num_samples = N
    st.next_sample_idx = N
    m = _Model()
    m.D = 1
    res = _Results()
    si, nl = np.zeros(max(N, 1), np.int64), np.zeros(max(N, 1), np.int64)
    ls, dp, lx = (np.zeros(max(N, 1)) for _ in range(3))
    lib().orc_to_results(ctypes.byref(m), ctypes.byref(st), ctypes.c_long(N), ctypes.byref(res), _lp(si), _lp(nl),
                         _dp(ls), _dp(dp), _dp(lx), None)
    return ({f: getattr(res, f) for f, _ in _Results._fields_}, si[:N], nl[:N], ls[:N], dp[:N], lx[:N])
