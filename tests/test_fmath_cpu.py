"""CPU tests of the fp32 elementary functions the sampler kernels use (gbns_fmath.h, built
from correctly rounded IEEE operations only, so the same bits on the device and here) and of
the oracle's fp32 kernel-arithmetic mode against its FP64 restatement."""
import numpy as np
import pytest

from tests.conftest import corr_gauss

scipy_special = pytest.importorskip("scipy.special")


def _ulps(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return np.abs(got - ref) / np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)


def test_exp_log_log1p_error_bounds(oracle_mod):
    x = np.linspace(-103.0, 88.0, 40001).astype(np.float32)
    assert np.max(_ulps(oracle_mod.fm("exp", x), np.exp(x.astype(np.float64)))) < 1.0
    x = np.logspace(-44, 38, 40001).astype(np.float32)
    assert np.max(_ulps(oracle_mod.fm("log", x), np.log(x.astype(np.float64)))) < 2.0
    x = np.logspace(-30, 0, 20001).astype(np.float32)
    assert np.max(_ulps(oracle_mod.fm("log1p", x), np.log1p(x.astype(np.float64)))) < 3.0
    # special values
    assert oracle_mod.fm("exp", np.float32([-np.inf]))[0] == 0.0
    assert oracle_mod.fm("exp", np.float32([0.0]))[0] == 1.0
    assert np.isneginf(oracle_mod.fm("log", np.float32([0.0]))[0])
    assert np.isnan(oracle_mod.fm("log", np.float32([-1.0]))[0])
    assert oracle_mod.fm("log1p", np.float32([0.0]))[0] == 0.0


def test_ndtri_and_jax_normal(oracle_mod):
    """Normal quantile (AS 241, about 1e-7 relative) of fp32 and FP64 arguments, and the jax
    float64 normal variate of a 64-bit draw: within 4e-7 relative of the FP64 values, with the
    tails formed exactly (u within 1e-12 of 0 or 1; p = (4M + 1) 2^-54 at the extremes)."""
    u = np.concatenate([np.linspace(1e-7, 1 - 1e-7, 20001), np.logspace(-44, -1, 3000)]).astype(np.float32)
    ref = scipy_special.ndtri(u.astype(np.float64))
    assert np.max(np.abs(oracle_mod.fm("ndtri", u) - ref) / np.maximum(np.abs(ref), 1e-30)) < 4e-7
    ud = np.array([1e-12, 1 - 1e-12, 3e-9, 1 - 3e-9, 0.3, 0.9])
    ref = scipy_special.ndtri(ud)
    ref[1], ref[3] = -ref[0], -ref[2]  # 1 - u rounds in FP64; the quantile is odd about 1/2
    assert np.max(np.abs(oracle_mod.fm("ndtri_d", ud) - ref) / np.abs(ref)) < 4e-7
    k = oracle_mod.PRNGKey(99)
    bits = oracle_mod.random_bits64(k, 5000)
    z32 = oracle_mod.fm("normal_from_bits", bits)
    z64 = oracle_mod.normal(k, 5000)
    assert np.max(np.abs(z32 - z64) / np.maximum(np.abs(z64), 1e-12)) < 4e-7
    M = np.array([0, 1, (1 << 51) - 1, 1 << 51, (1 << 52) - 1], np.uint64)
    z = oracle_mod.fm("normal_from_bits", M << np.uint64(12))
    p_lo = (4 * M.astype(np.float64) + 1) * 2.0 ** -54
    exact = scipy_special.ndtri(p_lo)
    exact[2] = -2.0 ** -54 * np.sqrt(2 * np.pi) * 3  # p = 1/2 - 3 2^-54: Phi^-1 ~ -3 2^-54 sqrt(2 pi)
    exact[3] = 2.0 ** -54 * np.sqrt(2 * np.pi)            # p = 1/2 + 2^-54
    exact[4] = -scipy_special.ndtri(3 * 2.0 ** -54)       # p = 1 - 3 2^-54
    np.testing.assert_allclose(z, exact, rtol=4e-7)


@pytest.mark.parametrize("D,n,S", [(2, 64, 8), (8, 256, 32), (24, 128, 24), (40, 96, 40)])
def test_fp32_chains_track_fp64_restatement(oracle_mod, D, n, S):
    """The fp32 kernel-arithmetic chains follow the FP64 chains except where a likelihood
    comparison sits within fp32 rounding of the contour: same evaluation counts and points
    within 2e-4 for at least 95 % of the chains (in practice all of them)."""
    from jaxns_gb300.engine import mvn_offset, mvn_params
    mu, cov = corr_gauss(D, D)
    om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    m32 = oracle_mod.model32(0, D, mvn_params(mu, cov), np.zeros(D), np.full(D, -10.0), np.full(D, 20.0))
    off = mvn_offset(cov)
    U = np.random.default_rng(D).uniform(0, 1, size=(8 * n, D)).astype(np.float32)
    L32 = oracle_mod.forward32(m32, U)
    keep = np.argsort(L32, kind="stable")[-n:]
    U, L32 = U[keep], L32[keep]
    s = n // 2
    key = oracle_mod.PRNGKey(1000 + D)
    U3, L3, E3, _, _ = oracle_mod.slice_shell32(m32, key, L32[s - 1], U, L32, s, S)
    Uo, Lo, Eo = oracle_mod.slice_shell(om, key, float(L32[s - 1]) + off, U.astype(np.float64),
                                        L32.astype(np.float64) + off, s, S)
    same = (E3 == Eo) & np.all(np.abs(U3 - Uo) < 2e-4, axis=1)
    assert same.mean() >= 0.95, same.mean()
    assert np.all(L3 > L32[s - 1])
