"""sample_evidence oracle against a direct restatement and against the evidence statistics;
JSON results in the reference's format (CPU only)."""
import json

import numpy as np
import pytest


def _restated_sample_evidence(oracle_mod, key, n, L, S):
    """utils.py:433-484 written out with the oracle's jax.random helpers, in numpy."""
    out = []
    for ks in oracle_mod.split(key, S):
        keys = oracle_mod.split(ks, len(L))
        log_Z, log_X = -np.inf, 0.0
        for i in range(len(L)):
            u = oracle_mod.uniform(keys[i], 1)[0]
            log_T = np.log(u) / n[i]
            log_nX = log_X + log_T
            log_dZ = log_X + np.log1p(-np.exp(log_T)) + L[i]
            log_Z = np.logaddexp(log_Z, log_dZ)
            log_X = log_nX
        out.append(log_Z)
    return np.array(out)


def test_sample_evidence_oracle_matches_restatement(oracle_mod):
    rng = np.random.default_rng(3)
    n = rng.integers(5, 40, size=60)
    L = np.sort(rng.normal(size=60)) * 3.0
    key = oracle_mod.PRNGKey(17)
    got = oracle_mod.sample_evidence(key, n, L, S=4)
    ref = _restated_sample_evidence(oracle_mod, key, n, L, 4)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-12)


def test_sample_evidence_agrees_with_evidence_stats(oracle_mod):
    """Constant n = 200: the replicas' mean and spread match compute_evidence_stats' log Z
    mean and uncertainty (the expectation uses the trapezoid rule, the replicas the sample's
    own L, so the means agree to the discretisation)."""
    n = np.full(4000, 200)
    X = np.exp(-np.arange(1, 4001) / 200.0)
    L = -0.5 * (X ** (2.0 / 3.0)) * 50.0                    # a D=3 Gaussian in X
    ev, _ = oracle_mod.compute_evidence_stats(L, n)
    mu, var = oracle_mod.linear_to_log_stats(ev["log_Z_mean"], ev["log_Z2_mean"])
    samples = oracle_mod.sample_evidence(oracle_mod.PRNGKey(0), n, L, S=400)
    assert abs(samples.mean() - mu) < 4 * samples.std() / np.sqrt(400) + 0.01
    assert 0.7 < samples.std() / np.sqrt(var) < 1.3


def test_results_json_roundtrip_reference_format(tmp_path):
    from jaxns_gb300.public import NestedSamplerResults
    from jaxns_gb300.utils import load_results, save_results
    rng = np.random.default_rng(0)
    M = 17
    res = NestedSamplerResults(
        log_Z_mean=-3.5, log_Z_uncert=0.1, ESS=120.0, H_mean=2.0, samples={"x": rng.normal(size=(M, 2))},
        parametrised_samples={"x": rng.normal(size=(M, 2))}, U_samples=rng.uniform(size=(M, 2)),
        log_L_samples=rng.normal(size=M), log_dp_mean=rng.normal(size=M), log_X_mean=-np.arange(M, dtype=float),
        log_posterior_density=rng.normal(size=M), num_live_points_per_sample=np.arange(M, dtype=np.int64),
        num_likelihood_evaluations_per_sample=np.ones(M, np.int64), total_num_samples=M, total_phantom_samples=0,
        total_num_likelihood_evaluations=3 * M, log_efficiency=-1.1, termination_reason=4)
    f = tmp_path / "res.json"
    save_results(res, str(f))
    raw = json.loads(f.read_text())
    assert raw["type"] == "__namedtuple__"
    assert raw["__class__"] == "jaxns.nested_samplers.common.types.NestedSamplerResults"
    assert raw["__data__"]["log_L_samples"]["type"] == "__jax_ndarray__"
    back = load_results(str(f))
    assert isinstance(back, NestedSamplerResults)
    for k in res._fields:
        a, b = getattr(res, k), getattr(back, k)
        if isinstance(a, dict):
            for kk in a:
                np.testing.assert_array_equal(a[kk], b[kk])
        else:
            np.testing.assert_array_equal(np.asarray(a), np.asarray(b))
    # a file in the reference's layout with numpy-tagged arrays loads too
    raw["__data__"]["log_X_mean"]["type"] = "__ndarray__"
    g = tmp_path / "ref.json"
    g.write_text(json.dumps(raw))
    back2 = load_results(str(g))
    np.testing.assert_array_equal(back2.log_X_mean, res.log_X_mean)


def test_trim_results_cuts_per_sample_arrays():
    """NestedSampler.trim_results (public.py:198-220): arrays of more than one element, also
    inside the samples dicts, keep their first total_num_samples rows; scalars stay."""
    torch = pytest.importorskip("torch")
    from jaxns_gb300.public import NestedSampler, NestedSamplerResults
    N, cap = 6, 10
    pad = lambda *s: np.arange(int(np.prod((cap,) + s)), dtype=np.float64).reshape((cap,) + s)
    res = NestedSamplerResults(
        log_Z_mean=-1.5, log_Z_uncert=0.1, ESS=50.0, H_mean=2.0,
        samples={"x": pad(3), "y": torch.arange(cap)}, parametrised_samples={"x": pad(3)},
        U_samples=pad(3), log_L_samples=torch.arange(cap, dtype=torch.float64), log_dp_mean=pad(),
        log_X_mean=pad(), log_posterior_density=pad(), num_live_points_per_sample=pad(),
        num_likelihood_evaluations_per_sample=np.arange(cap), total_num_samples=N, total_phantom_samples=0,
        total_num_likelihood_evaluations=123, log_efficiency=-0.7, termination_reason=4)
    t = NestedSampler.trim_results(res)
    assert t.U_samples.shape == (N, 3) and t.samples["x"].shape == (N, 3) and t.samples["y"].shape == (N,)
    assert t.log_L_samples.shape == (N,) and t.num_likelihood_evaluations_per_sample.shape == (N,)
    np.testing.assert_array_equal(t.log_dp_mean, np.arange(N))
    assert (t.log_Z_mean, t.total_num_samples, t.termination_reason) == (-1.5, N, 4)
    one = res._replace(log_dp_mean=np.zeros(1))
    assert NestedSampler.trim_results(one).log_dp_mean.shape == (1,)


def test_dead_set_log_weights():
    """DeadSet.from_results: log w_i = log dp_i - log L_i + log Z (experimental/
    evidence_maximisation.py:213), so at the run's own hyperparameters the reweighted evidence
    logsumexp_i(log L_i + log w_i) is log Z again (the normalised dp sum to one)."""
    torch = pytest.importorskip("torch")
    from scipy.special import logsumexp
    from jaxns_gb300.adjoint import DeadSet
    from jaxns_gb300.public import NestedSamplerResults
    rng = np.random.default_rng(4)
    M, P, N = 50, 3, 20
    log_L = np.sort(rng.standard_normal(M)) * 3
    log_dp = log_L + rng.standard_normal(M)
    log_dp -= logsumexp(log_dp)
    log_Z = -7.25
    res = NestedSamplerResults(
        log_Z_mean=log_Z, log_Z_uncert=0.1, ESS=10.0, H_mean=0.0, samples={}, parametrised_samples={},
        U_samples=torch.tensor(rng.random((M, P))), log_L_samples=torch.tensor(log_L),
        log_dp_mean=torch.tensor(log_dp), log_X_mean=None, log_posterior_density=None,
        num_live_points_per_sample=None, num_likelihood_evaluations_per_sample=None, total_num_samples=M,
        total_phantom_samples=0, total_num_likelihood_evaluations=0, log_efficiency=0.0, termination_reason=4)
    ds = DeadSet.from_results(res, rng.standard_normal((N, P)), rng.standard_normal(N))
    assert ds.U.dtype == torch.float64 and ds.log_w.dtype == torch.float64 and ds.Phi.dtype == torch.float32
    np.testing.assert_allclose(ds.log_w.numpy(), log_dp - log_L + log_Z, rtol=1e-14)
    assert logsumexp(log_L + ds.log_w.numpy()) == pytest.approx(log_Z, abs=1e-12)
