"""Posterior moments from the weighted samples (weights exp(log_dp_mean)) against the exact
posterior: a correlated Gaussian inside a wide uniform prior (mean mu, covariance Sigma) and
Bayesian linear regression (the analytic Gaussian posterior of w).  Tolerances are Monte-Carlo
errors from the run's Kish effective sample size."""
import numpy as np
import pytest

from tests.conftest import corr_gauss

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _weighted_moments(res, key):
    x = res.samples[key]
    x = (x.cpu().numpy() if hasattr(x, "cpu") else np.asarray(x)).astype(np.float64)
    ldp = res.log_dp_mean.cpu().numpy()
    w = np.exp(ldp - ldp.max())
    w /= w.sum()
    mean = w @ x
    cov = (x - mean).T @ ((x - mean) * w[:, None])
    ess = 1.0 / np.sum(w * w)
    return mean, cov, ess


def test_mvn_posterior_moments(gpu_lib):
    import jaxns_gb300 as gb
    D = 6
    mu, cov = corr_gauss(D, 11)

    def prior_model():
        x = yield gb.Prior(gb.Uniform(-10.0 * np.ones(D), 10.0 * np.ones(D)), name="x")
        return x

    ns = gb.NestedSampler(gb.Model(prior_model, gb.MultivariateNormalLikelihood(mu, cov)), num_live_points=1000)
    reason, state = ns(gb.random.PRNGKey(21), gb.TerminationCondition(dlogZ=1e-4))
    res = ns.to_results(reason, state)
    mean, C, ess = _weighted_moments(res, "x")
    sd = np.sqrt(np.diag(cov))
    # nested-sampling posterior samples are correlated across a shell; allow 6 Kish s.e.
    assert np.all(np.abs(mean - mu) < 6 * sd / np.sqrt(ess)), (mean - mu, sd / np.sqrt(ess))
    rel = np.abs(np.diag(C) / np.diag(cov) - 1.0)
    assert np.all(rel < 6 * np.sqrt(2.0 / ess) + 0.02), (rel, ess)
    corr = C / np.sqrt(np.outer(np.diag(C), np.diag(C)))
    corr_true = cov / np.outer(sd, sd)
    assert np.max(np.abs(corr - corr_true)) < 0.08


def test_blr_posterior_moments(gpu_lib):
    import jaxns_gb300 as gb
    rng = np.random.default_rng(8)
    N, P, sigma, tau = 800, 5, 0.5, 1.0
    Phi = rng.standard_normal((N, P))
    y = Phi @ rng.standard_normal(P) + sigma * rng.standard_normal(N)

    def prior_model():
        w = yield gb.Prior(gb.Normal(np.zeros(P), tau * np.ones(P)), name="w")
        return w

    ns = gb.NestedSampler(gb.Model(prior_model, gb.LinearGaussianLikelihood(Phi, y, sigma)), num_live_points=300)
    reason, state = ns(gb.random.PRNGKey(5))
    res = ns.to_results(reason, state)
    mean, C, ess = _weighted_moments(res, "w")
    Phi32, y32 = Phi.astype(np.float32).astype(np.float64), y.astype(np.float32).astype(np.float64)
    S = np.linalg.inv(np.eye(P) / tau ** 2 + Phi32.T @ Phi32 / sigma ** 2)
    m = S @ Phi32.T @ y32 / sigma ** 2
    sd = np.sqrt(np.diag(S))
    assert np.all(np.abs(mean - m) < 6 * sd / np.sqrt(ess)), ((mean - m) / sd, ess)
    rel = np.abs(np.diag(C) / np.diag(S) - 1.0)
    assert np.all(rel < 6 * np.sqrt(2.0 / ess) + 0.05), (rel, ess)
