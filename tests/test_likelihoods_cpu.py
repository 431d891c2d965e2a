"""Likelihood families (host side): the float64 reference of each family against scipy and
against the FP64 oracle, the packed parameter block the kernels read, and the log-L offsets."""
import numpy as np
import pytest

gb = pytest.importorskip("jaxns_gb300")
stats = pytest.importorskip("scipy.stats")


def test_mvn(oracle_mod):
    from jaxns_gb300.engine import mvn_offset, mvn_params
    rng = np.random.default_rng(0)
    D = 5
    A = rng.standard_normal((D, D))
    mu, cov = rng.standard_normal(D), A @ A.T / D + 0.1 * np.eye(D)
    lik = gb.MultivariateNormalLikelihood(mu, cov)
    X = rng.uniform(-3, 3, (50, D))
    np.testing.assert_allclose(lik(X), stats.multivariate_normal.logpdf(X, mu, cov), rtol=1e-10)
    om = oracle_mod.mvn_model(np.full(D, -3.0), np.full(D, 3.0), mu, cov)
    np.testing.assert_allclose(oracle_mod.forward(om, (X + 3.0) / 6.0), lik(X), rtol=1e-12)
    p = mvn_params(mu, cov).astype(np.float64)
    Linv = p[D:D + D * D].reshape(D, D)
    np.testing.assert_allclose(Linv @ np.linalg.cholesky(cov), np.eye(D), atol=1e-5)
    assert np.allclose(np.triu(Linv, 1), 0.0)
    assert p[-1] == pytest.approx(mvn_offset(cov), rel=1e-6)
    assert lik(mu) == pytest.approx(lik.log_L_offset(), rel=1e-12)   # at the mode log L is the offset


def test_shells(oracle_mod):
    from jaxns_gb300.engine import shells_params
    D = 4
    c1 = np.zeros(D); c1[0] = 2.0
    c2 = -c1
    lik = gb.GaussianShellsLikelihood(c1, c2, 1.5, 0.2)
    rng = np.random.default_rng(1)
    X = rng.uniform(-4, 4, (60, D))
    norm = np.log(np.sqrt(2 * np.pi * 0.2 ** 2))
    s1 = -0.5 * ((np.linalg.norm(X - c1, axis=1) - 1.5) / 0.2) ** 2 - norm
    s2 = -0.5 * ((np.linalg.norm(X - c2, axis=1) - 1.5) / 0.2) ** 2 - norm
    np.testing.assert_allclose(lik(X), np.logaddexp(s1, s2), rtol=1e-12)
    om = oracle_mod.shells_model(-4.0, 4.0, c1, c2, 1.5, 0.2)
    np.testing.assert_allclose(oracle_mod.forward(om, (X + 4.0) / 8.0), lik(X), rtol=1e-10)
    p = shells_params(c1, c2, 1.5, 0.2)
    assert len(p) == 2 * D + 3 and p[2 * D] == 1.5 and p[2 * D + 1] == pytest.approx(0.2)
    assert lik.log_L_offset() == pytest.approx(-norm)


def test_linear_gaussian(oracle_mod):
    rng = np.random.default_rng(2)
    N, P, sigma, tau = 30, 3, 0.4, 1.5
    Phi, y = rng.standard_normal((N, P)), rng.standard_normal(N)
    lik = gb.LinearGaussianLikelihood(Phi, y, sigma)
    W = rng.standard_normal((20, P))
    want = np.array([stats.norm.logpdf(y, Phi @ w, sigma).sum() for w in W])
    np.testing.assert_allclose(lik(W), want, rtol=1e-12)
    om = oracle_mod.lingauss_model(Phi, y, sigma, tau)
    U = stats.norm.cdf(W / tau)                                     # the Normal(0, tau^2) prior quantile's inverse
    np.testing.assert_allclose(oracle_mod.forward(om, U), want, rtol=1e-9)
    p = lik.params(None)
    assert len(p) == N * P + N + 1 and p[-1] == pytest.approx(sigma)
    np.testing.assert_allclose(p[:N * P].reshape(N, P), Phi, rtol=1e-6)
    assert lik.log_L_offset() == pytest.approx(-0.5 * N * np.log(2 * np.pi * sigma ** 2))


def test_dimension_checks():
    with pytest.raises(ValueError):
        gb.MultivariateNormalLikelihood(np.zeros(3), np.eye(3)).check(4)
    with pytest.raises(ValueError):
        gb.GaussianShellsLikelihood(np.zeros(3), np.zeros(2), 1.0, 0.1).check(3)
    with pytest.raises(ValueError):
        gb.LinearGaussianLikelihood(np.zeros((5, 2)), np.zeros(5), 1.0).check(3)
