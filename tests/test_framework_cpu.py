"""Model / Prior front end (framework/model.py:24, framework/prior.py:65): prior tables,
U -> X transform, prior density, name checks.  Host logic only."""
import numpy as np
import pytest

gb = pytest.importorskip("jaxns_gb300")
stats = pytest.importorskip("scipy.stats")


def _model():
    def prior_model():
        a = yield gb.Prior(gb.Uniform(-2.0, 3.0), name="a")                      # scalar
        v = yield gb.Prior(gb.Normal(np.array([0.0, 1.0, -1.0]), 2.0), name="v")  # vector, broadcast scale
        m = yield gb.Prior(gb.Uniform(np.zeros((2, 2)), np.ones((2, 2)) * 4.0), name="m")
        yield gb.Prior(gb.Normal(5.0, 0.5))                                    # unnamed
        return a, v, m
    return gb.Model(prior_model, gb.MultivariateNormalLikelihood(np.zeros(9), np.eye(9)))


def test_prior_tables():
    m = _model()
    assert m.U_ndims == 1 + 3 + 4 + 1
    np.testing.assert_array_equal(m.prior_kind, [0, 1, 1, 1, 0, 0, 0, 0, 1])
    np.testing.assert_allclose(m.prior_a, [-2.0, 0.0, 1.0, -1.0, 0, 0, 0, 0, 5.0])
    np.testing.assert_allclose(m.prior_b, [5.0, 2.0, 2.0, 2.0, 4, 4, 4, 4, 0.5])


def test_transform_shapes_and_values():
    m = _model()
    rng = np.random.default_rng(0)
    U = rng.random((7, m.U_ndims))
    X = m.transform(U)
    assert set(X) == {"a", "v", "m"}                       # unnamed priors are not reported
    assert X["a"].shape == (7,) and X["v"].shape == (7, 3) and X["m"].shape == (7, 2, 2)
    np.testing.assert_allclose(X["a"], -2.0 + 5.0 * U[:, 0])
    np.testing.assert_allclose(X["v"], stats.norm.ppf(U[:, 1:4], loc=[0.0, 1.0, -1.0], scale=2.0), rtol=1e-12)
    np.testing.assert_allclose(X["m"], 4.0 * U[:, 4:8].reshape(7, 2, 2))


def test_log_prob_prior():
    m = _model()
    rng = np.random.default_rng(1)
    U = rng.random((5, m.U_ndims))
    lp = np.asarray(m.log_prob_prior(U))
    X = m.transform_flat(U)
    want = (stats.uniform.logpdf(X[:, 0], -2.0, 5.0) + stats.norm.logpdf(X[:, 1:4], [0.0, 1.0, -1.0], 2.0).sum(1)
            + stats.uniform.logpdf(X[:, 4:8], 0.0, 4.0).sum(1) + stats.norm.logpdf(X[:, 8], 5.0, 0.5))
    np.testing.assert_allclose(lp, want, rtol=1e-12)
    import torch
    lp_t = m.log_prob_prior(torch.as_tensor(U))           # tensors in, tensors out
    assert isinstance(lp_t, torch.Tensor)
    np.testing.assert_allclose(lp_t.numpy(), want, rtol=1e-12)
    U_out = U.copy(); U_out[0, 0] = 1.0 + 1e-9          # outside the Uniform's support
    assert np.isneginf(m.log_prob_prior(U_out)[0])


def test_name_and_type_checks():
    def dup():
        yield gb.Prior(gb.Uniform(0.0, 1.0), name="x")
        yield gb.Prior(gb.Uniform(0.0, 1.0), name="x")
    with pytest.raises(gb.InvalidPriorName):
        gb.Model(dup, gb.MultivariateNormalLikelihood(np.zeros(2), np.eye(2)))

    def not_prior():
        yield 3.0
    with pytest.raises(ValueError):
        gb.Model(not_prior, gb.MultivariateNormalLikelihood(np.zeros(1), np.eye(1)))
    with pytest.raises(ValueError):
        gb.Prior(object(), name="z")


def test_likelihood_dimension_check():
    def pm():
        yield gb.Prior(gb.Uniform(np.zeros(3), np.ones(3)), name="x")
    with pytest.raises(Exception):
        gb.Model(pm, gb.MultivariateNormalLikelihood(np.zeros(4), np.eye(4)))


def test_multivariate_normal_tril_prior_and_fold():
    """MultivariateNormalTriL prior: X = loc + L ndtri(U), log density of N(loc, L L^T), and the
    folded correlated-Gaussian parameters give the likelihood of X exactly (FP64), mixed with a
    Uniform block ahead of it."""
    from scipy.special import ndtri
    from scipy.stats import multivariate_normal
    import jaxns_gb300 as gb
    rng = np.random.default_rng(0)
    D = 5
    A = rng.standard_normal((D, D))
    Lp = np.linalg.cholesky(A @ A.T / D + 0.3 * np.eye(D))
    loc = rng.standard_normal(D)
    mu = rng.standard_normal(D + 2)
    B = rng.standard_normal((D + 2, D + 2))
    cov = B @ B.T / D + 0.2 * np.eye(D + 2)

    def prior_model():
        a = yield gb.Prior(gb.Uniform(-2.0 * np.ones(2), 3.0 * np.ones(2)), name="a")
        x = yield gb.Prior(gb.MultivariateNormalTriL(loc, Lp), name="x")
        return a, x

    lik = gb.MultivariateNormalLikelihood(mu, cov)
    m = gb.Model(prior_model, lik)
    U = rng.uniform(0.05, 0.95, size=(50, D + 2))
    X = np.concatenate([-2.0 + 5.0 * U[:, :2], loc + ndtri(U[:, 2:]) @ Lp.T], 1)
    np.testing.assert_allclose(m.transform_flat(U), X, rtol=0, atol=1e-12)
    lp = np.log(1 / 5.0) * 2 + multivariate_normal(loc, Lp @ Lp.T).logpdf(X[:, 2:])
    np.testing.assert_allclose(m.log_prob_prior(U), lp, rtol=1e-10)
    # folded parameters, evaluated in FP64 on the kernels' per-dimension quantile outputs q
    A_, c_ = m.affine()
    Linv = np.linalg.inv(np.linalg.cholesky(cov))
    mu_q = np.linalg.solve(A_, mu - c_)
    q = np.concatenate([X[:, :2], ndtri(U[:, 2:])], 1)
    z = (q - mu_q) @ np.tril(Linv @ A_).T
    logL = -0.5 * np.sum(z * z, 1) + lik.log_L_offset()
    np.testing.assert_allclose(logL, multivariate_normal(mu, cov).logpdf(X), rtol=1e-9)
    p = m.family_params()  # the same fold, packed in fp32 for the device
    np.testing.assert_allclose(p[:D + 2], mu_q, rtol=1e-5, atol=1e-5)
    with pytest.raises(NotImplementedError):
        gb.Model(prior_model, gb.GaussianShellsLikelihood(np.zeros(D + 2), np.ones(D + 2), 1.0, 0.1)).family_params()
