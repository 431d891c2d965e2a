"""MultivariateNormalTriL priors on the GPU (framework/wrapped_tfp_distribution.py:77-84: the
standard normal quantile per dimension, then loc + L z).  With a correlated-Gaussian likelihood
the prior's triangular factor folds into the likelihood's, so the kernels run a correlated
Gaussian in z-space; these tests check that fold against the FP64 oracle, which applies the
prior map itself, and run the reference's own basic_mvn problem (tests/conftest.py:217-250,
the setting of benchmarks/gh168/main.py) against its analytic evidence."""
import numpy as np
import pytest

from tests.conftest import assert_shell_exact

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _basic_mvn(gb, D=8, prior_L=None):
    prior_mu = 15.0 * np.ones(D)
    prior_cov = np.eye(D)
    data_mu = np.zeros(D)
    data_cov = np.where(np.eye(D) == 1, 1.0, 0.99)
    L = np.linalg.cholesky(prior_cov) if prior_L is None else prior_L

    def prior_model():
        x = yield gb.Prior(gb.MultivariateNormalTriL(prior_mu, L), name="x")
        return x

    model = gb.Model(prior_model, gb.MultivariateNormalLikelihood(data_mu, data_cov))
    S = prior_cov + data_cov if prior_L is None else L @ L.T + data_cov
    diff = data_mu - prior_mu
    log_Z = float(-0.5 * diff @ np.linalg.solve(S, diff) - 0.5 * np.linalg.slogdet(2 * np.pi * S)[1])
    return model, prior_mu, L, data_mu, data_cov, log_Z


def test_tril_forward_matches_oracle(gpu_lib, oracle_mod):
    import jaxns_gb300 as gb
    from jaxns_gb300.engine import NSBatch
    rng = np.random.default_rng(4)
    D = 6
    A = rng.standard_normal((D, D))
    Lp = np.linalg.cholesky(A @ A.T / D + 0.5 * np.eye(D))  # a general lower-triangular prior factor
    model, loc, L, mu, cov, _ = _basic_mvn(gb, D, Lp)
    ns = gb.NestedSampler(model, num_live_points=64)
    spec = ns.nested_sampler.run_spec(gb.random.PRNGKey(0), ns.normalise_term_cond(None))
    b = NSBatch([spec])
    U = rng.uniform(0.05, 0.95, size=(300, D))
    got = b.forward(0, torch.tensor(U, dtype=torch.float32)).cpu().numpy()
    om = oracle_mod.mvn_tril_prior_model(loc, L, mu, cov)
    ref = oracle_mod.forward(om, U.astype(np.float32).astype(np.float64))
    np.testing.assert_allclose(got, ref, rtol=2e-4, atol=5e-3)
    # the model's own X map and prior density are the reference's
    from scipy.special import ndtri
    from scipy.stats import multivariate_normal
    X = loc + ndtri(U) @ L.T
    np.testing.assert_allclose(model.transform(U)["x"], X, rtol=0, atol=1e-12)
    np.testing.assert_allclose(model.log_prob_prior(U), multivariate_normal(loc, L @ L.T).logpdf(X), rtol=1e-10)


def test_tril_shell_parity(gpu_lib, oracle_mod):
    """One shell under the TriL prior: bit for bit the fp32 oracle of the folded model, and
    within fp32 rounding of the FP64 oracle that applies the prior map."""
    import jaxns_gb300 as gb
    from jaxns_gb300.engine import NSBatch
    model, loc, L, mu, cov, _ = _basic_mvn(gb)
    ns = gb.NestedSampler(model, num_live_points=256, num_slices=32)
    spec = ns.nested_sampler.run_spec(gb.random.PRNGKey(3), ns.normalise_term_cond(None))
    b = NSBatch([spec])
    b.init()
    b.iterate(4)  # move the contour towards the likelihood's mode
    torch.cuda.synchronize()
    live = b.live_view(0)
    s = spec.shell_size
    Ls_raw = float(live["log_L_raw"][s - 1].item())
    key = gb.random.PRNGKey(77)
    b.slice_shell(torch.tensor([Ls_raw]), torch.tensor(np.asarray(key).view(np.int32)).view(1, 2))
    torch.cuda.synchronize()
    U3, L3, E3 = assert_shell_exact(oracle_mod, b, 0, Ls_raw, key)
    om = oracle_mod.mvn_tril_prior_model(loc, L, mu, cov)
    U_o, L_o, E_o = oracle_mod.slice_shell(om, key, float(live["log_L"][s - 1].item()), live["U"].cpu().double().numpy(),
                                           live["log_L"].cpu().double().numpy(), s, 32)
    same = (E3 == E_o) & np.all(np.abs(U3 - U_o) < 2e-4, axis=1)
    assert same.mean() >= 0.9, same.mean()


def test_basic_mvn_log_Z(gpu_lib):
    """The reference's basic_mvn problem with NestedSampler's defaults (max_samples = 1e5):
    D = 8, prior N(15, I), likelihood N(0, Sigma) with 0.99 correlations."""
    import jaxns_gb300 as gb
    model, *_, log_Z = _basic_mvn(gb)
    ns = gb.NestedSampler(model, max_samples=100000)
    reason, state = ns(gb.random.PRNGKey(42))
    res = ns.to_results(reason, state)
    assert abs(res.log_Z_mean - log_Z) < 4 * res.log_Z_uncert + 0.05, (res.log_Z_mean, res.log_Z_uncert, log_Z)
    post = np.average(res.samples["x"].cpu().numpy(), axis=0,
                      weights=np.exp(res.log_dp_mean.cpu().numpy() - res.log_dp_mean.max().item()))
    # posterior mean of the conjugate pair: Sigma_d (Sigma_p + Sigma_d)^-1 mu_p (data mean 0)
    D = 8
    Sp, Sd = np.eye(D), np.where(np.eye(D) == 1, 1.0, 0.99)
    exact = Sd @ np.linalg.solve(Sp + Sd, 15.0 * np.ones(D))
    assert np.max(np.abs(post - exact)) < 0.15, (post, exact)
