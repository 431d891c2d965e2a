"""Device sample_evidence against the FP64 oracle on a real run's samples."""
import numpy as np
import pytest

from tests.conftest import corr_gauss

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_sample_evidence_device_matches_oracle(gpu_lib, oracle_mod):
    import jaxns_gb300 as gb
    D = 3
    mu, cov = corr_gauss(D, seed=5)

    def prior_model():
        x = yield gb.Prior(gb.Uniform(-10.0 * np.ones(D), 10.0 * np.ones(D)), name="x")
        return x

    ns = gb.NestedSampler(gb.Model(prior_model, gb.MultivariateNormalLikelihood(mu, cov)), num_live_points=128,
                          num_slices=4 * D)
    reason, state = ns(gb.random.PRNGKey(3), gb.TerminationCondition(dlogZ=1e-4))
    res = ns.to_results(reason, state)
    key = gb.random.PRNGKey(99)
    got = gb.sample_evidence(key, res.num_live_points_per_sample, res.log_L_samples, S=64).cpu().numpy()
    ref = oracle_mod.sample_evidence(key, res.num_live_points_per_sample.cpu().numpy(),
                                     res.log_L_samples.cpu().numpy(), S=64)
    np.testing.assert_allclose(got, ref, rtol=0, atol=1e-9)
    assert abs(got.mean() - res.log_Z_mean) < 4 * got.std() / np.sqrt(64) + 0.05
    assert 0.5 < got.std() / res.log_Z_uncert < 2.0
