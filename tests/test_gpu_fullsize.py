"""The headline workload at its full size (1024 independent Gaussian-shells runs, D=10,
n=1000, 50 slices), checked through properties that do not depend on a reference run:
every run's samples sorted by log L, live-point counts between 1 and n + 1 ending at 1,
posterior weights summing to 1, termination by dlogZ, and log Z near the FP64 quadrature.

At the end of these runs the contour is within ~1e-6 of the shell radius, below what fp32 U
(x quantised to ~7e-7) and the fp32 radius sqrt(sum e^2) - R resolve: the top of the live set
collapses onto one or two fp32 values of log L, so the no-seed-points (and sometimes plateau)
bits fire with, or in ~2 % of runs just before, the dlogZ bit."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_shells_1024_runs_properties(gpu_lib):
    import jaxns_gb300 as gb
    from jaxns_gb300.batched import BatchedNestedSampler
    from jaxns_gb300.replicas import replica_keys
    from tests.test_gpu_ns import shells_log_Z
    D, R, n = 10, 1024, 1000
    c1 = np.zeros(D)
    c1[0] = 3.5

    def prior_model():
        x = yield gb.Prior(gb.Uniform(-6.0 * np.ones(D), 6.0 * np.ones(D)), name="x")
        return x

    model = gb.Model(prior_model, gb.GaussianShellsLikelihood(c1, -c1, 2.0, 0.1))
    samplers = [gb.NestedSampler(model, num_live_points=n, num_slices=5 * D, max_samples=100000) for _ in range(R)]
    bns = BatchedNestedSampler(samplers, replica_keys(0, R), [gb.TerminationCondition(dlogZ=1e-4)] * R)
    reasons = bns(from_host=False)
    assert np.all((reasons & ~(4 | 128 | 1024)) == 0), np.unique(reasons)
    assert np.mean((reasons & 4) != 0) >= 0.95, np.unique(reasons, return_counts=True)
    b = bns.batch
    out = b.results(with_U=False)
    sc = out["scalars"].cpu().numpy()
    st = b.state()
    offs = b.offsets["store"]
    L = out["log_L_samples"].cpu().numpy()
    nl = out["num_live_points"].cpu().numpy()
    dp = out["log_dp_mean"].cpu().numpy()
    for r in range(0, R, 7):  # every 7th run in full
        o, N = int(offs[r]), int(st["num_samples"][r])
        Lr, nr, dpr = L[o:o + N], nl[o:o + N], dp[o:o + N]
        assert np.all(np.diff(Lr) >= 0)
        assert nr.min() >= 1 and nr.max() <= n + 1 and nr[-1] == 1
        w = np.exp(dpr - dpr.max())
        assert abs(np.exp(np.log(w.sum()) + dpr.max()) - 1.0) < 1e-6
    truth = shells_log_Z()
    dz = sc[:, 0] - truth
    assert np.mean(np.abs(dz) < 5 * sc[:, 1]) >= 0.99
    assert abs(np.mean(dz)) < 0.06  # the reference algorithm's own bias here is ~+0.02-0.03
