"""The deep-tail limit of the slice sampler belongs to the reference algorithm.

For a linear-regression evidence whose posterior sits far out in a Normal prior's tail, the
constrained region in U-space is many orders of magnitude thinner along that axis, random-
direction slice moves shrink to that width and the chains stop mixing.  The FP64 CPU oracle
(the reference algorithm restated, no fp32 or TF32 anywhere) shows the same failure as the
GPU runs: its log Z ensemble is unbiased with the posterior within 2 prior standard
deviations, single runs start to stray at 3.5, and from 4.5 on the ensemble is biased far
beyond its stated uncertainty with single runs off by many sigma.
"""
import numpy as np
import pytest


def _analytic_log_Z(Phi, y, sigma, tau):
    """log N(y; 0, sigma^2 I + tau^2 Phi Phi^T)."""
    N = len(y)
    C = sigma ** 2 * np.eye(N) + tau ** 2 * Phi @ Phi.T
    _, logdet = np.linalg.slogdet(C)
    return -0.5 * (y @ np.linalg.solve(C, y) + logdet + N * np.log(2 * np.pi))


def _ensemble(o, depth, seeds=8):
    g = np.random.default_rng(0)
    N, sigma, tau = 40, 0.2, 1.0
    Phi = g.standard_normal((N, 2))
    y = Phi @ np.array([depth * tau, 0.3]) + sigma * g.standard_normal(N)
    m = o.lingauss_model(Phi, y, sigma, tau)
    runs = [o.ns_run(m, o.PRNGKey(s), num_live_points=100, num_slices=10, max_samples=20000,
                     term_cond={"dlogZ": 1e-3}) for s in range(seeds)]
    err = np.array([r.results["log_Z_mean"] for r in runs]) - _analytic_log_Z(Phi, y, sigma, tau)
    unc = np.array([r.results["log_Z_uncert"] for r in runs])
    return err, unc


@pytest.mark.parametrize("depth", [0.5, 2.0])
def test_oracle_unbiased_within_the_prior_bulk(oracle_mod, depth):
    err, unc = _ensemble(oracle_mod, depth)
    assert abs(err.mean()) < 3 * unc.mean() / np.sqrt(len(err)), (depth, err, unc)
    assert np.all(np.abs(err) < 4 * unc)


def test_oracle_onset_at_three_and_a_half_sigma(oracle_mod):
    """At 3.5 prior sigma the ensemble mean still holds, single runs start to stray."""
    err, unc = _ensemble(oracle_mod, 3.5)
    assert abs(err.mean()) < 3 * unc.mean() / np.sqrt(len(err)), (err, unc)


@pytest.mark.parametrize("depth", [4.5, 5.5, 6.5])
def test_oracle_biased_deep_in_the_prior_tail(oracle_mod, depth):
    err, unc = _ensemble(oracle_mod, depth)
    assert abs(err.mean()) > 5 * unc.mean() / np.sqrt(len(err)), (depth, err, unc)
    assert np.max(np.abs(err) / unc) > 8, (depth, err, unc)


def _exact_sampling_ns(o, seed, D, n, iters=50):
    """The static-shell loop of _collect_shell (discard the lowest n/2, sender = the last
    discarded node, sorted live set) with exact, independent sampling above the contour in
    place of the slice chains: for a Gaussian likelihood {L > L*} is an ellipsoid, sampled
    uniformly through a ball (rejecting the rare points outside the prior box).  The samples
    go through the oracle's tree count and FP64 evidence statistics."""
    g = np.random.default_rng(5000 + seed)
    mu = np.linspace(-0.5, 0.5, D)
    A = np.random.default_rng(7).standard_normal((D, D))
    C = np.linalg.cholesky(A @ A.T / D + 0.1 * np.eye(D))
    Ci = np.linalg.inv(C)
    c0 = -np.sum(np.log(np.diag(C))) - 0.5 * D * np.log(2 * np.pi)

    def logL(x):
        z = (x - mu) @ Ci.T
        return c0 - 0.5 * np.sum(z * z, -1)

    def sample_above(Lstar, k):
        out = []
        while len(out) < k:
            if np.isfinite(Lstar):
                v = g.standard_normal((4 * k, D))
                v /= np.linalg.norm(v, axis=1, keepdims=True)
                x = mu + (v * np.sqrt(-2.0 * (Lstar - c0)) * g.random((4 * k, 1)) ** (1.0 / D)) @ C.T
            else:
                x = g.uniform(-10, 10, (4 * k, D))
            x = x[np.all(np.abs(x) <= 10, axis=1)]
            out.extend(x[logL(x) > Lstar] if np.isfinite(Lstar) else x)
        return np.array(out[:k])

    s = n // 2
    L = np.sort(logL(sample_above(-np.inf, n)))
    node = np.zeros(n, np.int64)
    SL, SS = [], []
    for _ in range(iters):
        SL.extend(L[:s])
        SS.extend(node[:s])
        sender, Lstar = len(SL), L[s - 1]
        L = np.concatenate([logL(sample_above(Lstar, s)), L[s:]])
        node = np.concatenate([np.full(s, sender), node[s:]])
        order = np.argsort(L, kind="stable")
        L, node = L[order], node[order]
    SL.extend(L)
    SS.extend(node)
    idx, nl = o.count_crossed_edges(np.array(SS), np.array(SL))
    fin, _ = o.compute_evidence_stats(np.array(SL)[idx], nl.astype(float))
    log_Z = 2 * fin["log_Z_mean"] - 0.5 * fin["log_Z2_mean"]
    return log_Z + D * np.log(20.0), np.sqrt(fin["log_Z2_mean"] - 2 * fin["log_Z_mean"])


@pytest.mark.parametrize("D", [2, 8])
def test_evidence_accounting_unbiased_with_exact_sampling(oracle_mod, D):
    """With independent samples the static-shell accounting (tree counts, FP64 recurrence) is
    unbiased and its stated uncertainty matches the run-to-run scatter; the positive bias of the
    slice-sampled runs at the same settings (+0.09 at D = 2, +0.18 at D = 8 over large oracle
    ensembles) therefore belongs to the slice sampler's correlated chains, not to the evidence."""
    res = np.array([_exact_sampling_ns(oracle_mod, k, D, 50 * D) for k in range(100)])
    err, unc = res[:, 0], res[:, 1]
    assert abs(err.mean()) < 3 * err.std(ddof=1) / np.sqrt(len(err)), (D, err.mean())
    assert 0.7 < err.std() / unc.mean() < 1.3, (D, err.std(), unc.mean())
