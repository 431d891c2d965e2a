"""End-to-end GPU nested sampling against the oracle and analytic evidences."""
import numpy as np
import pytest

from tests.conftest import corr_gauss

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _mvn_model(gb, D, seed, low=-10.0, high=10.0):
    mu, cov = corr_gauss(D, seed)

    def prior_model():
        x = yield gb.Prior(gb.Uniform(low * np.ones(D), high * np.ones(D)), name="x")
        return x

    return gb.Model(prior_model, gb.MultivariateNormalLikelihood(mu, cov)), mu, cov


def shells_log_Z(D=10, R=2.0, w=0.1, box=12.0):
    from scipy import integrate, special
    S = 2 * np.pi ** (D / 2) / special.gamma(D / 2)
    f = lambda r: r ** (D - 1) * np.exp(-0.5 * ((r - R) / w) ** 2) / np.sqrt(2 * np.pi * w * w)
    I, _ = integrate.quad(f, max(0.0, R - 12 * w), R + 12 * w, epsabs=0, epsrel=1e-12)
    return np.log(2 * S * I) - D * np.log(box)


def test_one_iteration_matches_oracle(gpu_lib, oracle_mod):
    import jaxns_gb300 as gb
    from jaxns_gb300.engine import NSBatch
    D, n = 8, 512
    model, mu, cov = _mvn_model(gb, D, 0)
    ns = gb.NestedSampler(model, num_live_points=n, num_slices=32)
    key = gb.random.PRNGKey(3)
    spec = ns.nested_sampler.run_spec(key, ns.normalise_term_cond(gb.TerminationCondition(dlogZ=1e-4)))
    b = NSBatch([spec])
    b.init()
    b.iterate(1)
    torch.cuda.synchronize()
    st = b.state()[0]
    om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    o = oracle_mod.ns_run(om, key, n, 32, max_samples=spec.max_samples, term_cond={"dlogZ": 1e-4},
                          max_iterations=1)
    s = n // 2
    assert int(st["num_samples"]) == s
    np.testing.assert_array_equal(np.array(st["key"], np.uint32), o.register["key"])
    # the discarded shell (identical initial live set) and its evidence register
    sv = b.store_view(0)
    np.testing.assert_array_equal(sv["sender"][:s].cpu().numpy(), 0)
    np.testing.assert_allclose(sv["log_L"][:s].cpu().numpy(), o.log_L[:s], rtol=2e-4, atol=2e-3)
    np.testing.assert_array_equal(sv["nevals"][:s].cpu().numpy(), o.nevals[:s])
    for f in ("log_X_mean", "log_X2_mean", "log_Z_mean", "log_ZX_mean", "log_Z2_mean", "log_dZ2_mean"):
        assert abs(st["ev"][f] - o.register["ev"][f]) < 1e-4 * max(1.0, abs(o.register["ev"][f])), f
    assert int(st["iterations"]) == 1


def test_results_on_gpu_store_match_oracle(gpu_lib, oracle_mod):
    """to_results on the GPU's own store vs the oracle's restatement on the same store:
    sample order and live-point counts bit-exact, FP64 evidence within 1e-6."""
    import jaxns_gb300 as gb
    D = 6
    model, mu, cov = _mvn_model(gb, D, 1)
    ns = gb.NestedSampler(model, num_live_points=300, num_slices=3 * D)
    reason, state = ns(gb.random.PRNGKey(11), gb.TerminationCondition(dlogZ=1e-4))
    res = ns.to_results(reason, state)
    sc = state.sample_collection
    sender = sc.sender_node_idx.cpu().numpy()
    L = sc.log_L.cpu().numpy()  # absolute log L (device fp32 + FP64 offset)
    si, nl = oracle_mod.count_crossed_edges(sender, L)
    np.testing.assert_array_equal(res.num_live_points_per_sample.cpu().numpy(), nl)
    ls = L[si]
    np.testing.assert_array_equal(res.log_L_samples.cpu().numpy(), ls)
    fin, per = oracle_mod.compute_evidence_stats(ls, nl.astype(np.float64))
    mu_o, var_o = oracle_mod.linear_to_log_stats(fin["log_Z_mean"], fin["log_Z2_mean"])
    assert abs(res.log_Z_mean - mu_o) < 1e-6
    assert abs(res.log_Z_uncert - np.sqrt(var_o)) < 1e-6
    np.testing.assert_allclose(res.log_X_mean.cpu().numpy(), per["log_X_mean"], rtol=1e-12, atol=1e-9)
    assert res.total_num_samples == len(L)
    assert res.total_num_likelihood_evaluations == int(sc.num_likelihood_evaluations.sum())


def test_config1_log_Z(gpu_lib):
    """D=8 correlated Gaussian in U[-10,10]^8, 512 live points, 32 slices, dlogZ < 1e-4."""
    import jaxns_gb300 as gb
    D = 8
    model, mu, cov = _mvn_model(gb, D, 0)
    ns = gb.NestedSampler(model, num_live_points=512, num_slices=32)
    truth = -D * np.log(20.0)
    zs = []
    for seed in range(4):
        reason, state = ns(gb.random.PRNGKey(seed), gb.TerminationCondition(dlogZ=1e-4))
        res = ns.to_results(reason, state)
        assert reason == 4
        assert abs(res.log_Z_mean - truth) < 4 * res.log_Z_uncert
        zs.append(res.log_Z_mean)
        # posterior mean of x against mu (the Gaussian lies well inside the box)
        w = torch.exp(res.log_dp_mean).cpu().numpy()
        xm = (w[:, None] * res.samples["x"].cpu().numpy()).sum(0)
        assert np.all(np.abs(xm - mu) < 0.2)
    assert abs(np.mean(zs) - truth) < 3 * 0.25 / np.sqrt(len(zs))


def test_graph_replay_equals_eager(gpu_lib):
    from jaxns_gb300.engine import NSBatch
    import jaxns_gb300 as gb
    D = 5
    model, _, _ = _mvn_model(gb, D, 2)
    ns = gb.NestedSampler(model, num_live_points=100, num_slices=10)
    spec = ns.nested_sampler.run_spec(gb.random.PRNGKey(5), ns.normalise_term_cond(None))
    a, b = NSBatch([spec]), NSBatch([spec])
    a.run(block=4, use_graph=True)
    b.run(block=4, use_graph=False)
    sa, sb = a.store_view(0), b.store_view(0)
    for k in ("log_L", "sender", "nevals"):
        assert torch.equal(sa[k], sb[k]), k


def test_batched_uneven_runs(gpu_lib):
    """Independent runs with different D, n and store sizes in one batch."""
    from jaxns_gb300.engine import NSBatch, RunSpec, mvn_offset, mvn_params
    specs = []
    Ds = [2, 3, 5, 8, 11, 16, 20, 33]
    for r, D in enumerate(Ds):
        mu, cov = corr_gauss(D, 100 + r)
        n = 25 * D
        s = n // 2
        cap = int(np.ceil(n * (3 * D + 25) / s)) * s
        specs.append(RunSpec(D=D, num_live_points=n, shell_size=s, num_slices=3 * D, family=0,
                             params=mvn_params(mu, cov), prior_kind=np.zeros(D, np.int32),
                             prior_a=np.full(D, -10.0), prior_b=np.full(D, 20.0), max_samples=cap,
                             term_cond={"dlogZ": 1e-4, "max_samples": float(cap)},
                             key=gb_key(r), store_U=False, log_L_offset=mvn_offset(cov)))
    b = NSBatch(specs)
    st = b.run(block=8)
    out = b.results(with_U=False)
    sc = out["scalars"].cpu().numpy()
    for r, D in enumerate(Ds):
        truth = -D * np.log(20.0)
        assert abs(sc[r, 0] - truth) < 4 * sc[r, 1] + 0.05, (D, sc[r, 0], sc[r, 1], truth)
        assert st["termination_reason"][r] & 4


def gb_key(r):
    from jaxns_gb300 import random
    return random.PRNGKey(1000 + r)


def test_config2_shells(gpu_lib):
    """D=10 Gaussian shells in U[-6,6]^10, 1000 live points, 50 slices: log Z vs FP64 quadrature."""
    pytest.importorskip("scipy")
    import jaxns_gb300 as gb
    D = 10
    c1 = np.zeros(D)
    c1[0] = 3.5

    def prior_model():
        x = yield gb.Prior(gb.Uniform(-6.0 * np.ones(D), 6.0 * np.ones(D)), name="x")
        return x

    model = gb.Model(prior_model, gb.GaussianShellsLikelihood(c1, -c1, 2.0, 0.1))
    ns = gb.NestedSampler(model, num_live_points=1000, num_slices=50)
    reason, state = ns(gb.random.PRNGKey(0), gb.TerminationCondition(dlogZ=1e-4))
    res = ns.to_results(reason, state)
    truth = shells_log_Z()
    assert abs(res.log_Z_mean - truth) < 4 * res.log_Z_uncert + 0.05, (res.log_Z_mean, res.log_Z_uncert, truth)


def test_phantoms_one_iteration_match_oracle(gpu_lib, oracle_mod):
    """k = 3 phantoms per chain (uni_slice_sampler.py:430-441, add_phantom_samples_to_state
    sharded_static.py:181-207): after one iteration the store holds the discarded shell and then
    s*k phantoms (phantom flag set, sender = the shell's sender), matching the oracle."""
    import jaxns_gb300 as gb
    from jaxns_gb300.engine import NSBatch
    D, n, S, K = 4, 256, 20, 3
    model, mu, cov = _mvn_model(gb, D, 1)
    ns = gb.NestedSampler(model, num_live_points=n * (K + 1), num_slices=S, k=K)
    key = gb.random.PRNGKey(5)
    spec = ns.nested_sampler.run_spec(key, ns.normalise_term_cond(gb.TerminationCondition(dlogZ=1e-4)))
    assert spec.num_phantom == K and spec.num_live_points == n
    b = NSBatch([spec])
    b.init()
    b.iterate(1)
    torch.cuda.synchronize()
    st = b.state()[0]
    s = n // 2
    assert int(st["num_samples"]) == s * (1 + K)
    sv = b.store_view(0)
    ph = sv["phantom"].cpu().numpy()
    np.testing.assert_array_equal(ph[:s], 0)
    np.testing.assert_array_equal(ph[s:s * (1 + K)], 1)
    np.testing.assert_array_equal(sv["nevals"][s:s * (1 + K)].cpu().numpy(), 0)
    om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    o = oracle_mod.ns_run(om, key, n, S, max_samples=spec.max_samples, num_phantom=K, term_cond={"dlogZ": 1e-4},
                          max_iterations=1)
    gL = sv["log_L"][s:s * (1 + K)].cpu().numpy()
    oL = o.log_L[s:s * (1 + K)]
    close = np.abs(gL - oL) <= 2e-3 + 2e-4 * np.abs(oL)
    assert close.mean() >= 0.9, close.mean()
    np.testing.assert_array_equal(np.array(st["key"], np.uint32), o.register["key"])


def test_parameter_estimation_and_difficult_model_log_Z(gpu_lib):
    """parameter_estimation (k = D phantoms) and difficult_model (no midpoint shrink, s = 10):
    log Z within 4 sigma of the analytic value; phantom count = k / (k + 1) of the samples."""
    import jaxns_gb300 as gb
    D = 4
    truth = -D * np.log(20.0)
    for kw in (dict(parameter_estimation=True), dict(difficult_model=True)):
        model, _, _ = _mvn_model(gb, D, 2)
        ns = gb.NestedSampler(model, num_live_points=400, **kw)
        reason, state = ns(gb.random.PRNGKey(8), gb.TerminationCondition(dlogZ=1e-4))
        res = ns.to_results(reason, state)
        assert abs(res.log_Z_mean - truth) < 4 * res.log_Z_uncert + 0.02, (kw, res.log_Z_mean, res.log_Z_uncert)
        if kw.get("parameter_estimation"):
            k = D
            assert res.total_phantom_samples > 0
            assert abs(res.total_phantom_samples / res.total_num_samples - k / (k + 1)) < 0.05


def test_peak_XL_frac_termination_matches_oracle(gpu_lib, oracle_mod):
    """TerminationCondition(peak_XL_frac) (termination.py:140-146): same iteration count and
    termination bit as the oracle."""
    import jaxns_gb300 as gb
    from jaxns_gb300.engine import NSBatch
    D, n = 3, 128
    model, mu, cov = _mvn_model(gb, D, 4)
    ns = gb.NestedSampler(model, num_live_points=n, num_slices=4 * D)
    key = gb.random.PRNGKey(12)
    tc = gb.TerminationCondition(peak_XL_frac=0.01)
    spec = ns.nested_sampler.run_spec(key, ns.normalise_term_cond(tc))
    b = NSBatch([spec])
    st = b.run(block=4)
    om = oracle_mod.mvn_model(-10 * np.ones(D), 10 * np.ones(D), mu, cov)
    o = oracle_mod.ns_run(om, key, n, 4 * D, max_samples=spec.max_samples, term_cond={"peak_XL_frac": 0.01})
    assert int(st["termination_reason"][0]) & 2048
    assert int(o.termination_reason) & 2048
    assert abs(int(st["iterations"][0]) - int(o.iterations)) <= 1
