"""NestedSampler's defaults and validation (public.py:69-137), host logic only: no kernel runs
until the sampler is called."""
import numpy as np
import pytest

gb = pytest.importorskip("jaxns_gb300")


def _model(D=3):
    def prior_model():
        x = yield gb.Prior(gb.Uniform(-10 * np.ones(D), 10 * np.ones(D)), name="x")
        return x
    return gb.Model(prior_model, gb.MultivariateNormalLikelihood(np.zeros(D), np.eye(D)))


def test_defaults():
    ns = gb.NestedSampler(_model(3))
    assert (ns.s, ns.num_slices, ns.k, ns.c, ns.max_samples) == (5, 15, 0, 90, 9000)
    assert ns.nested_sampler.sampler.midpoint_shrink and ns.nested_sampler.sampler.num_phantom_save == 0


def test_difficult_model():
    ns = gb.NestedSampler(_model(3), difficult_model=True)
    assert (ns.s, ns.num_slices, ns.c, ns.max_samples) == (10, 30, 300, 30000)
    assert not ns.nested_sampler.sampler.midpoint_shrink


def test_parameter_estimation_phantoms():
    ns = gb.NestedSampler(_model(3), parameter_estimation=True, num_live_points=100)
    # k = min(D, s D - 1) phantoms; c = num_live_points / (k + 1) chains; 100 shrinkages
    assert (ns.k, ns.c, ns.max_samples) == (3, 25, 25 * 4 * 100)
    assert ns.nested_sampler.sampler.num_phantom_save == 3


def test_explicit_values_and_gradient_guided():
    ns = gb.NestedSampler(_model(4), num_slices=7, num_live_points=64, max_samples=1234, gradient_guided=True)
    assert (ns.num_slices, ns.k, ns.c, ns.max_samples) == (7, 0, 64, 1234)
    assert ns.nested_sampler.sampler.gradient_guided


@pytest.mark.parametrize("kw", [{"s": 0}, {"k": 15}, {"k": -1}, {"c": 0}])
def test_invalid_arguments_raise(kw):
    with pytest.raises(ValueError):
        gb.NestedSampler(_model(3), **kw)


def test_post_analysis_utilities_attached():
    ns = gb.NestedSampler(_model(2))
    assert ns.save_results is gb.save_results and ns.load_results is gb.load_results


def test_batched_sampler_assembles_one_run_per_problem():
    from jaxns_gb300 import _ffi
    from jaxns_gb300.batched import BatchedNestedSampler
    samplers = [gb.NestedSampler(_model(D), num_live_points=20 * D) for D in (2, 5, 3)]
    keys = np.array([[0, 7], [1, 8], [2, 9]], np.uint32)
    tcs = [None, gb.TerminationCondition(dlogZ=0.5), gb.TerminationCondition(max_samples=500)]
    b = BatchedNestedSampler(samplers, keys, tcs, store_U=False, device="cpu")
    specs = b.batch.specs
    assert [s.D for s in specs] == [2, 5, 3] and [s.num_live_points for s in specs] == [40, 100, 60]
    for s, k in zip(specs, keys):
        np.testing.assert_array_equal(s.key, k)
        assert not s.store_U
    assert specs[0].term_cond["dlogZ"] == pytest.approx(np.log(1 + 1e-3))     # the default condition
    assert specs[1].term_cond["dlogZ"] == 0.5
    assert specs[2].term_cond["max_samples"] == 500                            # min(500, the sampler's cap)
    with pytest.raises(_ffi.GBNSError, match="no CPU path"):
        b()


@pytest.mark.parametrize("kw,exc", [({"num_slices": 0}, ValueError), ({"num_phantom_save": -1}, ValueError),
                                    ({"num_phantom_save": 5}, ValueError), ({"perfect": False}, ValueError),
                                    ({"adaptive_shrink": True}, NotImplementedError)])
def test_slice_sampler_validation(kw, exc):
    """samplers/uni_slice_sampler.py:276-326."""
    from jaxns_gb300.public import UniDimSliceSampler
    args = dict(model=_model(2), num_slices=5, num_phantom_save=0, midpoint_shrink=True, perfect=True)
    args.update(kw)
    with pytest.raises(exc):
        UniDimSliceSampler(**args)


def test_slice_sampler_gradient_options():
    """gradient_slice and gradient_guided reach the run spec for every family (the
    linear-Gaussian family takes them on its lock step)."""
    import jaxns_gb300 as gb
    from jaxns_gb300.public import ShardedStaticNestedSampler, UniDimSliceSampler
    m = _model(2)
    smp = UniDimSliceSampler(model=m, num_slices=5, num_phantom_save=0, midpoint_shrink=True, perfect=True,
                             gradient_slice=True)
    ns = ShardedStaticNestedSampler(model=m, max_samples=1000, init_efficiency_threshold=0.1, sampler=smp,
                                    num_live_points=20)
    spec = ns.run_spec(gb.random.PRNGKey(0), gb.TerminationCondition())
    assert spec.gradient_slice and not spec.gradient_guided
    Phi = np.ones((4, 2))

    def prior_model():
        w = yield gb.Prior(gb.Normal(np.zeros(2), np.ones(2)), name="w")
        return w

    lg = gb.Model(prior_model, gb.LinearGaussianLikelihood(Phi, np.ones(4), 0.5))
    smp = UniDimSliceSampler(model=lg, num_slices=5, num_phantom_save=0, midpoint_shrink=True, perfect=True,
                             gradient_guided=True)
    ns = ShardedStaticNestedSampler(model=lg, max_samples=1000, init_efficiency_threshold=0.1, sampler=smp,
                                    num_live_points=20)
    spec = ns.run_spec(gb.random.PRNGKey(0), gb.TerminationCondition())
    assert spec.gradient_guided and not spec.gradient_slice and spec.family == 2


def test_static_sampler_rounding():
    """sharded_static.py:577-594, :625-650: shell fraction at least 1/n, store capacity a
    multiple of one shell with its phantoms."""
    from jaxns_gb300.public import ShardedStaticNestedSampler, UniDimSliceSampler
    m = _model(2)
    sl = UniDimSliceSampler(model=m, num_slices=6, num_phantom_save=2, midpoint_shrink=True, perfect=True)
    ss = ShardedStaticNestedSampler(model=m, max_samples=1001, init_efficiency_threshold=0.1, sampler=sl,
                                    num_live_points=50)
    assert ss.shell_fraction == 0.5 and ss.num_live_points == 50
    assert ss.max_samples == 1050          # 25 discards x (1 + 2 phantoms) = 75 per shell
    one = ShardedStaticNestedSampler(model=m, max_samples=10, init_efficiency_threshold=0.1, sampler=sl,
                                     num_live_points=4, shell_fraction=0.1)
    assert one.shell_fraction == 0.25      # at least one discard per shell
    with pytest.raises(ValueError):
        ShardedStaticNestedSampler(model=m, max_samples=10, init_efficiency_threshold=0.1, sampler=sl,
                                   num_live_points=4, shell_fraction=1.5)


def test_termination_condition_fields_and_struct():
    """Every field of TerminationCondition reaches the device struct with its has_ flag."""
    from jaxns_gb300.engine import term_cond_struct
    from jaxns_gb300.public import TerminationConditionConjunction, TerminationConditionDisjunction
    tc = gb.TerminationCondition(ess=100, evidence_uncert=0.1, dlogZ=0.01, max_samples=1e4,
                                 max_num_likelihood_evaluations=1e6, log_L_contour=-3.0, efficiency_threshold=0.05,
                                 rtol=1e-3, atol=1e-4, peak_XL_frac=0.2)
    s = term_cond_struct(tc.as_dict())
    for flag, field, v in [("has_ess", "ess", 100), ("has_evidence_uncert", "evidence_uncert", 0.1),
                           ("has_dlogZ", "dlogZ", 0.01), ("has_max_samples", "max_samples", 1e4),
                           ("has_max_nlik", "max_nlik", 1e6), ("has_log_L_contour", "log_L_contour", -3.0),
                           ("has_efficiency", "efficiency_threshold", 0.05), ("has_rtol", "rtol", 1e-3),
                           ("has_atol", "atol", 1e-4), ("has_peak_XL", "peak_XL_frac", 0.2)]:
        assert getattr(s, flag) == 1 and getattr(s, field) == pytest.approx(v), field
    empty = term_cond_struct(gb.TerminationCondition().as_dict())
    assert empty.has_dlogZ == 0 and empty.has_max_samples == 0
    with pytest.warns(UserWarning):
        assert "live_evidence_frac" not in gb.TerminationCondition(live_evidence_frac=0.1).as_dict()
    assert isinstance(tc & tc, TerminationConditionConjunction) and isinstance(tc | tc, TerminationConditionDisjunction)
    ns = gb.NestedSampler(_model(2))
    with pytest.raises(TypeError):
        ns.normalise_term_cond(tc | tc)
    norm = ns.normalise_term_cond(gb.TerminationCondition(dlogZ=0.1))
    assert norm.max_samples == ns.nested_sampler.max_samples and norm.dlogZ == 0.1
