"""determine_termination (nested_samplers/common/termination.py:13-147): each condition and
its bit, on hand-built registers, against the rules as the reference states them; and the
reference's own round-up goldens (nested_samplers/sharded/tests/test_sharded_static.py:4-7)."""
import math

import numpy as np
import pytest


def _ev(log_Z_mean=-1.0, log_Z2_mean=-2.0, log_X_mean=-5.0, log_L=-1.0, log_dZ2_mean=-3.0):
    return dict(log_L=log_L, log_X_mean=log_X_mean, log_X2_mean=2 * log_X_mean, log_Z_mean=log_Z_mean,
                log_ZX_mean=-10.0, log_Z2_mean=log_Z2_mean, log_dZ_mean=-4.0, log_dZ2_mean=log_dZ2_mean)


def _reg(**kw):
    r = dict(num_samples_used=100, ev=_ev(), ev_rem=_ev(), num_likelihood_evaluations=1000, log_L_contour=-3.0,
             efficiency=0.5, plateau=0, no_seed_points=0, relative_spread=1.0, absolute_spread=1.0,
             peak_log_XL=-100.0)
    r.update(kw)
    return r


def _mu_var(f, f2):
    mu = 2 * f - 0.5 * f2
    return mu, max(f2 - 2 * f, 2.220446049250313e-16)


@pytest.mark.parametrize("tc,reg,bit,expect", [
    ({"max_samples": 100}, {}, 0, True),
    ({"max_samples": 101}, {}, 0, False),
    ({"evidence_uncert": 0.5}, {"ev_rem": _ev(log_Z_mean=-1.0, log_Z2_mean=-1.9)}, 1, True),    # var 0.1 <= 0.25
    ({"evidence_uncert": 0.2}, {"ev_rem": _ev(log_Z_mean=-1.0, log_Z2_mean=-1.9)}, 1, False),   # var 0.1 > 0.04
    ({"dlogZ": 0.1}, {"ev_rem": _ev(log_Z_mean=-0.95, log_Z2_mean=-1.9)}, 2, True),
    ({"dlogZ": 0.01}, {"ev_rem": _ev(log_Z_mean=-0.9, log_Z2_mean=-1.8)}, 2, False),
    ({"ess": 5.0}, {"ev_rem": _ev(log_Z_mean=0.0, log_dZ2_mean=-2.0)}, 3, True),                # exp(2*0+2) = 7.4
    ({"ess": 10.0}, {"ev_rem": _ev(log_Z_mean=0.0, log_dZ2_mean=-2.0)}, 3, False),
    ({"max_num_likelihood_evaluations": 1000}, {}, 4, True),
    ({"max_num_likelihood_evaluations": 1001}, {}, 4, False),
    ({"log_L_contour": -3.0}, {}, 5, True),
    ({"log_L_contour": -2.9}, {}, 5, False),
    ({"efficiency_threshold": 0.6}, {}, 6, True),
    ({"efficiency_threshold": 0.5}, {}, 6, False),
    ({}, {"plateau": 1}, 7, True),
    ({"rtol": 1.5}, {}, 8, True),
    ({"rtol": 1.0}, {}, 8, False),
    ({"atol": 1.5}, {}, 9, True),
    ({"atol": 0.5}, {}, 9, False),
    ({}, {"no_seed_points": 1}, 10, True),
    ({"peak_XL_frac": 0.5}, {"peak_log_XL": -5.0}, 11, True),    # log_X + log_L = -6 < -5 + log 0.5
    ({"peak_XL_frac": 0.5}, {"peak_log_XL": -5.9}, 11, False),   # -6 >= -5.9 - 0.69
])
def test_each_condition_sets_its_bit(oracle_mod, tc, reg, bit, expect):
    done, reason = oracle_mod.determine_termination(tc, _reg(**reg))
    assert bool(reason & (1 << bit)) == expect, (tc, reason)
    assert done == (reason != 0)


def test_dlogZ_rule_is_difference_of_log_means(oracle_mod):
    """dlogZ fires when E[log Z with remaining] - E[log Z] < dlogZ (termination.py:84-96)."""
    ev0, ev1 = _ev(log_Z_mean=-1.0, log_Z2_mean=-1.95), _ev(log_Z_mean=-0.97, log_Z2_mean=-1.9)
    m0, _ = _mu_var(ev0["log_Z_mean"], ev0["log_Z2_mean"])
    m1, _ = _mu_var(ev1["log_Z_mean"], ev1["log_Z2_mean"])
    gap = m1 - m0
    for dlogZ, expect in ((gap + 1e-9, True), (gap - 1e-9, False)):
        _, reason = oracle_mod.determine_termination({"dlogZ": dlogZ}, _reg(ev=ev0, ev_rem=ev1))
        assert bool(reason & 4) == expect


def test_reasons_accumulate(oracle_mod):
    done, reason = oracle_mod.determine_termination({"max_samples": 10, "log_L_contour": -5.0},
                                                    _reg(plateau=1, no_seed_points=1))
    assert done and reason == (1 << 0) + (1 << 5) + (1 << 7) + (1 << 10)


def test_round_up_goldens(oracle_mod):
    from jaxns_gb300.public import round_up_max_samples, round_up_num_live_points
    for f in (round_up_num_live_points, oracle_mod.round_up_num_live_points):
        assert f(10, 0.5, 1) == 10
        assert f(10, 0.5, 2) == 12
        assert f(10, 0.5, 3) == 12
    for f in (round_up_max_samples, oracle_mod.round_up_max_samples):
        assert f(1000, 256, 0) == 1024
        assert f(1000, 256, 3) == 1024
        assert f(1025, 256, 3) == 2048
