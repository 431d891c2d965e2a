"""Regression fixtures of the FP64 CPU oracle (``tests/golden/oracle_golden.json``, written by
``tests/golden/make_golden.py``): the oracle regenerates them and must agree.

Keys, 64-bit words, tree indices and live-point counts must match exactly everywhere.
Floating-point values are bit-exact on the platform the fixture was generated on; elsewhere
the host libm may differ in the last bits, so they are compared to a relative 1e-12 and the NS
runs (whose trajectories a last-bit difference can change) only on that platform.
"""
import json
import os
import platform

import numpy as np
import pytest

from tests.conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden", "oracle_golden.json")


@pytest.fixture(scope="module")
def pair(oracle_mod):
    from tests.golden.make_golden import generate
    with open(GOLDEN) as f:
        want = json.load(f)
    return want, generate()


def _same_platform(want):
    return want["platform"] == f"{platform.machine()}-{platform.system()}"


def _floats(hexes):
    return np.array([float.fromhex(h) for h in hexes])


def _close(want, got, same):
    if same:
        assert want == got
    else:
        np.testing.assert_allclose(_floats(got), _floats(want), rtol=1e-12, atol=0)


def test_rng_streams(pair):
    want, got = pair
    same = _same_platform(want)
    for seed, w in want["rng"].items():
        g = got["rng"][seed]
        assert g["key"] == w["key"] and g["split4"] == w["split4"] and g["bits64"] == w["bits64"], seed
        _close(w["uniform"], g["uniform"], same)
        _close(w["normal"], g["normal"], same)


def test_tree_count(pair):
    want, got = pair
    assert got["tree"] == want["tree"]
    # every live-point count is at least 1, and each sample index appears once
    nl = np.array(want["tree"]["num_live_points"])
    assert nl.min() >= 1
    idx = np.array(want["tree"]["samples_indices"])
    assert sorted(idx) == list(range(want["tree"]["N"]))


def test_tree_count_by_intervals(oracle_mod):
    """The crossed-edge recurrence equals a direct interval count: at sorted position t the
    live points are the samples whose parent is removed before t and that are removed at t or
    later (the root at position -1)."""
    g = np.random.default_rng(5)
    for N in (1, 2, 7, 60, 300):
        asc = np.round(np.sort(g.standard_normal(N)) * 3) / 3
        parent = np.array([int(g.choice(np.flatnonzero(asc < asc[i]))) if (asc < asc[i]).any() and g.random() < 0.8
                           else -1 for i in range(N)])
        perm = g.permutation(N)
        log_L = np.empty(N)
        sender = np.empty(N, np.int64)
        log_L[perm] = asc
        sender[perm] = np.where(parent >= 0, perm[np.maximum(parent, 0)] + 1, 0)
        idx, nl = oracle_mod.count_crossed_edges(sender, log_L)
        pos = np.empty(N, np.int64)
        pos[idx] = np.arange(N)
        ppos = np.where(sender > 0, pos[np.maximum(sender - 1, 0)], -1)
        direct = np.array([int(np.sum((ppos < t) & (pos >= t))) for t in range(N)])
        np.testing.assert_array_equal(nl, direct)
        np.testing.assert_array_equal(log_L[idx], np.sort(log_L, kind="stable"))


def test_evidence_stats(pair):
    want, got = pair
    w, g = want["evidence_stats"]["final"], got["evidence_stats"]["final"]
    assert set(w) == set(g)
    _close([w[k] for k in sorted(w)], [g[k] for k in sorted(g)], _same_platform(want))


@pytest.mark.parametrize("name", ["ns_mvn_D2", "ns_shells_D3_k2"])
def test_ns_runs(pair, name):
    want, got = pair
    if not _same_platform(want):
        pytest.skip(f"fixture generated on {want['platform']}; NS trajectories depend on the host libm")
    assert got[name] == want[name]


def test_ns_run_statistics(pair):
    """Platform-independent sanity of the frozen runs: log Z of the D = 2 correlated Gaussian
    (prior U[-10, 10]^2, fully inside the box) within 3 sigma of -2 log 20; phantoms recorded
    for the k = 2 run, two per sample drawn in the slice phase; termination by dlogZ (bit 4)."""
    want, _ = pair
    r = want["ns_mvn_D2"]
    lz, dz = float.fromhex(r["log_Z_mean"]), float.fromhex(r["log_Z_uncert"])
    assert abs(lz + 2 * np.log(20.0)) < 3 * dz
    assert r["termination_reason"] & 4
    s = want["ns_shells_D3_k2"]
    assert s["total_phantom_samples"] > 0 and s["total_phantom_samples"] % 2 == 0
    se = _floats(want["sample_evidence_mvn_D2"])
    assert abs(se.mean() - lz) < 3 * dz and se.std() > 0


def test_sample_evidence(pair):
    want, got = pair
    _close(want["sample_evidence_mvn_D2"], got["sample_evidence_mvn_D2"], _same_platform(want))
