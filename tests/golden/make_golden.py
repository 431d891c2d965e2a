"""Writes ``oracle_golden.json``: regression fixtures of the FP64 CPU oracle.

These are outputs of the oracle's restatement, not of the reference itself (the reference's
jax / jaxlib / tfp stack cannot be installed here, so no reference output exists to record).
They freeze the oracle's RNG streams (threefry split, 64-bit words, uniform and normal draws),
the live-point count of a seeded sample tree, the FP64 evidence statistics of a seeded sample
set, the stochastic-shrinkage replicas, and two complete small nested-sampling runs (one with
phantom points). ``tests/test_golden_cpu.py`` regenerates them and compares.

The integer parts (keys, words, indices, counts) are platform independent. The floating-point
parts depend on the host libm (log, exp, log1p), so the fixture records the platform it was
generated on and the NS-run comparison is exact only there.

Usage: python tests/golden/make_golden.py   (from the repository root)
"""
from __future__ import annotations

import hashlib
import json
import os
import platform
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(_HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

OUT = os.path.join(_HERE, "oracle_golden.json")


def _sha(a) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _f(x) -> str:
    """A float64 as its exact hex form (round-trips bit for bit)."""
    return float(x).hex()


def _run_summary(o, run) -> dict:
    r = run.results
    return {
        "termination_reason": run.termination_reason,
        "num_samples": run.num_samples,
        "iterations": run.iterations,
        "total_num_likelihood_evaluations": int(r["total_num_likelihood_evaluations"]),
        "total_phantom_samples": int(r["total_phantom_samples"]),
        "log_Z_mean": _f(r["log_Z_mean"]),
        "log_Z_uncert": _f(r["log_Z_uncert"]),
        "ESS": _f(r["ESS"]),
        "H_mean": _f(r["H_mean"]),
        "sender_sha256": _sha(run.sender.astype(np.int64)),
        "nevals_sha256": _sha(run.nevals.astype(np.int64)),
        "phantom_sha256": _sha(run.phantom.astype(np.int32)),
        "num_live_points_sha256": _sha(run.num_live_points.astype(np.int64)),
        "log_L_sha256": _sha(run.log_L.astype(np.float64)),
        "log_L_first": [_f(v) for v in run.log_L[:8]],
    }


def tree_inputs():
    """A seeded 200-sample tree with ties on a quarter grid: (sender node index, log L).  Every
    sender has a strictly lower log L; storage order shuffled; the sender is a node index, 0 the
    root and sample i node i + 1, as in SampleTreeGraph (internals/tree_structure.py:12-26)."""
    g = np.random.default_rng(11)
    N = 200
    asc = np.round(np.sort(g.standard_normal(N)) * 4) / 4
    parent = np.full(N, -1, np.int64)
    for i in range(N):
        lower = np.flatnonzero(asc < asc[i])
        if lower.size and g.random() < 0.9:
            parent[i] = int(lower[g.integers(max(0, lower.size - 30), lower.size)])
    perm = g.permutation(N)                 # storage slot of the i-th ascending sample
    log_L = np.empty(N)
    sender = np.empty(N, np.int64)
    log_L[perm] = asc
    sender[perm] = np.where(parent >= 0, perm[np.maximum(parent, 0)] + 1, 0)
    return sender, log_L


def evidence_inputs():
    """A seeded sample set for compute_evidence_stats: (sorted log L [500], live-point counts)."""
    g = np.random.default_rng(12)
    M = 500
    ll = np.sort(g.standard_normal(M)) * 3
    n = np.concatenate([np.full(M - 40, 40), np.arange(40, 0, -1)]).astype(np.float64)
    return ll, n


# the small complete run both fixture generators record (correlated Gaussian, D = 2)
MVN_RUN = {"mu": [0.3, -0.4], "cov": [[1.0, 0.4], [0.4, 0.6]], "low": -10.0, "high": 10.0,
           "num_live_points": 60, "num_slices": 10, "key_seed": 7, "dlogZ": 1e-3}


def generate() -> dict:
    from oracle import oracle as o
    o.build()
    out: dict = {"generator": "tests/golden/make_golden.py",
                 "platform": f"{platform.machine()}-{platform.system()}"}

    # RNG streams of jax.random under jax_threefry_partitionable=True
    rng = {}
    for seed in (0, 1, 42, 2 ** 31 - 1):
        k = o.PRNGKey(seed)
        rng[str(seed)] = {
            "key": [int(v) for v in k],
            "split4": [[int(a), int(b)] for a, b in o.split(k, 4)],
            "bits64": [str(int(v)) for v in o.random_bits64(k, 6)],
            "uniform": [_f(v) for v in o.uniform(k, 6)],
            "normal": [_f(v) for v in o.normal(k, 6)],
        }
    out["rng"] = rng

    # live-point count of a seeded tree with ties (tree_structure.py:33-108)
    sender, log_L = tree_inputs()
    idx, nl = o.count_crossed_edges(sender, log_L)
    out["tree"] = {"sender_seed": 11, "N": len(log_L), "samples_indices": [int(v) for v in idx],
                   "num_live_points": [int(v) for v in nl]}

    # FP64 evidence statistics (shrinkage_statistics.py:131-157)
    ll, n = evidence_inputs()
    fin, _ = o.compute_evidence_stats(ll, n)
    out["evidence_stats"] = {"seed": 12, "M": len(ll), "final": {k: _f(v) for k, v in fin.items()}}

    # a complete MVN run (D = 2) and a shells run with phantoms (D = 3, k = 2)
    c = MVN_RUN
    m1 = o.mvn_model(np.full(2, c["low"]), np.full(2, c["high"]), np.array(c["mu"]), np.array(c["cov"]))
    r1 = o.ns_run(m1, o.PRNGKey(c["key_seed"]), num_live_points=c["num_live_points"], num_slices=c["num_slices"],
                  term_cond={"dlogZ": c["dlogZ"]})
    m2 = o.shells_model(-6.0, 6.0, [3.5, 0.0, 0.0], [-3.5, 0.0, 0.0], 2.0, 0.3)
    r2 = o.ns_run(m2, o.PRNGKey(8), num_live_points=80, num_slices=15, num_phantom=2,
                  term_cond={"dlogZ": 1e-3})
    out["ns_mvn_D2"] = dict(_run_summary(o, r1), num_live_points=60, num_slices=10, key_seed=7)
    out["ns_shells_D3_k2"] = dict(_run_summary(o, r2), num_live_points=80, num_slices=15, num_phantom=2,
                                  key_seed=8)

    # stochastic-shrinkage replicas of the MVN run (utils.py:433-484)
    se = o.sample_evidence(o.PRNGKey(9), r1.num_live_points, r1.log_L_sorted, S=16)
    out["sample_evidence_mvn_D2"] = [_f(v) for v in se]
    return out


if __name__ == "__main__":
    with open(OUT, "w") as f:
        json.dump(generate(), f, indent=1)
        f.write("\n")
    print("wrote", OUT)
