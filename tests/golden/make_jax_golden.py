"""Writes ``jax_golden.json``: the reference's own outputs for the pieces the oracle restates,
so that the oracle (and through it every GPU parity test) can be pinned against jax itself.

jax, jaxlib, tensorflow_probability and jaxns cannot be installed where this repository is
built, so this script is meant for any machine that has them:

    python tests/golden/make_jax_golden.py [--jaxns-src PATH/TO/jaxns/src]

It records, under jax_threefry_partitionable=True and x64 (the settings jaxns's
internals/mixed_precision.py:11-15 makes):
  * PRNGKey, split(key, 4), bits(key, (6,), uint64), uniform(key, (6,), float64) and
    normal(key, (6,), float64) for four seeds;
  * count_crossed_edges (internals/tree_structure.py:33-108) of the tree in make_golden.py;
  * compute_evidence_stats (internals/shrinkage_statistics.py:131-157) of the sample set in
    make_golden.py;
  * one complete NestedSampler run (the D = 2 correlated Gaussian of make_golden.MVN_RUN,
    likelihood tfp MultivariateNormalTriL, prior Uniform[-10, 10]^2).
``tests/test_jax_golden_cpu.py`` compares the oracle with the file when it exists.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(_HERE, "jax_golden.json")


def _hex(a):
    return [float(v).hex() for v in np.asarray(a, np.float64).ravel()]


def generate() -> dict:
    import jax
    jax.config.update("jax_enable_x64", True)
    jax.config.update("jax_threefry_partitionable", True)
    import jax.numpy as jnp
    import jaxns
    import tensorflow_probability.substrates.jax as tfp
    from jaxns.internals.shrinkage_statistics import compute_evidence_stats
    from jaxns.internals.tree_structure import SampleTreeGraph, count_crossed_edges

    sys.path.insert(0, _HERE)
    from make_golden import MVN_RUN, evidence_inputs, tree_inputs

    tfpd = tfp.distributions
    out = {"generator": "tests/golden/make_jax_golden.py", "jax": jax.__version__,
           "jaxns": getattr(jaxns, "__version__", "unknown"),
           "platform": f"{platform.machine()}-{platform.system()}"}

    rng = {}
    for seed in (0, 1, 42, 2 ** 31 - 1):
        k = jax.random.PRNGKey(seed)
        rng[str(seed)] = {
            "key": [int(v) for v in np.asarray(k)],
            "split4": [[int(a), int(b)] for a, b in np.asarray(jax.random.split(k, 4))],
            "bits64": [str(int(v)) for v in np.asarray(jax.random.bits(k, (6,), jnp.uint64))],
            "uniform": _hex(jax.random.uniform(k, (6,), jnp.float64)),
            "normal": _hex(jax.random.normal(k, (6,), jnp.float64)),
        }
    out["rng"] = rng

    sender, log_L = tree_inputs()
    counts = count_crossed_edges(SampleTreeGraph(sender_node_idx=jnp.asarray(sender), log_L=jnp.asarray(log_L)))
    out["tree"] = {"samples_indices": [int(v) for v in np.asarray(counts.samples_indices)],
                   "num_live_points": [int(v) for v in np.asarray(counts.num_live_points)]}

    ll, n = evidence_inputs()
    final, _ = compute_evidence_stats(log_L=jnp.asarray(ll), num_live_points=jnp.asarray(n))
    out["evidence_stats"] = {f: float(getattr(final, f)).hex() for f in final._fields}

    c = MVN_RUN
    mu, L = np.asarray(c["mu"]), np.linalg.cholesky(np.asarray(c["cov"]))

    def prior_model():
        x = yield jaxns.Prior(tfpd.Uniform(low=c["low"] * jnp.ones(2), high=c["high"] * jnp.ones(2)), name="x")
        return x

    def log_likelihood(x):
        return tfpd.MultivariateNormalTriL(loc=jnp.asarray(mu), scale_tril=jnp.asarray(L)).log_prob(x)

    model = jaxns.Model(prior_model=prior_model, log_likelihood=log_likelihood)
    ns = jaxns.NestedSampler(model=model, num_live_points=c["num_live_points"], num_slices=c["num_slices"])
    reason, state = jax.jit(ns)(jax.random.PRNGKey(c["key_seed"]), jaxns.TerminationCondition(dlogZ=c["dlogZ"]))
    res = ns.to_results(termination_reason=reason, state=state)
    out["ns_mvn_D2"] = {
        "termination_reason": int(res.termination_reason),
        "num_samples": int(res.total_num_samples),
        "total_num_likelihood_evaluations": int(res.total_num_likelihood_evaluations),
        "log_Z_mean": float(res.log_Z_mean).hex(),
        "log_Z_uncert": float(res.log_Z_uncert).hex(),
        "log_L_first": _hex(np.asarray(res.log_L_samples)[:8]),
    }
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--jaxns-src", default=None, help="jaxns's src/ directory when jaxns is not installed")
    args = ap.parse_args()
    if args.jaxns_src:
        sys.path.insert(0, args.jaxns_src)
    with open(OUT, "w") as f:
        json.dump(generate(), f, indent=1)
        f.write("\n")
    print("wrote", OUT)
