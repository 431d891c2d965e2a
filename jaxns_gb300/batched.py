"""Many independent nested-sampling problems in one device batch.

``BatchedNestedSampler`` takes a list of configured ``NestedSampler`` objects (each with its
own model, live points and slices) and advances all of them together: one slice-sampler
launch per dimension bucket and one merge launch per iteration, replayed from a captured
CUDA graph every ``block`` iterations, until every run has terminated.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np
import torch

from .engine import FAMILY_LINGAUSS, NSBatch
from .public import NestedSampler, NestedSamplerResults, TerminationCondition, results_from_batch


class BatchedNestedSampler:
    def __init__(self, samplers: Sequence[NestedSampler], keys, term_conds: Optional[Sequence] = None,
                 block: int = 16, chains_per_item: int = 64, store_U: bool = False, lg_tensor_cores: bool = True,
                 autotune: bool = False, wide_chains_per_item: int = 0, device="cuda", chains_per_lane: int = 1,
                 warp_min_D: int = 17):
        self.samplers = list(samplers)
        keys = np.asarray(keys, np.uint32).reshape(len(self.samplers), 2)
        if term_conds is None:
            term_conds = [None] * len(self.samplers)
        specs = []
        for ns, k, tc in zip(self.samplers, keys, term_conds):
            spec = ns.nested_sampler.run_spec(k, ns.normalise_term_cond(tc))
            spec.store_U = store_U
            specs.append(spec)
        self.block = int(block)
        self.tuning = None
        if autotune and not any(s.family == FAMILY_LINGAUSS for s in specs):
            # launch shapes timed on this batch (results do not depend on them)
            from .autotune import autotune_launch
            self.tuning = autotune_launch(specs, device=device)
            chains_per_item = self.tuning["chains_per_item"]
            chains_per_lane = self.tuning["chains_per_lane"]
            wide_chains_per_item = self.tuning["wide_chains_per_item"]
            warp_min_D = self.tuning["warp_min_D"]
        self.batch = NSBatch(specs, device=device, chains_per_item=chains_per_item,
                             wide_chains_per_item=wide_chains_per_item, lg_tensor_cores=lg_tensor_cores,
                             chains_per_lane=chains_per_lane, warp_min_D=warp_min_D)
        self.state = None

    def __call__(self, from_host: bool = True, use_graph: bool = True, check: bool = True,
                 max_iterations: Optional[int] = None):
        """Run every problem to termination (or max_iterations).  Returns the termination
        reasons (host)."""
        self.batch.reset(from_host=from_host)
        self.state = self.batch.run(block=self.block, use_graph=use_graph, check=check, max_iterations=max_iterations)
        return self.state["termination_reason"].astype(np.int64)

    def summary(self):
        """log Z mean / uncert, ESS, H, sample and evaluation totals of every run, computed
        on the device and copied to the host as one [R, 8] array."""
        out = self.batch.results(with_U=False)
        return out["scalars"].cpu().numpy()

    def to_results(self, r: int) -> NestedSamplerResults:
        ns = self.samplers[r]
        return results_from_batch(ns.model, self.batch, r, int(self.state["termination_reason"][r]))
