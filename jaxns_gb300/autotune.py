"""Launch-shape autotuning of a batch.

The sampler's launch shape is free and the results do not depend on it within a kernel:
every chain's random stream and arithmetic are fixed by its index.  The shape is
  * the CTA width of the thread-per-chain kernel (``chains_per_item``) and the size of each
    CTA's chain pool in chains per lane (``chains_per_lane``),
  * the chains per item of the warp-cooperative correlated-Gaussian kernel
    (``wide_chains_per_item``),
  * which kernel runs correlated Gaussians with 8 < D <= 16 (``warp_min_D``: 9 moves them to
    the warp-cooperative kernel, 17 keeps them one thread per chain).  The two kernels sum the
    D squared components in different orders, so this choice can change the last bit of a
    log-likelihood; each is exact against the oracle's model of its own arithmetic.
``autotune_launch`` times the sampler launches (CUDA events recorded inside the captured graph)
over a few NS iterations of the real batch for each candidate, one dimension at a time, and
returns the fastest with the table of every timing.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence

import torch

from .engine import FAMILY_LINGAUSS, FAMILY_MVN, NSBatch, RunSpec

THREAD_WIDTHS = (32, 64, 128)
CHAINS_PER_LANE = (1, 2, 4)
WIDE_ITEMS = (128, 256, 512)


def _time(specs, device, iterations, **shape) -> float:
    b = NSBatch(specs, device=device, **shape)
    b.timing = True
    b.init()
    b.iterate_graph(1)          # capture and first replay (not timed)
    torch.cuda.synchronize()
    b._collect_timing()
    b.shell_ms = 0.0
    b.iterate_graph(iterations)
    torch.cuda.synchronize()
    b._collect_timing()
    ms = b.shell_ms
    del b
    torch.cuda.empty_cache()
    return ms


def autotune_launch(specs: Sequence[RunSpec], device="cuda", iterations: int = 2,
                    thread_widths: Optional[Sequence[int]] = None,
                    chains_per_lane: Optional[Sequence[int]] = None,
                    wide_items: Optional[Sequence[int]] = None, tune_kernel: bool = True) -> Dict:
    """{"chains_per_item", "chains_per_lane", "wide_chains_per_item", "warp_min_D", "sampler_ms",
    "table"} for this batch."""
    specs = list(specs)
    thread_runs = any(s.family != FAMILY_LINGAUSS and (s.family != FAMILY_MVN or s.D <= 16) for s in specs)
    wide_runs = any(s.family == FAMILY_MVN and s.D > 16 for s in specs)
    mid_mvn = any(s.family == FAMILY_MVN and 8 < s.D <= 16 for s in specs)
    best = {"chains_per_item": 64, "chains_per_lane": 1, "wide_chains_per_item": 0, "warp_min_D": 17}
    table: List[Dict] = []

    def trial(**change):
        shape = dict(best, **change)
        ms = _time(specs, device, iterations, **shape)
        table.append(dict(shape, sampler_ms=ms))
        return ms

    if thread_runs:
        cand = [(w, c) for w in (thread_widths or THREAD_WIDTHS) for c in (chains_per_lane or CHAINS_PER_LANE)]
        times = [trial(chains_per_item=w, chains_per_lane=c) for w, c in cand]
        w, c = cand[min(range(len(cand)), key=times.__getitem__)]
        best.update(chains_per_item=w, chains_per_lane=c)
    if wide_runs or (tune_kernel and mid_mvn):
        cand = list(wide_items or WIDE_ITEMS)
        times = [trial(wide_chains_per_item=wi) for wi in cand]
        best.update(wide_chains_per_item=cand[min(range(len(cand)), key=times.__getitem__)])
    if tune_kernel and mid_mvn:
        cand = [17, 9]
        times = [trial(warp_min_D=m) for m in cand]
        best.update(warp_min_D=cand[min(range(len(cand)), key=times.__getitem__)])
    best_ms = min((t["sampler_ms"] for t in table if all(t[k] == best[k] for k in best)), default=None)
    return dict(best, sampler_ms=best_ms, table=table)
