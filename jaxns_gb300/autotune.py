"""Launch-shape autotuning of a batch.

The sampler's launch shape is free: the CTA width of the thread-per-chain kernel (one chain
per thread, ``chains_per_item``) and the chains per item of the warp-cooperative kernel for
correlated Gaussians with D > 16 (``wide_chains_per_item``).  Every chain's random stream is
fixed by its index, so the results do not depend on the shape, only the time does.
``autotune_launch`` times the sampler launches (CUDA events recorded inside the captured graph)
over a few NS iterations of the real batch for each candidate and returns the fastest.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Sequence

import torch

from .engine import FAMILY_LINGAUSS, FAMILY_MVN, NSBatch, RunSpec

THREAD_WIDTHS = (32, 64, 128)
WIDE_ITEMS = (128, 256, 512)


def autotune_launch(specs: Sequence[RunSpec], device="cuda", iterations: int = 2,
                    thread_widths: Optional[Sequence[int]] = None,
                    wide_items: Optional[Sequence[int]] = None) -> Dict:
    """{"chains_per_item", "wide_chains_per_item", "sampler_ms", "table"} for this batch."""
    specs = list(specs)
    thread_runs = any(s.family != FAMILY_LINGAUSS and (s.family != FAMILY_MVN or s.D <= 16) for s in specs)
    wide_runs = any(s.family == FAMILY_MVN and s.D > 16 for s in specs)
    tw = tuple(thread_widths or THREAD_WIDTHS) if thread_runs else (64,)
    wi = tuple(wide_items or WIDE_ITEMS) if wide_runs else (0,)
    table: List[Dict] = []
    for cpi in tw:
        for wide in wi:
            b = NSBatch(specs, device=device, chains_per_item=cpi, wide_chains_per_item=wide)
            b.timing = True
            b.init()
            b.iterate_graph(1)          # capture and first replay (not timed)
            torch.cuda.synchronize()
            b._collect_timing()
            b.shell_ms = 0.0
            b.iterate_graph(iterations)
            torch.cuda.synchronize()
            b._collect_timing()
            table.append({"chains_per_item": cpi, "wide_chains_per_item": wide, "sampler_ms": b.shell_ms})
            del b
            torch.cuda.empty_cache()
    best = min(table, key=lambda t: t["sampler_ms"])
    return dict(best, table=table)
