"""Autotuner of the pair kernels' launch shapes.

The cell grid is not a free parameter here: it fixes the reference's output
order (stencil order over the reference's cells), so the tuner varies what
does not change results -- the count pass (each unordered cell pair once
into neighbour masks, for the systems whose 27-cell stencil has distinct
cells; one warp per home cell, staging the stencil in shared memory; or one
thread per home atom), the blocks per SM of the count / screening kernels and of the list
write kernel (how many home cells / atoms each warp walks) -- times every
candidate on the caller's own input with CUDA events, and keeps the fastest.
"""
from __future__ import annotations

import itertools
from typing import Dict, Iterable, Optional, Tuple

import torch

COUNT_KERNELS = (3, 1, 2)   # 3: symmetric where it applies, 1: warp per home cell, 2: thread per home atom
PAIR_BLOCKS = (4, 7, 14)
EMIT_BLOCKS = (8, 16, 32)


def _time_ms(fn, reps: int) -> float:
    ts = []
    for _ in range(reps):
        s = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        s.record()
        fn()
        e.record()
        e.synchronize()
        ts.append(s.elapsed_time(e))
    ts.sort()
    return ts[len(ts) // 2]


def autotune(runner, X: torch.Tensor, candidates: Optional[Iterable[Tuple[int, ...]]] = None,
             reps: int = 3) -> Dict:
    """Times runner.launch(X) for each (pair_blocks_per_sm, emit_blocks_per_sm
    [, count_kernel]) and leaves the fastest set on the runner (a
    NeighbourListEngine or a BatchNeighbourList).  Returns the choice and
    every trial."""
    cands = list(candidates) if candidates is not None else list(
        itertools.product(PAIR_BLOCKS, EMIT_BLOCKS, COUNT_KERNELS))
    runner.run(X)  # sizes the pair buffers
    trials = []
    for c in cands:
        p, e, k = (tuple(c) + (0,))[:3]
        runner.set_tuning(p, e, k)
        runner.launch(X)
        trials.append({"pair_blocks_per_sm": p, "emit_blocks_per_sm": e, "count_kernel": k,
                       "ms": _time_ms(lambda: runner.launch(X), reps)})
    runner.sync_status()
    best = min(trials, key=lambda t: t["ms"])
    runner.set_tuning(best["pair_blocks_per_sm"], best["emit_blocks_per_sm"], best["count_kernel"])
    return {"pair_blocks_per_sm": best["pair_blocks_per_sm"], "emit_blocks_per_sm": best["emit_blocks_per_sm"],
            "count_kernel": best["count_kernel"], "ms": best["ms"], "trials": trials}
