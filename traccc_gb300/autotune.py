"""Autotuner for the batched seeding launch.

The search space is the launch shape of the persistent seeding kernel
(``seedgb_tune``): warps per CTA, middle spacepoints per work item, the
neighbourhood capacity staged in shared memory, and resident CTAs per SM.
None of them changes the seeds; they trade load balance (small work items,
many warps) against per-item overhead (staging the neighbourhood once per
item) and shared-memory capacity (a larger neighbourhood tile leaves room for
fewer warps).

For a batch, every candidate is set, the graph is captured for the batch's
size, and the captured launch is timed with CUDA events on the launching
stream (median of ``reps`` after one warm-up launch) -- the library's own
search, seedgb_seeding_autotune, which C++ callers use directly.  The best
shape is stored in a JSON table keyed by the batch's mean-spacepoints-per-
event bucket, so a later process looks it up instead of searching again:

    table = autotune.load(path)
    shape = autotune.lookup(table, mean_sp)      # None: not tuned yet
    shape, report = autotune.tune(alg, events)   # search, then
    autotune.store(path, mean_sp, shape, report)
"""
from __future__ import annotations

import itertools
import json
import math
import os

from . import seeding

# 16 warps: as many as fit in shared memory with the neighbourhood capacity
WARPS = (8, 12, 16)
MIDDLES = (64, 256, 384, 512, 1024)
NEIGHBOURHOOD = (1536, 2048, 2560, 3072)
CTAS = (1, 2)


def candidates(warps=WARPS, middles=MIDDLES, neighbourhood=NEIGHBOURHOOD, ctas=CTAS):
    """All launch shapes of the grid (the library clamps or rejects shapes
    that do not fit in shared memory)."""
    return list(itertools.product(warps, middles, neighbourhood, ctas))


def bucket(mean_sp: float) -> str:
    """Power-of-two bucket of the mean spacepoint count per event."""
    b = 1 << max(10, math.ceil(math.log2(max(1.0, mean_sp))))
    return f"le{b}"


def tune(alg, events, outs=None, shapes=None, reps=3, stream=None):
    """Search the launch shapes for this batch (seedgb_seeding_autotune).
    Returns (best shape, report sorted by time); leaves the best shape set
    and the graph captured for the batch's size."""
    import torch
    stream = stream or torch.cuda.current_stream()
    outs = outs or [seeding.SeedBuffer(alg.max_seeds(len(e)), device=e.global_.device)
                    for e in events]
    best, times = alg.autotune(events, outs, candidates=shapes or candidates(), reps=reps,
                               stream=stream.cuda_stream)
    report = sorted(({"shape": list(sh), "ms": ms} for sh, ms in times if ms is not None),
                    key=lambda r: r["ms"])
    return tuple(best), report


def load(path: str) -> dict:
    if not os.path.exists(path):
        return {}
    with open(path) as f:
        return json.load(f)


def lookup(table: dict, mean_sp: float):
    e = table.get(bucket(mean_sp))
    return tuple(e["shape"]) if e else None


def store(path: str, mean_sp: float, shape, report) -> dict:
    table = load(path)
    table[bucket(mean_sp)] = {"shape": list(shape), "ms": report[0]["ms"] if report else None,
                              "measured": len(report)}
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    return table
