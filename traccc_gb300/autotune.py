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
stream (median of ``reps`` after one warm-up launch).  The best shape is
stored in a JSON table keyed by the batch's mean-spacepoints-per-event
bucket, so a later process looks it up instead of searching again:

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
import statistics

from . import seeding

# 16 warps: as many as fit in shared memory with the neighbourhood capacity
WARPS = (8, 12, 16)
MIDDLES = (64, 256, 1024)
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


def _time_graph(alg, events, outs, stream, reps):
    import torch
    alg.graph_launch(events, outs, stream=stream.cuda_stream)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * reps)]
    times = []
    for r in range(reps):
        ev[2 * r].record(stream)
        alg.graph_launch(events, outs, stream=stream.cuda_stream)
        ev[2 * r + 1].record(stream)
    stream.synchronize()
    for r in range(reps):
        times.append(ev[2 * r].elapsed_time(ev[2 * r + 1]))
    return statistics.median(times)


def tune(alg, events, outs=None, shapes=None, reps=3, stream=None):
    """Search the launch shapes for this batch.  Returns (best shape,
    report); leaves the best shape set and the graph captured for the
    batch's size.  Every candidate must end with status OK."""
    import torch
    stream = stream or torch.cuda.current_stream()
    outs = outs or [seeding.SeedBuffer(alg.max_seeds(len(e)), device=e.global_.device)
                    for e in events]
    total_sp = sum(len(e) for e in events)
    report = []
    best = None
    for shape in shapes or candidates():
        try:
            eff = alg.set_tune(*shape)
        except seeding.SeedingError:
            continue  # does not fit in shared memory
        if any(r["shape"] == list(eff) for r in report):
            continue  # clamped to a shape already measured
        alg.graph_create(len(events), total_sp)
        ms = _time_graph(alg, events, outs, stream, reps)
        st = alg.last_status(stream.cuda_stream)
        if st != seeding.OK:
            raise seeding.SeedingError(st, f"tuning shape {eff}")
        report.append({"shape": list(eff), "ms": ms})
        if best is None or ms < best[1]:
            best = (tuple(eff), ms)
    if best is None:
        raise RuntimeError("no launch shape fits this device")
    alg.set_tune(*best[0])
    alg.graph_create(len(events), total_sp)
    report.sort(key=lambda r: r["ms"])
    return best[0], report


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
