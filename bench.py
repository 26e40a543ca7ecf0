#!/usr/bin/env python
"""Seeding throughput: events/s of traccc-style triplet seeding on one GB300.

Workload (the ~100k-spacepoint configuration the metric is quoted on): 20
synthetic events from seeds 0-19, each 9000 helices with pT ~ exp(mean
0.6 GeV) truncated at 0.1 GeV, |eta| < 1.5, plus 12 % noise spacepoints
(~88k spacepoints per event) in a 10-layer barrel, 2 T field.  The seeding
config is the reference default.

One step = the whole stage for all 20 events: spacepoint binning, doublets,
triplets, seed filtering (one batched launch sequence) and track-parameter
estimation (one batched launch for all events).

  value : events/s with inputs resident in HBM (device time, CUDA events on
          the launching stream, L2 flushed between steps by a 256 MiB write)
  e2e   : events/s through the public API from pinned host buffers: the
          spacepoint columns are copied in, seeds and parameters copied out
          every step (two steps in flight: step k+1's inputs are copied in
          and step k-1's results copied out on two copy streams while step k
          computes)
  cpu_baseline : the oracle (restated reference host seeding, libm phi) on a
          bounded sample of the same events, one event per host thread

Also in the JSON line (one GPU):
  learned : the same 20-event step with the learned doublet filter gating
            whole middles (a subset of the plain seeds by construction),
            trained on the GPU by the library's kernels (200 pileup9k events),
            gate thresholds per event-size class calibrated for 99.9 % seed
            recall (99.8 % on every event) on 144 held-out events (a margin
            above the 99.5 % target);
            events/s, speed-up against the plain step, per-event recall,
            seeds outside the plain set, pruned fraction, fallback events,
            training report
  batched : the 64-event uneven batch (5k-114k spacepoints per event) through
            the captured graph with the autotuned launch shape, plain and
            with the filter: events/s, p50/p99 batch latency (device and end
            to end one batch at a time), end-to-end throughput with two
            batches in flight, autotuner report

``--impl reference`` times the reference's CPU seeding path (the oracle port;
the reference itself cannot be built: its seeding path needs vecmem, detray,
covfie and the ACTS logger, none of them vendored) with all host
threads on the same workload and metric.

Multi-GPU (``torchrun --nproc-per-node N``): replicas only -- every rank seeds
its own copy of the 20 events, no collective on the data path; value = events
of all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "events/s seeding @100k SP/event, plain vs learned-pruned at >=99.5% seed recall"
WORKLOAD = ("pileup9k: 20 synthetic events (seeds 0-19), 9000 helices + 12% noise, "
            "~88k spacepoints/event, reference default seeding config")
N_EVENTS = 20
L2_FLUSH_BYTES = 256 << 20


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=30)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="seedgb", choices=["seedgb", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--events", type=int, default=N_EVENTS)
    p.add_argument("--no-batched", action="store_true",
                   help="skip the 64-event graph-launched batch")
    p.add_argument("--retune", action="store_true",
                   help="search launch shapes even if the tuning table has an entry")
    p.add_argument("--no-learned", action="store_true",
                   help="skip training and timing the learned doublet filter")
    p.add_argument("--filter-events", type=int, default=FILTER_TRAIN_EVENTS)
    p.add_argument("--profile-case", choices=["plain4", "plain20", "learned4", "train", "batch64",
                                              "gbts1"],
                   help="run one small fixed workload for an ncu capture and exit")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(values, device):
    """Element-wise maximum of per-rank timings over all ranks (the slowest
    replica sets the job's time)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor(values, dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def job_throughput(events_per_rank_step, steps, world, seconds):
    """Events of all ranks per second of the slowest rank."""
    return world * events_per_rank_step * steps / seconds


def make_events(n):
    from traccc_gb300 import synth
    return [synth.workload_event("pileup9k", s) for s in range(n)]


BATCH_EVENTS = 64
BATCH_SEED = 3
BATCH_WORKLOAD = ("uneven64: 64 synthetic events (batch seed 3) with U(500, 12000) helices each "
                  "+ 12% noise, pileup9k pT/eta/z0 statistics, one graph launch per batch")


def quantile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q
    lo, hi = int(np.floor(k)), int(np.ceil(k))
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


def tune_table_path():
    return os.environ.get("SEEDGB_TUNE_TABLE",
                          os.path.join(ROOT, "traccc_gb300", "_lib", "tune_table.json"))


class BatchInputs:
    """The uneven 64-event batch, resident on the device and pinned on the
    host (for the end-to-end timing)."""

    def __init__(self, dev):
        import torch

        from traccc_gb300 import seeding, synth
        events = synth.batch_events(BATCH_EVENTS, BATCH_SEED)
        self.sizes = [len(e["layer"]) for e in events]
        offs = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)
        self.total = int(offs[-1])

        def cat(key, dt, shape=()):
            return np.ascontiguousarray(np.concatenate(
                [np.asarray(e[key]).reshape((-1,) + shape) for e in events]).astype(dt))

        host = {"mi1": cat("measurement_index_1", np.uint32).view(np.int32),
                "mi2": cat("measurement_index_2", np.uint32).view(np.int32),
                "glob": cat("global", np.float32, (3,)),
                "zvar": cat("z_variance", np.float32),
                "rvar": cat("radius_variance", np.float32)}
        self.pinned = {k: torch.from_numpy(v).pin_memory() for k, v in host.items()}
        self.dcols = {k: v.to(dev) for k, v in self.pinned.items()}
        # a second device copy for the pipelined end-to-end loop
        self.dcols2 = {k: torch.empty_like(v) for k, v in self.dcols.items()}

        def views(d):
            out = []
            for e in range(BATCH_EVENTS):
                a, b = int(offs[e]), int(offs[e + 1])
                out.append(seeding.SpacepointCollection(d["mi1"][a:b], d["mi2"][a:b],
                                                        d["glob"][a:b], d["zvar"][a:b],
                                                        d["rvar"][a:b]))
            return out

        self.sps = views(self.dcols)
        self.sps2 = views(self.dcols2)


def run_batched(args, dev, stream, flush_buf, inputs, model=None):
    """The uneven 64-event batch through the captured graph (with the learned
    filter when `model` is given): autotuned launch shape, events/s over K
    batches, p50/p99 per-batch latency (device time of one graph launch, L2
    flushed before each), the same end to end (pinned host columns in, seeds
    out, wall clock) one batch at a time, and the end-to-end throughput with
    two batches in flight.  Returns (report, seed buffers of the last
    latency-loop batch)."""
    import torch

    from traccc_gb300 import autotune, seeding
    alg = seeding.TripletSeedingAlgorithm()
    if model is not None:
        alg.set_filter(model.struct())
    sps, total = inputs.sps, inputs.total
    outs = []
    size_all = torch.zeros(BATCH_EVENTS, dtype=torch.int32, device=dev)
    for e in range(BATCH_EVENTS):
        so = seeding.SeedBuffer(alg.max_seeds(len(sps[e])), device=dev)
        so.size = size_all[e:e + 1]
        outs.append(so)
    mean_sp = total / BATCH_EVENTS
    path = tune_table_path()
    if model is not None:
        path = path.replace(".json", "_learned.json")
    table = autotune.load(path)
    shape = None if args.retune else autotune.lookup(table, mean_sp)
    t0 = time.perf_counter()
    if shape is None:
        shape, report = autotune.tune(alg, sps, outs, stream=stream)
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            autotune.store(path, mean_sp, shape, report)
        except OSError:
            pass
        tuned = {"shape": list(shape), "source": "searched", "measured": len(report),
                 "search_s": time.perf_counter() - t0,
                 "top3": report[:3], "default_ms": next(
                     (r["ms"] for r in report if r["shape"][1:] == [256, 2048, 1]), None)}
    else:
        alg.set_tune(*shape)
        alg.graph_create(BATCH_EVENTS, total)
        tuned = {"shape": list(alg.get_tune()), "source": "table " + os.path.basename(path)}
    sptr = stream.cuda_stream
    for _ in range(max(3, args.warmup)):
        alg.graph_launch(sps, outs, stream=sptr)
    torch.cuda.synchronize()
    st = alg.last_status(sptr)
    if st != seeding.OK:
        raise RuntimeError(f"batched seeding status {st}")
    n_seeds = int(size_all.sum().item())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    for k in range(args.steps):
        flush_buf.fill_(1)
        ev[2 * k].record(stream)
        alg.graph_launch(sps, outs, stream=sptr)
        ev[2 * k + 1].record(stream)
    torch.cuda.synchronize()
    lat = [ev[2 * k].elapsed_time(ev[2 * k + 1]) for k in range(args.steps)]
    # end to end: columns in from pinned memory, seeds out, per batch
    h_size = torch.zeros(BATCH_EVENTS, dtype=torch.int32).pin_memory()
    h_seeds = torch.empty((4, sum(o.capacity for o in outs)), dtype=torch.int32).pin_memory()
    h2d = sum(v.numel() * v.element_size() for v in inputs.pinned.values())

    def e2e_batch():
        for k in inputs.dcols:
            inputs.dcols[k].copy_(inputs.pinned[k], non_blocking=True)
        alg.graph_launch(sps, outs, stream=sptr)
        h_size.copy_(size_all, non_blocking=True)
        stream.synchronize()
        o, d2h = 0, 4 * BATCH_EVENTS
        for e in range(BATCH_EVENTS):
            ns = int(h_size[e])
            so = outs[e]
            for j, col in enumerate((so.bottom_index, so.middle_index, so.top_index)):
                h_seeds[j, o:o + ns].copy_(col[:ns], non_blocking=True)
            h_seeds[3, o:o + ns].copy_(so.quality[:ns].view(torch.int32), non_blocking=True)
            o += ns
            d2h += 16 * ns
        stream.synchronize()
        return d2h

    for _ in range(max(1, args.warmup)):
        e2e_batch()
    e2e_lat, d2h = [], 0
    for _ in range(args.steps):
        flush_buf.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d2h = e2e_batch()
        e2e_lat.append(1e3 * (time.perf_counter() - t0))

    # End to end, pipelined two deep (throughput): batch k+1's columns are
    # copied in and batch k-1's seeds copied out on two copy streams while
    # batch k runs through the graph (two input, output and host sets).
    outs2 = []
    size2 = torch.zeros(BATCH_EVENTS, dtype=torch.int32, device=dev)
    for e in range(BATCH_EVENTS):
        so = seeding.SeedBuffer(alg.max_seeds(len(sps[e])), device=dev)
        so.size = size2[e:e + 1]
        outs2.append(so)
    out_sets = [(outs, size_all), (outs2, size2)]
    in_sets = [(inputs.sps, inputs.dcols), (inputs.sps2, inputs.dcols2)]
    h2d_stream = torch.cuda.Stream(device=dev)
    copy_stream = torch.cuda.Stream(device=dev)
    h2d_done = [torch.cuda.Event() for _ in range(2)]
    computed = [torch.cuda.Event() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    h_sizes = [torch.zeros(BATCH_EVENTS, dtype=torch.int32).pin_memory() for _ in range(2)]
    h_seed_sets = [torch.empty((4, sum(o.capacity for o in outs)), dtype=torch.int32).pin_memory()
                   for _ in range(2)]

    def p_issue(k):
        b = k % 2
        o, sz = out_sets[b]
        isp, icols = in_sets[b]
        with torch.cuda.stream(h2d_stream):
            h2d_stream.wait_event(computed[b])  # batch k-2 read this input set
            for key, col in icols.items():
                col.copy_(inputs.pinned[key], non_blocking=True)
            h2d_done[b].record(h2d_stream)
        stream.wait_event(copied[b])  # batch k-2's seeds were copied out of this set
        flush_buf.fill_(1)
        stream.wait_event(h2d_done[b])
        alg.graph_launch(isp, o, stream=sptr)
        h_sizes[b].copy_(sz, non_blocking=True)
        computed[b].record(stream)

    def p_collect(k):
        b = k % 2
        o, _ = out_sets[b]
        computed[b].synchronize()
        hs = h_seed_sets[b]
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(computed[b])
            off = 0
            for e in range(BATCH_EVENTS):
                ns = int(h_sizes[b][e])
                so = o[e]
                for j, col in enumerate((so.bottom_index, so.middle_index, so.top_index)):
                    hs[j, off:off + ns].copy_(col[:ns], non_blocking=True)
                hs[3, off:off + ns].copy_(so.quality[:ns].view(torch.int32), non_blocking=True)
                off += ns
            copied[b].record(copy_stream)

    def p_run(n):
        for k in range(n):
            p_issue(k)
            if k >= 1:
                p_collect(k - 1)
        p_collect(n - 1)
        copy_stream.synchronize()

    p_run(max(2, args.warmup))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    p_run(args.steps)
    torch.cuda.synchronize()
    pipelined_s = time.perf_counter() - t0
    rep = {
        "workload": BATCH_WORKLOAD, "events_per_batch": BATCH_EVENTS,
        "spacepoints_per_batch": total,
        "min_max_spacepoints": [min(inputs.sizes), max(inputs.sizes)],
        "seeds_per_batch": n_seeds,
        "value": BATCH_EVENTS * args.steps / (sum(lat) / 1e3), "unit": "events/s",
        "latency_ms": {"p50": quantile(lat, 0.5), "p99": quantile(lat, 0.99),
                       "max": max(lat), "batches": len(lat)},
        "e2e": {"value": BATCH_EVENTS * args.steps / (sum(e2e_lat) / 1e3), "unit": "events/s",
                "latency_ms": {"p50": quantile(e2e_lat, 0.5), "p99": quantile(e2e_lat, 0.99)},
                "h2d_bytes_per_batch": int(h2d), "d2h_bytes_per_batch": int(d2h),
                "timing": "one batch at a time: columns in, graph launch, seeds out, wall clock"},
        "e2e_pipelined": {"value": BATCH_EVENTS * args.steps / pipelined_s, "unit": "events/s",
                          "h2d_bytes_per_batch": int(h2d), "d2h_bytes_per_batch": int(d2h),
                          "timing": "wall clock over K batches, two in flight: the column copy "
                                    "of batch k+1 and the seed copy of batch k-1 overlap batch "
                                    "k on two copy streams"},
        "autotune": tuned,
        "gpu_launches_per_batch": len(seeding.KERNEL_NAMES) + (4 if model is not None else 0),
        "l2": "flushed before each batch (256 MiB write)",
    }
    if model is not None:
        per, fb, _ = alg.filter_stats(BATCH_EVENTS)
        frac = (per[:, 1] + per[:, 3]) / np.maximum(per[:, 0] + per[:, 2], 1)
        rep["pruned_fraction"] = {"mean": float(frac.mean()), "min": float(frac.min()),
                                  "max": float(frac.max())}
        rep["fallback_events"] = int(fb.sum())
    return rep, outs


def run_trk1000(args, stream, flush_buf):
    """The 1000-track event (trk1000, seed 0, ~10k spacepoints, 10 % noise):
    ms per event through the per-event API (seeding then parameters), device
    time with the L2 flushed before each event, and its parity with the
    committed oracle outputs (tests/golden/trk1000_s0.npz): seeds bit-exact,
    parameters within 1e-5 relative."""
    import torch

    from traccc_gb300 import seeding, synth
    ev = synth.workload_event("trk1000", 0)
    f, g, fl, tp = seeding.default_configs()
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    est = seeding.SeedParameterEstimationAlgorithm(tp)
    sps = seeding.SpacepointCollection.from_numpy(ev)
    meas = seeding.MeasurementCollection.from_numpy(ev)
    out = seeding.SeedBuffer(alg.max_seeds(len(sps)))
    par = seeding.ParamsBuffer(out.capacity)
    bf = (0.0, 0.0, float(f.bFieldInZ))
    sptr = stream.cuda_stream

    def one():
        alg(sps, out, stream=sptr)
        est(bf, meas, sps, out, par, stream=sptr)

    for _ in range(max(3, args.warmup)):
        one()
    torch.cuda.synchronize()
    ev_t = [torch.cuda.Event(enable_timing=True) for _ in range(2 * args.steps)]
    for k in range(args.steps):
        flush_buf.fill_(1)
        ev_t[2 * k].record(stream)
        one()
        ev_t[2 * k + 1].record(stream)
    torch.cuda.synchronize()
    ms = [ev_t[2 * k].elapsed_time(ev_t[2 * k + 1]) for k in range(args.steps)]
    gold = np.load(os.path.join(ROOT, "tests", "golden", "trk1000_s0.npz"))
    got = out.to_numpy()
    seeds_ok = bool(np.array_equal(got, gold["seeds"]))
    gp, rp = par.to_numpy(), gold["params"]
    params_ok = False
    if seeds_ok and len(gp) == len(rp):
        a, b = gp["params"].astype(np.float64), rp["params"].astype(np.float64)
        d = np.abs(a - b)
        d[:, 2] = np.abs((a[:, 2] - b[:, 2] + np.pi) % (2 * np.pi) - np.pi)
        params_ok = bool(np.all(gp["surface_link"] == rp["surface_link"]) and
                         np.all(d <= 1e-5 * 0.5 * (np.abs(a) + np.abs(b)) + 1e-30))
    return {"workload": f"trk1000: 1 synthetic event (seed 0), 1000 helices, pT log-U(0.5, 20) "
                        f"GeV, 10% noise, {len(sps)} spacepoints",
            "ms_per_event": statistics.median(ms), "ms_per_event_mean": sum(ms) / len(ms),
            "events_per_s": 1e3 * len(ms) / sum(ms), "seeds": len(got),
            "parity": {"seeds_bit_exact": seeds_ok, "params_within_1e-5": params_ok,
                       "against": "tests/golden/trk1000_s0.npz (oracle outputs)"},
            "timing": "per-event API (seedgb_seeding_run + seedgb_params_run), device "
                      "time, L2 flushed before each event"}


FILTER_TRAIN_EVENTS = 200
FILTER_CALIB_EVENTS = 144
# thresholds and band per event size (spacepoints): the calibration events
# span 5k-135k spacepoints, and sparse events need a lower threshold for the
# same recall
FILTER_SIZE_CLASSES = (25000, 50000, 80000, 1 << 31)
# calibrated with a margin above the 99.5 % recall target, for events the
# calibration did not see (at 99.7 % / 99.5 % on 48 events, 4 of the 64
# batch events and 1 of the 20 bench events came out just below 99.5 %; at
# 99.8 % / 99.7 % on 96 events, 1 batch event at 99.45 %)
FILTER_CALIB_TARGET = 0.999
# and at least this recall on every held-out event
FILTER_CALIB_MIN_EVENT = 0.998


def run_formation(args, stream, meas, n_sp_total):
    """Spacepoint formation in front of the step: the 20 events' measurements
    on the synthetic barrel's cylinder surfaces -> spacepoints, device time
    per step (i) in one launch sequence for all events on a device-resident
    surface table (seedgb_formation_run_batch) and (ii) event by event
    (seedgb_form_spacepoints, which uploads the surface table and finishes
    each call before returning).  Fusing formation into binning would save
    at most the spacepoint columns' write and re-read (28 + 12 bytes per
    spacepoint), which the batched figure bounds."""
    import torch

    from traccc_gb300 import seeding, synth
    surf = np.zeros(len(synth.LAYER_RADII) + 1, seeding.SURFACE_DTYPE)
    for layer, r in enumerate(synth.LAYER_RADII):
        surf[layer + 1]["type"] = seeding.SURFACE_CYLINDER
        surf[layer + 1]["radius"] = r
        surf[layer + 1]["rotation"] = np.eye(3, dtype=np.float32).reshape(-1)
    sptr = stream.cuda_stream
    reps = max(1, min(args.steps, 5))
    # (i) batched
    form = seeding.SpacepointFormationAlgorithm(surf)
    outs, counts = form.run_batch(meas, stream=sptr)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    batched = []
    for _ in range(reps):
        e0.record(stream)
        form.run_batch(meas, outs=outs, stream=sptr)
        e1.record(stream)
        e1.synchronize()
        batched.append(e0.elapsed_time(e1))
    formed = int(counts.sum().item())
    # (ii) event by event
    for m in meas:
        seeding.form_spacepoints(surf, m, stream=sptr)
    ev_t = [torch.cuda.Event(enable_timing=True) for _ in range(2 * len(meas))]
    per_event = 0.0
    for _ in range(reps):
        for i, m in enumerate(meas):
            ev_t[2 * i].record(stream)
            seeding.form_spacepoints(surf, m, stream=sptr)
            ev_t[2 * i + 1].record(stream)
        torch.cuda.synchronize()
        per_event += sum(ev_t[2 * i].elapsed_time(ev_t[2 * i + 1]) for i in range(len(meas)))
    return {"batched_ms_per_step": statistics.median(batched),
            "per_event_calls_ms_per_step": per_event / reps, "events": len(meas),
            "spacepoints_formed": formed, "fusion_saving_bound_bytes": 40 * n_sp_total,
            "timing": "device time, CUDA events on the launching stream; batched: one "
                      "seedgb_formation_run_batch call for the step's events (median of "
                      f"{reps}); per event: the seedgb_form_spacepoints calls summed over the "
                      f"events (mean of {reps})"}


GBTS_EDGES_FACTOR = 40


def gbts_setup(events):
    """GBTS on the synthetic barrel: layer table, linked eta bins and
    geometry-id binning from synth.gbts_geometry (10 barrel layers, 0.2 eta
    bins), the reference's default cuts at min_pt 900 MeV with
    max_edges_factor 40 (the reference default of 10 truncates the graph of
    a 100k-spacepoint event of this 10-layer detector), per-measurement
    barcodes and cluster diameters from synth.gbts_measurements."""
    from traccc_gb300 import gbts, seeding, synth
    layers, pairs, geoid = synth.gbts_geometry()
    cfg = gbts.config_default()
    cfg.max_edges_factor = GBTS_EDGES_FACTOR
    alg = gbts.GbtsSeedingAlgorithm(cfg, layers, pairs, geoid, min_pt=900.0)
    data, host = [], []
    for s, ev in enumerate(events):
        link, dia = synth.gbts_measurements(ev, s)
        host.append((ev, link, dia))
        data.append((seeding.SpacepointCollection.from_numpy(ev),
                     seeding.MeasurementCollection.from_numpy(dict(surface_link=link,
                                                                   diameter=dia))))
    outs = [seeding.SeedBuffer(alg.max_seeds(len(ev["global"]))) for ev in events]
    return alg, data, outs, host, (layers, pairs, geoid, cfg)


def run_gbts(args, stream, flush_buf, events):
    """GBTS seeding (the alternative seeder on the same spacepoints) of the
    step's 20 events, one seedgb_gbts_run call per event: events/s over the
    timed steps (CUDA events on the launching stream around each step,
    which include the two waits per call for the path-store size), the first
    event's seeds against the oracle, and the oracle's own time for one
    event on one host thread."""
    import torch

    import oracle
    alg, data, outs, host, (layers, pairs, geoid, cfg) = gbts_setup(events)
    sptr = stream.cuda_stream

    def step():
        for (sp, m), o in zip(data, outs):
            alg(sp, m, o, stream=sptr)

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    steps = max(1, min(args.steps, 10))
    ms = []
    for _ in range(steps):
        flush_buf.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    counters = alg.counters()  # of the last event
    status = alg.last_status(stream=sptr)
    # the same events through seedgb_gbts_run_batch (one call per step)
    sps_l = [d[0] for d in data]
    meas_l = [d[1] for d in data]
    for _ in range(max(3, args.warmup)):
        alg.run_batch(sps_l, meas_l, outs, stream=sptr)
    torch.cuda.synchronize()
    ms_b = []
    for _ in range(steps):
        flush_buf.fill_(1)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        alg.run_batch(sps_l, meas_l, outs, stream=sptr)
        e1.record(stream)
        e1.synchronize()
        ms_b.append(e0.elapsed_time(e1))
    status_b = alg.last_status(stream=sptr)
    # end to end through the same call: every step copies the events' columns
    # in from pinned host memory and the seeds (sizes, then the seeds) out
    cols = []
    for sp, m in data:
        cols.append([(torch.empty_like(t, device="cpu").pin_memory(), t) for t in
                     (sp.measurement_index_1, sp.measurement_index_2, sp.global_, sp.z_variance,
                      sp.radius_variance, m.surface_link, m.diameter)])
    for c_ in cols:
        for h_, d_ in c_:
            h_.copy_(d_)
    h2d = sum(h_.numel() * h_.element_size() for c_ in cols for h_, _ in c_)
    h_size = torch.zeros(len(outs), dtype=torch.int32).pin_memory()
    h_out = [torch.empty((4, max(1, o.capacity)), dtype=torch.int32).pin_memory() for o in outs]

    def e2e_step():
        with torch.cuda.stream(stream):
            for c_ in cols:
                for h_, d_ in c_:
                    d_.copy_(h_, non_blocking=True)
            alg.run_batch(sps_l, meas_l, outs, stream=sptr)
            for i, o in enumerate(outs):
                h_size[i:i + 1].copy_(o.size, non_blocking=True)
        stream.synchronize()
        nbytes = 4 * h_size.numel()
        with torch.cuda.stream(stream):
            for i, o in enumerate(outs):
                ns = int(h_size[i])
                for j, col in enumerate((o.bottom_index, o.middle_index, o.top_index)):
                    h_out[i][j, :ns].copy_(col[:ns], non_blocking=True)
                h_out[i][3, :ns].copy_(o.quality[:ns].view(torch.int32), non_blocking=True)
                nbytes += 16 * ns
        stream.synchronize()
        return nbytes

    for _ in range(2):
        e2e_step()
    t0 = time.perf_counter()
    d2h = 0
    for _ in range(steps):
        d2h = e2e_step()
    e2e_s = time.perf_counter() - t0
    got = outs[0].to_numpy()
    ev, link, dia = host[0]
    oc = oracle.GbtsConfig()
    import ctypes as C
    C.memmove(C.byref(oc), C.byref(cfg), C.sizeof(oc))
    t0 = time.perf_counter()
    ref, rctr = oracle.gbts(ev, link, dia, layers, pairs, geoid, cfg=oc, min_pt=900.0)
    cpu_s = time.perf_counter() - t0
    # one event per host thread (the C call releases the GIL)
    threads = cpu_threads()
    sample = [host[i % len(host)] for i in range(threads)]
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(lambda h: oracle.gbts(h[0], h[1], h[2], layers, pairs, geoid, cfg=oc,
                                          min_pt=900.0), sample))
    cpu_mt_s = time.perf_counter() - t0
    same = bool(len(got) == len(ref) and all(np.array_equal(got[k], ref[k]) for k in
                                             ("bottom", "middle", "top")) and
                np.array_equal(got["quality"].view(np.uint32), ref["quality"].view(np.uint32)))
    n_ev = len(events)
    med = statistics.median(ms)
    return {"workload": f"pileup9k: the step's {n_ev} events; GBTS on the synthetic barrel "
                        f"(10 layers, 0.2 eta bins, {len(pairs)} linked bin pairs), reference "
                        f"default cuts at min_pt 900 MeV, max_edges_factor {GBTS_EDGES_FACTOR}",
            "value": 1e3 * n_ev / med, "unit": "events/s", "ms_per_step": med,
            "ms_per_event": med / n_ev, "status": int(status),
            "e2e": {"value": n_ev * steps / e2e_s, "unit": "events/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h),
                    "timing": "wall clock over the steps: the events' spacepoint and measurement "
                              "columns in from pinned host memory, one seedgb_gbts_run_batch "
                              "call, the seed counts and then the seeds out"},
            "batch": {"value": 1e3 * n_ev / statistics.median(ms_b), "unit": "events/s",
                      "ms_per_step": statistics.median(ms_b), "status": int(status_b),
                      "timing": "one seedgb_gbts_run_batch call per step (event e + 1's kernels "
                                "queued before the wait for event e's path-store size), same "
                                "outputs"},
            "last_event_counters": counters,
            "parity": {"event0_seeds_bit_exact": same, "seeds": len(got),
                       "oracle_seeds": len(ref), "against": "the C oracle (parity unpinned: "
                                                            "the reference has no GBTS tests)"},
            "cpu_oracle": {"s_per_event": cpu_s, "events_per_s": 1.0 / cpu_s, "cores": 1,
                           "sample": "event 0, one host thread"},
            "cpu_oracle_all_cores": {"events_per_s": len(sample) / cpu_mt_s, "cores": threads,
                                     "sample": f"{len(sample)} of the step's events, one per "
                                               f"thread on {threads} threads ({cpu_model()})"},
            "timing": f"median of {steps} steps, each the {n_ev} per-event calls back to back "
                      "on one stream, L2 flushed before each step; CUDA events on the stream"}


FILTER_TRAIN_SEED0 = 1000


def train_filter(args):
    """Learned doublet filter (middle gate): 200 training events of the
    100k-spacepoint workload's statistics (pileup9k, 9000 tracks, seeds
    1000-1199, disjoint from the bench events), labels from the plain seeder,
    trained with the library's kernels; the gate threshold and band
    calibrated per event-size class on 144 held-out events spanning the
    uneven batch's sizes (U(500, 12000) tracks, batch seed 20) for >= 99.9 %
    seed recall over each class's events and >= 99.8 % on each of them (a
    margin above the 99.5 % target for unseen events)."""
    from traccc_gb300 import learned, seeding, synth
    t0 = time.perf_counter()
    train_ev = [synth.workload_event("pileup9k", FILTER_TRAIN_SEED0 + s)
                for s in range(args.filter_events)]
    calib_ev = synth.batch_events(FILTER_CALIB_EVENTS, 20)
    gen_s = time.perf_counter() - t0
    alg = seeding.TripletSeedingAlgorithm()
    model, rep = learned.build_filter(
        alg, train_ev, calib_ev, epochs=4, target=FILTER_CALIB_TARGET, class_max=FILTER_SIZE_CLASSES,
        min_event=FILTER_CALIB_MIN_EVENT)
    rep["generate_s"] = gen_s
    rep["train_workload"] = (f"pileup9k statistics, {len(train_ev)} events (seeds "
                             f"{FILTER_TRAIN_SEED0}-{FILTER_TRAIN_SEED0 + len(train_ev) - 1})")
    rep["calib_workload"] = f"{FILTER_CALIB_EVENTS} uneven events (batch seed 20), size classes"
    rep["mode"] = "middle gate"
    rep.pop("candidates", None)
    return model, rep


def _finite(v):
    """JSON-safe float: None for infinities (a role the filter keeps whole)."""
    v = float(v)
    return v if np.isfinite(v) else None


def recall_report(plain, learned_keys):
    from traccc_gb300 import learned
    rec, out = learned.compare(plain, learned_keys)
    n_plain = sum(len(p) for p in plain)
    return {"min": float(rec.min()), "mean": float(rec.mean()),
            "per_event_ge_0.995": int((rec >= 0.995).sum()), "events": len(rec),
            "outside_plain_set": int(out.sum()),
            "outside_fraction": float(out.sum() / max(n_plain, 1))}


# ---------------------------------------------------------------------------
# CPU side (oracle): baseline and the reference arm
# ---------------------------------------------------------------------------

def cpu_seed_event(ev):
    import oracle
    f, g, fl, tp = oracle.default_configs()
    seeds, _ = oracle.seeding(ev, f, g, fl, phi_mode=oracle.PHI_LIBM)
    oracle.track_params(ev, seeds, (0.0, 0.0, float(f.bFieldInZ)), tp)
    return len(seeds)


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def cpu_run(events, threads):
    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        n_seeds = sum(ex.map(cpu_seed_event, events))
    return time.perf_counter() - t0, n_seeds


def cpu_model():
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def cpu_baseline(events):
    threads = cpu_threads()
    sample = [events[i % len(events)] for i in range(min(threads, 2 * len(events)))]
    dt, _ = cpu_run(sample, threads)
    return {"value": len(sample) / dt, "unit": "events/s", "cores": threads,
            "kind": "port",
            "sample": f"{len(sample)} pileup9k events (seeds 0-{min(len(events), len(sample)) - 1}), "
                      f"one per thread on {threads} threads ({cpu_model()}), oracle with libm "
                      f"phi, seeding + params, {dt:.1f} s"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    threads = cpu_threads()
    from traccc_gb300 import synth
    warm = [synth.workload_event("trk100", s) for s in range(threads)]
    events = make_events(min(threads, args.events))
    sample = [events[i % len(events)] for i in range(threads)]
    for _ in range(args.warmup):
        cpu_run(warm, threads)
    times = []
    for _ in range(args.steps):
        dt, _ = cpu_run(sample, threads)
        times.append(dt)
    tot = sum(times)
    value = len(sample) * args.steps / tot
    line = {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * tot / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": WORKLOAD, "step": f"{len(sample)} events, one per host thread",
                   "l2": "n/a (CPU)"},
        "cpu_baseline": {"value": value, "unit": "events/s", "cores": threads,
                         "kind": "port",
                         "sample": f"{len(sample)} pileup9k events per step on {threads} threads "
                                   f"({cpu_model()}); warm-up steps on trk100 events"},
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.samples.append(parts)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        s = self.samples
        if not s:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(x[1]) for x in s if x[1].replace(".", "").isdigit()]
        mx = [float(x[2]) for x in s if x[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for x in s for n, v in zip(names, x[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(s)}


def load_profile_traffic(kernel, n_events):
    """DRAM bytes and warp instructions per launch of `kernel` from the
    committed ncu summary (profiles/traffic.json), or None when the summary
    is for another number of events than this run's launch."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as fh:
            prof = json.load(fh).get(kernel)
    except Exception:
        return None
    return prof if prof and prof.get("events") == n_events else None


def load_op_model(n_events):
    """Reference FP32 work of the bench events (profiles/op_model.json,
    counted by the oracle offline), or None when it does not cover them."""
    p = os.path.join(ROOT, "profiles", "op_model.json")
    try:
        with open(p) as fh:
            m = json.load(fh)
    except Exception:
        return None
    if m.get("events") != n_events or [e["seed"] for e in m["per_event"]] != list(range(n_events)):
        return None
    return m


def run_gpu(args):
    import torch
    import torch.distributed as dist

    from traccc_gb300 import seeding

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if world > 1:
            dist.barrier()

    events = make_events(args.events)
    n_ev = len(events)
    sizes = [len(e["layer"]) for e in events]
    offs = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
    total = int(offs[-1])

    def cat(key, dt, shape=()):
        return np.ascontiguousarray(np.concatenate([np.asarray(e[key]).reshape((-1,) + shape)
                                                    for e in events]).astype(dt))

    host_cols = {
        "mi1": cat("measurement_index_1", np.uint32).view(np.int32),
        "mi2": cat("measurement_index_2", np.uint32).view(np.int32),
        "glob": cat("global", np.float32, (3,)),
        "zvar": cat("z_variance", np.float32),
        "rvar": cat("radius_variance", np.float32),
        "lp": cat("local_position", np.float32, (2,)),
        "sl": cat("surface_link", np.uint64).view(np.int64),
    }
    dev = torch.device("cuda", local)
    pinned = {k: torch.from_numpy(v).pin_memory() for k, v in host_cols.items()}
    dcols = {k: torch.empty_like(v, device=dev) for k, v in pinned.items()}
    for k in dcols:
        dcols[k].copy_(pinned[k])
    f, g, fl, tp = seeding.default_configs()
    bfield = (0.0, 0.0, float(f.bFieldInZ))
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    est = seeding.SeedParameterEstimationAlgorithm(tp)
    alg.reserve(n_ev, total)
    # launch shape of the seeding kernel for this step: the autotuner's
    # table entry for its events-size bucket, else a search (seeds do not
    # depend on the shape)
    from traccc_gb300 import autotune
    t_path = tune_table_path()
    shape = None if args.retune else autotune.lookup(autotune.load(t_path), total / n_ev)
    t0 = time.perf_counter()
    if shape is None:
        probe = [seeding.SpacepointCollection(
            dcols["mi1"][int(offs[e]):int(offs[e + 1])], dcols["mi2"][int(offs[e]):int(offs[e + 1])],
            dcols["glob"][int(offs[e]):int(offs[e + 1])], dcols["zvar"][int(offs[e]):int(offs[e + 1])],
            dcols["rvar"][int(offs[e]):int(offs[e + 1])]) for e in range(n_ev)]
        shape, t_rep = autotune.tune(alg, probe)
        try:
            os.makedirs(os.path.dirname(t_path), exist_ok=True)
            autotune.store(t_path, total / n_ev, shape, t_rep)
        except OSError:
            pass
        step_tune = {"shape": list(shape), "source": "searched", "measured": len(t_rep),
                     "search_s": time.perf_counter() - t0, "top3": t_rep[:3],
                     "default_ms": next((r["ms"] for r in t_rep
                                         if r["shape"] == [16, 256, 2048, 1]), None)}
    else:
        alg.set_tune(*shape)
        step_tune = {"shape": list(alg.get_tune()), "source": "table " + os.path.basename(t_path)}
    alg.set_option(seeding.OPTION_KERNEL_TIMING, 1)

    def make_views(cols):
        sps, meas = [], []
        for e in range(n_ev):
            a, b = int(offs[e]), int(offs[e + 1])
            sps.append(seeding.SpacepointCollection(cols["mi1"][a:b], cols["mi2"][a:b],
                                                    cols["glob"][a:b], cols["zvar"][a:b],
                                                    cols["rvar"][a:b]))
            meas.append(seeding.MeasurementCollection(cols["lp"][a:b], cols["sl"][a:b]))
        return sps, meas

    sps, meas = make_views(dcols)

    def make_outputs():
        """Seed and parameter buffers of the 20 events, sizes in one array
        (seeds first, then parameters)."""
        size_all = torch.zeros(2 * n_ev, dtype=torch.int32, device=dev)
        souts, pouts = [], []
        for e in range(n_ev):
            so = seeding.SeedBuffer(alg.max_seeds(int(offs[e + 1] - offs[e])), device=dev)
            so.size = size_all[e:e + 1]
            po = seeding.ParamsBuffer(so.capacity, device=dev)
            po.size = size_all[n_ev + e:n_ev + e + 1]
            souts.append(so)
            pouts.append(po)
        return souts, pouts, size_all

    souts, pouts, size_all = make_outputs()
    stream = torch.cuda.current_stream()
    flush_buf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device=dev)

    def step_device(outs=None, ins=None):
        so, po = (souts, pouts) if outs is None else outs
        sp, me = (sps, meas) if ins is None else ins
        alg.run_batch(sp, so, stream=stream)
        est.run_batch(bfield, me, sp, so, po, stream=stream)

    # End to end, pipelined two deep: step k's inputs are copied in on an
    # input stream while step k-1 computes, step k's seeds and parameters are
    # computed on the compute stream while step k-1's results are copied out
    # on an output stream (two input sets, two output sets, two host result
    # sets).  Every step copies its whole input in from pinned memory and its
    # seeds and parameters out.
    out_sets = [(souts, pouts, size_all), make_outputs()]
    dcols2 = {k: torch.empty_like(v) for k, v in dcols.items()}
    in_sets = [(sps, meas), make_views(dcols2)]
    in_cols = [dcols, dcols2]
    h2d_stream = torch.cuda.Stream(device=dev)
    h2d_done = [torch.cuda.Event() for _ in range(2)]
    copy_stream = torch.cuda.Stream(device=dev)
    h_sizes = [torch.zeros(2 * n_ev, dtype=torch.int32).pin_memory() for _ in range(2)]
    h_seeds = [[torch.empty((4, max(1, so.capacity)), dtype=torch.int32).pin_memory()
                for so in out_sets[0][0]] for _ in range(2)]
    h_params = [[torch.empty(po.data.numel(), dtype=torch.uint8).pin_memory()
                 for po in out_sets[0][1]] for _ in range(2)]
    computed = [torch.cuda.Event() for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    h2d_bytes = sum(v.numel() * v.element_size() for v in pinned.values())

    def e2e_issue(k):
        b = k % 2
        so, po, sz = out_sets[b]
        with torch.cuda.stream(h2d_stream):
            # step k-2 computed from this input set
            h2d_stream.wait_event(computed[b])
            for key, col in in_cols[b].items():
                col.copy_(pinned[key], non_blocking=True)
            h2d_done[b].record(h2d_stream)
        # the copies of step k-2 read this output set
        stream.wait_event(copied[b])
        flush_buf.fill_(1)
        stream.wait_event(h2d_done[b])
        step_device((so, po), in_sets[b])
        h_sizes[b].copy_(sz, non_blocking=True)
        computed[b].record(stream)

    def e2e_collect(k):
        b = k % 2
        so, po, _ = out_sets[b]
        computed[b].synchronize()
        d2h = h_sizes[b].numel() * 4
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(computed[b])
            for e in range(n_ev):
                ns, npar = int(h_sizes[b][e]), int(h_sizes[b][n_ev + e])
                for j, col in enumerate((so[e].bottom_index, so[e].middle_index,
                                         so[e].top_index)):
                    h_seeds[b][e][j, :ns].copy_(col[:ns], non_blocking=True)
                h_seeds[b][e][3, :ns].copy_(so[e].quality[:ns].view(torch.int32),
                                            non_blocking=True)
                nb = npar * seeding.PARAMS_DTYPE.itemsize
                h_params[b][e][:nb].copy_(po[e].data[:nb], non_blocking=True)
                d2h += 16 * ns + nb
            copied[b].record(copy_stream)
        return d2h

    def run_e2e(n_steps):
        d2h = 0
        for k in range(n_steps):
            e2e_issue(k)
            if k >= 1:
                d2h = e2e_collect(k - 1)
        d2h = e2e_collect(n_steps - 1)
        copy_stream.synchronize()
        return d2h

    # -- warm-up (also checks the device status once)
    for _ in range(max(3, args.warmup)):
        step_device()
    torch.cuda.synchronize()
    st = alg.last_status(stream)
    if st != seeding.OK:
        raise RuntimeError(f"seeding status {st}")
    counters = alg.counters()

    # -- timed: device-resident inputs
    sampler = ClockSampler(local)
    kt_sum = {k: 0.0 for k in seeding.KERNEL_NAMES}
    step_ms = []
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    torch.cuda.synchronize()
    sampler.start()
    wall0 = time.perf_counter()
    for _ in range(args.steps):
        flush_buf.fill_(1)
        e0.record(stream)
        step_device()
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        for k, v in alg.kernel_times().items():
            kt_sum[k] += v
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    barrier()
    dev_s = sum(step_ms) / 1e3

    # -- timed: end to end through the API from host buffers (pipelined)
    run_e2e(max(2, args.warmup))
    torch.cuda.synchronize()
    barrier()
    t0 = time.perf_counter()
    d2h_bytes = run_e2e(args.steps)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    barrier()

    trk1000 = run_trk1000(args, stream, flush_buf) if world == 1 else None
    formation = run_formation(args, stream, meas, total) if world == 1 else None
    gbts_line = run_gbts(args, stream, flush_buf, events) if world == 1 else None

    learned_line = None
    batched = None
    if world == 1 and not args.no_learned:
        from traccc_gb300 import learned
        # plain seeds of the 20 events (the last step's output)
        step_device()
        torch.cuda.synchronize()
        plain_keys = learned.seed_keys(souts)
        model, train_rep = train_filter(args)
        alg.set_filter(model.struct())
        for _ in range(max(3, args.warmup)):
            step_device()
        torch.cuda.synchronize()
        if alg.last_status(stream) != seeding.OK:
            raise RuntimeError("learned seeding failed")
        lkeys = learned.seed_keys(souts)
        per, fb, _ = alg.filter_stats(n_ev)
        lms = []
        for _ in range(args.steps):
            flush_buf.fill_(1)
            e0.record(stream)
            step_device()
            e1.record(stream)
            e1.synchronize()
            lms.append(e0.elapsed_time(e1))
        alg.set_filter(None)
        frac = (per[:, 1] + per[:, 3]) / np.maximum(per[:, 0] + per[:, 2], 1)
        l_value = n_ev * args.steps / (sum(lms) / 1e3)
        learned_line = {
            "value": l_value, "unit": "events/s", "workload": WORKLOAD,
            "ms_per_step": sum(lms) / args.steps,
            "speedup_vs_plain": l_value / job_throughput(n_ev, args.steps, 1, dev_s),
            "recall": recall_report(plain_keys, lkeys),
            "pruned_fraction": {"mean": float(frac.mean()), "min": float(frac.min()),
                                "max": float(frac.max())},
            "fallback_events": int(fb.sum()),
            "mode": "middle gate (prune_top = SEEDGB_FILTER_GATE_MIDDLE)",
            "threshold": [_finite(v) for v in model.threshold],
            "band": [float(v) for v in model.band],
            "size_classes": [[int(m), [_finite(t) for t in th], [float(b) for b in bd]]
                             for m, th, bd in (model.classes or [])],
            "training": train_rep,
        }
    if not args.no_batched and world == 1:
        inputs = BatchInputs(dev)
        b_plain, outs_plain = run_batched(args, dev, stream, flush_buf, inputs)
        batched = {"plain": b_plain}
        if learned_line is not None:
            from traccc_gb300 import learned
            pk = learned.seed_keys(outs_plain)
            b_learn, outs_learn = run_batched(args, dev, stream, flush_buf, inputs, model)
            b_learn["recall"] = recall_report(pk, learned.seed_keys(outs_learn))
            b_learn["speedup_vs_plain_batched"] = b_learn["value"] / b_plain["value"]
            b_learn["speedup_vs_plain_pileup9k"] = (
                b_learn["value"] / job_throughput(n_ev, args.steps, 1, dev_s))
            batched["learned"] = b_learn
    clocks = sampler.stop()

    dev_s, e2e_s = max_over_ranks([dev_s, e2e_s], dev)
    value = job_throughput(n_ev, args.steps, world, dev_s)
    e2e_value = job_throughput(n_ev, args.steps, world, e2e_s)

    # roofline of the dominant kernel (seed_fast).  Its binding limit is
    # instruction issue: the headline is warp instructions issued per second
    # against SMs x 4 schedulers x clock.  HBM (algorithmic bytes) and the
    # reference-equivalent FP32 op rate are reported beside it.
    dom = max(kt_sum, key=kt_sum.get)
    dom_ms = kt_sum[dom] / args.steps
    n_valid, n_seeds = counters["n_valid"], counters["n_seeds"]
    # algorithmic bytes of seed_fast per launch: every valid spacepoint read
    # once as a middle (x,y,z,r 16 B + its index 4 B), its seed count written
    # (1 B), and per seed the slot (16 B) plus the two partner indices (8 B)
    alg_bytes = {"seed_fast": 21 * n_valid + 24 * n_seeds,
                 "bin_count": 20 * total + 4 * total,
                 "bin_scatter": 20 * total + 4 * total + 28 * n_valid}
    ab = alg_bytes.get(dom, 21 * n_valid + 24 * n_seeds)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = ab / (dom_ms * 1e-3) / 1e9
    prof = load_profile_traffic(dom, n_ev) or {}
    sm_mhz = clocks.get("sm_mhz") or float(peaks.get("sm_max_mhz", 2070.0))
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    hbm = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
        "frac": achieved / hbm_peak, "algorithmic_bytes_per_launch": int(ab),
        "traffic": prof.get("dram_bytes_per_launch"),
        "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else
                       "fallback 6800 GB/s (of fallback)",
    }
    fp32 = None
    om = load_op_model(n_ev) if dom == "seed_fast" else None
    if om is not None:
        peak_fma = n_sm * 128 * 2 * sm_mhz * 1e6
        ach = om["flop_seeding_total"] / (dom_ms * 1e-3)
        fp32 = {
            "bound": "fp32", "flop_per_launch": om["flop_seeding_total"],
            "achieved": ach / 1e12, "peak": peak_fma / 1e12, "unit": "TFLOP/s",
            "frac": ach / peak_fma, "frac_of_fma_free_peak": 2 * ach / peak_fma,
            "source": "profiles/op_model.json: FP32 operations of the reference's doublet "
                      "and triplet tests and lin_circles for these 20 events, counted by "
                      "the oracle; peak = SMs x 128 lanes x 2 (FMA) x median SM clock. The "
                      "build is FMA-free (bit-exact cuts), so half that peak is attainable; "
                      "the GPU skips most triplet tests (exact cot(theta) window), so this "
                      "is a reference-work-equivalent rate"}
    common = {"kernel": dom, "avg_launch_ms": dom_ms,
              "share": kt_sum[dom] / max(1e-12, sum(step_ms)),
              "sm_mhz": sm_mhz, "sms": n_sm}
    if prof.get("inst_issued_per_launch"):
        peak_issue = n_sm * 4 * sm_mhz * 1e6
        ach_issue = prof["inst_issued_per_launch"] / (dom_ms * 1e-3)
        roofline = dict(common, **{
            "bound": "issue", "achieved": ach_issue / 1e9, "peak": peak_issue / 1e9,
            "unit": "G warp-instructions/s", "frac": ach_issue / peak_issue,
            "traffic": prof.get("dram_bytes_per_launch"),
            "inst_issued_per_launch": prof["inst_issued_per_launch"],
            "count_source": prof.get("source"),
            "duration": "average launch time of this run (CUDA events on the launching "
                        "stream); peak = SMs x 4 schedulers x median SM clock of this run",
            "hbm": hbm})
        if fp32 is not None:
            roofline["fp32_op_model"] = fp32
    elif fp32 is not None:
        roofline = dict(common, **fp32, traffic=prof.get("dram_bytes_per_launch"), hbm=hbm)
    else:
        roofline = dict(common, **hbm)

    kernels = {k: v / args.steps for k, v in kt_sum.items()}
    line = {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * dev_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "impl": "seedgb",
        "config": {"workload": WORKLOAD, "events_per_step": n_ev,
                   "spacepoints_per_step": total, "parallelism": f"replicas{world}",
                   "l2": "flushed between steps (256 MiB write)",
                   "path": "plain (no learned filter)",
                   "launch_shape": step_tune},
        "e2e": {"value": e2e_value, "unit": "events/s", "h2d_bytes_per_step": int(h2d_bytes),
                "d2h_bytes_per_step": int(d2h_bytes),
                "ms_per_step": e2e_s * 1e3 / args.steps,
                "timing": "wall clock over all steps, host->device input copy, seeding, "
                          "parameters and device->host result copy of every step; two steps "
                          "in flight (the input copy of step k+1 and the result copy of "
                          "step k-1 overlap step k, on two copy streams)"},
        "gpu_launches": len(seeding.KERNEL_NAMES) + 1,
        "kernel_ms_per_step": kernels,
        "wall_s_timed": wall,
        "roofline": roofline,
        "clocks": clocks,
        "work": {"valid_spacepoints": n_valid, "seeds": n_seeds,
                 "triplets": counters["n_triplets"],
                 "overflow_middles": counters["n_overflow_middles"]},
    }
    if trk1000 is not None:
        line["trk1000"] = trk1000
    if formation is not None:
        line["formation"] = formation
    if gbts_line is not None:
        line["gbts"] = gbts_line
    if learned_line is not None:
        line["learned"] = learned_line
    if batched is not None:
        line["batched"] = batched
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(events)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# Profile cases: small fixed workloads for ncu captures of single kernels.
# `python bench.py --profile-case <case>` sets the case up (for the learned
# filter it also trains and calibrates), then runs the launches to capture
# inside the NVTX range "profile", so that
#     ncu --nvtx --nvtx-include "profile/" -k regex:<kernel> -c <n> ... \
#         python bench.py --profile-case <case>
# captures exactly those launches however many came before.  Cases:
#   plain4    plain seeding of 4 events of the 100k-spacepoint workload
#   plain20   the same for the bench step's 20 events
#   learned4  the same 4 events with the learned doublet filter (trained on
#             16 events, calibrated on 4)
#   train     one gradient step of the filter's network on the doublets of
#             4 events (the tensor-core training kernel)
#   batch64   one graph launch of the 64-event uneven batch
#   gbts1     GBTS seeding of one event of the 100k-spacepoint workload
# ---------------------------------------------------------------------------

def _events(n, seed0=0):
    from traccc_gb300 import synth
    return [synth.workload_event("pileup9k", seed0 + s) for s in range(n)]


def _range(torch, fn):
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("profile")
    fn()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()


def _case_plain(n):
    import torch

    from traccc_gb300 import seeding
    from traccc_gb300 import autotune
    sps = [seeding.SpacepointCollection.from_numpy(e) for e in _events(n)]
    alg = seeding.TripletSeedingAlgorithm()
    # the launch shape the bench runs with (its tune table's entry for these
    # events, when a bench run stored one), so the counters match its launch
    shape = autotune.lookup(autotune.load(tune_table_path()),
                            sum(len(s) for s in sps) / len(sps))
    if shape is not None:
        alg.set_tune(*shape)
    outs = [seeding.SeedBuffer(alg.max_seeds(len(s))) for s in sps]
    for _ in range(2):
        alg.run_batch(sps, outs)
    _range(torch, lambda: alg.run_batch(sps, outs))
    assert alg.last_status() == seeding.OK


def case_plain4():
    _case_plain(4)


def case_plain20():
    # the bench step's 20 events (seeds 0-19): for single-pass counters of
    # the exact launch the bench times
    _case_plain(N_EVENTS)


def _trained_model(alg):
    from traccc_gb300 import learned, synth
    model, rep = learned.build_filter(alg, synth.batch_events(16, 10), synth.batch_events(4, 20),
                                      epochs=3, target=0.995)
    return model, rep


def case_learned4():
    import torch

    from traccc_gb300 import seeding
    alg = seeding.TripletSeedingAlgorithm()
    model, rep = _trained_model(alg)
    sps = [seeding.SpacepointCollection.from_numpy(e) for e in _events(4)]
    outs = [seeding.SeedBuffer(alg.max_seeds(len(s))) for s in sps]
    alg.set_filter(model.struct())
    for _ in range(2):
        alg.run_batch(sps, outs)
    _range(torch, lambda: alg.run_batch(sps, outs))
    assert alg.last_status() == seeding.OK
    per, fb, _ = alg.filter_stats(4)
    print("pruned fraction per event:", ((per[:, 1] + per[:, 3]) / per[:, 2].clip(1)).round(3),
          "fallback:", fb.tolist(), "threshold:", model.threshold)


def case_train():
    import torch

    from traccc_gb300 import learned, seeding
    alg = seeding.TripletSeedingAlgorithm()
    data = learned.collect(alg, _events(4, 100), neg_keep=0.05)
    n = len(data.labels)
    P = torch.from_numpy(learned.init_params(0)).cuda()
    norm = torch.from_numpy(learned.feature_norm(data.features)).cuda()
    G = torch.empty_like(P)
    L = torch.empty(1, dtype=torch.float32, device="cuda")
    pw = float((n - data.labels.sum()) / data.labels.sum())
    for _ in range(2):
        seeding.mlp_grad(P, norm, data.features, data.labels, pw, G, L)
    _range(torch, lambda: seeding.mlp_grad(P, norm, data.features, data.labels, pw, G, L))
    print(f"{n} samples, loss {float(L.item()):.4f}")


def case_batch64():
    import torch

    from traccc_gb300 import seeding, synth
    sps = [seeding.SpacepointCollection.from_numpy(e) for e in synth.batch_events(64, 3)]
    alg = seeding.TripletSeedingAlgorithm()
    outs = [seeding.SeedBuffer(alg.max_seeds(len(s))) for s in sps]
    alg.graph_create(64, sum(len(s) for s in sps))
    for _ in range(2):
        alg.graph_launch(sps, outs)
    _range(torch, lambda: alg.graph_launch(sps, outs))
    assert alg.last_status() == seeding.OK


def case_gbts1():
    import torch
    alg, data, outs, _, _ = gbts_setup(_events(1))
    (sp, m), o = data[0], outs[0]
    for _ in range(2):
        alg(sp, m, o)
    _range(torch, lambda: alg(sp, m, o))
    assert alg.last_status() == 0
    print(alg.counters())


PROFILE_CASES = {"plain4": case_plain4, "plain20": case_plain20, "learned4": case_learned4,
                 "train": case_train, "batch64": case_batch64, "gbts1": case_gbts1}


def main():
    args = parse()
    if args.profile_case:
        PROFILE_CASES[args.profile_case]()
        return 0
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
