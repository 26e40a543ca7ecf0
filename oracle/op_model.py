"""Algorithmic work of the 100k-spacepoint bench workload, counted by the
oracle (test infrastructure: this script is run by hand, its output is a
committed constant file; nothing on the product path runs it).

Writes profiles/op_model.json: for each of the 20 events the bench seeds
(synthetic, 9000 helices + 12 % noise, seeds 0-19) the reference host
algorithm's work as the oracle executes it:

* n_pair_tests     (middle, neighbour) visits, both roles
                   (doublet_finding.hpp:62-106)
* n_window_pairs   of those, pairs inside the doublet window (first stage of
                   doublet_finding_helper::isCompatible, :59-82)
* n_mb, n_mt       doublets, each transformed once (transform_coordinates,
                   doublet_finding_helper.hpp:218-272: 27 operations)
* n_triplet_tests  middle-bottom x middle-top pairs tested
                   (triplet_finding.hpp:70-182)
* ops_doublet_tests, ops_triplet_tests
                   FP32 operations (+ - * / sqrt, one each) of the doublet
                   and triplet tests as written, counted per stage reached
                   (doublet: 8 window + 39 helix; triplet: 11 + 5 scattering
                   + 1 + 8 helix diameter + 15 remainder)

flop_seeding = ops_doublet_tests + ops_triplet_tests + 27 (n_mb + n_mt) per
event: the FP32 work of the reference's seeding for the event.  The GPU
path skips most triplet tests (exact cot(theta) window), so this count over
the GPU time is a reference-work-equivalent rate.

Usage: python -m oracle.op_model  (from the repository root)
"""
import json
import multiprocessing as mp
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OUT = os.path.join(ROOT, "profiles", "op_model.json")
SEEDS = tuple(range(20))
OPS_LIN_CIRCLE = 27
KEYS = ("n_sp", "n_valid", "n_pair_tests", "n_window_pairs", "n_mb", "n_mt",
        "n_triplet_tests", "n_triplets", "n_seeds", "ops_doublet_tests",
        "ops_triplet_tests")


def event_counts(seed):
    """The oracle's work counters for one event of the bench workload."""
    sys.path.insert(0, ROOT)
    import oracle
    from traccc_gb300 import synth
    ev = synth.workload_event("pileup9k", seed)
    _, st = oracle.seeding(ev, phi_mode=oracle.PHI_CR)
    d = {k: int(st[k]) for k in KEYS}
    d["seed"] = seed
    d["flop_seeding"] = (d["ops_doublet_tests"] + d["ops_triplet_tests"] +
                         OPS_LIN_CIRCLE * (d["n_mb"] + d["n_mt"]))
    return d


def main():
    sys.path.insert(0, ROOT)
    import oracle
    oracle.build()
    with mp.get_context("spawn").Pool(min(len(SEEDS), os.cpu_count() or 1)) as pool:
        per = pool.map(event_counts, SEEDS)
    total = sum(d["flop_seeding"] for d in per)
    out = {
        "workload": "pileup9k: synthetic, 9000 helices + 12% noise, seeds 0-19",
        "events": len(per),
        "ops_lin_circle": OPS_LIN_CIRCLE,
        "flop_seeding_total": total,
        "flop_seeding_per_event": total / len(per),
        "per_event": per,
        "generated_by": "python -m oracle.op_model",
    }
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(f"{OUT}: {total / len(per) / 1e9:.2f} GFLOP per event")


if __name__ == "__main__":
    main()
