"""Generates tests/golden/workload_hashes.json: for every event of the two
full-size workloads -- the 20 events of the 100k-spacepoint workload (seeds
0-19) and the 64-event uneven batch (batch seed 3) -- the SHA-256 of its
spacepoint columns and of the oracle's seeds (correctly rounded phi), with
the seed count.  The GPU test compares the GPU's seeds of the whole
workloads against these digests without running the oracle; the input
digests show that the event generator reproduced the same events.

    python tests/golden/make_workload_hashes.py
"""
import hashlib
import json
import multiprocessing as mp
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "workload_hashes.json")
INPUT_COLUMNS = ("measurement_index_1", "measurement_index_2", "global", "z_variance",
                 "radius_variance")


def input_digest(ev):
    h = hashlib.sha256()
    for k in INPUT_COLUMNS:
        h.update(np.ascontiguousarray(ev[k]).tobytes())
    return h.hexdigest()


def seed_digest(seeds):
    return hashlib.sha256(np.ascontiguousarray(seeds).tobytes()).hexdigest()


def workloads():
    """(name, events) of the two workloads."""
    sys.path.insert(0, ROOT)
    from traccc_gb300 import synth
    return [("pileup9k", [synth.workload_event("pileup9k", s) for s in range(20)]),
            ("uneven64", synth.batch_events(64, 3))]


def _oracle_entry(args):
    name, i = args
    sys.path.insert(0, ROOT)
    import oracle
    from traccc_gb300 import synth
    ev = (synth.workload_event("pileup9k", i) if name == "pileup9k"
          else synth.batch_events(64, 3)[i])
    seeds, _ = oracle.seeding(ev, phi_mode=oracle.PHI_CR)
    return {"n_sp": int(len(ev["global"])), "input": input_digest(ev),
            "n_seeds": int(len(seeds)), "seeds": seed_digest(seeds)}


def main():
    sys.path.insert(0, ROOT)
    import oracle
    oracle.build()
    jobs = [("pileup9k", i) for i in range(20)] + [("uneven64", i) for i in range(64)]
    with mp.get_context("spawn").Pool(os.cpu_count() or 1) as pool:
        res = pool.map(_oracle_entry, jobs)
    out = {"pileup9k": res[:20], "uneven64": res[20:],
           "generated_by": "python tests/golden/make_workload_hashes.py"}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(OUT, sum(r["n_seeds"] for r in res), "seeds")


if __name__ == "__main__":
    main()
