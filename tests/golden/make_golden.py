"""Generates the golden fixtures of the seeding tests.

Each fixture holds one event's spacepoint and measurement columns and the
oracle's outputs on it: the phi-z grid, the seeds (correctly rounded phi and
this machine's libm phi), the track parameters and the oracle's work counters.
The GPU tests compare against these files, so they do not depend on the event
generator or the C library of the machine that runs them.

    python tests/golden/make_golden.py        # rewrites tests/golden/*.npz

Events: the 100-track workload (seeds 0-2), the 1000-track workload (seed 0),
and an edge-case event: the 1000-track workload (seed 5) with nonzero
spacepoint variances, two non-finite spacepoints, one at z = zMax exactly, one
beyond rMax, and 40 exact duplicates of existing spacepoints (exact ties in
the final seed sort).
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from traccc_gb300 import synth  # noqa: E402

COLUMNS = ("measurement_index_1", "measurement_index_2", "global", "z_variance",
           "radius_variance", "local_position", "surface_link", "layer")


def edge_event():
    ev = synth.workload_event("trk1000", 5)
    rng = np.random.default_rng(12345)
    n = len(ev["layer"])
    ev["z_variance"] = rng.uniform(0.0, 0.05, n).astype(np.float32)
    ev["radius_variance"] = rng.uniform(0.0, 0.01, n).astype(np.float32)
    extra = np.array([[np.nan, 50.0, 10.0], [np.inf, 10.0, 0.0],
                      [60.0, 40.0, 2000.0], [250.0, 10.0, 5.0]], np.float32)
    dup = rng.choice(n, 40, replace=False)
    g = np.concatenate([ev["global"], extra, ev["global"][dup]])
    m = len(g)
    out = {
        "global": g,
        "measurement_index_1": np.arange(m, dtype=np.uint32),
        "measurement_index_2": np.full(m, 0xFFFFFFFF, np.uint32),
        "z_variance": np.concatenate([ev["z_variance"], np.zeros(4, np.float32),
                                      ev["z_variance"][dup]]),
        "radius_variance": np.concatenate([ev["radius_variance"], np.zeros(4, np.float32),
                                           ev["radius_variance"][dup]]),
        "local_position": np.concatenate([ev["local_position"], np.zeros((4, 2), np.float32),
                                          ev["local_position"][dup]]),
        "surface_link": np.concatenate([ev["surface_link"], np.zeros(4, np.uint64),
                                        ev["surface_link"][dup]]),
        "layer": np.concatenate([ev["layer"], np.zeros(4, np.uint32), ev["layer"][dup]]),
    }
    return out


def fixtures():
    yield "trk100_s0", synth.workload_event("trk100", 0)
    yield "trk100_s1", synth.workload_event("trk100", 1)
    yield "trk100_s2", synth.workload_event("trk100", 2)
    yield "trk1000_s0", synth.workload_event("trk1000", 0)
    yield "edge", edge_event()


def main():
    f, g, fl, tp = O.default_configs()
    bfield = (0.0, 0.0, float(f.bFieldInZ))
    for name, ev in fixtures():
        off, bsp, _, _ = O.binning(ev, f, g, phi_mode=O.PHI_CR)
        seeds, st = O.seeding(ev, f, g, fl, phi_mode=O.PHI_CR)
        seeds_libm, _ = O.seeding(ev, f, g, fl, phi_mode=O.PHI_LIBM)
        params = O.track_params(ev, seeds, bfield, tp)
        data = {k: np.asarray(ev[k]) for k in COLUMNS}
        data.update(bin_offsets=off, bin_sps=bsp, seeds=seeds, seeds_libm=seeds_libm,
                    params=params,
                    stats_keys=np.array(list(st.keys())),
                    stats_vals=np.array(list(st.values()), np.uint64))
        path = os.path.join(HERE, f"{name}.npz")
        np.savez_compressed(path, **data)
        print(f"{name}: {len(ev['global'])} spacepoints, {len(seeds)} seeds -> {path}")


if __name__ == "__main__":
    main()
