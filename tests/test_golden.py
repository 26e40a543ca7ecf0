"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py).

CPU: the oracle reproduces its committed outputs (grids and seeds exactly;
track parameters within the reference's 1e-5 comparison, since asin/atan2/sin
come from the machine's C library).  GPU: the seeding library reproduces the
committed grids and seed sets bit for bit, and the parameters within 1e-5, on
the same spacepoints -- including the edge-case event (nonzero variances,
non-finite spacepoints, z = zMax, duplicated spacepoints with exact ties).
"""
import glob
import os

import numpy as np
import pytest

import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
FILES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
NAMES = [os.path.basename(f)[:-4] for f in FILES]


def load(name):
    with np.load(os.path.join(HERE, "golden", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def same_params(a, b, tol=1e-5):
    """is_same_object<bound_track_parameters> (performance/src/performance/
    details/is_same_object.cpp:23-35) over arrays."""
    ok = a["surface_link"] == b["surface_link"]
    pa, pb = a["params"].astype(np.float64), b["params"].astype(np.float64)
    for k in (0, 1, 3, 4, 5):
        ok &= np.abs(pa[:, k] - pb[:, k]) <= tol * (np.abs(pa[:, k]) + np.abs(pb[:, k])) / 2
    d = (pa[:, 2] - pb[:, 2] + np.pi) % (2 * np.pi) - np.pi
    mean = (pb[:, 2] + 0.5 * d + np.pi) % (2 * np.pi) - np.pi
    ok &= np.abs(d) <= tol * np.abs(mean)
    return ok


def test_fixtures_present():
    assert {"trk100_s0", "trk1000_s0", "edge"} <= set(NAMES)


@pytest.mark.parametrize("name", NAMES)
def test_oracle_reproduces_golden(name):
    g = load(name)
    f, gc, fl, tp = O.default_configs()
    off, bsp, _, _ = O.binning(g, f, gc, phi_mode=O.PHI_CR)
    assert np.array_equal(off, g["bin_offsets"])
    assert np.array_equal(bsp, g["bin_sps"])
    seeds, _ = O.seeding(g, f, gc, fl, phi_mode=O.PHI_CR)
    assert np.array_equal(seeds, g["seeds"])
    p = O.track_params(g, seeds, (0.0, 0.0, float(f.bFieldInZ)), tp)
    assert same_params(p, g["params"]).all()


@pytest.mark.parametrize("name", NAMES)
def test_libm_phi_differences_are_bin_edge_cases(name):
    """Seeds with this machine's atan2f differ from the correctly rounded
    ones only if some spacepoint sits within an ulp of a phi-bin edge."""
    g = load(name)
    f, gc, fl, tp = O.default_configs()
    seeds_libm, st = O.seeding(g, f, gc, fl, phi_mode=O.PHI_LIBM)
    if not np.array_equal(seeds_libm, g["seeds"]):
        assert st["near_bin_edges"] > 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", NAMES)
def test_gpu_reproduces_golden(name):
    import torch

    from traccc_gb300 import seeding
    g = load(name)
    f, gc, fl, tp = seeding.default_configs()
    alg = seeding.TripletSeedingAlgorithm(f, gc, fl)
    sps = seeding.SpacepointCollection.from_numpy(g)
    seeds = alg(sps)
    est = seeding.SeedParameterEstimationAlgorithm(tp)
    params = est((0.0, 0.0, float(f.bFieldInZ)), seeding.MeasurementCollection.from_numpy(g),
                 sps, seeds)
    torch.cuda.synchronize()
    assert alg.last_status() == seeding.OK
    off, bsp = alg.grid(0, len(g["global"]))
    assert np.array_equal(off, g["bin_offsets"])
    assert np.array_equal(bsp, g["bin_sps"])
    got = seeds.to_numpy()
    assert np.array_equal(got, g["seeds"])
    gp = params.to_numpy()
    assert len(gp) == len(g["params"])
    ok = same_params(gp, g["params"])
    assert ok.all(), np.nonzero(~ok)[0][:10]
