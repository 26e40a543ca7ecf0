"""GPU seeding vs the CPU oracle (restated reference host seeding).

Bit-exact grids and seed sets (the oracle in correctly-rounded phi mode);
parameters within the reference's own 1e-5 relative comparison
(performance/src/performance/details/is_same_scalar.cpp:16-18,
is_same_angle.cpp)."""
import numpy as np
import pytest

import oracle
from traccc_gb300 import seeding, synth

pytestmark = pytest.mark.gpu

PARAM_TOL = 1e-5
# The reference's angle comparison (is_same_angle.cpp) is relative to the
# angle itself, so it is ill-conditioned near phi = 0: there both sides carry
# the absolute float rounding of the direction they take the angle of, and a
# relative 1e-5 would ask for ~1e-12 rad at phi ~ 1e-7.  Such angles pass
# within this absolute bound instead; tests count them and keep them rare (on
# the 1.03 M parameter sets of the 100k-spacepoint bench events: 2, the
# largest difference 1.9e-9 rad).
ANGLE_ABS_TOL = 1e-8


def run_gpu(ev, cfgs=None, exhaustive=False):
    import torch
    f, g, fl, tp = cfgs or seeding.default_configs()
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    if exhaustive:
        alg.set_option(seeding.OPTION_EXHAUSTIVE_TRIPLETS, 1)
    sps = seeding.SpacepointCollection.from_numpy(ev)
    out = alg(sps)
    torch.cuda.synchronize()
    st = alg.last_status()
    return alg, sps, out, st


def same_params(a, b, tol=PARAM_TOL, angle_abs=0.0, counts=None):
    """is_same_object<bound_track_parameters> semantics, vectorised; with
    angle_abs > 0 an angle also passes within that absolute difference
    (counted in counts["angle_abs"] when counts is a dict)."""
    ok = a["surface_link"] == b["surface_link"]
    pa, pb = a["params"].astype(np.float64), b["params"].astype(np.float64)
    for k in (0, 1, 3, 4, 5):
        ok &= np.abs(pa[:, k] - pb[:, k]) <= tol * (np.abs(pa[:, k]) + np.abs(pb[:, k])) / 2
    d = (pa[:, 2] - pb[:, 2] + np.pi) % (2 * np.pi) - np.pi
    mean = pb[:, 2] + 0.5 * d
    mean = (mean + np.pi) % (2 * np.pi) - np.pi
    rel = np.abs(d) <= tol * np.abs(mean)
    absol = np.abs(d) <= angle_abs
    if counts is not None:
        counts["angle_abs"] = counts.get("angle_abs", 0) + int((ok & absol & ~rel).sum())
        bad = ok & ~(rel | absol)
        counts["worst_angle_diff"] = max(counts.get("worst_angle_diff", 0.0),
                                         float(np.abs(d[~rel]).max()) if (~rel).any() else 0.0)
        counts["bad_examples"] = counts.get("bad_examples", []) + [
            (float(pa[i, 2]), float(pb[i, 2])) for i in np.nonzero(bad)[0][:3]]
    return ok & (rel | absol)


@pytest.mark.parametrize("name,seed", [("trk100", 0), ("trk100", 1), ("trk1000", 0), ("trk1000", 3)])
def test_seeds_and_grid_match_oracle(name, seed):
    ev = synth.workload_event(name, seed)
    alg, sps, out, st = run_gpu(ev)
    assert st == seeding.OK
    off, bsp = alg.grid(0, len(ev["layer"]))
    roff, rsp, _, _ = oracle.binning(ev, phi_mode=oracle.PHI_CR)
    assert np.array_equal(off, roff)
    assert np.array_equal(bsp, rsp)
    got = out.to_numpy()
    ref, _ = oracle.seeding(ev, phi_mode=oracle.PHI_CR)
    assert len(got) == len(ref)
    assert np.array_equal(got, ref)


def test_params_match_oracle():
    import torch
    ev = synth.workload_event("trk1000", 5)
    f, g, fl, tp = seeding.default_configs()
    alg, sps, out, st = run_gpu(ev)
    est = seeding.SeedParameterEstimationAlgorithm(tp)
    meas = seeding.MeasurementCollection.from_numpy(ev)
    bf = (0.0, 0.0, float(f.bFieldInZ))
    p = est(bf, meas, sps, out)
    torch.cuda.synchronize()
    gp = p.to_numpy()
    rp = oracle.track_params(ev, out.to_numpy(), bf)
    assert len(gp) == len(rp) > 0
    ok = same_params(gp, rp)
    assert ok.all(), np.nonzero(~ok)[0][:10]


def test_small_seed_buffer_reports_overflow():
    """A seed buffer smaller than the event's seeds: the call reports
    SEEDGB_CAPACITY_OVERFLOW through the device status, the buffer holds the
    first seeds in host order and its size is its capacity; the next run
    with room is complete again."""
    import torch
    ev = synth.workload_event("trk1000", 2)
    ref, _ = oracle.seeding(ev, phi_mode=oracle.PHI_CR)
    assert len(ref) > 40
    alg = seeding.TripletSeedingAlgorithm()
    sps = seeding.SpacepointCollection.from_numpy(ev)
    small = seeding.SeedBuffer(37, device=sps.global_.device)
    out = alg(sps, small)
    torch.cuda.synchronize()
    assert alg.last_status() == seeding.CAPACITY_OVERFLOW
    got = out.to_numpy()
    assert len(got) == 37
    assert np.array_equal(got, ref[:37])
    full = alg(sps)
    torch.cuda.synchronize()
    assert alg.last_status() == seeding.OK
    assert np.array_equal(full.to_numpy(), ref)


def test_params_batch_equals_per_event():
    """seedgb_params_run_batch (one launch for several events) gives the same
    bytes as one seedgb_params_run per event, and the oracle's parameters."""
    import torch
    evs = [synth.workload_event("trk1000", s) for s in (5, 6, 7)]
    f, g, fl, tp = seeding.default_configs()
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    sps = [seeding.SpacepointCollection.from_numpy(e) for e in evs]
    meas = [seeding.MeasurementCollection.from_numpy(e) for e in evs]
    outs = alg.run_batch(sps)
    est = seeding.SeedParameterEstimationAlgorithm(tp)
    bf = (0.0, 0.0, float(f.bFieldInZ))
    batch = est.run_batch(bf, meas, sps, outs)
    single = [est(bf, m, s, o) for m, s, o in zip(meas, sps, outs)]
    torch.cuda.synchronize()
    for e, ev in enumerate(evs):
        a, b = batch[e].to_numpy(), single[e].to_numpy()
        assert len(a) == len(b) > 0
        assert a.tobytes() == b.tobytes()
        ok = same_params(a, oracle.track_params(ev, outs[e].to_numpy(), bf))
        assert ok.all()


def test_pileup9k_event_matches_oracle():
    ev = synth.workload_event("pileup9k", 0)
    alg, sps, out, st = run_gpu(ev)
    assert st == seeding.OK
    got = out.to_numpy()
    ref, stats = oracle.seeding(ev, phi_mode=oracle.PHI_CR)
    assert np.array_equal(got, ref)
    c = alg.counters()
    # doublet counters skip middles that can have no top (or no bottom)
    # doublet at all; the triplet count covers the same work as the oracle's
    assert c["n_triplets"] == stats["n_triplets"]
    assert c["n_seeds"] == stats["n_seeds"] == len(ref)
    assert c["n_valid"] == stats["n_valid"]


@pytest.mark.parametrize("name,seed", [("trk1000", 7), ("pileup9k", 3), ("pileup9k", 11)])
def test_fast_paths_equal_exhaustive(name, seed):
    """The cot(theta) window and the fast helix pre-check give exactly the
    results of evaluating every pair with the reference arithmetic."""
    ev = synth.workload_event(name, seed, n_tracks=12000 if name == "pileup9k" else None)
    _, _, a, sa = run_gpu(ev)
    _, _, b, sb = run_gpu(ev, exhaustive=True)
    assert sa == sb == seeding.OK
    assert np.array_equal(a.to_numpy(), b.to_numpy())
