"""Spacepoint formation on the GPU against the oracle: bit-identical
spacepoints (cylinder and rotated-plane surfaces, pixel / strip mix, unknown
surfaces), measurement order kept, and formation -> seeding gives the
oracle's seeds on the formed spacepoints."""
import numpy as np
import pytest

import oracle as O
from traccc_gb300 import synth

pytestmark = pytest.mark.gpu


def _surfaces(seed=0):
    from tests.test_io_formation import barrel_surfaces
    s = barrel_surfaces()
    rng = np.random.default_rng(seed)
    planes = np.zeros(5, O.SURFACE_DTYPE)
    for k in range(5):
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        planes[k]["type"] = 0
        planes[k]["rotation"] = R.astype(np.float32).reshape(-1)
        planes[k]["translation"] = rng.uniform(-500, 500, 3).astype(np.float32)
    return np.concatenate([s, planes])


def test_formation_matches_oracle():
    import torch

    from traccc_gb300 import seeding
    ev = synth.workload_event("trk1000", 6)
    n = len(ev["global"])
    rng = np.random.default_rng(1)
    link = np.asarray(ev["surface_link"], np.uint64).copy()
    link[rng.choice(n, 300, replace=False)] = rng.integers(11, 16, 300)  # planes
    link[rng.choice(n, 50, replace=False)] = 1000                        # unknown
    dims = np.full(n, 2, np.uint8)
    dims[rng.choice(n, 200, replace=False)] = 1
    surf = _surfaces()
    ref = O.form_spacepoints(surf, ev["local_position"], link, dims)
    meas = seeding.MeasurementCollection.from_numpy(dict(local_position=ev["local_position"],
                                                         surface_link=link))
    sps, k = seeding.form_spacepoints(surf, meas, torch.from_numpy(dims).cuda())
    torch.cuda.synchronize()
    assert k == len(ref["global"])
    got_g = sps.global_.cpu().numpy()
    assert np.array_equal(sps.measurement_index_1.cpu().numpy().view(np.uint32),
                          ref["measurement_index_1"])
    assert np.all(sps.measurement_index_2.cpu().numpy().view(np.uint32) == 0xFFFFFFFF)
    # cos / sin in double rounded to float: identical except where the two
    # libraries' double results straddle a float rounding boundary
    same = np.all(got_g.view(np.uint32) == ref["global"].view(np.uint32), axis=1)
    assert same.mean() > 0.9999
    assert np.abs(got_g - ref["global"]).max() < 1e-3


def test_formation_then_seeding():
    import torch

    from traccc_gb300 import seeding
    ev = synth.workload_event("trk1000", 8)
    surf = _surfaces()
    meas = seeding.MeasurementCollection.from_numpy(ev)
    sps, k = seeding.form_spacepoints(surf, meas)
    alg = seeding.TripletSeedingAlgorithm()
    out = alg(sps)
    assert alg.last_status() == seeding.OK
    got = out.to_numpy()
    g = sps.global_.cpu().numpy()
    formed = {"measurement_index_1": sps.measurement_index_1.cpu().numpy().view(np.uint32),
              "measurement_index_2": sps.measurement_index_2.cpu().numpy().view(np.uint32),
              "global": g, "z_variance": np.zeros(k, np.float32),
              "radius_variance": np.zeros(k, np.float32)}
    ref, _ = O.seeding(formed)
    assert np.array_equal(got, ref)
    torch.cuda.synchronize()


def test_formation_telescope_known_answer():
    """tests/cpu/test_spacepoint_formation.cpp:82-88 on the GPU: nine planes
    at x = 20 ... 180 mm, local axes along global y and z; (7, 2) on the first
    plane -> (20, 7, 2), (10, 15) on the last -> (180, 10, 15)."""
    import torch

    from traccc_gb300 import seeding
    planes = np.zeros(9, O.SURFACE_DTYPE)
    for k, x in enumerate((20., 40., 60., 80., 100., 120., 140., 160., 180.)):
        planes[k]["type"] = 0
        planes[k]["rotation"] = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]],
                                         np.float32).reshape(-1)
        planes[k]["translation"] = (x, 0., 0.)
    meas = seeding.MeasurementCollection.from_numpy(dict(
        local_position=np.array([[7., 2.], [10., 15.]], np.float32),
        surface_link=np.array([0, 8], np.uint64)))
    sps, k = seeding.form_spacepoints(planes, meas,
                                      torch.tensor([2, 2], dtype=torch.uint8, device="cuda"))
    torch.cuda.synchronize()
    assert k == 2
    assert np.array_equal(sps.global_.cpu().numpy()[:2],
                          np.array([[20., 7., 2.], [180., 10., 15.]], np.float32))


def test_batched_formation_equals_per_event_calls():
    """seedgb_formation_run_batch (surface table resident on the device, one
    launch sequence for the batch) forms the same spacepoints, in the same
    order and with the same counts, as seedgb_form_spacepoints event by
    event -- with mixed surfaces, pixel / strip dimensions, unknown surfaces
    and an empty event in the batch -- on two batches in a row (the two
    descriptor slots)."""
    import torch

    from traccc_gb300 import seeding
    surf = _surfaces()
    rng = np.random.default_rng(3)
    events, dims = [], []
    for s in range(4):
        ev = synth.workload_event("trk1000", 30 + s)
        n = len(ev["global"])
        link = np.asarray(ev["surface_link"], np.uint64).copy()
        link[rng.choice(n, 200, replace=False)] = rng.integers(11, 16, 200)
        link[rng.choice(n, 30, replace=False)] = 1000
        d = np.full(n, 2, np.uint8)
        d[rng.choice(n, 100, replace=False)] = 1
        events.append(dict(local_position=ev["local_position"], surface_link=link))
        dims.append(d)
    events.insert(2, dict(local_position=np.zeros((0, 2), np.float32),
                          surface_link=np.zeros(0, np.uint64)))
    dims.insert(2, np.zeros(0, np.uint8))
    meas = [seeding.MeasurementCollection.from_numpy(e) for e in events]
    ddims = [torch.from_numpy(d).cuda() for d in dims]
    alg = seeding.SpacepointFormationAlgorithm(surf)
    for _ in range(2):
        outs, counts = alg.run_batch(meas, ddims)
        torch.cuda.synchronize()
        counts = counts.cpu().numpy()
        for e, (m, d, o) in enumerate(zip(meas, ddims, outs)):
            ref, k = seeding.form_spacepoints(surf, m, d)
            assert counts[e] == k
            for col in ("measurement_index_1", "measurement_index_2", "global_", "z_variance",
                        "radius_variance"):
                a = getattr(o, col)[:k].cpu().numpy()
                b = getattr(ref, col)[:k].cpu().numpy()
                assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), (e, col)
    assert counts[2] == 0
