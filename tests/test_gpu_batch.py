"""Batched, graph-captured seeding and the autotuner.

GPU: one captured graph serves uneven batches of any size within its
capacity (including an empty event) and gives exactly the seeds of the direct
batched run and of the oracle; batches launched back to back through the two
alternating graph slots do not disturb each other; every launch shape of the
autotuner's search space gives the same seeds.  CPU: the tuning table.
"""
import numpy as np
import pytest

import oracle as O
from traccc_gb300 import autotune, synth

EMPTY = {"measurement_index_1": np.zeros(0, np.uint32),
         "measurement_index_2": np.zeros(0, np.uint32),
         "global": np.zeros((0, 3), np.float32),
         "z_variance": np.zeros(0, np.float32),
         "radius_variance": np.zeros(0, np.float32)}


def _batch(seed, n, lo, hi):
    evs = synth.batch_events(n, seed, lo, hi)
    evs.insert(n // 2, EMPTY)
    return evs


def _collections(seeding, evs):
    return [seeding.SpacepointCollection.from_numpy(e) for e in evs]


def _seeds(outs):
    return [o.to_numpy() for o in outs]


def test_bucket_and_table(tmp_path):
    assert autotune.bucket(1000) == "le1024"
    assert autotune.bucket(88000) == "le131072"
    assert autotune.bucket(3) == "le1024"
    path = str(tmp_path / "tune.json")
    assert autotune.lookup(autotune.load(path), 5000) is None
    autotune.store(path, 5000, (8, 64, 2048, 1), [{"shape": [8, 64, 2048, 1], "ms": 1.5}])
    autotune.store(path, 90000, (6, 128, 2560, 1), [{"shape": [6, 128, 2560, 1], "ms": 9.0}])
    t = autotune.load(path)
    assert autotune.lookup(t, 6000) == (8, 64, 2048, 1)
    assert autotune.lookup(t, 100000) == (6, 128, 2560, 1)
    assert autotune.lookup(t, 200) is None
    assert len(autotune.candidates()) == 3 * 5 * 4 * 2


@pytest.mark.gpu
def test_graph_matches_direct_batch_and_oracle():
    import torch

    from traccc_gb300 import seeding
    alg = seeding.TripletSeedingAlgorithm()
    evs = _batch(7, 9, 100, 1500)
    cols = _collections(seeding, evs)
    total = sum(len(c) for c in cols)
    alg.graph_create(len(cols) + 2, total + 5000)
    got_graph = _seeds(alg.graph_launch(cols))
    assert alg.last_status() == seeding.OK
    direct = _seeds(alg.run_batch(cols))
    assert alg.last_status() == seeding.OK
    torch.cuda.synchronize()
    f, g, fl, _ = O.default_configs()
    for k, (a, b) in enumerate(zip(got_graph, direct)):
        assert np.array_equal(a, b), k
    for k in (0, len(evs) // 2, len(evs) - 1):
        if len(evs[k]["global"]) == 0:
            assert len(got_graph[k]) == 0
            continue
        ref, _ = O.seeding(evs[k], f, g, fl, phi_mode=O.PHI_CR)
        assert np.array_equal(got_graph[k], ref), k


@pytest.mark.gpu
def test_graph_slots_back_to_back():
    """Three different batches launched without a host sync in between (the
    host refills a slot while the other one runs)."""
    import torch

    from traccc_gb300 import seeding
    alg = seeding.TripletSeedingAlgorithm()
    batches = [_batch(s, n, 100, 2500) for s, n in ((1, 6), (2, 11), (3, 3))]
    cols = [_collections(seeding, b) for b in batches]
    cap_sp = max(sum(len(c) for c in cs) for cs in cols)
    alg.graph_create(12, cap_sp)
    outs = [alg.graph_launch(cs) for cs in cols]
    assert alg.last_status() == seeding.OK
    got = [_seeds(o) for o in outs]
    direct = seeding.TripletSeedingAlgorithm()
    for cs, g in zip(cols, got):
        want = _seeds(direct.run_batch(cs))
        assert direct.last_status() == seeding.OK
        for a, b in zip(g, want):
            assert np.array_equal(a, b)
    torch.cuda.synchronize()


@pytest.mark.gpu
def test_graph_rejects_batches_beyond_capacity():
    from traccc_gb300 import seeding
    alg = seeding.TripletSeedingAlgorithm()
    cols = _collections(seeding, synth.batch_events(4, 5, 100, 400))
    total = sum(len(c) for c in cols)
    alg.graph_create(3, total)
    with pytest.raises(seeding.SeedingError) as e:
        alg.graph_launch(cols)
    assert e.value.status == seeding.SIZE_LIMIT
    alg.graph_create(4, total - 1)
    with pytest.raises(seeding.SeedingError) as e:
        alg.graph_launch(cols)
    assert e.value.status == seeding.SIZE_LIMIT


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(4, 8, 256, 1), (10, 32, 1536, 2), (6, 512, 3072, 1),
                                   (8, 4096, 8192, 1)])
def test_launch_shapes_do_not_change_seeds(shape):
    from traccc_gb300 import seeding
    evs = _batch(11, 5, 500, 9000)
    base = seeding.TripletSeedingAlgorithm()
    cols = _collections(seeding, evs)
    want = _seeds(base.run_batch(cols))
    assert base.last_status() == seeding.OK
    alg = seeding.TripletSeedingAlgorithm()
    eff = alg.set_tune(*shape)
    assert eff[1:] == shape[1:] and 1 <= eff[0] <= shape[0]
    alg.graph_create(len(cols), sum(len(c) for c in cols))
    got = _seeds(alg.graph_launch(cols))
    assert alg.last_status() == seeding.OK
    for a, b in zip(got, want):
        assert np.array_equal(a, b)
    # a direct run, a tune change, then the graph again (re-captured)
    direct = _seeds(alg.run_batch(cols))
    for a, b in zip(direct, want):
        assert np.array_equal(a, b)
    alg.set_tune(6, 128, 2560, 1)
    got2 = _seeds(alg.graph_launch(cols))
    assert alg.last_status() == seeding.OK
    for a, b in zip(got2, want):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_autotuner_picks_a_measured_shape(tmp_path):
    from traccc_gb300 import seeding
    alg = seeding.TripletSeedingAlgorithm()
    cols = _collections(seeding, synth.batch_events(6, 21, 500, 4000))
    shapes = [(4, 64, 2048, 1), (8, 128, 2560, 1), (6, 32, 1536, 2)]
    best, report = autotune.tune(alg, cols, shapes=shapes, reps=2)
    assert tuple(report[0]["shape"]) == best
    assert alg.get_tune() == best
    path = str(tmp_path / "t.json")
    mean = sum(len(c) for c in cols) / len(cols)
    autotune.store(path, mean, best, report)
    assert autotune.lookup(autotune.load(path), mean) == best
    alg.graph_launch(cols)
    assert alg.last_status() == seeding.OK
