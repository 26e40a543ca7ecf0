"""Host-side logic without a GPU: the event generator and the multi-rank
aggregation of bench.py (world size 2 over gloo, as the replica path runs
over NCCL on GPUs)."""
import os
import socket

import numpy as np
import pytest

from traccc_gb300 import synth

LAYERS = np.array([32., 72., 116., 172., 260., 360., 500., 600., 700., 820.])


def test_generator_is_deterministic():
    a = synth.workload_event("trk1000", 3)
    b = synth.workload_event("trk1000", 3)
    c = synth.workload_event("trk1000", 4)
    for k in a:
        assert np.array_equal(a[k], b[k])
    assert not np.array_equal(a["global"][:100], c["global"][:100])


def test_generator_geometry_and_sizes():
    ev = synth.workload_event("pileup9k", 0)
    n = len(ev["layer"])
    assert 80_000 < n < 100_000  # ~100k spacepoints per event
    r = np.hypot(ev["global"][:, 0].astype(np.float64), ev["global"][:, 1])
    assert np.allclose(r, LAYERS[ev["layer"]], atol=1e-3)
    assert np.all(np.abs(ev["global"][:, 2]) <= 1000.01)
    assert np.array_equal(ev["measurement_index_1"], np.arange(n, dtype=np.uint32))
    assert np.all(ev["measurement_index_2"] == 0xFFFFFFFF)
    noise = np.count_nonzero(ev["particle"] < 0)
    assert abs(noise / (n - noise) - 0.12) < 0.01


def test_batch_sizes_follow_the_uneven_distribution():
    evs = synth.batch_events(6, seed=1)
    sizes = [len(e["layer"]) for e in evs]
    assert len(set(sizes)) == 6
    assert all(4_000 < s < 140_000 for s in sizes)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks([1.0 + rank, 10.0 - rank], "cpu")
    v = bench.job_throughput(20, 5, world, t[0])
    dist.destroy_process_group()
    q.put((rank, t, v))


def test_replica_aggregation_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in res:
        assert t == [2.0, 10.0]          # max over ranks
        assert v == pytest.approx(2 * 20 * 5 / 2.0)


def test_roofline_constants_only_for_their_event_count():
    """The committed per-launch ncu figures of the seeding kernel and the
    oracle's op model are used only for a launch over the events they were
    taken on (a 4-event run must not divide 20 events' instructions by its
    time)."""
    import bench
    prof = bench.load_profile_traffic("seed_fast", 20)
    assert prof is not None and prof["inst_issued_per_launch"] > 0
    assert bench.load_profile_traffic("seed_fast", 4) is None
    assert bench.load_profile_traffic("no_such_kernel", 20) is None
    assert bench.load_op_model(20) is not None
    assert bench.load_op_model(4) is None
