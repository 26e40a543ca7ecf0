"""The allocation-free binning entry point.

seedgb_spacepoint_binning_noalloc exists for callers that cannot allocate
device memory on their event path (code running during stream capture,
trigger processes that reserve all memory at start-up, plugins of frameworks
that own every allocation).  Its scratch is a fixed array in the library's
device image that every call shares.  These tests call it through the C ABI
and compare its grid with the one the handle-based seeding path builds
(integer output: identical), for two calls in a row on different events, so a
call that inherits the previous call's scratch contents is covered.  The file
is collected last so that a run stopping at the first failure has already run
every other test; it also passes on its own in a fresh process.
"""
import numpy as np
import pytest

from traccc_gb300 import seeding, synth

pytestmark = pytest.mark.gpu


def _noalloc_grid(f, g, ev):
    import torch
    ax = seeding.get_axes(g)
    nb = ax.phi_bins * ax.z_bins
    sps = seeding.SpacepointCollection.from_numpy(ev)
    off = torch.full((nb + 1,), -1, dtype=torch.int32, device="cuda")
    bsp = torch.full((max(1, len(sps)),), -1, dtype=torch.int32, device="cuda")
    st = seeding.spacepoint_binning_noalloc(f, g, sps, off, bsp)
    assert st == seeding.OK, seeding.STATUS.get(st, st)
    torch.cuda.synchronize()
    o = off.cpu().numpy().view(np.uint32)
    return o, bsp.cpu().numpy().view(np.uint32)[: int(o[-1])]


def _handle_grid(f, g, fl, ev):
    import torch
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    alg(seeding.SpacepointCollection.from_numpy(ev))
    torch.cuda.synchronize()
    return alg.grid(0, len(ev["layer"]))


def test_noalloc_binning_equals_seeding_grid_two_calls():
    f, g, fl, _ = seeding.default_configs()
    events = [synth.workload_event("trk1000", 21), synth.workload_event("pileup9k", 22, 5000)]
    # two calls in a row on the shared scratch, then the reference grids
    got = [_noalloc_grid(f, g, ev) for ev in events]
    for ev, (off, bsp) in zip(events, got):
        roff, rbsp = _handle_grid(f, g, fl, ev)
        assert np.array_equal(off, roff)
        assert np.array_equal(bsp, rbsp)
        assert off[-1] > 0


def _padded(ev, n):
    """The event followed by spacepoints far outside the finder's z range
    (dropped by every binning), n spacepoints in all."""
    k = len(ev["global"])
    pad = n - k
    g = np.concatenate([np.asarray(ev["global"], np.float32),
                        np.tile(np.array([[100.0, 0.0, 1.0e6]], np.float32), (pad, 1))])
    return {"measurement_index_1": np.arange(n, dtype=np.uint32),
            "measurement_index_2": np.full(n, 0xFFFFFFFF, np.uint32), "global": g,
            "z_variance": np.zeros(n, np.float32), "radius_variance": np.zeros(n, np.float32),
            "layer": np.zeros(n, np.uint32)}


def test_noalloc_under_stream_capture_replays_on_new_events():
    """The use the entry point exists for: one eager call (caches the scratch
    address), then the call captured into a CUDA graph on a side stream and
    replayed on two events written into the same input buffers; each replay
    gives the handle path's grid."""
    import torch
    f, g, fl, _ = seeding.default_configs()
    ax = seeding.get_axes(g)
    nb = ax.phi_bins * ax.z_bins
    raw = [synth.workload_event("trk1000", 31), synth.workload_event("trk1000", 32)]
    n = max(len(e["global"]) for e in raw) + 17
    events = [_padded(e, n) for e in raw]
    sps = seeding.SpacepointCollection.from_numpy(events[0])
    off = torch.full((nb + 1,), -1, dtype=torch.int32, device="cuda")
    bsp = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    assert seeding.spacepoint_binning_noalloc(f, g, sps, off, bsp) == seeding.OK
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        st = seeding.spacepoint_binning_noalloc(f, g, sps, off, bsp,
                                                stream=torch.cuda.current_stream())
    assert st == seeding.OK
    for ev in events:
        src = seeding.SpacepointCollection.from_numpy(ev)
        for col in ("measurement_index_1", "measurement_index_2", "global_", "z_variance",
                    "radius_variance"):
            getattr(sps, col).copy_(getattr(src, col))
        off.fill_(-1)
        bsp.fill_(-1)
        graph.replay()
        torch.cuda.synchronize()
        o = off.cpu().numpy().view(np.uint32)
        b = bsp.cpu().numpy().view(np.uint32)[: int(o[-1])]
        roff, rbsp = _handle_grid(f, g, fl, ev)
        assert np.array_equal(o, roff) and np.array_equal(b, rbsp)
        assert o[-1] > 0


def test_noalloc_rejects_events_above_its_capacity():
    import torch
    f, g, _, _ = seeding.default_configs()
    n = seeding.NOALLOC_MAX_SPACEPOINTS + 1
    ev = {"measurement_index_1": np.arange(n, dtype=np.uint32),
          "measurement_index_2": np.full(n, 0xFFFFFFFF, np.uint32),
          "global": np.ones((n, 3), np.float32),
          "z_variance": np.zeros(n, np.float32),
          "radius_variance": np.zeros(n, np.float32)}
    sps = seeding.SpacepointCollection.from_numpy(ev)
    off = torch.zeros(1024, dtype=torch.int32, device="cuda")
    bsp = torch.zeros(n, dtype=torch.int32, device="cuda")
    assert seeding.spacepoint_binning_noalloc(f, g, sps, off, bsp) == seeding.SIZE_LIMIT


def test_noalloc_refuses_a_grid_that_cannot_place_the_finders_phi():
    """A grid phi range far narrower than the finder's (here [-0.5, 0.5]
    against [-pi, pi]) cannot place every accepted spacepoint.  The handle
    path reports that after the run (SEEDGB_BAD_CONFIG from last_status);
    the allocation-free entry point refuses the configuration before it
    launches anything, so it never returns SEEDGB_OK with spacepoints left
    out of the grid."""
    import torch
    f, g, fl, _ = seeding.default_configs()
    g.phiMin, g.phiMax = -0.5, 0.5
    ev = synth.workload_event("trk1000", 23)
    alg = seeding.TripletSeedingAlgorithm(f, g, fl)
    alg(seeding.SpacepointCollection.from_numpy(ev))
    torch.cuda.synchronize()
    assert alg.last_status() == seeding.BAD_CONFIG
    ax = seeding.get_axes(g)
    sps = seeding.SpacepointCollection.from_numpy(ev)
    off = torch.full((ax.phi_bins * ax.z_bins + 1,), -1, dtype=torch.int32, device="cuda")
    bsp = torch.full((len(sps),), -1, dtype=torch.int32, device="cuda")
    assert seeding.spacepoint_binning_noalloc(f, g, sps, off, bsp) == seeding.BAD_CONFIG
    torch.cuda.synchronize()
    assert int(off.max().item()) == -1  # nothing was written


def test_noalloc_narrower_grid_that_wraps_equals_seeding_grid():
    """A grid phi range narrower than the finder's whose circular axis still
    wraps every accepted phi ([-2, 2] against [-pi, pi]) is accepted and
    gives the handle path's grid, on two calls in a row."""
    f, g, fl, _ = seeding.default_configs()
    g.phiMin, g.phiMax = -2.0, 2.0
    events = [synth.workload_event("trk1000", 24), synth.workload_event("trk1000", 25)]
    got = [_noalloc_grid(f, g, ev) for ev in events]
    for ev, (off, bsp) in zip(events, got):
        roff, rbsp = _handle_grid(f, g, fl, ev)
        assert np.array_equal(off, roff)
        assert np.array_equal(bsp, rbsp)
