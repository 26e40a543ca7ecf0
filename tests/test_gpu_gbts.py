"""GBTS seeding on the GPU against the oracle: identical seeds (indices and
quality bits, in the same canonical order) and identical counters, on clean
and dense events, with the edge budget binding and not, with end-cap layer
types and the tau lookup table, at another pT threshold; plus empty events,
events with no usable spacepoint, bad measurement indices and a seed
buffer too small."""
import numpy as np
import pytest

import oracle as O
from traccc_gb300 import gbts, synth

pytestmark = pytest.mark.gpu


def _run(ev, link, dia, layers, pairs, geoid, cfg=None, min_pt=900.0, tau_lut=None, cap=None):
    import torch

    from traccc_gb300 import seeding
    alg = gbts.GbtsSeedingAlgorithm(cfg, layers, pairs, geoid, min_pt=min_pt, tau_lut=tau_lut)
    sps = seeding.SpacepointCollection.from_numpy(ev)
    meas = seeding.MeasurementCollection.from_numpy(dict(surface_link=link, diameter=dia))
    out = seeding.SeedBuffer(cap if cap is not None else alg.max_seeds(len(ev["global"])))
    alg(sps, meas, out)
    torch.cuda.synchronize()
    return alg, out


def _compare(ev, link, dia, layers, pairs, geoid, cfg=None, min_pt=900.0, tau_lut=None):
    alg, out = _run(ev, link, dia, layers, pairs, geoid, cfg, min_pt, tau_lut)
    assert alg.last_status() == 0
    ref, rctr = O.gbts(ev, link, dia, layers, pairs, geoid,
                       cfg=None if cfg is None else _oracle_cfg(cfg), min_pt=min_pt,
                       tau_lut=tau_lut)
    got = out.to_numpy()
    assert alg.counters() == rctr
    assert len(got) == len(ref)
    for k in ("bottom", "middle", "top"):
        assert np.array_equal(got[k], ref[k]), k
    assert np.array_equal(got["quality"].view(np.uint32), ref["quality"].view(np.uint32))
    return got, rctr


def _oracle_cfg(cfg):
    import ctypes as C
    o = O.GbtsConfig()
    C.memmove(C.byref(o), C.byref(cfg), C.sizeof(o))
    return o


@pytest.mark.parametrize("name,seed", [("trk100", 0), ("trk1000", 0), ("trk1000", 5)])
def test_gbts_matches_oracle(name, seed):
    layers, pairs, geoid = synth.gbts_geometry()
    ev = synth.workload_event(name, seed)
    link, dia = synth.gbts_measurements(ev, seed)
    got, ctr = _compare(ev, link, dia, layers, pairs, geoid)
    assert ctr["seeds"] > 0


def test_gbts_dense_event_full_and_capped_edge_budget():
    """100k spacepoints: with max_edges_factor 40 the graph is complete; with
    the reference default (10) the edge budget binds and the first edges in
    the canonical order are kept."""
    layers, pairs, geoid = synth.gbts_geometry()
    ev = synth.workload_event("pileup9k", 0)
    link, dia = synth.gbts_measurements(ev)
    for factor in (40, 10):
        cfg = gbts.config_default()
        cfg.max_edges_factor = factor
        got, ctr = _compare(ev, link, dia, layers, pairs, geoid, cfg=cfg)
        if factor == 10:
            assert ctr["edges"] > 10 * ctr["nodes"]
        assert ctr["seeds"] > 0


def test_gbts_lower_pt_threshold():
    layers, pairs, geoid = synth.gbts_geometry()
    ev = synth.workload_event("trk1000", 2)
    link, dia = synth.gbts_measurements(ev, 2)
    _compare(ev, link, dia, layers, pairs, geoid, min_pt=500.0)


def test_gbts_endcap_types_and_tau_table():
    """Layers of type 1 / 2 (wide clusters on type 1 dropped, diameters
    replaced by -type under doTauCut), then the tau window from a lookup
    table instead of the linear formula."""
    layers, pairs, geoid = synth.gbts_geometry()
    layers = layers.copy()
    layers["type"][7] = 1
    layers["type"][9] = 2
    ev = synth.workload_event("trk1000", 4)
    link, dia = synth.gbts_measurements(ev, 4)
    _compare(ev, link, dia, layers, pairs, geoid)
    cfg = gbts.config_default()
    cfg.useTauLUT = 1
    cfg.tau_lut_inv_bin = 20.0
    n_bins = 16
    lut = np.zeros(5 * n_bins, np.float32)
    for b in range(n_bins):
        w = (b + 1) / 20.0
        lut[5 * b:5 * b + 5] = (w, max(0.0, 6.5 * (w - 0.25)), 1.8 + 6.5 * w, -1.0, -1.0)
    cfg.tauLutSize = len(lut) - 5
    _compare(ev, link, dia, layers, pairs, geoid, cfg=cfg, tau_lut=lut)


def test_gbts_empty_and_unmapped_events():
    layers, pairs, geoid = synth.gbts_geometry()
    ev = synth.workload_event("trk100", 1)
    link, dia = synth.gbts_measurements(ev)
    # every barcode in a volume the binning does not know
    bad = (np.uint64(4000) << np.uint64(52)) | (link & np.uint64((1 << 52) - 1))
    alg, out = _run(ev, bad, dia, layers, pairs, geoid)
    assert alg.last_status() == 0 and len(out.to_numpy()) == 0
    assert alg.counters()["nodes"] == 0
    z = {k: v[:0] for k, v in ev.items()}
    alg, out = _run(z, link[:0], dia[:0], layers, pairs, geoid)
    assert alg.last_status() == 0 and len(out.to_numpy()) == 0


def test_gbts_bad_measurement_index_and_small_buffer():
    layers, pairs, geoid = synth.gbts_geometry()
    ev = synth.workload_event("trk100", 2)
    link, dia = synth.gbts_measurements(ev, 2)
    ref, _ = O.gbts(ev, link, dia, layers, pairs, geoid)
    alg, out = _run(ev, link, dia, layers, pairs, geoid, cap=10)
    assert alg.last_status() == 4  # SEEDGB_CAPACITY_OVERFLOW
    got = out.to_numpy()
    assert len(got) == 10
    assert np.array_equal(got["top"], ref["top"][:10])
    ev2 = dict(ev)
    mi = ev["measurement_index_1"].copy()
    mi[5] = 10 ** 6
    ev2["measurement_index_1"] = mi
    alg, out = _run(ev2, link, dia, layers, pairs, geoid)
    assert alg.last_status() == 6  # SEEDGB_INVALID_ARGUMENT


def test_gbts_batch_equals_per_event_calls():
    """seedgb_gbts_run_batch (events alternating over two work areas, each
    event's kernels queued before the previous event's wait) gives the seeds
    of one call per event -- on a batch with an empty event, a small and a
    100k-spacepoint event -- twice in a row."""
    import torch

    from traccc_gb300 import seeding
    layers, pairs, geoid = synth.gbts_geometry()
    cfg = gbts.config_default()
    cfg.max_edges_factor = 40
    alg = gbts.GbtsSeedingAlgorithm(cfg, layers, pairs, geoid)
    evs = [synth.workload_event("trk1000", 11), synth.workload_event("pileup9k", 12),
           synth.workload_event("trk100", 13), synth.workload_event("pileup9k", 14, 3000)]
    evs.insert(2, {k: v[:0] for k, v in evs[0].items()})
    sps, meas = [], []
    for s, ev in enumerate(evs):
        link, dia = synth.gbts_measurements(ev, s) if len(ev["global"]) else (
            np.zeros(0, np.uint64), np.zeros(0, np.float32))
        sps.append(seeding.SpacepointCollection.from_numpy(ev))
        meas.append(seeding.MeasurementCollection.from_numpy(dict(surface_link=link, diameter=dia)))
    single = []
    for sp, m in zip(sps, meas):
        single.append(alg(sp, m).to_numpy())
    assert alg.last_status() == 0
    for _ in range(2):
        outs = alg.run_batch(sps, meas)
        torch.cuda.synchronize()
        assert alg.last_status() == 0
        for got, ref in zip(outs, single):
            g = got.to_numpy()
            assert len(g) == len(ref)
            for k in ("bottom", "middle", "top"):
                assert np.array_equal(g[k], ref[k])
            assert np.array_equal(g["quality"].view(np.uint32), ref["quality"].view(np.uint32))
    assert len(single[2]) == 0 and len(single[1]) > 0


def _long_chain_event():
    """24 barrel layers 30 mm apart and straight tracks from the beam line:
    chains of up to 23 edges, past the automaton's 15 iterations, plus
    tracks crossing only the first 12 layers (chains that settle)."""
    radii = 40.0 + 30.0 * np.arange(24)
    layers = np.zeros(len(radii), gbts.LAYER_DTYPE)
    for i in range(len(radii)):
        layers[i] = (0, i, 1, -5.0, 10.0)          # one eta bin per layer
    pairs = np.array([(i, i + 1) for i in range(len(radii) - 1)], np.uint32)
    geoid = np.zeros(len(radii), [("barcode", np.uint64), ("layer", np.int16)])
    geoid["barcode"] = (np.arange(1, len(radii) + 1, dtype=np.uint64) << np.uint64(52))
    geoid["layer"] = np.arange(len(radii))
    pts, lay, part = [], [], []
    rng = np.random.default_rng(5)
    for k, phi in enumerate(rng.uniform(-3.0, 3.0, 12)):
        tau = rng.uniform(0.2, 1.2)
        z0 = rng.uniform(-50.0, 50.0)
        n_layers = len(radii) if k % 2 == 0 else 12
        for i in range(n_layers):
            r = radii[i]
            pts.append((r * np.cos(phi), r * np.sin(phi), z0 + tau * r))
            lay.append(i)
            part.append(k)
    g = np.asarray(pts, np.float32)
    n = len(g)
    ev = {"measurement_index_1": np.arange(n, dtype=np.uint32),
          "measurement_index_2": np.full(n, 0xFFFFFFFF, np.uint32), "global": g,
          "z_variance": np.zeros(n, np.float32), "radius_variance": np.zeros(n, np.float32),
          "layer": np.asarray(lay, np.uint32), "particle": np.asarray(part, np.int32)}
    link = (np.asarray(lay, np.uint64) + np.uint64(1)) << np.uint64(52)
    dia = np.zeros(n, np.float32)      # no cluster width: the full tau window
    return ev, link, dia, layers, pairs, geoid


def test_gbts_chains_longer_than_the_automaton():
    ev, link, dia, layers, pairs, geoid = _long_chain_event()
    got, ctr = _compare(ev, link, dia, layers, pairs, geoid)
    assert ctr["connected_edges"] > 0 and ctr["seeds"] > 0
    # a 24-layer track's 23-edge chain: its 8 innermost edges would need more
    # than 15 iterations, are capped and never enter a path, so its seeds
    # start at layer 8; a 12-layer track's seeds start at layer 0
    part = ev["particle"]
    lay = ev["layer"]
    assert np.all(part[got["bottom"]] == part[got["top"]])
    for k in range(12):
        b = lay[got["bottom"][part[got["bottom"]] == k]]
        assert len(b) > 0
        assert b.min() == (8 if k % 2 == 0 else 0), (k, b.min())


def _bundle_event(n=600, n_long=30, seed=11):
    """Four barrel layers 30 mm apart and a bundle of straight tracks 5 mrad
    wide in phi: 600 tracks cross the first two layers, 30 of them all four.
    Every outer node of layer 1 pairs with the inner nodes of each 128-node
    chunk of layer 0, so a quarter of a work item holds 150-160 outer nodes
    with edges: more than the edge walk's 128-record stage, which sends those
    units through the two-walk fallback (count, then write)."""
    radii = np.array([50.0, 80.0, 110.0, 140.0])
    layers = np.zeros(len(radii), gbts.LAYER_DTYPE)
    for i in range(len(radii)):
        layers[i] = (0, i, 1, -5.0, 10.0)          # one eta bin per layer
    pairs = np.array([(0, 1), (1, 2), (2, 3)], np.uint32)
    geoid = np.zeros(len(radii), [("barcode", np.uint64), ("layer", np.int16)])
    geoid["barcode"] = np.arange(1, len(radii) + 1, dtype=np.uint64) << np.uint64(52)
    geoid["layer"] = np.arange(len(radii))
    rng = np.random.default_rng(seed)
    phi = rng.uniform(0.500, 0.505, n)
    tau = rng.uniform(0.40, 0.42, n)
    z0 = rng.uniform(-2.0, 2.0, n)
    pts, lay = [], []
    for k in range(n):
        for i in range(len(radii) if k < n_long else 2):
            r = radii[i]
            pts.append((r * np.cos(phi[k]), r * np.sin(phi[k]), z0[k] + tau[k] * r))
            lay.append(i)
    g = np.asarray(pts, np.float32)
    m = len(g)
    ev = {"measurement_index_1": np.arange(m, dtype=np.uint32),
          "measurement_index_2": np.full(m, 0xFFFFFFFF, np.uint32), "global": g,
          "z_variance": np.zeros(m, np.float32), "radius_variance": np.zeros(m, np.float32)}
    link = (np.asarray(lay, np.uint64) + np.uint64(1)) << np.uint64(52)
    return ev, link, np.zeros(m, np.float32), layers, pairs, geoid


def test_gbts_dense_bundle_past_the_edge_record_stage():
    ev, link, dia, layers, pairs, geoid = _bundle_event()
    cfg = gbts.config_default()
    cfg.max_edges_factor = 400      # every edge of the bundle is kept
    got, ctr = _compare(ev, link, dia, layers, pairs, geoid, cfg=cfg)
    assert ctr["edges"] > 90000 and ctr["connections"] > 0 and ctr["seeds"] > 0
