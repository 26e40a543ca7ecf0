"""GBTS without a GPU: the oracle's seeds on clean events are the particles'
own hits, the linking scheme follows setLinkingScheme's rules, the library's
config defaults equal the oracle's bit for bit, and the configuration
directory reader reads the reference's format.

The reference has no host GBTS implementation and no GBTS tests, so the
oracle is "parity unpinned": these checks pin its behaviour by physics
(pure seeds, every particle of a clean event found) and by the reference's
configuration logic."""
import ctypes as C

import numpy as np
import pytest

import oracle as O
from traccc_gb300 import gbts, synth


def _purity(ev, seeds):
    part = ev["particle"]
    b, m, t = seeds["bottom"], seeds["middle"], seeds["top"]
    pure = (part[b] == part[m]) & (part[m] == part[t]) & (part[b] >= 0)
    return pure, part


def test_config_defaults_match_the_oracle_bit_for_bit():
    a, b = gbts.config_default(), O.gbts_config_default()
    assert C.sizeof(a) == C.sizeof(b)
    assert bytes(a) == bytes(b)
    # gbts_seeding_config.hpp: qual_scale = 0.01 * INT_MAX / (add_hit * max_cca_iter)
    assert a.qual_scale == np.float32(np.float32(0.01) * np.float32(2147483647.0) /
                                      (np.float32(14.0) * np.float32(15.0)))
    assert (a.cut_zMinU, a.cut_zMaxU) == (-160.0 - 350.0 * 45.0, 160.0 + 350.0 * 45.0)


def test_oracle_finds_every_particle_of_a_clean_event():
    layers, pairs, geoid = synth.gbts_geometry()
    ev = synth.workload_event("trk100", 0)
    link, dia = synth.gbts_measurements(ev)
    seeds, ctr = O.gbts(ev, link, dia, layers, pairs, geoid)
    pure, part = _purity(ev, seeds)
    assert pure.all()
    assert len(np.unique(part[seeds["bottom"]])) == len(np.unique(part[part >= 0]))
    # bottom / middle / top run outwards
    r = np.hypot(ev["global"][:, 0], ev["global"][:, 1])
    assert np.all(r[seeds["bottom"]] < r[seeds["middle"]])
    assert np.all(r[seeds["middle"]] < r[seeds["top"]])
    assert ctr["seeds"] == len(seeds) and ctr["props"] >= ctr["rejected"]


def test_oracle_on_1000_tracks_is_deterministic_and_mostly_pure():
    layers, pairs, geoid = synth.gbts_geometry()
    ev = synth.workload_event("trk1000", 3)
    link, dia = synth.gbts_measurements(ev)
    s1, c1 = O.gbts(ev, link, dia, layers, pairs, geoid)
    s2, c2 = O.gbts(ev, link, dia, layers, pairs, geoid)
    assert np.array_equal(s1, s2) and c1 == c2
    pure, _ = _purity(ev, s1)
    assert pure.mean() > 0.98


def test_pt_threshold_scales_the_cuts():
    """setLinkingScheme scales the phi windows and max curvature by
    900 MeV / minPt: a lower threshold finds more (lower-pT) particles."""
    layers, pairs, geoid = synth.gbts_geometry()
    ev = synth.workload_event("trk1000", 1)
    link, dia = synth.gbts_measurements(ev)
    c900, _, _ = O.gbts_linking(O.gbts_config_default(), geoid, 900.0)
    c450, _, _ = O.gbts_linking(O.gbts_config_default(), geoid, 450.0)
    assert c450.max_Kappa == np.float32(np.float32(3.75e-4) * np.float32(2.0))
    assert c450.min_delta_phi == np.float32(np.float32(0.015) * np.float32(2.0))
    assert c900.max_Kappa == np.float32(3.75e-4)
    hi, _ = O.gbts(ev, link, dia, layers, pairs, geoid, min_pt=900.0)
    lo, _ = O.gbts(ev, link, dia, layers, pairs, geoid, min_pt=450.0)
    ph, part = _purity(ev, hi)
    pl, _ = _purity(ev, lo)
    assert len(np.unique(part[lo["bottom"][pl]])) > len(np.unique(part[hi["bottom"][ph]]))


def test_linking_scheme_rules():
    """gbts_seeding_config.cpp:19-142: one volume on one layer maps to the
    layer; a volume over several layers maps to -(first surface-map entry +
    1) and lists its surfaces; volumes up to the largest that are absent map
    to 0, the next (largest + 1) entries to SHRT_MAX."""
    def bc(vol, idx):
        return (vol << 52) | (idx << 27)
    geoid = np.zeros(6, [("barcode", np.uint64), ("layer", np.int16)])
    geoid[:] = [(bc(5, 1), 3), (bc(5, 2), 3), (bc(7, 1), 0), (bc(7, 2), 1), (bc(7, 3), 1),
                (bc(2, 9), 4)]
    c, vmap, smap = O.gbts_linking(O.gbts_config_default(), geoid, 900.0)
    assert len(vmap) == 2 * (7 + 1)
    assert vmap[5] == 3 and vmap[2] == 4
    assert vmap[7] == -1                       # split: surfaces from map entry 0
    assert vmap[0] == 0 and vmap[3] == 0       # absent, below the largest
    assert np.all(vmap[8:] == 32767)
    # volume 7's surfaces in descending barcode order
    assert smap.tolist() == [[3, 1], [2, 1], [1, 0]]


def test_config_dir_round_trip(tmp_path):
    layers, pairs, geoid = synth.gbts_geometry()
    gbts.write_config_dir(str(tmp_path), layers, pairs, geoid)
    l2, p2, g2 = gbts.read_config_dir(str(tmp_path))
    assert np.array_equal(p2, pairs)
    assert np.array_equal(g2["barcode"], geoid["barcode"])
    assert np.array_equal(g2["layer"], geoid["layer"].astype(np.int32))
    for k in ("type", "eta_bin0", "n_eta_bins", "min_eta", "eta_bin_width"):
        assert np.array_equal(l2[k], layers[k].astype(l2[k].dtype)), k


def test_config_dir_errors_are_statuses(tmp_path):
    with pytest.raises(RuntimeError):
        gbts.read_config_dir(str(tmp_path / "missing"))
    layers, pairs, geoid = synth.gbts_geometry()
    gbts.write_config_dir(str(tmp_path), layers, pairs, geoid)
    (tmp_path / "binTables.txt").write_text("3\n1 2\n3\n")
    with pytest.raises(RuntimeError):
        gbts.read_config_dir(str(tmp_path))


def test_create_refuses_bad_tables_before_device_work():
    """seedgb_gbts_create checks the linking inputs on the host first:
    setLinkingScheme's own failures and tables the kernels could not index
    give SEEDGB_BAD_CONFIG, missing arguments SEEDGB_INVALID_ARGUMENT (no
    GPU is touched on these paths)."""
    L = gbts.lib()
    layers, pairs, geoid = synth.gbts_geometry()
    lay = np.ascontiguousarray(layers.astype(gbts.LAYER_DTYPE))
    prs = np.ascontiguousarray(pairs, np.uint32)
    geo = np.zeros(len(geoid), gbts.GEOID_DTYPE)
    geo["barcode"] = geoid["barcode"]
    geo["layer"] = geoid["layer"]
    cfg = gbts.config_default()

    def create(c=cfg, lay=lay, prs=prs, geo=geo, min_pt=900.0, lut=None, nlut=0):
        h = C.c_void_p()
        return L.seedgb_gbts_create(C.byref(c), lay.ctypes.data if lay is not None else None,
                                    0 if lay is None else len(lay), prs.ctypes.data, len(prs),
                                    geo.ctypes.data, len(geo), min_pt, lut, nlut, C.byref(h))

    BAD, INV = 2, 6
    bad_layer = geo.copy()
    bad_layer["layer"][3] = len(lay)           # a layer the table does not have
    assert create(geo=bad_layer) == BAD
    bad_pair = prs.copy()
    bad_pair[0, 1] = 10 ** 6                   # an eta bin past the last layer's
    assert create(prs=bad_pair) == BAD
    assert create(lay=lay[:0]) == BAD          # no layers
    assert create(min_pt=0.0) == BAD
    c2 = gbts.config_default()                 # decoded volumes >= SHRT_MAX (9 << 12)
    c2.volume_shift, c2.volume_bits = 40, 20
    assert create(c=c2) == BAD
    c3 = gbts.config_default()
    c3.useTauLUT = 1
    lut = np.zeros(7, np.float32)              # not a multiple of 5
    assert create(c=c3, lut=lut.ctypes.data, nlut=7) == BAD
    assert create(c=c3) == BAD                 # the table is missing
    assert L.seedgb_gbts_create(None, lay.ctypes.data, len(lay), prs.ctypes.data, len(prs),
                                geo.ctypes.data, len(geo), 900.0, None, 0,
                                C.byref(C.c_void_p())) == INV
    from traccc_gb300 import seeding
    v = seeding._SpacepointView()
    b = seeding._SeedBuffer()
    assert L.seedgb_gbts_run(None, C.byref(v), None, None, 0, C.byref(b), None) == INV
