"""GBTS (graph-based track seeding) through the library's C ABI.

Mirrors traccc's GBTS interface: ``gbts_seedfinder_config`` with
``setLinkingScheme`` (core/include/traccc/gbts_seeding/gbts_seeding_config.hpp,
core/src/gbts_seeding/gbts_seeding_config.cpp) and
``traccc::cuda::gbts_seeding_algorithm`` whose ``operator()(spacepoints,
measurements)`` returns a seed buffer
(device/common/include/traccc/gbts_seeding/device/gbts_seeding_algorithm.hpp:
94-96), plus the reader of the reference's configuration directory
(examples/options/src/track_gbts_seeding.cpp:158-226).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import seeding as _s

_FLOATS_1 = ("tMin_slope", "offset", "tMax_min", "tMax_correction", "tMax_slope", "maxTau")
_FLOATS_2 = ("minDeltaRadius", "min_z0", "max_z0", "maxOuterRadius", "tau_roi", "cut_zMinU",
             "cut_zMaxU", "max_Kappa", "low_Kappa_d0", "high_Kappa_d0", "cut_dphi_max",
             "cut_dcurv_max", "cut_tau_ratio_max", "min_delta_phi", "dphi_coeff",
             "min_delta_phi_low_dr", "dphi_coeff_low_dr", "low_dr_threshold",
             "type1_max_width")
_FLOATS_3 = ("sigmaMS", "radLen", "sigma_x", "sigma_y", "weight_x", "weight_y", "maxDChi2_x",
             "maxDChi2_y", "add_hit", "qual_scale", "inv_max_curvature")
_FLOATS_4 = ("dropout_dcurv_m", "force_dropout_max_curv_m", "best_hit_frac",
             "tight_bid_cot_threshold")
_UINTS = ("n_phi_bins", "max_num_neighbours", "minLevel", "max_edges_factor",
          "edge_bidding_rounds", "volume_shift", "volume_bits", "index_shift", "index_bits")


class GbtsConfig(C.Structure):
    """seedgb_gbts_config: gbts_seedfinder_config's parameters, flattened."""
    _fields_ = ([(n, C.c_float) for n in _FLOATS_1]
                + [("useTauLUT", C.c_int32), ("tau_lut_inv_bin", C.c_float),
                   ("tauLutSize", C.c_uint32)]
                + [(n, C.c_float) for n in _FLOATS_2]
                + [("doTauCut", C.c_int32)]
                + [(n, C.c_float) for n in _FLOATS_3]
                + [("use_dropout", C.c_int32)]
                + [(n, C.c_float) for n in _FLOATS_4]
                + [(n, C.c_uint32) for n in _UINTS])


class GbtsLayer(C.Structure):
    _fields_ = [("type", C.c_int32), ("eta_bin0", C.c_uint32), ("n_eta_bins", C.c_uint32),
                ("min_eta", C.c_float), ("eta_bin_width", C.c_float)]


class GbtsGeoid(C.Structure):
    _fields_ = [("barcode", C.c_uint64), ("layer", C.c_int32)]


LAYER_DTYPE = np.dtype([("type", np.int32), ("eta_bin0", np.uint32), ("n_eta_bins", np.uint32),
                        ("min_eta", np.float32), ("eta_bin_width", np.float32)])
GEOID_DTYPE = np.dtype([("barcode", np.uint64), ("layer", np.int32)], align=True)
COUNTERS = ("nodes", "edges", "connections", "connected_edges", "terminus", "paths", "props",
            "rejected", "seeds")

_ready = False


def lib():
    global _ready
    L = _s.lib()
    if not _ready:
        P, vp = C.POINTER, C.c_void_p
        L.seedgb_gbts_config_default.argtypes = [P(GbtsConfig)]
        L.seedgb_gbts_config_default.restype = None
        L.seedgb_gbts_create.argtypes = [P(GbtsConfig), vp, C.c_uint32, vp, C.c_uint32, vp,
                                         C.c_uint32, C.c_float, vp, C.c_uint32, P(vp)]
        L.seedgb_gbts_create.restype = C.c_int
        L.seedgb_gbts_destroy.argtypes = [vp]
        L.seedgb_gbts_destroy.restype = C.c_int
        L.seedgb_gbts_get_config.argtypes = [vp, P(GbtsConfig), P(C.c_uint32), P(C.c_uint32),
                                             P(C.c_uint32)]
        L.seedgb_gbts_get_config.restype = C.c_int
        L.seedgb_gbts_run.argtypes = [vp, P(_s._SpacepointView), vp, vp, C.c_uint32,
                                      P(_s._SeedBuffer), vp]
        L.seedgb_gbts_run.restype = C.c_int
        L.seedgb_gbts_run_batch.argtypes = [vp, vp, vp, vp, vp, C.c_uint32, vp, vp]
        L.seedgb_gbts_run_batch.restype = C.c_int
        L.seedgb_gbts_last_status.argtypes = [vp, vp]
        L.seedgb_gbts_last_status.restype = C.c_int
        L.seedgb_gbts_counters.argtypes = [vp, P(C.c_uint64)]
        L.seedgb_gbts_counters.restype = C.c_int
        L.seedgb_gbts_read_config_dir.argtypes = [C.c_char_p, vp, P(C.c_uint32), vp,
                                                  P(C.c_uint32), vp, P(C.c_uint32)]
        L.seedgb_gbts_read_config_dir.restype = C.c_int
        _ready = True
    return L


def config_default() -> GbtsConfig:
    c = GbtsConfig()
    lib().seedgb_gbts_config_default(C.byref(c))
    return c


def read_config_dir(path):
    """(layers, bin_pairs [n, 2], geoid_binning) from the reference's GBTS
    configuration directory (geoidBinning.txt, binTables.txt, layerInfo.txt)."""
    L = lib()
    nl, npairs, ng = C.c_uint32(0), C.c_uint32(0), C.c_uint32(0)
    p = os.fsencode(path)
    _s._check(L.seedgb_gbts_read_config_dir(p, None, C.byref(nl), None, C.byref(npairs), None,
                                            C.byref(ng)), "seedgb_gbts_read_config_dir")
    layers = np.zeros(nl.value, LAYER_DTYPE)
    pairs = np.zeros((npairs.value, 2), np.uint32)
    geoid = np.zeros(ng.value, GEOID_DTYPE)
    _s._check(L.seedgb_gbts_read_config_dir(p, layers.ctypes.data, C.byref(nl),
                                            pairs.ctypes.data, C.byref(npairs),
                                            geoid.ctypes.data, C.byref(ng)),
              "seedgb_gbts_read_config_dir")
    return layers, pairs, geoid


def write_config_dir(path, layers, pairs, geoid):
    """Write the three files in the format the reference reads."""
    os.makedirs(path, exist_ok=True)
    with open(os.path.join(path, "geoidBinning.txt"), "w") as f:
        f.write(f"{len(geoid)}\n")
        for g in geoid:
            f.write(f"{int(g['barcode'])} {int(g['layer'])}\n")
    with open(os.path.join(path, "binTables.txt"), "w") as f:
        f.write(f"{len(pairs)}\n")
        for a, b in np.asarray(pairs).reshape(-1, 2):
            f.write(f"{int(a)} {int(b)}\n")
    with open(os.path.join(path, "layerInfo.txt"), "w") as f:
        f.write(f"{len(layers)}\n")
        for l in layers:
            f.write(f"{int(l['type'])} {int(l['eta_bin0'])} {int(l['n_eta_bins'])} "
                    f"{float(l['min_eta']):.9g} {float(l['eta_bin_width']):.9g}\n")


class GbtsSeedingAlgorithm:
    """traccc::cuda::gbts_seeding_algorithm: setLinkingScheme(bin pairs, layers,
    geometry-id binning, min_pt) at construction; __call__(spacepoints,
    measurements) -> SeedBuffer (measurements need surface_link and diameter)."""

    def __init__(self, config: GbtsConfig | None, layers, bin_pairs, geoid_binning,
                 min_pt: float = 900.0, tau_lut=None):
        L = lib()
        cfg = config if config is not None else config_default()
        lay = np.ascontiguousarray(np.asarray(layers).astype(LAYER_DTYPE))
        prs = np.ascontiguousarray(np.asarray(bin_pairs, np.uint32).reshape(-1, 2))
        geo = np.zeros(len(geoid_binning), GEOID_DTYPE)
        geo["barcode"] = np.asarray(geoid_binning["barcode"], np.uint64)
        geo["layer"] = np.asarray(geoid_binning["layer"], np.int32)
        lut = None if tau_lut is None else np.ascontiguousarray(tau_lut, np.float32)
        self._h = C.c_void_p()
        _s._check(L.seedgb_gbts_create(C.byref(cfg), lay.ctypes.data, len(lay), prs.ctypes.data,
                                       len(prs), geo.ctypes.data, len(geo), float(min_pt),
                                       None if lut is None else lut.ctypes.data,
                                       0 if lut is None else len(lut), C.byref(self._h)),
                  "seedgb_gbts_create")

    def __del__(self):
        h = getattr(self, "_h", None)
        if h and h.value:
            lib().seedgb_gbts_destroy(h)
            self._h = None

    def config(self):
        """(config after setLinkingScheme's scaling, eta bins, volume map
        entries, surface map entries)."""
        c = GbtsConfig()
        ne, nv, ns = C.c_uint32(0), C.c_uint32(0), C.c_uint32(0)
        _s._check(lib().seedgb_gbts_get_config(self._h, C.byref(c), C.byref(ne), C.byref(nv),
                                               C.byref(ns)), "seedgb_gbts_get_config")
        return c, ne.value, nv.value, ns.value

    @staticmethod
    def max_seeds(n_spacepoints: int) -> int:
        return 3 * max(1, int(n_spacepoints))

    def __call__(self, spacepoints, measurements, out=None, stream=None):
        if measurements.diameter is None:
            raise ValueError("GBTS seeding needs the measurements' cluster diameters")
        if out is None:
            out = _s.SeedBuffer(self.max_seeds(len(spacepoints)),
                                device=spacepoints.global_.device)
        v = spacepoints.view()
        b = out.buf()
        _s._check(lib().seedgb_gbts_run(self._h, C.byref(v), measurements.surface_link.data_ptr(),
                                        measurements.diameter.data_ptr(),
                                        int(measurements.surface_link.shape[0]), C.byref(b),
                                        _s._stream_ptr(stream)), "seedgb_gbts_run")
        return out

    def run_batch(self, spacepoints, measurements, outs=None, stream=None):
        """seedgb_gbts_run_batch: the events in one call (same seeds as one
        call per event)."""
        n = len(spacepoints)
        if len(measurements) != n:
            raise ValueError("run_batch: one measurement collection per event")
        if any(m.diameter is None for m in measurements):
            raise ValueError("GBTS seeding needs the measurements' cluster diameters")
        if outs is None:
            outs = [_s.SeedBuffer(self.max_seeds(len(sp)), device=sp.global_.device)
                    for sp in spacepoints]
        views = (_s._SpacepointView * n)(*[sp.view() for sp in spacepoints])
        bufs = (_s._SeedBuffer * n)(*[o.buf() for o in outs])
        links = (C.c_void_p * n)(*[m.surface_link.data_ptr() for m in measurements])
        dias = (C.c_void_p * n)(*[m.diameter.data_ptr() for m in measurements])
        nm = (C.c_uint32 * n)(*[int(m.surface_link.shape[0]) for m in measurements])
        _s._check(lib().seedgb_gbts_run_batch(self._h, views, links, dias, nm, n, bufs,
                                              _s._stream_ptr(stream)), "seedgb_gbts_run_batch")
        return outs

    def last_status(self, stream=None) -> int:
        return int(lib().seedgb_gbts_last_status(self._h, _s._stream_ptr(stream)))

    def counters(self) -> dict:
        arr = (C.c_uint64 * len(COUNTERS))()
        _s._check(lib().seedgb_gbts_counters(self._h, arr), "seedgb_gbts_counters")
        return {k: int(v) for k, v in zip(COUNTERS, arr)}
