"""ctypes front-end of the CPU seeding oracle.

TEST INFRASTRUCTURE ONLY.  The oracle is a plain-C restatement of traccc's
host seeding (``core/src/seeding/*``) and host track-parameter estimation
(``core/src/seeding/track_params_estimation.cpp``).  Only the tests, the smoke
check and bench.py's CPU-baseline leg import this module; the product package
``traccc_gb300`` never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_lib", "libseedoracle.so")

PHI_LIBM = 0
PHI_CR = 1


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (-O2 -ffp-contract=off) into oracle/_lib."""
    srcs = [os.path.join(_HERE, f) for f in ("seeding_oracle.c", "gbts_oracle.c")]
    deps = srcs + [os.path.join(_HERE, f) for f in ("seeding_oracle.h", "gbts_oracle.h")]
    if (not force and os.path.exists(_LIB_PATH)
            and all(os.path.getmtime(_LIB_PATH) >= os.path.getmtime(d) for d in deps)):
        return _LIB_PATH
    os.makedirs(os.path.dirname(_LIB_PATH), exist_ok=True)
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-std=c11", "-D_GNU_SOURCE", "-shared", "-o", _LIB_PATH] + srcs + ["-lm"]
    subprocess.run(cmd, check=True)
    return _LIB_PATH


class FinderConfig(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "zMin", "zMax", "rMax", "rMin", "collisionRegionMin",
        "collisionRegionMax", "phiMin", "phiMax", "minPt", "cotThetaMax",
        "deltaRMin", "deltaRMax", "deltaZMax", "impactMax", "sigmaScattering",
        "maxPtScattering")] + [
        ("maxSeedsPerSpM", C.c_uint32), ("bFieldInZ", C.c_float),
        ("beamPos", C.c_float * 2)] + [(n, C.c_float) for n in (
            "radLengthPerSeed", "zAlign", "rAlign", "sigmaError", "highland",
            "maxScatteringAngle2", "pTPerHelixRadius", "minHelixDiameter2",
            "minHelixRadius", "pT2perRadius")] + [
        ("phiBinDeflectionCoverage", C.c_int32),
        ("neighbor_scope", C.c_uint32 * 2)]


class GridConfig(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "bFieldInZ", "minPt", "rMax", "zMax", "zMin", "deltaRMax",
        "cotThetaMax", "impactMax", "phiMin", "phiMax")] + [
        ("phiBinDeflectionCoverage", C.c_int32)]


class FilterConfig(C.Structure):
    _fields_ = [(n, C.c_float) for n in (
        "deltaInvHelixDiameter", "impactWeightFactor", "compatSeedWeight",
        "deltaRMin")] + [("compatSeedLimit", C.c_uint64)] + [
        (n, C.c_float) for n in (
            "good_spB_min_radius", "good_spB_weight_increase",
            "good_spT_max_radius", "good_spT_weight_increase",
            "good_spB_min_weight", "seed_min_weight", "spB_min_radius")]


class TPConfig(C.Structure):
    _fields_ = [("initial_sigma", C.c_float * 6),
                ("initial_sigma_qopt", C.c_float),
                ("initial_sigma_pt_rel", C.c_float),
                ("initial_inflation", C.c_float * 6)]


class Axes(C.Structure):
    _fields_ = [("phi_bins", C.c_uint32), ("phi_min", C.c_float),
                ("phi_max", C.c_float), ("z_bins", C.c_uint32),
                ("z_min", C.c_float), ("z_max", C.c_float)]


class Spacepoints(C.Structure):
    _fields_ = [("measurement_index_1", C.POINTER(C.c_uint32)),
                ("measurement_index_2", C.POINTER(C.c_uint32)),
                ("glob", C.POINTER(C.c_float)),
                ("z_variance", C.POINTER(C.c_float)),
                ("radius_variance", C.POINTER(C.c_float)),
                ("size", C.c_uint32)]


class Measurements(C.Structure):
    _fields_ = [("local_position", C.POINTER(C.c_float)),
                ("surface_link", C.POINTER(C.c_uint64)),
                ("size", C.c_uint32)]


SEED_DTYPE = np.dtype([("bottom", "<u4"), ("middle", "<u4"), ("top", "<u4"),
                       ("quality", "<f4")])
PARAMS_DTYPE = np.dtype([("surface_link", "<u8"), ("params", "<f4", (6,)),
                         ("cov", "<f4", (36,))])

_STATS_FIELDS = (
    "n_sp", "n_valid", "n_pair_tests", "n_mb", "n_mt", "n_middles_with_mb",
    "n_middles_both", "n_triplet_tests", "n_triplets", "n_triplets_after_cut",
    "n_seeds", "max_mb_per_middle", "max_mt_per_middle",
    "max_triplets_per_mb", "max_triplets_per_middle", "max_bin_size",
    "max_neighbourhood", "near_doublet_cuts", "near_triplet_cuts",
    "near_bin_edges", "phi_cr_undecided", "n_scored_mb", "n_scored_mt",
    "n_pruned_mb", "n_pruned_mt", "n_window_pairs", "ops_doublet_tests",
    "ops_triplet_tests")


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in _STATS_FIELDS]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n in _STATS_FIELDS}


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        P = C.POINTER
        L.or_finder_config_default.argtypes = [P(FinderConfig)]
        L.or_finder_config_setup.argtypes = [P(FinderConfig)]
        L.or_grid_config_from_finder.argtypes = [P(GridConfig), P(FinderConfig)]
        L.or_filter_config_default.argtypes = [P(FilterConfig)]
        L.or_tp_config_default.argtypes = [P(TPConfig)]
        L.or_get_axes.argtypes = [P(GridConfig), P(Axes)]
        L.or_get_axes.restype = C.c_int
        for f in ("or_regular_bin", "or_circular_bin"):
            getattr(L, f).argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_float]
            getattr(L, f).restype = C.c_uint32
        for f in ("or_regular_range", "or_circular_range"):
            getattr(L, f).argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_float,
                                      P(C.c_uint32), P(C.c_uint32)]
        for f in ("or_regular_zone", "or_circular_zone"):
            getattr(L, f).argtypes = [C.c_uint32, C.c_float, C.c_float, C.c_float,
                                      P(C.c_uint32), P(C.c_uint32), C.c_uint32]
            getattr(L, f).restype = C.c_uint32
        L.or_circular_remap.argtypes = [C.c_uint32, C.c_uint32, C.c_int32]
        L.or_circular_remap.restype = C.c_uint32
        L.or_sp_phi.argtypes = [C.c_float, C.c_float, C.c_int, P(C.c_int)]
        L.or_sp_phi.restype = C.c_float
        L.or_is_valid_sp.argtypes = [P(FinderConfig), C.c_float, C.c_float,
                                     C.c_float, C.c_int]
        L.or_is_valid_sp.restype = C.c_int
        L.or_binning.argtypes = [P(FinderConfig), P(Axes), P(Spacepoints), C.c_int,
                                 P(C.c_uint32), P(C.c_uint32), P(C.c_uint32),
                                 P(Stats)]
        L.or_binning.restype = C.c_int
        L.or_seeding.argtypes = [P(FinderConfig), P(GridConfig), P(FilterConfig),
                                 P(Spacepoints), C.c_int, C.c_void_p, C.c_uint32,
                                 P(C.c_uint32), P(Stats)]
        L.or_seeding.restype = C.c_int
        L.or_seeding_ex.argtypes = [P(FinderConfig), P(GridConfig), P(FilterConfig),
                                    P(Spacepoints), C.c_int, P(DoubletFilter), C.c_void_p,
                                    C.c_uint64, P(C.c_uint64), C.c_void_p, C.c_uint64,
                                    P(C.c_uint64), C.c_void_p, C.c_uint32,
                                    P(C.c_uint32), P(Stats)]
        L.or_seeding_ex.restype = C.c_int
        L.or_form_spacepoints.argtypes = [C.c_void_p, C.c_uint32, P(Measurements), C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]
        L.or_form_spacepoints.restype = C.c_uint32
        L.or_mlp_logit.argtypes = [P(DoubletFilter), P(C.c_float)]
        L.or_mlp_logit.restype = C.c_float
        L.or_bf16_round.argtypes = [C.c_float]
        L.or_bf16_round.restype = C.c_float
        L.or_track_params.argtypes = [P(TPConfig), P(Measurements), P(Spacepoints),
                                      C.c_void_p, C.c_uint32, P(C.c_float),
                                      C.c_void_p]
        L.or_track_params.restype = C.c_int
        fa = P(C.c_float)
        L.or_doublet_compatible.argtypes = [C.c_int, fa, fa, P(FinderConfig)]
        L.or_doublet_compatible.restype = C.c_int
        L.or_transform_coordinates.argtypes = [C.c_int, fa, fa, fa]
        L.or_triplet_compatible.argtypes = [fa, fa, fa, P(FinderConfig), C.c_float,
                                            C.c_float, fa, fa]
        L.or_triplet_compatible.restype = C.c_int
        _lib = L
    return _lib


def default_configs():
    """Reference default finder/grid/filter/params configs."""
    L = lib()
    f, g, fl, tp = FinderConfig(), GridConfig(), FilterConfig(), TPConfig()
    L.or_finder_config_default(C.byref(f))
    L.or_grid_config_from_finder(C.byref(g), C.byref(f))
    L.or_filter_config_default(C.byref(fl))
    L.or_tp_config_default(C.byref(tp))
    return f, g, fl, tp


def grid_from_finder(f):
    g = GridConfig()
    lib().or_grid_config_from_finder(C.byref(g), C.byref(f))
    return g


def get_axes(g):
    a = Axes()
    rc = lib().or_get_axes(C.byref(g), C.byref(a))
    if rc:
        raise ValueError(f"get_axes domain error {rc}")
    return a


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def sp_struct(ev):
    """Build an oracle spacepoint view over a dict of numpy columns.
    Keeps references alive on the returned tuple."""
    keep = (_u32(ev["measurement_index_1"]), _u32(ev["measurement_index_2"]),
            _f32(ev["global"]).reshape(-1), _f32(ev["z_variance"]),
            _f32(ev["radius_variance"]))
    s = Spacepoints(keep[0].ctypes.data_as(C.POINTER(C.c_uint32)),
                    keep[1].ctypes.data_as(C.POINTER(C.c_uint32)),
                    keep[2].ctypes.data_as(C.POINTER(C.c_float)),
                    keep[3].ctypes.data_as(C.POINTER(C.c_float)),
                    keep[4].ctypes.data_as(C.POINTER(C.c_float)),
                    len(keep[0]))
    return s, keep


def binning(ev, f=None, g=None, phi_mode=PHI_CR):
    """Returns (bin_offsets[nbins+1], bin_sps[n_valid], axes, stats)."""
    if f is None:
        f, g, _, _ = default_configs()
    a = get_axes(g)
    s, keep = sp_struct(ev)
    nb = a.phi_bins * a.z_bins
    off = np.zeros(nb + 1, np.uint32)
    sps = np.zeros(max(1, s.size), np.uint32)
    nv = C.c_uint32(0)
    st = Stats()
    rc = lib().or_binning(C.byref(f), C.byref(a), C.byref(s), phi_mode,
                          off.ctypes.data_as(C.POINTER(C.c_uint32)),
                          sps.ctypes.data_as(C.POINTER(C.c_uint32)),
                          C.byref(nv), C.byref(st))
    if rc:
        raise RuntimeError(f"or_binning failed {rc}")
    return off, sps[: nv.value].copy(), a, st.as_dict()


def seeding(ev, f=None, g=None, fl=None, phi_mode=PHI_CR):
    """Host seeding.  Returns (seeds structured array, stats dict)."""
    if f is None:
        f, g, fl, _ = default_configs()
    s, keep = sp_struct(ev)
    cap = max(16, 5 * s.size)
    out = np.zeros(cap, SEED_DTYPE)
    n = C.c_uint32(0)
    st = Stats()
    rc = lib().or_seeding(C.byref(f), C.byref(g), C.byref(fl), C.byref(s),
                          phi_mode, out.ctypes.data, cap, C.byref(n), C.byref(st))
    if rc == -1:
        cap = n.value
        out = np.zeros(cap, SEED_DTYPE)
        st = Stats()
        rc = lib().or_seeding(C.byref(f), C.byref(g), C.byref(fl), C.byref(s),
                              phi_mode, out.ctypes.data, cap, C.byref(n),
                              C.byref(st))
    if rc:
        raise RuntimeError(f"or_seeding failed {rc}")
    return out[: n.value].copy(), st.as_dict()


MLP_IN, MLP_H, MAX_BAND_EDGES = 8, 32, 15

DOUBLET_DTYPE = np.dtype([("middle", "<u4"), ("other", "<u4"), ("top", "<u4"),
                          ("feat", "<f4", (MLP_IN,)), ("logit", "<f4")])


class DoubletFilter(C.Structure):
    """or_doublet_filter: the learned doublet filter's network, input
    standardisation, threshold and radial band edges."""
    _fields_ = [("mu", C.c_float * MLP_IN), ("isd", C.c_float * MLP_IN),
                ("w1", C.c_float * (MLP_IN * MLP_H)), ("b1", C.c_float * MLP_H),
                ("w2", C.c_float * (MLP_H * MLP_H)), ("b2", C.c_float * MLP_H),
                ("w3", C.c_float * MLP_H), ("b3", C.c_float),
                ("threshold", C.c_float * 2), ("n_edges", C.c_uint32),
                ("edges", C.c_float * MAX_BAND_EDGES),
                ("prune_bottom", C.c_uint32), ("prune_top", C.c_uint32),
                ("gate_max_tops", C.c_uint32)]


FILTER_KEEP, FILTER_PRUNE_DOUBLETS, FILTER_GATE_MIDDLE = 0, 1, 2


def doublet_filter(model: dict, threshold, prune_bottom=True, prune_top=True, gate_max_tops=0):
    """A DoubletFilter from a model dict with numpy arrays mu, isd, w1 (8x32),
    b1, w2 (32x32), b2, w3 (32), b3 and edges; threshold = (middle-bottom,
    middle-top) logit thresholds (or one for both).  prune_bottom / prune_top:
    False / True (keep / drop doublets below the threshold) or a FILTER_*
    mode (prune_top = FILTER_GATE_MIDDLE gates whole middles)."""
    f = DoubletFilter()
    def put(name, arr):
        arr = np.asarray(arr, np.float32).reshape(-1)
        getattr(f, name)[:] = arr.tolist()
    for k in ("mu", "isd", "w1", "b1", "w2", "b2", "w3"):
        put(k, model[k])
    f.b3 = float(np.float32(model["b3"]))
    th = np.broadcast_to(np.asarray(threshold, np.float32), (2,))
    f.threshold[0] = float(th[0])
    f.threshold[1] = float(th[1])
    edges = np.asarray(model["edges"], np.float32)
    f.n_edges = len(edges)
    f.edges[: len(edges)] = edges.tolist()
    f.prune_bottom = int(prune_bottom)
    f.prune_top = int(prune_top)
    f.gate_max_tops = int(gate_max_tops)
    return f


def bf16_round(x):
    """Round float32 values to bf16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(x, np.float32).view(np.uint32).astype(np.uint64)
    nan = ((u & 0x7f800000) == 0x7f800000) & ((u & 0x007fffff) != 0)
    r = ((u + 0x7fff + ((u >> 16) & 1)) & 0xffff0000)
    r = np.where(nan, (u | 0x00400000) & 0xffff0000, r)
    return r.astype(np.uint32).view(np.float32).reshape(np.shape(x))


TRIPLET_DTYPE = np.dtype([("middle", "<u4"), ("bottom", "<u4"), ("top", "<u4"),
                          ("event", "<u4")])


def seeding_ex(ev, f=None, g=None, fl=None, phi_mode=PHI_CR, filt=None, dump=False,
               triplets=False):
    """Host seeding with the learned doublet filter (filt: DoubletFilter or
    None) and/or dumps of every scored doublet and every triplet of the
    scored middles.  Returns (seeds, stats, doublets or None[, triplets])."""
    if f is None:
        f, g, fl, _ = default_configs()
    s, keep = sp_struct(ev)
    cap = max(16, 5 * s.size)
    dcap = tcap = 0
    for _ in range(3):
        out = np.zeros(cap, SEED_DTYPE)
        drec = np.zeros(max(1, dcap), DOUBLET_DTYPE)
        trec = np.zeros(max(1, tcap), TRIPLET_DTYPE)
        n = C.c_uint32(0)
        nd = C.c_uint64(0)
        nt = C.c_uint64(0)
        st = Stats()
        rc = lib().or_seeding_ex(
            C.byref(f), C.byref(g), C.byref(fl), C.byref(s), phi_mode,
            C.byref(filt) if filt is not None else None,
            drec.ctypes.data if dump else None, dcap, C.byref(nd),
            trec.ctypes.data if triplets else None, tcap, C.byref(nt),
            out.ctypes.data, cap, C.byref(n), C.byref(st))
        if rc not in (0, -1):
            raise RuntimeError(f"or_seeding_ex failed {rc}")
        if rc == 0 and (not dump or nd.value <= dcap) and (not triplets or nt.value <= tcap):
            break
        cap = max(cap, n.value)
        dcap = nd.value
        tcap = nt.value
    res = (out[: n.value].copy(), st.as_dict(), (drec[: nd.value].copy() if dump else None))
    return res + (trec[: nt.value].copy(),) if triplets else res


SURFACE_DTYPE = np.dtype([("type", "<u4"), ("radius", "<f4"), ("rotation", "<f4", (9,)),
                          ("translation", "<f4", (3,))])


def form_spacepoints(surfaces, local_position, surface_link, dimensions=None):
    """Spacepoint formation: returns the spacepoint columns (dict) of the
    2-dimensional measurements, in measurement order."""
    surfaces = np.ascontiguousarray(surfaces, SURFACE_DTYPE)
    lp = np.ascontiguousarray(local_position, np.float32).reshape(-1)
    sl = np.ascontiguousarray(surface_link, np.uint64)
    n = len(sl)
    m = Measurements(lp.ctypes.data_as(C.POINTER(C.c_float)),
                     sl.ctypes.data_as(C.POINTER(C.c_uint64)), n)
    dims = None if dimensions is None else np.ascontiguousarray(dimensions, np.uint8)
    out = {"measurement_index_1": np.zeros(n, np.uint32),
           "measurement_index_2": np.zeros(n, np.uint32),
           "global": np.zeros((n, 3), np.float32),
           "z_variance": np.zeros(n, np.float32),
           "radius_variance": np.zeros(n, np.float32)}
    k = lib().or_form_spacepoints(
        surfaces.ctypes.data if len(surfaces) else None, len(surfaces), C.byref(m),
        dims.ctypes.data if dims is not None else None,
        out["measurement_index_1"].ctypes.data, out["measurement_index_2"].ctypes.data,
        out["global"].ctypes.data, out["z_variance"].ctypes.data,
        out["radius_variance"].ctypes.data)
    return {key: v[:k].copy() for key, v in out.items()}


def track_params(ev, seeds, bfield, tp=None):
    if tp is None:
        _, _, _, tp = default_configs()
    s, keep = sp_struct(ev)
    lp = _f32(ev["local_position"]).reshape(-1)
    sl = np.ascontiguousarray(ev["surface_link"], dtype=np.uint64)
    m = Measurements(lp.ctypes.data_as(C.POINTER(C.c_float)),
                     sl.ctypes.data_as(C.POINTER(C.c_uint64)), len(sl))
    seeds = np.ascontiguousarray(seeds, dtype=SEED_DTYPE)
    out = np.zeros(max(1, len(seeds)), PARAMS_DTYPE)
    b = (C.c_float * 3)(*[float(v) for v in bfield])
    rc = lib().or_track_params(C.byref(tp), C.byref(m), C.byref(s),
                               seeds.ctypes.data, len(seeds), b, out.ctypes.data)
    if rc:
        raise RuntimeError(f"or_track_params failed {rc}")
    return out[: len(seeds)].copy()


# ---------------------------------------------------------------------------
# GBTS seeding (gbts_oracle.c)
# ---------------------------------------------------------------------------
_GBTS_FLOATS_1 = ("tMin_slope", "offset", "tMax_min", "tMax_correction", "tMax_slope", "maxTau")
_GBTS_FLOATS_2 = ("minDeltaRadius", "min_z0", "max_z0", "maxOuterRadius", "tau_roi",
                  "cut_zMinU", "cut_zMaxU", "max_Kappa", "low_Kappa_d0", "high_Kappa_d0",
                  "cut_dphi_max", "cut_dcurv_max", "cut_tau_ratio_max", "min_delta_phi",
                  "dphi_coeff", "min_delta_phi_low_dr", "dphi_coeff_low_dr",
                  "low_dr_threshold", "type1_max_width")
_GBTS_FLOATS_3 = ("sigmaMS", "radLen", "sigma_x", "sigma_y", "weight_x", "weight_y",
                  "maxDChi2_x", "maxDChi2_y", "add_hit", "qual_scale", "inv_max_curvature")
_GBTS_FLOATS_4 = ("dropout_dcurv_m", "force_dropout_max_curv_m", "best_hit_frac",
                  "tight_bid_cot_threshold")
_GBTS_UINTS = ("n_phi_bins", "max_num_neighbours", "minLevel", "max_edges_factor",
               "edge_bidding_rounds", "volume_shift", "volume_bits", "index_shift",
               "index_bits")


class GbtsConfig(C.Structure):
    """or_gbts_config: gbts_seedfinder_config's parameters, flattened."""
    _fields_ = ([(n, C.c_float) for n in _GBTS_FLOATS_1]
                + [("useTauLUT", C.c_int32), ("tau_lut_inv_bin", C.c_float),
                   ("tauLutSize", C.c_uint32)]
                + [(n, C.c_float) for n in _GBTS_FLOATS_2]
                + [("doTauCut", C.c_int32)]
                + [(n, C.c_float) for n in _GBTS_FLOATS_3]
                + [("use_dropout", C.c_int32)]
                + [(n, C.c_float) for n in _GBTS_FLOATS_4]
                + [(n, C.c_uint32) for n in _GBTS_UINTS])


class GbtsTables(C.Structure):
    _fields_ = [("n_layers", C.c_uint32), ("layer_type", C.c_void_p),
                ("eta_bin0", C.c_void_p), ("n_eta", C.c_void_p), ("min_eta", C.c_void_p),
                ("eta_width", C.c_void_p), ("n_pairs", C.c_uint32), ("pairs", C.c_void_p),
                ("n_volumes", C.c_uint32), ("volume_map", C.c_void_p),
                ("n_surfaces", C.c_uint32), ("surface_map", C.c_void_p),
                ("n_tau_lut", C.c_uint32), ("tau_lut", C.c_void_p),
                ("n_eta_bins", C.c_uint32)]


GBTS_COUNTERS = ("nodes", "edges", "connections", "connected_edges", "terminus", "paths",
                 "props", "rejected", "seeds")


def _gbts_lib():
    L = lib()
    if not hasattr(L, "_gbts_ready"):
        P = C.POINTER
        L.or_gbts_config_default.argtypes = [P(GbtsConfig)]
        L.or_gbts_linking.argtypes = [P(GbtsConfig), C.c_float, C.c_void_p, C.c_void_p,
                                      C.c_uint32, C.c_void_p, C.c_uint32, P(C.c_uint32),
                                      C.c_void_p, C.c_uint32, P(C.c_uint32)]
        L.or_gbts_linking.restype = C.c_int
        L.or_gbts_run.argtypes = [P(GbtsConfig), P(GbtsTables), C.c_uint32, C.c_void_p,
                                  C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_uint64, P(C.c_uint64), C.c_void_p]
        L.or_gbts_run.restype = C.c_int
        L._gbts_ready = True
    return L


def gbts_config_default():
    c = GbtsConfig()
    _gbts_lib().or_gbts_config_default(C.byref(c))
    return c


def gbts_linking(cfg, geoid, min_pt=900.0):
    """setLinkingScheme on a copy of `cfg`: (scaled config, volume map,
    surface map [n, 2])."""
    L = _gbts_lib()
    c = GbtsConfig()
    C.memmove(C.byref(c), C.byref(cfg), C.sizeof(GbtsConfig))
    ids = np.ascontiguousarray(geoid["barcode"], np.uint64)
    lay = np.ascontiguousarray(geoid["layer"], np.int16)
    vcap = 2 * (1 << int(cfg.volume_bits)) if cfg.volume_bits <= 15 else 1 << 16
    vmap = np.zeros(vcap, np.int16)
    smap = np.zeros(2 * (len(ids) + 1), np.uint32)
    nv, ns = C.c_uint32(0), C.c_uint32(0)
    rc = L.or_gbts_linking(C.byref(c), min_pt, ids.ctypes.data, lay.ctypes.data, len(ids),
                           vmap.ctypes.data, vcap, C.byref(nv), smap.ctypes.data,
                           len(ids) + 1, C.byref(ns))
    if rc:
        raise RuntimeError("or_gbts_linking rejected the geometry binning")
    return c, vmap[: nv.value].copy(), smap[: 2 * ns.value].reshape(-1, 2).copy()


def gbts(ev, surface_link, diameter, layers, pairs, geoid, cfg=None, min_pt=900.0,
         tau_lut=None):
    """GBTS seeding of one event: (seeds in SEED_DTYPE, counters dict)."""
    L = _gbts_lib()
    if cfg is None:
        cfg = gbts_config_default()
    c, vmap, smap = gbts_linking(cfg, geoid, min_pt)
    ltype = np.ascontiguousarray(layers["type"], np.int8)
    bin0 = np.ascontiguousarray(layers["eta_bin0"], np.uint32)
    neta = np.ascontiguousarray(layers["n_eta_bins"], np.uint32)
    meta = np.ascontiguousarray(layers["min_eta"], np.float32)
    weta = np.ascontiguousarray(layers["eta_bin_width"], np.float32)
    prs = np.ascontiguousarray(pairs, np.uint32).reshape(-1)
    lut = np.ascontiguousarray(tau_lut if tau_lut is not None else np.zeros(1), np.float32)
    smap_flat = np.ascontiguousarray(smap.reshape(-1), np.uint32)
    t = GbtsTables(len(ltype), ltype.ctypes.data, bin0.ctypes.data, neta.ctypes.data,
                   meta.ctypes.data, weta.ctypes.data, len(prs) // 2, prs.ctypes.data,
                   len(vmap), vmap.ctypes.data, len(smap), smap_flat.ctypes.data,
                   0 if tau_lut is None else len(lut), lut.ctypes.data,
                   int((bin0 + neta).max()) if len(bin0) else 0)
    g = np.ascontiguousarray(ev["global"], np.float32)
    mi = np.ascontiguousarray(ev["measurement_index_1"], np.uint32)
    link = np.ascontiguousarray(surface_link, np.uint64)
    dia = np.ascontiguousarray(diameter, np.float32)
    cap = max(64, 3 * len(g))
    out = np.zeros(cap, SEED_DTYPE)
    n = C.c_uint64(0)
    ctr = np.zeros(len(GBTS_COUNTERS), np.uint64)
    rc = L.or_gbts_run(C.byref(c), C.byref(t), len(g), g.ctypes.data, mi.ctypes.data,
                       len(link), link.ctypes.data, dia.ctypes.data, out.ctypes.data, cap,
                       C.byref(n), ctr.ctypes.data)
    if rc == 1:
        raise RuntimeError("or_gbts_run: seed capacity exceeded")
    if rc not in (0, 2):
        raise RuntimeError(f"or_gbts_run failed {rc}")
    return out[: n.value].copy(), dict(zip(GBTS_COUNTERS, (int(v) for v in ctr)))
