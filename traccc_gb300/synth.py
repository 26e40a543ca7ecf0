"""Seeded synthetic helix events (the stand-in for the reference's data files).

The generator itself is C (``csrc/synth_events.c``); this module wraps it and
names the benchmark workloads:

* ``trk100``: 100 tracks, pT U(1, 10) GeV, 5 % noise           (~1k spacepoints)
* ``trk1000``: 1000 tracks, pT log-U(0.5, 20) GeV, 10 % noise   (~11k)
* ``pileup9k``: 9000 tracks, pT exp(mean 0.6 GeV) >= 0.1 GeV, 12 % noise (~100k)
* ``uneven64``: batch events as pileup9k with U(500, 12000) tracks per event

All share the detector (10 barrel layers, |z| <= 1000 mm), a 2 T field along
z, |eta| < 1.5, z0 ~ N(0, 50 mm), d0 ~ N(0, 0.02 mm), smearing 15 um (r*phi)
and 50 um (z).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _build


class SynthConfig(C.Structure):
    _fields_ = [("n_tracks", C.c_uint32), ("pt_dist", C.c_int32),
                ("pt_a", C.c_double), ("pt_b", C.c_double),
                ("eta_max", C.c_double), ("noise_frac", C.c_double),
                ("z0_sigma", C.c_double), ("d0_sigma", C.c_double),
                ("smear_rphi", C.c_double), ("smear_z", C.c_double),
                ("bz_tesla", C.c_double), ("seed", C.c_uint64)]


class SynthOutput(C.Structure):
    _fields_ = [("glob", C.c_void_p), ("measurement_index_1", C.c_void_p),
                ("measurement_index_2", C.c_void_p), ("z_variance", C.c_void_p),
                ("radius_variance", C.c_void_p), ("layer", C.c_void_p),
                ("particle", C.c_void_p), ("local_position", C.c_void_p),
                ("surface_link", C.c_void_p), ("capacity", C.c_uint32)]


# layer radii (mm) of the synthetic barrel, as generated by synth_events.c;
# measurement surface_link = layer index + 1
LAYER_RADII = (32.0, 72.0, 116.0, 172.0, 260.0, 360.0, 500.0, 600.0, 700.0, 820.0)

WORKLOADS = {
    "trk100": dict(n_tracks=100, pt_dist=0, pt_a=1.0, pt_b=10.0, noise_frac=0.05),
    "trk1000": dict(n_tracks=1000, pt_dist=1, pt_a=0.5, pt_b=20.0, noise_frac=0.10),
    "pileup9k": dict(n_tracks=9000, pt_dist=2, pt_a=0.6, pt_b=0.1, noise_frac=0.12),
}

_lib = None


def _load():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.synth_library())
        _lib.synth_event.argtypes = [C.POINTER(SynthConfig), C.POINTER(SynthOutput)]
        _lib.synth_event.restype = C.c_uint32
    return _lib


def make_event(n_tracks, pt_dist, pt_a, pt_b, noise_frac, seed, eta_max=1.5,
               z0_sigma=50.0, d0_sigma=0.02, smear_rphi=0.015, smear_z=0.05,
               bz_tesla=2.0):
    """One event as a dict of numpy columns in the reference's SoA layout:
    measurement_index_1/2 (u32), global (n,3 f32), z_variance, radius_variance
    (f32); plus layer (u32), particle (i32), and the measurement columns
    local_position (n,2 f32) and surface_link (u64)."""
    cfg = SynthConfig(n_tracks, pt_dist, pt_a, pt_b, eta_max, noise_frac,
                      z0_sigma, d0_sigma, smear_rphi, smear_z, bz_tesla, seed)
    cap = int(n_tracks * 10 * (1.0 + noise_frac)) + 64
    while True:
        ev = {
            "global": np.zeros((cap, 3), np.float32),
            "measurement_index_1": np.zeros(cap, np.uint32),
            "measurement_index_2": np.zeros(cap, np.uint32),
            "z_variance": np.zeros(cap, np.float32),
            "radius_variance": np.zeros(cap, np.float32),
            "layer": np.zeros(cap, np.uint32),
            "particle": np.zeros(cap, np.int32),
            "local_position": np.zeros((cap, 2), np.float32),
            "surface_link": np.zeros(cap, np.uint64),
        }
        out = SynthOutput(*(ev[k].ctypes.data for k in (
            "global", "measurement_index_1", "measurement_index_2", "z_variance",
            "radius_variance", "layer", "particle", "local_position",
            "surface_link")), cap)
        n = _load().synth_event(C.byref(cfg), C.byref(out))
        if n <= cap:
            return {k: v[:n].copy() for k, v in ev.items()}
        cap = n + 64


def workload_event(name: str, seed: int, n_tracks: int | None = None):
    """An event of a named workload (trk100, trk1000, pileup9k) with the given seed."""
    kw = dict(WORKLOADS[name])
    if n_tracks is not None:
        kw["n_tracks"] = n_tracks
    return make_event(seed=seed, **kw)


def batch_events(n_events: int, seed: int, lo: int = 500, hi: int = 12000):
    """The uneven batch: pileup9k statistics with U(lo, hi) tracks per event."""
    rng = np.random.default_rng(seed)
    counts = rng.integers(lo, hi + 1, size=n_events)
    return [workload_event("pileup9k", seed * 100003 + i, int(c))
            for i, c in enumerate(counts)]


# --------------------------------------------------------------------------
# GBTS inputs for the synthetic barrel: the layer table, the linked eta bins,
# the geometry-id binning and per-measurement surface barcodes and cluster
# diameters.  Barcodes use the detray layout the GBTS library decodes by
# default: volume in bits 52-63, surface index in bits 27-47.
# --------------------------------------------------------------------------
GBTS_SECTORS = 16


def gbts_volume(layer):
    """Volume of a barrel layer: layers 0 and 1 share volume 1 (a volume split
    over two layers, resolved through the surface map), layer L >= 2 is
    volume L."""
    layer = np.asarray(layer)
    return np.where(layer <= 1, 1, layer).astype(np.uint64)


def gbts_barcode(layer, sector):
    layer = np.asarray(layer, np.uint64)
    index = layer * np.uint64(GBTS_SECTORS) + np.asarray(sector, np.uint64)
    return (gbts_volume(layer) << np.uint64(52)) | (index << np.uint64(27))


def gbts_geometry(eta_bin_width=0.2, z0_max=160.0, eta_max=1.5, z_max=1000.0, skip=2):
    """(layers, bin_pairs, geoid_binning) of the synthetic barrel.

    layers: structured array (type, eta_bin0, n_eta_bins, min_eta, eta_bin_width),
    all type 0 (barrel), eta bins of `eta_bin_width` covering the hits of
    |eta| < eta_max tracks from |z0| < z0_max.  bin_pairs: (bin on layer L1,
    bin on layer L2) for L2 = L1 + 1 ... L1 + skip whose z ranges overlap for
    straight lines from |z0| <= z0_max (10 % slack for the helix).
    geoid_binning: (barcode, layer) of every surface (GBTS_SECTORS phi sectors
    per layer)."""
    radii = LAYER_RADII
    n_layers = len(radii)
    layers = np.zeros(n_layers, [("type", np.int32), ("eta_bin0", np.uint32),
                                 ("n_eta_bins", np.uint32), ("min_eta", np.float32),
                                 ("eta_bin_width", np.float32)])
    bin0 = 0
    for L, r in enumerate(radii):
        zl = min(z_max, z0_max + 1.15 * r * np.sinh(eta_max))
        lim = np.arcsinh(zl / r)
        n = int(np.ceil(2 * lim / eta_bin_width))
        layers[L] = (0, bin0, n, np.float32(-n * eta_bin_width / 2), np.float32(eta_bin_width))
        bin0 += n
    pairs = []
    for L1 in range(n_layers):
        r1 = radii[L1]
        for L2 in range(L1 + 1, min(n_layers, L1 + 1 + skip)):
            r2 = radii[L2]
            k = r2 / r1
            for b1 in range(int(layers[L1]["n_eta_bins"])):
                a = float(layers[L1]["min_eta"]) + b1 * eta_bin_width
                z1lo, z1hi = r1 * np.sinh(a), r1 * np.sinh(a + eta_bin_width)
                z2lo = z1lo * k - z0_max * (k - 1)
                z2hi = z1hi * k + z0_max * (k - 1)
                z2lo -= 0.1 * abs(z2lo)
                z2hi += 0.1 * abs(z2hi)
                e2lo, e2hi = np.arcsinh(z2lo / r2), np.arcsinh(z2hi / r2)
                for b2 in range(int(layers[L2]["n_eta_bins"])):
                    c = float(layers[L2]["min_eta"]) + b2 * eta_bin_width
                    if c + eta_bin_width >= e2lo and c <= e2hi:
                        pairs.append((int(layers[L1]["eta_bin0"]) + b1,
                                      int(layers[L2]["eta_bin0"]) + b2))
    lay = np.repeat(np.arange(n_layers), GBTS_SECTORS)
    sec = np.tile(np.arange(GBTS_SECTORS), n_layers)
    geoid = np.zeros(len(lay), [("barcode", np.uint64), ("layer", np.int16)])
    geoid["barcode"] = gbts_barcode(lay, sec)
    geoid["layer"] = lay
    return layers, np.asarray(pairs, np.uint32).reshape(-1, 2), geoid


def gbts_measurements(ev, seed=0):
    """(surface_link, diameter) per measurement of a synthetic event for GBTS:
    the barcode of the hit's layer and phi sector, and a cluster diameter
    consistent with the particle's |cot(theta)| (w = 0.2 + max(0, |tau| / 7 -
    0.003), inside the default tau window of the barrel) or, for noise hits,
    uniform in [0.2, 0.55]."""
    g = np.asarray(ev["global"], np.float64)
    layer = np.asarray(ev["layer"], np.int64)
    part = np.asarray(ev["particle"], np.int64)
    phi = np.arctan2(g[:, 1], g[:, 0])
    sector = np.floor((phi + np.pi) / (2 * np.pi) * GBTS_SECTORS).astype(np.int64) % GBTS_SECTORS
    link = gbts_barcode(layer, sector)
    r = np.hypot(g[:, 0], g[:, 1])
    z = g[:, 2]
    rng = np.random.default_rng(seed)
    diam = rng.uniform(0.2, 0.55, len(r))
    real = part >= 0
    if real.any():
        p = part[real]
        n = np.bincount(p).astype(np.float64)
        sr = np.bincount(p, r[real])
        sz = np.bincount(p, z[real])
        srr = np.bincount(p, r[real] * r[real])
        srz = np.bincount(p, r[real] * z[real])
        den = n * srr - sr * sr
        tau = np.where(den > 0, (n * srz - sr * sz) / np.where(den > 0, den, 1.0), 0.0)
        diam[real] = 0.2 + np.maximum(0.0, np.abs(tau[p]) / 7.0 - 0.003)
    m = np.asarray(ev["measurement_index_1"], np.int64)
    n_meas = int(m.max()) + 1 if len(m) else 0
    out_link = np.zeros(n_meas, np.uint64)
    out_diam = np.zeros(n_meas, np.float32)
    out_link[m] = link
    out_diam[m] = diam.astype(np.float32)
    return out_link, out_diam
