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
