"""The C ABI without a GPU: the library loads, exports every function
include/seedgb.h declares, derives the reference's configs bit for bit like
the oracle, and reports errors as status codes (no exceptions, no crashes)."""
import ctypes as C
import os
import re

import numpy as np

import oracle as O
from traccc_gb300 import seeding

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "seedgb.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*[A-Za-z_][\w\s\*]*?\b(seedgb_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_function():
    names = declared_functions()
    assert len(names) >= 20
    lib = C.CDLL(seeding.library_path())
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def _fields(s):
    out = {}
    for name, _ in s._fields_:
        v = getattr(s, name)
        out[name] = list(v) if hasattr(v, "__len__") else v
    return out


def _bits(d):
    return {k: (np.asarray(v, np.float32).view(np.uint32).tolist()
                if isinstance(v, (float, list)) else v) for k, v in d.items()}


def test_configs_match_the_oracle_bit_for_bit():
    f, g, fl, tp = seeding.default_configs()
    of, og, ofl, otp = O.default_configs()
    for ours, theirs in ((f, of), (g, og), (fl, ofl), (tp, otp)):
        a, b = _fields(ours), _fields(theirs)
        assert a.keys() == b.keys()
        assert _bits(a) == _bits(b)


def test_axes_match_the_oracle():
    f, g, _, _ = seeding.default_configs()
    a = seeding.get_axes(g)
    b = O.get_axes(O.default_configs()[1])
    assert (a.phi_bins, a.z_bins, a.phi_min, a.phi_max, a.z_min, a.z_max) == \
        (b.phi_bins, b.z_bins, b.phi_min, b.phi_max, b.z_min, b.z_max)
    # a modified config follows setup() identically
    f.minPt = 0.9
    f.setup()
    of = O.default_configs()[0]
    of.minPt = 0.9
    O.lib().or_finder_config_setup(C.byref(of))
    assert _bits(_fields(f)) == _bits(_fields(of))


def test_bad_config_is_a_status_not_an_exception():
    f, g, fl, _ = seeding.default_configs()
    g.minPt = 0.01
    a = seeding.GridAxes()
    assert seeding.lib().seedgb_get_axes(C.byref(g), C.byref(a)) == seeding.BAD_CONFIG


def test_status_strings():
    L = seeding.lib()
    for s in range(9):
        assert L.seedgb_status_string(s)
    assert L.seedgb_status_string(99) == b"unknown status"
    assert L.seedgb_abi_version() == 1


def test_invalid_arguments_are_rejected_before_device_work():
    L = seeding.lib()
    assert L.seedgb_seeding_run(None, None, None, None) == seeding.INVALID_ARGUMENT
    assert L.seedgb_seeding_destroy(None) == seeding.INVALID_ARGUMENT
    f, g, _, _ = seeding.default_configs()
    v = seeding._SpacepointView(0, 0, 1, 0, 0, seeding.NOALLOC_MAX_SPACEPOINTS + 1)
    st = L.seedgb_spacepoint_binning_noalloc(C.byref(f), C.byref(g), C.byref(v),
                                             C.c_void_p(1), C.c_void_p(1), None)
    assert st == seeding.SIZE_LIMIT


def test_noalloc_refuses_a_grid_too_narrow_for_the_finder_before_device_work():
    """The allocation-free binning checks on the host that the grid's
    circular phi axis can place every phi the finder accepts; a grid range of
    [-0.5, 0.5] against the finder's [-pi, pi] is refused (no launch, so no
    GPU is needed), a wrapping [-2, 2] grid passes the check (and then fails
    only for want of a device here)."""
    L = seeding.lib()
    f, g, _, _ = seeding.default_configs()
    v = seeding._SpacepointView(0, 0, 1, 0, 0, 10)
    g.phiMin, g.phiMax = -0.5, 0.5
    st = L.seedgb_spacepoint_binning_noalloc(C.byref(f), C.byref(g), C.byref(v),
                                             C.c_void_p(1), C.c_void_p(1), None)
    assert st == seeding.BAD_CONFIG
    g.phiMin, g.phiMax = -2.0, 2.0
    st = L.seedgb_spacepoint_binning_noalloc(C.byref(f), C.byref(g), C.byref(v),
                                             C.c_void_p(1), C.c_void_p(1), None)
    assert st != seeding.BAD_CONFIG


def test_ckf_record_layout():
    """The CKF hand-off record: parameter vector (24 B), 64-bit barcode at
    offset 24, 6 x 6 covariance at offset 32, 176 bytes, as declared in
    seedgb.h (and the converter refuses null or misaligned buffers without
    touching a device)."""
    dt = seeding.CKF_PARAMS_DTYPE
    assert dt.itemsize == 176
    assert dt.fields["barcode"][1] == 24 and dt.fields["covariance"][1] == 32
    L = seeding.lib()
    assert L.seedgb_params_to_ckf(None, None, 0, None, None) == seeding.INVALID_ARGUMENT
    b = seeding._ParamsBuffer(16, 4, 16)
    assert L.seedgb_params_to_ckf(C.byref(b), C.c_void_p(24), 4, None, None) == \
        seeding.INVALID_ARGUMENT


def test_batched_formation_arguments_are_checked_before_device_work():
    """seedgb_formation_run_batch refuses, before touching a device, a batch
    above 65535 events and an output whose capacity is below its event's
    measurement count (a handle without surfaces needs no device)."""
    L = seeding.lib()
    assert L.seedgb_formation_run_batch(None, None, None, None, 1, None) == \
        seeding.INVALID_ARGUMENT
    assert L.seedgb_formation_destroy(None) == seeding.INVALID_ARGUMENT
    bad = C.c_void_p()
    assert L.seedgb_formation_create(None, 3, C.byref(bad)) == seeding.INVALID_ARGUMENT
    h = C.c_void_p()
    assert L.seedgb_formation_create(None, 0, C.byref(h)) == seeding.OK
    m = seeding._MeasurementView(16, 16, 10)
    small = seeding._SpacepointBuffer(16, 16, 16, 16, 16, 9, 16)
    assert L.seedgb_formation_run_batch(h, C.byref(m), None, C.byref(small), 1, None) == \
        seeding.INVALID_ARGUMENT
    n = 65536
    ms = (seeding._MeasurementView * n)()
    outs = (seeding._SpacepointBuffer * n)()
    assert L.seedgb_formation_run_batch(h, ms, None, outs, n, None) == seeding.SIZE_LIMIT
    L.seedgb_formation_destroy(h)
