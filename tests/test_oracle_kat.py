"""The oracle against the known answers in the reference's own tests.

* tests/cpu/test_seeding.cpp:35-181 -- two 5-spacepoint muon events; with the
  tests' config tweaks (deltaRMax = 100 mm and maxPtScattering = 0.5 GeV set
  after the grid config was copied) each gives exactly one seed and one set of
  track parameters.
* tests/cpu/test_track_params_estimation.cpp:34-144 -- three spacepoints on a
  helix (p = sqrt(2) GeV, B = 2 T, charge -1 / +1) give |p - sqrt(2)| < 2e-4
  and the right q/p sign.  The points are regenerated here from the helix
  equation (detray's helix class is not available).
* tests/cpu/test_axis.cpp:26-161 -- regular and circular axis bin / range /
  zone / remap known answers (binned neighbourhoods).
* core/include/traccc/seeding/detail/seeding_config.hpp:120-138 -- derived
  seed-finder constants for the default config.
* tests/cpu/test_spacepoint_formation.cpp:21-89 -- a telescope of nine planes
  at x = 20 ... 180 mm (normals along x, local axes along global y and z): the
  measurement (7, 2) on the first plane forms the spacepoint (20, 7, 2), the
  measurement (10, 15) on the last plane (180, 10, 15).  detray's telescope
  builder is not available; its plane placement is written here as a rotation
  and a translation of the library's surface table.
"""
import ctypes as C
import math

import numpy as np
import pytest

import oracle as O

INVALID = 0xFFFFFFFF


def _event(points):
    n = len(points)
    return {"measurement_index_1": np.arange(n, dtype=np.uint32),
            "measurement_index_2": np.full(n, INVALID, np.uint32),
            "global": np.asarray(points, np.float32),
            "z_variance": np.zeros(n, np.float32),
            "radius_variance": np.zeros(n, np.float32),
            "local_position": np.zeros((n, 2), np.float32),
            "surface_link": np.zeros(n, np.uint64)}


def _case_configs():
    f, g, fl, tp = O.default_configs()
    # tests/cpu/test_seeding.cpp:43-44: tweak the finder after the grid copy
    f.deltaRMax = 100.0
    f.maxPtScattering = 0.5
    return f, g, fl, tp


CASE1 = [(36.6706, 10.6472, 104.131), (94.2191, 29.6699, 113.628),
         (149.805, 47.9518, 122.979), (218.514, 70.3049, 134.029),
         (275.359, 88.668, 143.378)]
CASE2 = [(36.301, 13.1197, 106.83), (93.9366, 33.7101, 120.978),
         (149.192, 52.0562, 134.678), (218.398, 73.1025, 151.979),
         (275.322, 89.0663, 166.229)]


@pytest.mark.parametrize("points", [CASE1, CASE2], ids=["case1", "case2"])
@pytest.mark.parametrize("phi_mode", [O.PHI_LIBM, O.PHI_CR])
def test_seeding_cases_give_one_seed(points, phi_mode):
    f, g, fl, tp = _case_configs()
    ev = _event(points)
    seeds, st = O.seeding(ev, f, g, fl, phi_mode=phi_mode)
    assert len(seeds) == 1
    b = (0.0, 0.0, 2.0 * 0.000299792458)
    params = O.track_params(ev, seeds, b, tp)
    assert len(params) == 1
    # only the three spacepoints with r < 200 mm are binned (is_valid_sp)
    assert st["n_valid"] == 3
    assert (seeds["bottom"][0], seeds["middle"][0], seeds["top"][0]) == (0, 1, 2)


def _helix_points(q, s_values):
    """Positions at path lengths s on the helix from the origin with
    direction (1, 0, 1)/sqrt(2), |p| = sqrt(2) GeV, in B = (0, 0, 2 T):
    dt/ds = (q/p) t x B, so the transverse direction turns at
    dphi/ds = -(q/p) Bz."""
    bz = 2.0 * 0.000299792458
    qop = q / math.sqrt(2.0)
    st = ct = 1.0 / math.sqrt(2.0)
    w = -qop * bz
    pts = []
    for s in s_values:
        phi = w * s
        pts.append((st / w * math.sin(phi), -st / w * (math.cos(phi) - 1.0), ct * s))
    return pts


@pytest.mark.parametrize("q", [-1.0, 1.0], ids=["negative", "positive"])
def test_track_params_on_helix(q):
    f, g, fl, tp = O.default_configs()
    ev = _event(_helix_points(q, [50.0, 100.0, 150.0]))
    seeds = np.zeros(1, O.SEED_DTYPE)
    seeds[0] = (0, 1, 2, 0.0)
    p = O.track_params(ev, seeds, (0.0, 0.0, 2.0 * 0.000299792458), tp)
    qop = float(p["params"][0][4])
    assert abs(abs(q / qop) - math.sqrt(2.0)) < 2e-4
    assert (qop < 0) == (q < 0)
    # covariance diagonal as in track_params_estimation.cpp:64-86
    cov = p["cov"][0].reshape(6, 6)
    assert np.count_nonzero(cov - np.diag(np.diag(cov))) == 0
    assert cov[0, 0] == np.float32(1.0) and cov[1, 1] == np.float32(1.0)


def _u2(a, b):
    return (C.c_uint32 * 2)(a, b)


def _zone(fn, n, mn, mx, v, nh):
    out = (C.c_uint32 * 128)()
    k = fn(n, mn, mx, v, _u2(*nh), out, 128)
    return [out[i] for i in range(k)]


def _range(fn, n, mn, mx, v, nh):
    out = (C.c_uint32 * 2)()
    fn(n, mn, mx, v, _u2(*nh), out)
    return [out[0], out[1]]


def test_regular_axis_known_answers():
    L = O.lib()
    n, mn, mx = 10, -3.0, 7.0
    assert L.or_regular_bin(n, mn, mx, -4.0) == 0
    assert L.or_regular_bin(n, mn, mx, 2.5) == 5
    assert L.or_regular_bin(n, mn, mx, 8.0) == 9
    rr = lambda v, nh: _range(L.or_regular_range, n, mn, mx, v, nh)
    assert rr(2.5, (0, 0)) == [5, 5]
    assert rr(2.5, (1, 1)) == [4, 6]
    assert rr(2.5, (0, 1)) == [5, 6]
    assert rr(1.5, (4, 4)) == [0, 8]
    assert rr(5.5, (5, 5)) == [3, 9]
    rz = lambda v, nh: _zone(L.or_regular_zone, n, mn, mx, v, nh)
    assert rz(2.5, (0, 0)) == [5]
    assert rz(2.5, (0, 1)) == [5, 6]
    assert rz(2.5, (1, 1)) == [4, 5, 6]
    assert rz(1.5, (4, 4)) == list(range(9))


def test_circular_axis_known_answers():
    L = O.lib()
    pi = float(np.float32(math.pi))
    eps = float(np.float32(10.0) * np.finfo(np.float32).eps)
    half = float(np.float32(pi) / np.float32(72.0))
    mn = float(np.float32(-pi) + np.float32(half))
    mx = float(np.float32(pi) - np.float32(half))
    n = 36
    pe = float(np.float32(pi) + np.float32(eps))
    pm = float(np.float32(pi) - np.float32(eps))
    assert L.or_circular_bin(n, mn, mx, pm) == 0
    assert L.or_circular_bin(n, mn, mx, pe) == 0
    assert L.or_circular_bin(n, mn, mx, 0.0) == 18
    rm = lambda b, s: L.or_circular_remap(n, b, s)
    assert (rm(4, -1), rm(4, 1), rm(0, -1), rm(0, -2), rm(1, -1), rm(35, 1)) == \
        (3, 5, 35, 34, 0, 0)
    rr = lambda nh: _range(L.or_circular_range, n, mn, mx, pe, nh)
    assert rr((0, 0)) == [0, 0]
    assert rr((0, 1)) == [0, 1]
    assert rr((1, 1)) == [35, 1]
    assert rr((2, 2)) == [34, 2]
    assert _zone(L.or_circular_zone, n, mn, mx, pe, (2, 2)) == [34, 35, 0, 1, 2]


def test_default_config_derived_constants():
    f, g, fl, tp = O.default_configs()
    assert abs(f.highland - 2.694866e-3) < 1e-9
    assert abs(f.maxScatteringAngle2 - 2.904921e-5) < 1e-11
    assert abs(f.minHelixDiameter2 - 2.789318e6) < 1.0
    assert abs(f.pT2perRadius - 20.25688) < 1e-4
    a = O.get_axes(g)
    assert (a.phi_bins, a.z_bins) == (78, 1)


def test_bad_grid_config_is_rejected():
    f, g, fl, tp = O.default_configs()
    g.minPt = 0.01  # minHelixRadius < rMax / 2: std::domain_error in get_axes
    with pytest.raises(ValueError):
        O.get_axes(g)


def test_spacepoint_formation_on_a_telescope():
    planes = np.zeros(9, O.SURFACE_DTYPE)
    for k, x in enumerate((20., 40., 60., 80., 100., 120., 140., 160., 180.)):
        planes[k]["type"] = 0  # plane: local (u, v) -> global R (u, v, 0) + t
        # local u -> global y, local v -> global z, local normal -> global x
        planes[k]["rotation"] = np.array([[0, 0, 1], [1, 0, 0], [0, 1, 0]],
                                         np.float32).reshape(-1)
        planes[k]["translation"] = (x, 0., 0.)
    sp = O.form_spacepoints(planes, np.array([[7., 2.], [10., 15.]], np.float32),
                            np.array([0, 8], np.uint64), np.array([2, 2], np.uint8))
    assert len(sp["global"]) == 2
    assert np.array_equal(sp["global"], np.array([[20., 7., 2.], [180., 10., 15.]], np.float32))
    assert np.array_equal(sp["measurement_index_1"], np.array([0, 1], np.uint32))
