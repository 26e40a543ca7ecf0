"""CSV input and spacepoint formation on the CPU.

* The library's CSV readers (traccc's hit / measurement / measurement-hit-id
  files, columns by name) give back exactly the columns written, map hits to
  measurements like io/src/csv/read_spacepoints.cpp (first map row per hit,
  unmapped hits invalid), decode local_key like make_measurement_edm.cpp, and
  reject malformed files with a status.
* The oracle's spacepoint formation on the synthetic barrel (cylinder
  surfaces) reproduces the events' global positions, keeps measurement order
  and skips non-pixel measurements and unknown surfaces.
"""
import os

import numpy as np
import pytest

import oracle as O
from traccc_gb300 import seeding, synth

RADII = synth.LAYER_RADII


def barrel_surfaces():
    s = np.zeros(len(RADII) + 1, O.SURFACE_DTYPE)
    for layer, r in enumerate(RADII):
        s[layer + 1]["type"] = 1
        s[layer + 1]["radius"] = r
        s[layer + 1]["rotation"] = np.eye(3, dtype=np.float32).reshape(-1)
    return s


def write_csv(path, header, rows):
    with open(path, "w") as f:
        f.write(",".join(header) + "\n")
        for r in rows:
            f.write(",".join(r) + "\n")


def test_csv_spacepoints_round_trip(tmp_path):
    ev = synth.workload_event("trk100", 3)
    g = np.asarray(ev["global"], np.float32)
    n = len(g)
    hits = tmp_path / "event000000000-hits.csv"
    cols = ["particle_id", "geometry_id", "tx", "ty", "tz", "tt", "tpx", "tpy", "tpz", "te",
            "deltapx", "deltapy", "deltapz", "deltae", "index"]
    write_csv(hits, cols, [[str(7), str(100 + i % 5)] + [repr(float(v)) for v in g[i]] +
                           ["0"] * 9 + [str(i)] for i in range(n)])
    # every hit but the last two has a measurement; hit 3 is listed twice
    mh = tmp_path / "event000000000-measurement-simhit-map.csv"
    rows = [[str(n - 1 - i), str(i)] for i in range(n - 2)] + [["999", "3"]]
    write_csv(mh, ["measurement_id", "hit_id"], rows)
    sp = seeding.read_spacepoints_csv(hits, mh)
    assert np.array_equal(sp["global"].view(np.uint32), g.view(np.uint32))
    want = np.array([n - 1 - i for i in range(n - 2)] + [0xFFFFFFFF, 0xFFFFFFFF], np.uint32)
    assert np.array_equal(sp["measurement_index_1"], want)
    assert np.all(sp["measurement_index_2"] == 0xFFFFFFFF)
    assert not sp["z_variance"].any() and not sp["radius_variance"].any()
    # without a map every spacepoint is unmatched
    sp2 = seeding.read_spacepoints_csv(hits)
    assert np.all(sp2["measurement_index_1"] == 0xFFFFFFFF)
    # the oracle seeds the read spacepoints like the generated ones
    s1, _ = O.seeding(ev)
    ev2 = dict(ev, **{k: sp[k] for k in ("global", "z_variance", "radius_variance")})
    s2, _ = O.seeding(ev2)
    assert np.array_equal(s1, s2)


def test_csv_measurements(tmp_path):
    meas = tmp_path / "event000000000-measurements.csv"
    cols = ["measurement_id", "geometry_id", "local_key", "local0", "local1", "phi", "theta",
            "time", "var_local0", "var_local1", "var_phi", "var_theta", "var_time"]
    write_csv(meas, cols, [
        ["0", "1152921779484753920", "6", "1.5", "-2.25", "0", "0", "0", "1", "1", "0", "0", "0"],
        ["1", "1152921779484753921", "2", "3.5", "7.0", "0", "0", "0", "1", "1", "0", "0", "0"],
        ["2", "1152921779484753922", "4", "3.5", "-1e-3", "0", "0", "0", "1", "1", "0", "0", "0"]])
    m = seeding.read_measurements_csv(meas)
    assert list(m["dimensions"]) == [2, 1, 1]
    assert m["local_position"].tolist() == [[1.5, -2.25], [3.5, 0.0], [0.0, np.float32(-1e-3)]]
    assert m["surface_link"].tolist() == [1152921779484753920, 1152921779484753921,
                                          1152921779484753922]


def test_csv_errors(tmp_path):
    bad = tmp_path / "hits.csv"
    write_csv(bad, ["tx", "ty"], [["1", "2"]])
    with pytest.raises(seeding.SeedingError) as e:
        seeding.read_spacepoints_csv(bad)
    assert e.value.status == seeding.INVALID_ARGUMENT
    bad2 = tmp_path / "hits2.csv"
    write_csv(bad2, ["tx", "ty", "tz"], [["1", "2", "x"]])
    with pytest.raises(seeding.SeedingError):
        seeding.read_spacepoints_csv(bad2)
    with pytest.raises(seeding.SeedingError):
        seeding.read_spacepoints_csv(tmp_path / "missing.csv")


def test_oracle_formation_on_the_barrel():
    ev = synth.workload_event("trk1000", 2)
    sp = O.form_spacepoints(barrel_surfaces(), ev["local_position"], ev["surface_link"])
    assert len(sp["global"]) == len(ev["global"])
    assert np.array_equal(sp["measurement_index_1"], np.arange(len(ev["global"]), dtype=np.uint32))
    assert np.all(sp["measurement_index_2"] == 0xFFFFFFFF)
    assert np.abs(sp["global"] - ev["global"]).max() < 1e-3
    # strips and unknown surfaces form no spacepoint; order is kept
    dims = np.full(len(ev["global"]), 2, np.uint8)
    dims[::7] = 1
    link = np.asarray(ev["surface_link"], np.uint64).copy()
    link[5::11] = 99
    sp2 = O.form_spacepoints(barrel_surfaces(), ev["local_position"], link, dims)
    keep = np.nonzero((dims == 2) & (link < 11))[0]
    assert np.array_equal(sp2["measurement_index_1"], keep.astype(np.uint32))
    assert np.array_equal(sp2["global"], sp["global"][keep])


MOCK = "/root/reference/tests/io/mock_data"


@pytest.mark.skipif(not os.path.isdir(MOCK), reason="the reference's test data is not here")
def test_csv_readers_on_the_reference_mock_event():
    """The reference's own CSV test event (tests/io/mock_data, used by
    tests/io/test_event_data.cpp:66-140: three particles, one hit and one
    measurement each).  The hits become three spacepoints with the files'
    positions (decimal -> float, correctly rounded) and measurement indices
    0, 1, 2 through the measurement-hit-id map, as
    io/src/csv/read_spacepoints.cpp:39-77 builds them.  The three
    measurements keep their geometry id; their local_key column holds the raw
    byte 0x06 (the reference's uint8_t field, read as one character), so loc0
    and loc1 are both active (io/src/csv/make_measurement_edm.cpp:36-52) and
    the local positions are the files' local0 / local1."""
    sp = seeding.read_spacepoints_csv(os.path.join(MOCK, "event000000000-hits.csv"),
                                      os.path.join(MOCK, "event000000000-measurement-simhit-map.csv"))
    want = np.array([[39.2037048, 0.352969825, -1502.5],
                     [31.5048428, 5.16000509, -1502.5],
                     [90.4015808, 0.7420941, -1502.5]], np.float32)
    assert np.array_equal(sp["global"], want)
    assert sp["measurement_index_1"].tolist() == [0, 1, 2]
    assert np.all(sp["measurement_index_2"] == 0xFFFFFFFF)
    assert not sp["z_variance"].any() and not sp["radius_variance"].any()
    m = seeding.read_measurements_csv(os.path.join(MOCK, "event000000000-measurements.csv"))
    assert m["surface_link"].tolist() == [1224979236083738112] * 3
    assert m["dimensions"].tolist() == [2, 2, 2]
    assert np.array_equal(m["local_position"], np.array(
        [[4.2657785415649414, 11.742777824401855], [2.4493119716644287, -17.223770141601562],
         [3.1442358493804932, 21.099834442138672]], np.float32))
    # the read columns feed the seeding path: all three are inside the
    # default finder's z and radius range and are binned
    off, bins, _, st = O.binning(dict(sp))
    assert sorted(bins.tolist()) == [0, 1, 2]
