"""The oracle's C++ face (oracle/seeding_algorithm.hpp: the reference's
host::seeding_algorithm and track_params_estimation constructor and
operator() names) compiled with g++ against the oracle library: the same
seeds and parameters as the oracle's Python entry points, and a grid
configuration the reference's get_axes rejects throws std::domain_error."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from traccc_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_oracle_cpp_classes(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    lib = O.build()
    exe = str(tmp_path / "oracle_host_check")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "oracle"),
                    os.path.join(ROOT, "tests", "cpp", "oracle_host_check.cpp"),
                    "-L", os.path.dirname(lib), "-lseedoracle",
                    "-Wl,-rpath," + os.path.dirname(lib), "-o", exe], check=True)
    ev = synth.workload_event("trk1000", 6)
    n = len(ev["global"])
    inp = tmp_path / "event.bin"
    with open(inp, "wb") as f:
        np.array([n, len(ev["surface_link"])], np.uint32).tofile(f)
        np.asarray(ev["measurement_index_1"], np.uint32).tofile(f)
        np.asarray(ev["measurement_index_2"], np.uint32).tofile(f)
        np.asarray(ev["global"], np.float32).tofile(f)
        np.asarray(ev["z_variance"], np.float32).tofile(f)
        np.asarray(ev["radius_variance"], np.float32).tofile(f)
        np.asarray(ev["local_position"], np.float32).tofile(f)
        np.asarray(ev["surface_link"], np.uint64).tofile(f)
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(inp), str(out)], check=True)
    raw = out.read_bytes()
    ns = int(np.frombuffer(raw[:4], np.uint32)[0])
    seeds = np.frombuffer(raw[4:4 + 16 * ns], O.SEED_DTYPE)
    off = 4 + 16 * ns
    params = np.frombuffer(raw[off:off + O.PARAMS_DTYPE.itemsize * ns], O.PARAMS_DTYPE)
    threw = int(np.frombuffer(raw[off + O.PARAMS_DTYPE.itemsize * ns:], np.int32)[0])
    f, g, fl, tp = O.default_configs()
    ref, _ = O.seeding(ev, f, g, fl, phi_mode=O.PHI_CR)
    assert ns == len(ref) > 0
    assert np.array_equal(seeds, ref)
    refp = O.track_params(ev, ref, (0.0, 0.0, float(f.bFieldInZ)), tp)
    assert params.tobytes() == refp.tobytes()
    assert threw == 1
