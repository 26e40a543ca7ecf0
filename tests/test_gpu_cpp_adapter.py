"""The C++ algorithm classes of include/seedgb.hpp (the reference's
triplet_seeding_algorithm / seed_parameter_estimation_algorithm surface)
compiled against the library and run like traccc's examples run theirs:
same seeds and parameters as the oracle, the batch call gives the same seeds,
a rejected configuration throws std::domain_error; and the C++ surface of the
additions (the CKF hand-off, the autotuner, filter training and gate
calibration) works from C++ alone."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O
from traccc_gb300 import synth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def test_cpp_adapter(tmp_path):
    from traccc_gb300 import seeding
    lib = seeding.library_path()
    exe = str(tmp_path / "adapter_check")
    subprocess.run([_nvcc(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "adapter_check.cpp"),
                    "-L", os.path.dirname(lib), "-lseedgb",
                    "-Xlinker", "-rpath=" + os.path.dirname(lib), "-o", exe], check=True)
    ev = synth.workload_event("trk1000", 4)
    n = len(ev["global"])
    inp = tmp_path / "event.bin"
    with open(inp, "wb") as f:
        np.array([n, n], np.uint32).tofile(f)
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
    batch = np.frombuffer(raw[off + O.PARAMS_DTYPE.itemsize * ns:], np.uint32)
    f, g, fl, tp = O.default_configs()
    ref, _ = O.seeding(ev, f, g, fl, phi_mode=O.PHI_CR)
    assert np.array_equal(seeds, ref)
    refp = O.track_params(ev, ref, (0.0, 0.0, float(f.bFieldInZ)), tp)
    assert np.array_equal(params["surface_link"], refp["surface_link"])
    assert np.allclose(params["params"], refp["params"], rtol=1e-5, atol=1e-6)
    assert list(batch) == [ns, ns]
