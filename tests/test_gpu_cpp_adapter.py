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
import sys

import numpy as np
import pytest

import oracle as O
from traccc_gb300 import synth

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests"))


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


def test_cpp_full_chain(tmp_path):
    """The whole stage from C++ through include/seedgb.hpp (formation of
    three events in one call, seeding, parameters, the hand-off to the track
    finding's records): the seeds are the oracle's on the formed
    spacepoints, the handed-off parameters the oracle's estimation of those
    seeds (1e-5, the covariance stored as an array of columns), and the
    barcodes the bottom measurements' surfaces."""
    from test_gpu_parity import same_params

    from traccc_gb300 import seeding
    lib = seeding.library_path()
    exe = str(tmp_path / "full_chain_check")
    subprocess.run([_nvcc(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "full_chain_check.cpp"),
                    "-L", os.path.dirname(lib), "-lseedgb",
                    "-Xlinker", "-rpath=" + os.path.dirname(lib), "-o", exe], check=True)
    surf = np.zeros(len(synth.LAYER_RADII) + 1, seeding.SURFACE_DTYPE)
    for layer, r in enumerate(synth.LAYER_RADII):
        surf[layer + 1]["type"] = seeding.SURFACE_CYLINDER
        surf[layer + 1]["radius"] = r
        surf[layer + 1]["rotation"] = np.eye(3, dtype=np.float32).reshape(-1)
    events = [synth.workload_event("trk1000", 50 + s) for s in range(3)]
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([len(events), len(surf)], np.uint32).tofile(f)
        surf.tofile(f)
        for ev in events:
            np.array([len(ev["global"])], np.uint32).tofile(f)
            np.asarray(ev["local_position"], np.float32).tofile(f)
            np.asarray(ev["surface_link"], np.uint64).tofile(f)
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(inp), str(out)], check=True)
    raw = out.read_bytes()
    off = 0
    f, g, fl, tp = O.default_configs()
    bf = (0.0, 0.0, float(f.bFieldInZ))
    for ev in events:
        n_sp, n_seeds = np.frombuffer(raw[off:off + 8], np.uint32)
        off += 8
        glob = np.frombuffer(raw[off:off + 12 * n_sp], np.float32).reshape(-1, 3)
        off += 12 * n_sp
        seeds = np.frombuffer(raw[off:off + 16 * n_seeds], O.SEED_DTYPE)
        off += 16 * n_seeds
        ckf = np.frombuffer(raw[off:off + 176 * n_seeds], seeding.CKF_PARAMS_DTYPE)
        off += 176 * n_seeds
        assert n_sp == len(ev["global"]) and n_seeds > 0
        formed = dict(ev, **{"global": glob.copy(),
                             "measurement_index_1": np.arange(n_sp, dtype=np.uint32),
                             "measurement_index_2": np.full(n_sp, 0xFFFFFFFF, np.uint32),
                             "z_variance": np.zeros(n_sp, np.float32),
                             "radius_variance": np.zeros(n_sp, np.float32)})
        ref, _ = O.seeding(formed, f, g, fl, phi_mode=O.PHI_CR)
        assert np.array_equal(seeds, ref)
        rp = O.track_params(formed, ref, bf, tp)
        got = np.zeros(len(ckf), O.PARAMS_DTYPE)
        got["surface_link"] = ckf["barcode"]
        got["params"] = ckf["vector"]
        got["cov"] = ckf["covariance"].reshape(-1, 6, 6).transpose(0, 2, 1).reshape(-1, 36)
        assert same_params(got, rp).all()
        assert np.array_equal(got["cov"], rp["cov"]) or np.allclose(got["cov"], rp["cov"],
                                                                     rtol=1e-5, atol=0)
    assert off == len(raw)


def test_cpp_gbts_from_config_directory(tmp_path):
    """GBTS from C++: the configuration directory in the reference's format
    (written here from the synthetic barrel) read by
    gbts_seedfinder_config::from_directory, seeds equal to the oracle's."""
    from traccc_gb300 import gbts, seeding
    lib = seeding.library_path()
    exe = str(tmp_path / "gbts_check")
    subprocess.run([_nvcc(), "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "gbts_check.cpp"),
                    "-L", os.path.dirname(lib), "-lseedgb",
                    "-Xlinker", "-rpath=" + os.path.dirname(lib), "-o", exe], check=True)
    layers, pairs, geoid = synth.gbts_geometry()
    cfgdir = tmp_path / "gbts_config"
    gbts.write_config_dir(str(cfgdir), layers, pairs, geoid)
    ev = synth.workload_event("trk1000", 7)
    link, dia = synth.gbts_measurements(ev, 7)
    inp = tmp_path / "event.bin"
    with open(inp, "wb") as f:
        np.array([len(ev["global"]), len(link)], np.uint32).tofile(f)
        np.asarray(ev["measurement_index_1"], np.uint32).tofile(f)
        np.asarray(ev["global"], np.float32).tofile(f)
        np.asarray(link, np.uint64).tofile(f)
        np.asarray(dia, np.float32).tofile(f)
    out = tmp_path / "out.bin"
    subprocess.run([exe, str(cfgdir), str(inp), str(out)], check=True)
    raw = out.read_bytes()
    ns = int(np.frombuffer(raw[:4], np.uint32)[0])
    got = np.frombuffer(raw[4:4 + 16 * ns], O.SEED_DTYPE)
    l2, p2, g2 = gbts.read_config_dir(str(cfgdir))
    ref, _ = O.gbts(ev, link, dia, l2, p2, g2)
    assert len(ref) > 0 and np.array_equal(got, ref)
