"""In-tree build of the native libraries (no cmake, no pip install).

* ``_lib/libseedgb.so``       -- the CUDA seeding library (C ABI), sm_103a only.
* ``_lib/libseedgb_synth.so`` -- the synthetic event generator (host C).

Both are rebuilt when a source is newer than the library.  CUDA sources are
compiled in parallel, one translation unit per nvcc process.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "_lib")
REPO = os.path.dirname(HERE)
INCLUDE = os.path.join(REPO, "include")

CUDA_SOURCES = ["seedgb_kernels.cu", "seedgb_api.cu", "seedgb_noalloc.cu", "seedgb_learned.cu",
                "seedgb_formation.cu", "seedgb_handoff.cu", "seedgb_host.cu", "seedgb_gbts.cu"]
HOST_SOURCES = ["seedgb_config.cpp", "seedgb_io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# The cut arithmetic must match the reference's host float semantics: no FMA
# contraction, IEEE division and square root, no flush-to-zero.
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-fmad=false", "--prec-div=true", "--prec-sqrt=true",
                     "--ftz=false", "-I", INCLUDE, "-I", CSRC]


def _nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    p = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(p):
        return p
    raise RuntimeError("nvcc not found: the CUDA toolkit is required")


def _stale(out, deps):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def synth_library(force: bool = False) -> str:
    out = os.path.join(LIBDIR, "libseedgb_synth.so")
    src = os.path.join(CSRC, "synth_events.c")
    if force or _stale(out, [src]):
        os.makedirs(LIBDIR, exist_ok=True)
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-std=c11",
                        "-D_GNU_SOURCE", "-shared", "-o", out, src, "-lm"],
                       check=True)
    return out


def _headers():
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC)
           if f.endswith((".h", ".cuh", ".hpp"))]
    return hs


def cuda_library(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA seeding library for sm_103a and return its path."""
    out = os.path.join(LIBDIR, "libseedgb.so")
    srcs = [os.path.join(CSRC, s) for s in CUDA_SOURCES + HOST_SOURCES]
    deps = srcs + _headers()
    if not force and not _stale(out, deps):
        return out
    os.makedirs(os.path.join(LIBDIR, "obj"), exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(LIBDIR, "obj", os.path.basename(src) + ".o")
        if src.endswith(".cu"):
            cmd = [nvcc] + NVCC_FLAGS + ["-dc" if False else "-c", src, "-o", obj]
            if verbose:
                cmd += ["-Xptxas", "-v"]
        else:
            cmd = ["g++", "-O2", "-ffp-contract=off", "-fPIC", "-std=c++17",
                   "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return obj, (r.stdout + r.stderr)

    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        results = list(ex.map(compile_one, srcs))
    if verbose:
        for _, log in results:
            if log.strip():
                print(log)
    objs = [o for o, _ in results]
    cmd = [nvcc] + ARCH + ["-shared", "-o", out] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return out


def build_all(force: bool = False, verbose: bool = False):
    return synth_library(force), cuda_library(force, verbose)
