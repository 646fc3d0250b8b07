"""Builds the native libraries in-tree.

* ``lfm_public_gb300/liblfm_gpu.so``  -- the product: sm_103a CUDA kernels, the
  C ABI of include/lfm_gpu.h and the OpenFOAM-free host plugins.
* ``lfm_public_gb300/lfm_solve_gpu``  -- the command-line solver (the
  reference's lfm_solve on the device path).
* ``oracle/port/liblfm_port.so``      -- the CPU restatement used by tests and
  the CPU baseline (test infrastructure).
* ``oracle/_ref/lfm_oracle``          -- the reference solver built from its own
  sources, only where those sources are present.

Objects are compiled in parallel with one ``-gencode`` for sm_103a.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(ROOT, "_build")
INCLUDES = [os.path.join(ROOT, "include"), os.path.join(ROOT, "include", "lfm"), os.path.join(CSRC, "host"),
            os.path.join(CSRC, "cuda")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_SOURCES = ["foam_io.cpp", "foam_case.cpp", "dict_reader.cpp", "poly_mesh_reader.cpp", "run_time_manager.cpp",
                "input_reader.cpp", "renumber.cpp", "hpath.cpp", "case_setup.cpp", "tiles.cpp", "capi_case.cpp"]
CUDA_SOURCES = ["solver_kernels.cu", "solver_kernels_fp32.cu", "flux_staged_fp32.cu", "batch_kernels.cu",
                "tile_kernels.cu", "post_kernels.cu", "capi_solver.cu", "capi_batch.cu", "capi_server.cu"]
CLI_SOURCES = ["gpu_mesh.cpp", "lfm_solve_gpu.cpp"]
# The FP32-bulk kernels are compiled without implicit FMA contraction (explicit
# fmaf/fma calls stay fused): every kernel that inlines the same device
# function then rounds identically, so a case gives the same bits in the
# single-case solver, in any batch-kernel variant and in any mix of cases.
# The post-processing kernels follow the reference's CPU arithmetic, which is
# not contracted either.
CUDA_FLAGS = {"solver_kernels_fp32.cu": ["-fmad=false"], "flux_staged_fp32.cu": ["-fmad=false"],
              "batch_kernels.cu": ["-fmad=false"],
              "tile_kernels.cu": ["-fmad=false"], "post_kernels.cu": ["-fmad=false"]}

LIB = os.path.join(PKG, "liblfm_gpu.so")
CLI = os.path.join(PKG, "lfm_solve_gpu")
PORT = os.path.join(ROOT, "oracle", "port", "liblfm_port.so")
# The reference sources, when a checkout is at hand: $LFM_REFERENCE_DIR, else a
# checkout named "reference" beside this repository. Without one the reference
# oracle is not built (the CPU restatement in oracle/port is always built).
REF_DIR = os.environ.get("LFM_REFERENCE_DIR") or os.path.join(os.path.dirname(ROOT), "reference")


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblfm_gpu.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def _newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _headers():
    out = [os.path.abspath(__file__)]   # flags live here: a change rebuilds everything
    for d in INCLUDES:
        for n in os.listdir(d):
            if n.endswith((".h", ".cuh")):
                out.append(os.path.join(d, n))
    return out


def build_library(verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    inc = [f"-I{d}" for d in INCLUDES]
    hdrs = _headers()
    jobs = []
    objs = []
    for s in HOST_SOURCES:
        src = os.path.join(CSRC, "host", s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + hdrs):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", *inc, "-c", src, "-o", obj])
    for s in CUDA_SOURCES:
        src = os.path.join(CSRC, "cuda", s)
        obj = os.path.join(BUILD, s + ".o")
        objs.append(obj)
        if not _newer(obj, [src] + hdrs):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", *CUDA_FLAGS.get(s, []), "-Xcompiler", "-fPIC",
                         *inc, "-c", src, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout, r.stderr)
    if not _newer(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    cli_objs = []
    cli_jobs = []
    for s in CLI_SOURCES:
        src = os.path.join(CSRC, "host", s)
        if not os.path.exists(src):
            continue
        obj = os.path.join(BUILD, s + ".o")
        cli_objs.append(obj)
        if not _newer(obj, [src] + hdrs):
            cli_jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", *inc, "-c", src, "-o", obj])
    for j in cli_jobs:
        _run(j)
    if cli_objs and not _newer(CLI, cli_objs + [LIB]):
        _run(["g++", "-o", CLI, *cli_objs, f"-L{PKG}", "-llfm_gpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


def build_port() -> str:
    """The oracle's CPU restatement: the stage loop (lfm_port.c) and its own
    case set-up (lfm_port_setup.c), one shared library that needs nothing
    from liblfm_gpu.so."""
    srcs = [os.path.join(ROOT, "oracle", "port", n) for n in ("lfm_port.c", "lfm_port_setup.c")]
    hdr = [os.path.join(ROOT, "oracle", "port", "lfm_port.h"), os.path.join(ROOT, "include", "lfm_gpu.h")]
    if not _newer(PORT, srcs + hdr):
        _run(["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared", f"-I{os.path.join(ROOT, 'include')}",
              "-o", PORT, *srcs, "-lm"])
    return PORT


def build_reference_oracle() -> str | None:
    """Builds oracle/_ref/lfm_oracle from the reference sources when present."""
    if not os.path.isdir(os.path.join(REF_DIR, "src")):
        return None
    r = subprocess.run(["make", "-s", "-j", str(os.cpu_count() or 4), f"REF={REF_DIR}"],
                       cwd=os.path.join(ROOT, "oracle"), capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference oracle build failed:\n" + r.stdout + r.stderr)
    return os.path.join(ROOT, "oracle", "_ref", "lfm_oracle")


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        futs = [ex.submit(build_library, verbose), ex.submit(build_port), ex.submit(build_reference_oracle)]
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", LIB, PORT)
