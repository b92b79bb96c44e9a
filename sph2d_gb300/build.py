"""Builds the native libraries in-tree (no cmake, no pip install).

- ``sph2d_gb300/librrsph_cuda.so``: the CUDA kernels (sm_103a) and the C ABI
  declared in ``include/rrsph_cuda.h`` (solver, parameters, CSV layers);
- ``sph2d_gb300/rrsph_run``: the command-line runner linked against it.

The CPU checkers (the oracle) have their own recipe, ``oracle/build.py``.

Translation units compile in parallel; a rebuild is skipped when every output
is newer than its inputs.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "sph2d_gb300"
CSRC = PKG / "csrc"
HOST = PKG / "host"
BUILD = PKG / "_build"
LIB = PKG / "librrsph_cuda.so"
RUNNER = PKG / "rrsph_run"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CU_SOURCES = ["sort.cu", "kernels_common.cu", "kernels_fp64.cu", "kernels_mixed.cu", "kernels_reuse.cu", "solver.cu",
              "sort_noalloc.cu", "run_loop.cu", "adjoint.cu"]
CPP_SOURCES = ["params.cpp", "layers.cpp"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build sph2d_gb300")
    return cand


def _newer(out: Path, inputs) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(i).stat().st_mtime <= t for i in inputs)


def _run(cmd, verbose: bool) -> None:
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(str(c) for c in cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, flush=True)


def _headers():
    return (
        list(CSRC.glob("*.cuh"))
        + list(HOST.glob("*.hpp"))
        + list(HOST.glob("*.def"))
        + [ROOT / "include" / "rrsph_cuda.h"]
    )


def build_cuda(verbose: bool = False, extra_nvcc=()) -> Path:
    """Compiles and links ``librrsph_cuda.so``; returns its path."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = _headers()
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = CSRC / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if not _newer(o, [s, *headers]):
            jobs.append(
                [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-O3",
                 *extra_nvcc, "-c", s, "-o", o]
            )
    for src in CPP_SOURCES:
        s = HOST / src
        o = BUILD / (src + ".o")
        objs.append(o)
        if not _newer(o, [s, *headers]):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(lambda c: _run(c, verbose), jobs))
    if jobs or not _newer(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, ARCH, "-shared", "-o", tmp, *objs, "-lcudart_static", "-lrt", "-ldl", "-lpthread"], verbose)
        os.replace(tmp, LIB)
    # the command-line runner (links the library, found next to it at run time)
    main_src = HOST / "rrsph_run_main.cpp"
    if not _newer(RUNNER, [main_src, LIB, ROOT / "include" / "rrsph_cuda.h"]):
        _run(["g++", "-O2", "-std=c++17", "-Wall", "-o", RUNNER, main_src, "-L", PKG, "-lrrsph_cuda",
              "-Wl,-rpath,$ORIGIN"], verbose)
    return LIB


def build_all(verbose: bool = False) -> None:
    build_cuda(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", LIB, RUNNER)
