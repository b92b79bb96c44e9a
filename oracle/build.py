"""Builds the CPU checkers in-tree (TEST INFRASTRUCTURE; no cmake, no install).

- ``oracle/liboracle.so``: the C restatement of RRSPH_OMP's step (plain C +
  OpenMP, ``-ffp-contract=off``), used by the tests, the smoke check and the
  benchmark's CPU arms.
- ``oracle/_ref/rrsph_ref``: the reference's own OMP compute core with
  ``oracle/ref_driver.cpp`` (``oracle/build_ref.sh``). The recipe reads the
  reference sources where they lie (``$RRSPH_REFERENCE``, by default the
  reference checkout of the build machine) and stages the few files it
  compiles under ``oracle/_ref/src/``, so that a machine without the
  reference checkout (but with that staged copy) builds the same core.

A rebuild is skipped when every output is newer than its inputs.
"""

from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
ORACLE_LIB = HERE / "liboracle.so"
REF_DIR = HERE / "_ref"
REF_BIN = REF_DIR / "rrsph_ref"
REF_STAGED = REF_DIR / "src"
DEFAULT_REFERENCE = "/root/reference"


def reference_root() -> Path:
    """The reference checkout the recipe reads ($RRSPH_REFERENCE or the default)."""
    return Path(os.environ.get("RRSPH_REFERENCE", DEFAULT_REFERENCE))


def _newer(out: Path, inputs) -> bool:
    if not out.exists():
        return False
    t = out.stat().st_mtime
    return all(Path(i).stat().st_mtime <= t for i in inputs)


def _run(cmd, verbose: bool, env=None) -> None:
    if verbose:
        print(" ".join(str(c) for c in cmd), flush=True)
    res = subprocess.run([str(c) for c in cmd], capture_output=True, text=True, env=env)
    if res.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(str(c) for c in cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and (res.stdout or res.stderr):
        print(res.stdout + res.stderr, flush=True)


def build_oracle(verbose: bool = False) -> Path:
    """Compiles the C oracle into ``oracle/liboracle.so``."""
    srcs = [HERE / "rrsph_oracle.c", HERE / "rrsph_tangent.c"]
    hdrs = [HERE / "rrsph_oracle.h", ROOT / "include" / "rrsph_cuda.h"]
    if not _newer(ORACLE_LIB, [*srcs, *hdrs]):
        tmp = ORACLE_LIB.with_suffix(".so.tmp")
        _run(["gcc", "-std=c11", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-Wall", "-o", tmp,
              *srcs, "-lm"], verbose)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def reference_sources_available() -> bool:
    return (reference_root() / "sources" / "RRSPH_OMP" / "src").is_dir() or (REF_STAGED / "sources").is_dir()


def build_reference(verbose: bool = False) -> Path | None:
    """Builds the reference's compute core where its sources (the checkout or
    the staged copy) are present; returns the binary or None."""
    if not reference_sources_available():
        return None
    inputs = [HERE / "ref_driver.cpp", HERE / "build_ref.sh", HERE / "ref_params_driver.cpp",
              *sorted((ROOT / "sph2d_gb300" / "integration").glob("*"))]
    if not _newer(REF_BIN, inputs):
        env = dict(os.environ)
        env.setdefault("RRSPH_REFERENCE", str(reference_root()))
        _run(["sh", str(HERE / "build_ref.sh")], verbose, env=env)
    return REF_BIN if REF_BIN.exists() else None


def build_all(verbose: bool = False) -> None:
    build_oracle(verbose)
    build_reference(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print("built", ORACLE_LIB, REF_BIN if REF_BIN.exists() else "(no reference core)")
