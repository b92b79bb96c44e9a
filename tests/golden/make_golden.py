"""Writes tests/golden/reference_fixtures.npz from the reference's own code.

Runs the reference's RRSPH_OMP compute core (built from its sources into
oracle/_ref/rrsph_ref by oracle/build_ref.sh) on seeded synthetic cases from
sph2d_gb300.cases and stores its outputs, so that machines without the
reference sources can still pin the oracle and the CUDA path to the
reference's results.

Cases (small versions of the benchmark workloads, to keep the file small):
  dam: dam_break_2d(nx=50, ny=25, seed=1), continuity density
  flume: piston_flume_2d(nx=120, ny=20, seed=7), summation density, piston on
Outputs per case: grid hashes (keys, sorted grid, cells_start, neighbour
counts and lists), density, force terms on a seeded velocity field, and the
state after N loop steps.

Usage: python tests/golden/make_golden.py   (needs oracle/_ref/rrsph_ref)
"""

from __future__ import annotations

import hashlib
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "reference_fixtures.npz"
RUN_STEPS = {"dam": 30, "flume": 30}


def fixture_cases():
    from sph2d_gb300 import cases

    return {
        "dam": cases.dam_break_2d(nx=50, ny=25, seed=1, density_treatment=1),
        "flume": cases.piston_flume_2d(nx=120, ny=20, seed=7, density_treatment=0),
    }


def velocity_field(case, seed=5):
    rng = np.random.default_rng(seed)
    return rng.normal(0.0, 0.3, size=case.r.shape)


def digest(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main() -> None:
    from oracle import binding as O
    from sph2d_gb300 import capi

    if not O.ref_available():
        raise SystemExit("reference core not built: run oracle/build_ref.sh where the reference sources are")
    out = {}
    for name, case in fixture_cases().items():
        p = case.params()
        g = O.ref_run(p, "grid", case.r, case.v, case.rho, case.itype)
        out[f"{name}/grid_sha"] = np.array(digest(g["keys"], g["grid"], g["cells_start"]))
        out[f"{name}/pairs_sha"] = np.array(digest(g["counts"], g["list"]))
        out[f"{name}/pairs"] = np.array(int(g["counts"].sum()))
        d = O.ref_run(p, "density", case.r, case.v, case.rho, case.itype)
        out[f"{name}/density"] = d["density"]
        out[f"{name}/density_p"] = d["pout"]
        v = velocity_field(case)
        q = p.copy()
        q.dt_correction_method = 2
        pres = O.eos_p(q, case.rho)
        t = O.ref_run(q, f"terms:{capi.TERM_ALL}", case.r, v, case.rho, case.itype, pres=pres)
        out[f"{name}/terms_a"] = t["a"]
        out[f"{name}/terms_mu"] = t["mu"]
        n = RUN_STEPS[name]
        run = O.ref_run(p, f"run:{n}", case.r, case.v, case.rho, case.itype)
        for k in ("r_out", "v_out", "rho_out", "p_out"):
            out[f"{name}/run_{k[:-4]}"] = run[k]
        out[f"{name}/run_itype"] = run["itype_out"]
        out[f"{name}/run_time"] = np.array(run["timing"]["time"])
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT} ({OUT.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
