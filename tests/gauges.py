"""Gauge free-surface elevation over a run: FP32-mixed vs FP64 GPU step vs the
CPU oracle.

The gauge is the reference's WaterProfile measure
(tools/WaterProfile/include/HeightTesting.h:25-54): the largest y among fluid
particles with |x - x_gauge| < search_n * h (search_n = 3), sampled every
`--every` steps.

  python tests/gauges.py --case flume --steps 20000 --every 200
         [--gauges 2,5,10] [--oracle-steps N] [--out series.csv]

Prints one JSON line with the maximum and mean relative gauge differences:
mixed vs FP64 GPU over the whole run, and FP64 GPU vs the oracle over the
first --oracle-steps steps (the oracle is the C restatement of RRSPH_OMP).
"""

from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))

FLUID = 2


def gauges(r: np.ndarray, itype: np.ndarray, xs, radius: float) -> np.ndarray:
    """maxInLayer for each gauge position (0 where no fluid particle is near)."""
    out = np.zeros(len(xs))
    fl = itype == FLUID
    x, y = r[:, 0], r[:, 1]
    for k, xg in enumerate(xs):
        m = fl & (np.abs(x - xg) < radius)
        out[k] = max(0.0, float(y[m].max())) if m.any() else 0.0
    return out


def run_gpu(p, case, precision: str, steps: int, every: int, xs, radius: float, stats: dict | None = None):
    """Gauge series of a GPU run sampled every `every` steps; `stats` (if
    given) receives the directed pairs summed over the run."""
    from sph2d_gb300 import Solver

    series = []
    t = 0.0
    with Solver(p, precision) as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        st = s.download()
        series.append((0, t, gauges(st["r"], st["itype"], xs, radius)))
        done = 0
        t0 = time.perf_counter()
        while done < steps:
            k = min(every, steps - done)
            t = s.step(k, t)
            done += k
            st = s.download()
            series.append((done, t, gauges(st["r"], st["itype"], xs, radius)))
        wall = time.perf_counter() - t0
        if stats is not None:
            stats["pairs_total"] = s.pair_count()[1]
    return series, wall


def run_oracle(p, case, steps: int, every: int, xs, radius: float):
    from oracle import binding as O

    series = []
    t = 0.0
    r, v, rho, itype = case.r.copy(), case.v.copy(), case.rho.copy(), case.itype.copy()
    a = drho = pres = None
    series.append((0, t, gauges(r, itype, xs, radius)))
    done = 0
    while done < steps:
        k = min(every, steps - done)
        res = O.run(p, r, v, rho, itype, nsteps=k, time=t, pres=pres, a=a, drho=drho, itimestep=done)
        r, v, rho, itype, a, drho, pres, t = (res["r"], res["v"], res["rho"], res["itype"], res["a"], res["drho"],
                                              res["p"], res["time"])
        done += k
        series.append((done, t, gauges(r, itype, xs, radius)))
    return series


def compare(a, b):
    """Relative gauge differences |a - b| / b over matching samples (b > 0)."""
    ea = np.array([g for _, _, g in a])
    eb = np.array([g for _, _, g in b])
    n = min(len(ea), len(eb))
    ea, eb = ea[:n], eb[:n]
    ok = eb > 0
    rel = np.abs(ea - eb)[ok] / eb[ok]
    return {"max": float(rel.max()) if rel.size else 0.0, "mean": float(rel.mean()) if rel.size else 0.0,
            "samples": int(n)}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--case", default="flume", choices=["flume", "dam"])
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--every", type=int, default=200)
    ap.add_argument("--gauges", default=None)
    ap.add_argument("--oracle-steps", type=int, default=0)
    ap.add_argument("--search-n", type=float, default=3.0)
    ap.add_argument("--out", default=None)
    args = ap.parse_args()
    from sph2d_gb300 import cases

    if args.case == "flume":
        case = cases.piston_flume_2d()
        xs = [2.0, 5.0, 10.0]
    else:
        case = cases.dam_break_2d()
        xs = [0.2, 0.6, 0.95]
    if args.gauges:
        xs = [float(x) for x in args.gauges.split(",")]
    p = case.params()
    radius = args.search_n * p.hsml
    mixed, wall_m = run_gpu(p, case, "mixed", args.steps, args.every, xs, radius)
    fp64, wall_d = run_gpu(p, case, "fp64", args.steps, args.every, xs, radius)
    result = {
        "case": args.case, "n_particles": case.ntotal, "steps": args.steps, "every": args.every, "gauges_x": xs,
        "simulated_time": mixed[-1][1], "wall_s": {"mixed": wall_m, "fp64": wall_d},
        "mixed_vs_fp64_gpu": compare(mixed, fp64),
    }
    orc = None
    if args.oracle_steps > 0:
        n = min(args.oracle_steps, args.steps)
        orc = run_oracle(p, case, n, args.every, xs, radius)
        result["fp64_gpu_vs_oracle"] = compare(fp64[: len(orc)], orc)
        result["mixed_vs_oracle"] = compare(mixed[: len(orc)], orc)
        result["oracle_steps"] = n
    if args.out:
        with open(args.out, "w") as f:
            cols = ["step", "time"] + [f"{src}_x{x:g}" for src in ("mixed", "fp64") for x in xs]
            if orc:
                cols += [f"oracle_x{x:g}" for x in xs]
            f.write(",".join(cols) + "\n")
            for i, (st, t, g) in enumerate(mixed):
                row = [str(st), repr(float(t))] + [repr(float(v)) for v in g] + [repr(float(v)) for v in fp64[i][2]]
                if orc:
                    row += [repr(float(v)) for v in orc[i][2]] if i < len(orc) else [""] * len(xs)
                f.write(",".join(row) + "\n")
    print(json.dumps(result), flush=True)


if __name__ == "__main__":
    main()
