"""Generates tests/golden/flume_gauges_full.npz: the free-surface elevation of
the 2D piston flume over its full 20,000 steps, computed on the CPU by the
reference's own RRSPH_OMP compute core (oracle/_ref/rrsph_ref, built from the
reference sources by oracle/build_ref.sh), or by the C restatement of it
(oracle/liboracle.so) where the reference core is absent.

The gauge is WaterProfile's measure (tools/WaterProfile/include/HeightTesting.h:25-54):
the largest y among water particles with |x - x_gauge| < 3 h, at x = 2, 5 and
10 m, sampled at step 0 and after every 200 steps. The loop is the reference's
(sources/RRSPH_OMP/src/TimeIntegration.cpp:60-100) with the piston call enabled.

  python tests/golden/make_flume_gauges.py [--steps 20000] [--every 200] [--threads 8]

This takes about 35 minutes on 8 host cores. The GPU tests in
tests/test_gpu_gauges.py compare the CUDA step's series with this file.
"""

from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

OUT = Path(__file__).resolve().parent / "flume_gauges_full.npz"
GAUGES_X = (2.0, 5.0, 10.0)
SEARCH_N = 3.0
WATER = 2


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--every", type=int, default=200)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--out", default=str(OUT))
    args = ap.parse_args()

    from oracle import binding as O
    from oracle import params as OP
    from sph2d_gb300 import cases

    case = cases.piston_flume_2d()
    p = OP.case_params(case)
    t0 = time.perf_counter()
    if O.ref_available():
        res = O.ref_run(p, f"run:{args.steps}", case.r, case.v, case.rho, case.itype, threads=args.threads,
                        timeout=6 * 3600, gauges=(args.every, SEARCH_N, WATER, GAUGES_X))
        series = res["gauges"]
        pairs = res["pairs"]
        source = "reference RRSPH_OMP compute core (oracle/_ref/rrsph_ref)"
        final_time = res["timing"]["time"]
    else:
        if args.threads:
            O.set_threads(args.threads)
        rows = [[O.gauge(p, case.r, case.itype, x, SEARCH_N, WATER) for x in GAUGES_X]]
        st = {"r": case.r, "v": case.v, "rho": case.rho, "itype": case.itype, "p": None, "a": None, "drho": None,
              "time": 0.0}
        pairs = []
        done = 0
        while done < args.steps:
            k = min(args.every, args.steps - done)
            st = O.run(p, st["r"], st["v"], st["rho"], st["itype"], nsteps=k, time=st["time"], pres=st["p"],
                       a=st["a"], drho=st["drho"], itimestep=done)
            done += k
            rows.append([O.gauge(p, st["r"], st["itype"], x, SEARCH_N, WATER) for x in GAUGES_X])
        series = np.array(rows)
        pairs = np.zeros(0, dtype=np.uint64)
        source = "C restatement of RRSPH_OMP (oracle/liboracle.so)"
        final_time = st["time"]
    wall = time.perf_counter() - t0
    steps = np.arange(series.shape[0], dtype=np.int64) * args.every
    meta = {"source": source, "steps": args.steps, "every": args.every, "gauges_x": list(GAUGES_X),
            "search_n": SEARCH_N, "type_filter": WATER, "ntotal": int(p.ntotal), "hsml": float(p.hsml),
            "dt": float(p.dt), "mass": float(p.mass), "final_time": float(final_time), "wall_s": wall}
    np.savez_compressed(args.out, gauges=np.asarray(series, dtype=np.float64), steps=steps,
                        pairs=np.asarray(pairs, dtype=np.uint64), meta=json.dumps(meta))
    print(json.dumps(meta))


if __name__ == "__main__":
    main()
