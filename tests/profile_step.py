"""Runs a few steps of a workload, for profilers (ncu) to capture.

  python tests/profile_step.py [--precision mixed|fp64] [--steps N]
                                     [--case flume|dam|dam3d] [--nx 4000 --ny 100]
                                     [--dx3d 0.0026] [--no-graph]

The default is the full 2D piston flume (409k particles, about 0.2 GB on the
device); dam3d is the 3D dam break (6.5M particles at dx 2.6 mm, about 20 GB
with the mixed step's lists; a larger --dx3d makes it smaller). Warm-up steps
run first, so `ncu -s <k>` can skip them.
"""

from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--nx", type=int, default=4000)
    ap.add_argument("--ny", type=int, default=100)
    ap.add_argument("--case", default="flume", choices=["flume", "dam", "dam3d"])
    ap.add_argument("--dx3d", type=float, default=0.0026)
    ap.add_argument("--no-graph", action="store_true", help="launch kernels directly (per-phase events)")
    args = ap.parse_args()
    from sph2d_gb300 import Solver, cases

    if args.case == "flume":
        case = cases.piston_flume_2d(nx=args.nx, ny=args.ny)
    elif args.case == "dam3d":
        case = cases.dam_break_3d(dx=args.dx3d)
    else:
        case = cases.dam_break_2d()
    p = case.params()
    with Solver(p, args.precision) as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        if args.no_graph:
            s.set_phase_timing(True)
        t = s.step(args.warmup, 0.0)
        t = s.step(args.steps, t)
        last, total = s.pair_count()
        if args.no_graph:
            phases, n = s.phase_times()
            print("phases ms/step:", {k: round(v / max(n, 1), 4) for k, v in phases.items()})
        print(f"profile_step: n={case.ntotal} precision={args.precision} steps={args.warmup}+{args.steps} "
              f"pairs/step={last} t={t:.6f} launches={s.kernel_launches()}")


if __name__ == "__main__":
    main()
