"""Gradient of the gauge misfit by the piston's Fourier coefficients: the GPU
adjoint (rrsph_adjoint_forward/reverse) against central finite differences of
the FP64 GPU forward run and, where the oracle can afford the run, against the
oracle's FP64 forward-mode derivatives.

  python tests/adjoint_check.py [--nx 2000 --ny 100 --steps 5000]
         [--checkpoint-every 100] [--eps 1e-6] [--oracle]

Loss: mean over the samples of (gauge - target)^2, the target series being the
gauges of the run with the target seed's coefficients. Prints one JSON line.
"""

from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--nx", type=int, default=2000)
    ap.add_argument("--ny", type=int, default=100)
    ap.add_argument("--steps", type=int, default=5000)
    ap.add_argument("--checkpoint-every", type=int, default=100)
    ap.add_argument("--eps", default="1e-6", help="comma-separated finite-difference steps")
    ap.add_argument("--fd-coefs", default=None, help="comma-separated coefficient indices (default: all)")
    ap.add_argument("--gauge-x", type=float, default=0.3)
    ap.add_argument("--window", type=float, default=0.1)
    ap.add_argument("--oracle", action="store_true", help="also run the oracle's forward-mode reference")
    args = ap.parse_args()
    from sph2d_gb300 import Solver, cases

    case = cases.adjoint_flume_2d(nx=args.nx, ny=args.ny, steps=args.steps, gauge_x=args.gauge_x,
                                  window=args.window)
    p = case.params()
    om, coef, tcoef = case.notes["omega"], case.notes["coef"], case.notes["target_coef"]
    sf, se, gx, K = case.notes["sample_from"], case.notes["sample_every"], case.notes["gauge_x"], args.checkpoint_every

    with Solver(p, "fp64") as s:
        def forward(cf):
            s.upload(case.r, case.v, case.rho, case.itype)
            s.set_piston_fourier(om, cf)
            return s.adjoint_forward(args.steps, gx, sf, se, K)[0]

        target = forward(tcoef)
        s.upload(case.r, case.v, case.rho, case.itype)
        s.set_piston_fourier(om, coef)
        t0 = time.perf_counter()
        s.step(args.steps, 0.0)
        t_fwd = time.perf_counter() - t0
        t0 = time.perf_counter()
        g = forward(coef)
        t1 = time.perf_counter()
        w = 2.0 * (g - target) / len(g)
        dcoef, dvx = s.adjoint_reverse(w)
        t2 = time.perf_counter()
        loss = float(np.mean((g - target) ** 2))
        idx = [int(k) for k in args.fd_coefs.split(",")] if args.fd_coefs else list(range(len(coef)))
        fds = {}
        for eps in [float(e) for e in args.eps.split(",")]:
            fd = np.zeros(len(idx))
            for j, k in enumerate(idx):
                cp, cm = coef.copy(), coef.copy()
                cp[k] += eps
                cm[k] -= eps
                fd[j] = (np.mean((forward(cp) - target) ** 2) - np.mean((forward(cm) - target) ** 2)) / (2 * eps)
            fds[eps] = fd
    res = {
        "particles": case.ntotal, "steps": args.steps, "checkpoint_every": K, "samples": len(g),
        "sample_from": sf, "sample_every": se, "gauge_x": gx, "loss": loss,
        "dloss_dcoef_adjoint": dcoef.tolist(), "fd_coefs": idx,
        "fd": {f"{e:g}": {"dloss_dcoef": fd.tolist(),
                          "rel_err": float(np.linalg.norm(dcoef[idx] - fd) / np.linalg.norm(fd))}
               for e, fd in fds.items()},
        "forward_s": t_fwd, "adjoint_forward_s": t1 - t0, "adjoint_reverse_s": t2 - t1,
        "gradient_cost_vs_forward": (t2 - t0) / t_fwd,
    }
    if args.oracle:
        from oracle import binding as O

        t0 = time.perf_counter()
        go, dgo, _ = O.piston_tangent_run(p, case.r, case.v, case.rho, case.itype, args.steps, om, coef, gx,
                                          sample_from=sf, sample_every=se)
        want = dgo.T @ w
        res.update({
            "oracle_s": time.perf_counter() - t0,
            "gauges_rel_err_vs_oracle": float(np.abs(g - go).max() / np.abs(go).max()),
            "dloss_dcoef_forward_mode": want.tolist(),
            "rel_err_vs_forward_mode": float(np.linalg.norm(dcoef - want) / np.linalg.norm(want)),
        })
    print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
