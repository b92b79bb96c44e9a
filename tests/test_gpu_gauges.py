"""Gauge free-surface elevation over full runs. The gauge is the reference's
WaterProfile measure (tools/WaterProfile/include/HeightTesting.h:25-54): the
largest y among water particles within 3 h of the gauge's x.

- The 2D piston flume (408,970 particles) over its full 20,000 steps, against
  the series of the reference's own RRSPH_OMP compute core committed in
  tests/golden/flume_gauges_full.npz (made by tests/golden/make_flume_gauges.py
  on the CPU): the FP64 and the FP32-mixed GPU steps within 1% of it at
  x = 2, 5 and 10 m, and the mixed step within 1e-3 of the FP64 GPU step.
- The 2D dam break over its full 2,000 steps against the CPU oracle.
"""

import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FLUME_FIXTURE = Path(__file__).resolve().parent / "golden" / "flume_gauges_full.npz"


def _rel_series(a, b):
    """max and mean of |a - b| / b over the samples where b > 0."""
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    ok = b > 0
    rel = np.abs(a - b)[ok] / b[ok]
    return float(rel.max()), float(rel.mean())


def test_flume_gauges_full_run_vs_reference(gpu_available):
    from gauges import run_gpu
    from sph2d_gb300 import cases

    fx = np.load(FLUME_FIXTURE)
    meta = json.loads(str(fx["meta"]))
    ref = fx["gauges"]
    case = cases.piston_flume_2d()
    p = case.params()
    assert int(p.ntotal) == meta["ntotal"] and float(p.dt) == meta["dt"] and float(p.hsml) == meta["hsml"]
    xs = meta["gauges_x"]
    radius = meta["search_n"] * p.hsml
    steps, every = meta["steps"], meta["every"]
    assert steps == 20000 and ref.shape == (steps // every + 1, len(xs))
    series, pairs = {}, {}
    for prec in ("mixed", "fp64"):
        stats = {}
        out, _ = run_gpu(p, case, prec, steps, every, xs, radius, stats)
        assert [s for s, _, _ in out] == list(fx["steps"])
        series[prec] = np.array([g for _, _, g in out])
        pairs[prec] = stats["pairs_total"]
        assert out[-1][1] == pytest.approx(meta["final_time"], rel=1e-12)
    e64 = _rel_series(series["fp64"], ref)
    emx = _rel_series(series["mixed"], ref)
    emf = _rel_series(series["mixed"], series["fp64"])
    report = {"fp64_vs_reference": e64, "mixed_vs_reference": emx, "mixed_vs_fp64": emf,
              "pairs": {k: int(v) for k, v in pairs.items()}, "pairs_reference": int(fx["pairs"].sum())}
    print("flume gauges over 20,000 steps (max, mean relative):", json.dumps(report))
    assert e64[0] < 1e-2, ("FP64 GPU vs reference", e64)
    assert emx[0] < 1e-2, ("mixed vs reference", emx)
    assert emf[0] < 1e-3, ("mixed vs FP64 GPU", emf)
    # the run's directed pairs, summed over the 20,000 steps, against the reference's find_neighbours
    # (the trajectories separate slowly: 1.5e-6 for FP64 and 2.3e-5 for the mixed step measured)
    ref_pairs = float(fx["pairs"].sum())
    assert abs(pairs["fp64"] - ref_pairs) / ref_pairs < 1e-5, (pairs, ref_pairs)
    assert abs(pairs["mixed"] - ref_pairs) / ref_pairs < 1e-4, (pairs, ref_pairs)
    # water stands at every gauge for the whole run
    assert np.all(ref > 0.3) and np.all(series["mixed"] > 0.3)


def test_dam_break_gauges_over_full_run(gpu_available):
    from gauges import compare, run_gpu, run_oracle
    from sph2d_gb300 import cases

    case = cases.dam_break_2d()
    p = case.params()
    xs = [0.2, 0.6, 0.95]
    radius = 3.0 * p.hsml
    steps, every = 2000, 100
    mixed, _ = run_gpu(p, case, "mixed", steps, every, xs, radius)
    fp64, _ = run_gpu(p, case, "fp64", steps, every, xs, radius)
    orc = run_oracle(p, case, steps, every, xs, radius)
    assert len(mixed) == len(fp64) == len(orc) == steps // every + 1
    e_fp64 = compare(fp64, orc)
    e_mixed = compare(mixed, fp64)
    assert e_fp64["max"] < 1e-2, e_fp64
    assert e_mixed["max"] < 1e-3, e_mixed
    # water stands at the first two stations for the whole run
    assert all(g[0] > 0.3 and g[1] > 0.3 for _, _, g in fp64)
