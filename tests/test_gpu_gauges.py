"""Gauge free-surface elevation over a full run of the 2D dam break workload
(2,000 steps): the FP64 GPU step against the CPU oracle (bar: within 1%), and
the FP32-mixed step against the FP64 GPU step (bar: within 1e-3). The gauge is
the reference's WaterProfile measure (HeightTesting.h:25-54)."""

import pytest

pytestmark = pytest.mark.gpu


def test_dam_break_gauges_over_full_run(gpu_available):
    from sph2d_gb300 import cases
    from sph2d_gb300.validate import compare, run_gpu, run_oracle

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
