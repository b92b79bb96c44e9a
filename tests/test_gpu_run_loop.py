"""The time loop with layer output (rrsph_run and the rrsph_run command):
file names and timing of data/dump layers as RRSPHOutput writes them
(Output.cpp:45-79, 223-446), the layer contents against the oracle, and the
crash dump of a CONSISTENCY_STOP failure."""

import math
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

RUNNER = Path(__file__).resolve().parent.parent / "sph2d_gb300" / "rrsph_run"


def _digits(val):
    """format_count_decimal_digits (TimeFormat.cpp:36-49)."""
    if val > 10:
        return 0
    if val > 1:
        return 1
    count = 1
    while val < 1:
        val *= 10
        count += 1
    return count


def _expected_layers(t0, dt, sim_time, save_time, dump_time, use_dump):
    """The layer times update_step would write (Output.cpp:366-446)."""
    saves, dumps, save_steps = [t0], [], [0]
    t, last_s, last_d, steps = t0, t0, t0, 0
    while t <= sim_time:
        t = t + dt
        steps += 1
        if (t - last_s) > save_time:
            saves.append(t)
            save_steps.append(steps)
            last_s = t
        if use_dump and (t - last_d) > dump_time:
            dumps.append(t)
            last_d = t
    return saves, dumps, steps, save_steps


def _experiment(tmp_path, **model):
    from sph2d_gb300 import cases

    case = cases.dam_break_2d(nx=40, ny=20)
    dt = case.model["dt"]
    case.model.update({"simulation_time": 37 * dt, "save_time": 10 * dt, "dump_time": 25 * dt, "use_dump": True})
    case.model.update(model)
    case.write_experiment(tmp_path)
    return case


def test_runner_writes_the_reference_layers(gpu_available, tmp_path):
    from oracle import binding as O
    from sph2d_gb300 import read_layer

    case = _experiment(tmp_path)
    p = case.params()
    res = subprocess.run([str(RUNNER), str(tmp_path), "--precision", "fp64"], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    saves, dumps, steps, save_steps = _expected_layers(0.0, p.dt, p.simulation_time, p.save_time, p.dump_time, True)
    sd, dd = _digits(p.save_time), _digits(p.dump_time)
    data = sorted(f.name for f in (tmp_path / "data").iterdir())
    assert data == sorted(f"{t:.{sd}f}.csv" for t in saves)
    dump_files = sorted(f.name for f in (tmp_path / "dump").iterdir())
    assert dump_files == sorted({"0.csv"} | {f"{t:.{dd}f}.csv" for t in dumps})
    assert f"{steps} steps" in res.stdout
    # the last data layer against the oracle run from the same (printed) start layer
    r0, v0, rho0, _, it0 = read_layer(tmp_path / "dump" / "0.csv", p)
    ref = O.run(p, r0, v0, rho0, it0, nsteps=save_steps[-1])
    last = tmp_path / "data" / f"{saves[-1]:.{sd}f}.csv"
    q = p.copy()
    r, v, rho, pres, itype = read_layer(last, q)
    assert np.allclose(r, ref["r"], atol=6e-7) and np.allclose(v, ref["v"], atol=6e-7)
    assert np.allclose(rho, ref["rho"], atol=6e-7) and np.array_equal(itype, ref["itype"])


def test_run_api_mixed_and_restart_from_dump(gpu_available, tmp_path):
    """rrsph_run from Python; then a restart from the written dump continues
    the run as the reference's dump/resume does (Input.cpp:258)."""
    from sph2d_gb300 import Solver, derive, load_params, read_layer

    case = _experiment(tmp_path, simulation_time=0.0, use_dump=True)
    p = case.params()
    p.simulation_time = 30 * p.dt
    with Solver(p, "mixed") as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        t, n = s.run(tmp_path, 0.0)
    assert n in (30, 31) and math.isclose(t, n * p.dt, rel_tol=1e-12)
    dumps = sorted((tmp_path / "dump").glob("*.csv"), key=lambda f: float(f.stem))
    assert len(dumps) >= 2
    p0 = load_params(tmp_path)
    r, v, rho, pres, itype = read_layer(dumps[-1], p0)
    assert itype.shape[0] == case.ntotal and np.all(np.isfinite(r))
    q = derive(p0, r)
    q.start_simulation_time = float(dumps[-1].stem)
    with Solver(q, "fp64") as s:
        s.upload(r, v, rho, itype)
        t2 = s.step(5, q.start_simulation_time)
    assert t2 > q.start_simulation_time


def test_consistency_stop_writes_a_crash_dump(gpu_available, tmp_path):
    from sph2d_gb300 import RrsphError, Solver, capi

    case = _experiment(tmp_path, consistency_treatment=1)
    p = case.params()
    v = case.v.copy()
    v[0] = [0.0, -1.0e4]
    with Solver(p, "fp64") as s:
        s.upload(case.r, v, case.rho, case.itype)
        with pytest.raises(RrsphError) as e:
            s.run(tmp_path, 0.0)
        assert e.value.code == capi.ERR_OUTSIDE_GEOMETRY
    crash = list(tmp_path.glob("crash_dump_*.csv"))
    assert len(crash) == 1
    assert crash[0].read_text().splitlines()[0] == "x,y,itype,vx,vy,rho,p"


def test_run_3d_layers_match_the_oracle(gpu_available, tmp_path):
    """rrsph_run of a 3D case (FP32-mixed step, neighbour reuse): the data
    layer names, the 3D columns, and the last layer against the oracle run
    for the same steps (mixed-precision tolerance)."""
    from oracle import binding as O
    from sph2d_gb300 import Solver, cases, read_layer

    case = cases.dam_break_3d(dx=0.02, block=(0.3, 0.3, 0.3), density_treatment=0)
    dt = case.model["dt"]
    case.model.update({"simulation_time": 12 * dt, "save_time": 5 * dt, "use_dump": False})
    case.write_experiment(tmp_path)
    p = case.params()
    with Solver(p, "mixed") as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        t, n = s.run(tmp_path, 0.0)
    saves, _, steps, save_steps = _expected_layers(0.0, p.dt, p.simulation_time, p.save_time, p.dump_time, False)
    assert n == steps
    sd = _digits(p.save_time)
    data = sorted((tmp_path / "data").iterdir(), key=lambda f: float(f.stem))
    assert [f.name for f in data] == [f"{t:.{sd}f}.csv" for t in saves]
    assert data[-1].read_text().splitlines()[0].startswith("x,y,z,itype,vx,vy,vz")
    ref = O.run(p, case.r, case.v, case.rho, case.itype, nsteps=save_steps[-1])
    r, v, rho, pres, itype = read_layer(data[-1], p)
    # the layer prints six decimals; the mixed step adds float rounding
    assert np.array_equal(itype, ref["itype"])
    assert np.allclose(r, ref["r"], rtol=0.0, atol=1e-6)
    assert rel_l2(v, ref["v"]) < 1e-4
    assert rel_l2(rho, ref["rho"]) < 1e-6
