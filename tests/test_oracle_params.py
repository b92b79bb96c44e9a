"""The oracle's own parameter loading and derivation (oracle/params.py) against
the GPU library's (rrsph_experiment_load_params + rrsph_params_derive), and the
benchmark's reference arm, which uses the former and must not load the GPU
library. CPU only."""

import ctypes as C
import json
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _same(a, b):
    from sph2d_gb300 import capi

    return [(f, getattr(a, f), getattr(b, f)) for f, _ in capi.RrsphParams._fields_ if getattr(a, f) != getattr(b, f)]


def test_struct_mirrors_agree():
    from oracle.params import OracleParams
    from sph2d_gb300 import capi

    assert [f for f, _ in OracleParams._fields_] == [f for f, _ in capi.RrsphParams._fields_]
    assert [t for _, t in OracleParams._fields_] == [t for _, t in capi.RrsphParams._fields_]
    assert C.sizeof(OracleParams) == C.sizeof(capi.RrsphParams) == capi.lib().rrsph_params_sizeof()


def _variants():
    from sph2d_gb300 import cases

    out = [("flume", cases.piston_flume_2d(nx=400, ny=40)), ("dam", cases.dam_break_2d()),
           ("dam3d", cases.dam_break_3d(dx=0.02)), ("adjoint", cases.adjoint_flume_2d(nx=200, ny=20))]
    base = cases.dam_break_2d(nx=40, ny=20)
    for name, upd in (("cfl_dt", {"dt_correction_method": 1}),
                      ("dynamic_dt", {"dt_correction_method": 2}),
                      ("piston_2nd", {"nwm": 3, "nwm_wave_length": 3.0, "nwm_wave_magnitude": 0.04,
                                      "nwm_direction": 1}),
                      ("solitary", {"nwm": 5, "nwm_wave_magnitude": 0.05}),
                      ("wall", {"nwm": 4, "nwm_time_start": 0.1}),
                      ("specific_c", {"eos_sound_vel_method": 1, "eos_sound_vel": 900.0}),
                      ("gauss", {"density_skf": 2, "intf_skf": 2, "artificial_viscosity_skf": 2,
                                 "average_velocity_skf": 2, "artificial_pressure_skf": 2}),
                      ("old_version", {"params_target_version_minor": 0, "params_target_version_patch": 0}),
                      ("version_3_0_5", {"params_target_version_minor": 0, "params_target_version_patch": 5}),
                      ("no_version", {"params_target_version_major": 0, "params_target_version_minor": 0,
                                      "params_target_version_patch": 0, "nwm_direction": 0})):
        c = cases.dam_break_2d(nx=40, ny=20)
        c.model = dict(base.model, **upd)
        out.append((name, c))
    c = cases.dam_break_2d(nx=40, ny=20)
    c.particle = dict(c.particle)
    c.particle.pop("depth", None)  # found from the fluid rows
    out.append(("find_depth", c))
    return out


@pytest.mark.parametrize("name,case", _variants(), ids=[n for n, _ in _variants()])
def test_oracle_derivation_equals_library(name, case):
    from oracle import params as OP

    lib_p = case.params()
    orc_p = OP.case_params(case)
    assert _same(lib_p, orc_p) == []


def test_reference_case_loading_and_eos_sound_velocity():
    """The reference's own dam-break experiment: both loaders agree field for
    field, and the derivation reproduces the speed of sound that the
    reference's fileInput wrote back into that ModelParams.json
    (postFillInModelParams, Input.cpp:112-116). The build that wrote the file
    held g as the float 9.81f (its other values are float-rounded too, e.g.
    CFL_coef 0.20000000298023224): with that g the derivation gives the file's
    value bit for bit; with the double 9.81 of this step, sqrt(7848)."""
    from conftest import GOLDEN_CASE

    if not GOLDEN_CASE.is_dir():
        pytest.skip("reference sources not present on this machine")
    from oracle import params as OP
    from sph2d_gb300 import derive, load_params

    a = load_params(GOLDEN_CASE)
    b = OP.load_experiment(GOLDEN_CASE)
    assert _same(a, b) == []
    model = json.loads((GOLDEN_CASE / "ModelParams.json").read_text())
    d = OP.derive(b, None)
    assert d.eos_sound_vel == np.sqrt(200 * 9.81 * 2.0 * 2.0)
    for q in (b.copy(), a.copy()):
        q.g = float(np.float32(9.81))
        dq = OP.derive(q, None) if isinstance(q, OP.OracleParams) else derive(q, None)
        assert dq.eos_sound_vel == model["eos_sound_vel"]
    assert d.hsml == b.delta * b.intf_hsml_coef and d.maxn == 32768 and d.mass == 1000.0 * (b.delta * b.delta)


def test_version_comparison_is_the_references():
    """ModelParams.json older than 3.1.4 gets nwm_direction = 1
    (backward_compatibility_model_params, ModelParams.cpp:162-167), with the
    reference's component-wise comparison (Version.h:17-21)."""
    from oracle import params as OP
    from sph2d_gb300 import cases, params_from_json

    c = cases.dam_break_2d(nx=10, ny=5)
    for ver, old in (((3, 1, 4), False), ((0, 0, 0), True), ((3, 1, 3), True), ((3, 0, 5), False),
                     ((2, 5, 0), False), ((3, 0, 0), True)):
        m = dict(c.model, nwm_direction=0, params_target_version_major=ver[0], params_target_version_minor=ver[1],
                 params_target_version_patch=ver[2])
        assert OP.load(m, c.particle).nwm_direction == (1 if old else 0), ver
        assert params_from_json(m, c.particle).nwm_direction == (1 if old else 0), ver


def test_loading_errors_match_the_reference_messages():
    from oracle import params as OP
    from sph2d_gb300 import cases

    c = cases.dam_break_2d(nx=10, ny=5)
    bad = dict(c.model)
    bad.pop("save_time")
    with pytest.raises(OP.ParamsError, match="Mandatory param not specified: save_time"):
        OP.load(bad, c.particle)
    bad = dict(c.model, visc=True)
    with pytest.raises(OP.ParamsError, match="Not implemented: visc"):
        OP.load(bad, c.particle)
    bad = dict(c.model, nwm=2)
    with pytest.raises(OP.ParamsError, match="Need optional param: nwm_wave_length"):
        OP.load(bad, c.particle)


def test_reference_arm_does_not_load_the_gpu_library():
    """bench.py --impl reference on a bounded sample: its JSON line, and a
    process in which neither the sph2d_gb300 package nor librrsph_cuda.so was
    loaded."""
    code = (
        "import sys, runpy, json\n"
        "sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', '--warmup', '0']\n"
        "runpy.run_path('bench.py', run_name='__main__')\n"
        "maps = open('/proc/self/maps').read()\n"
        "print(json.dumps({'pkg': any(m == 'sph2d_gb300' or m.startswith('sph2d_gb300.') for m in sys.modules),\n"
        "                  'lib': 'librrsph_cuda' in maps}))\n"
    )
    res = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    line, probe = json.loads(lines[0]), json.loads(lines[-1])
    assert probe == {"pkg": False, "lib": False}
    assert line["impl"] == "reference" and line["steps"] == 1 and line["value"] > 0
    assert line["config"]["pairs_first_step"] > 7_900_000
    assert line["cpu_baseline"]["kind"] in ("reference", "port")
    assert np.isfinite(line["ms_per_step"])
