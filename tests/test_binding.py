"""The RRSPH_CUDA binding (sph2d_gb300/integration/), compiled against the
reference's headers by oracle/build_ref.sh where the reference sources (or
their staged copy) are present:

- fill_rrsph_params_from puts every ExperimentParams field
  (sources/RRSPH_PARAMS/include/Params.h:8-196) into the rrsph_params field of
  the same name (``ref_params --mapping``);
- on real experiment directories, the reference's own loaders
  (ParticleParams.cpp:22-149, ModelParams.cpp:110-311) followed by
  fill_rrsph_params_from give the same rrsph_params, field for field, as this
  library's rrsph_experiment_load_params (so also after rrsph_params_derive);
- the binding's time_integration compiles against the reference's headers
  (checked by the build itself).
CPU only.
"""

import subprocess
from pathlib import Path

import pytest

REF_PARAMS = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "ref_params"

pytestmark = pytest.mark.skipif(not REF_PARAMS.exists(), reason="binding check not built (reference sources absent)")


def _ref_load(directory):
    from sph2d_gb300 import capi, default_params

    res = subprocess.run([str(REF_PARAMS), str(directory)], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0, res.stderr
    p = default_params()
    types = dict(capi.RrsphParams._fields_)
    for line in res.stdout.splitlines():
        name, value = line.split()
        setattr(p, name, float(value) if types[name] is capi.f64 else int(value))
    return p


def _diff(a, b):
    from sph2d_gb300 import capi

    return [(f, getattr(a, f), getattr(b, f)) for f, _ in capi.RrsphParams._fields_ if getattr(a, f) != getattr(b, f)]


def test_mapping_field_by_field():
    res = subprocess.run([str(REF_PARAMS), "--mapping"], capture_output=True, text=True, timeout=60)
    assert res.returncode == 0 and res.stdout.strip() == "mapping ok", res.stdout + res.stderr


def _experiments():
    from sph2d_gb300 import cases

    out = [("flume", cases.piston_flume_2d(nx=200, ny=20)), ("dam_sum", cases.dam_break_2d(nx=40, ny=20)),
           ("dam_con", cases.dam_break_2d(nx=40, ny=20, density_treatment=1)),
           ("dam3d", cases.dam_break_3d(dx=0.04))]
    for name, upd in (("delta_sph", {"density_treatment": 2, "density_delta_sph_coef": 0.1}),
                      ("cfl_dt", {"dt_correction_method": 1}),
                      ("switches", {"artificial_pressure": True, "average_velocity": True,
                                    "average_velocity_coef": 0.05, "intf_sph_approximation": 1,
                                    "boundary_treatment": 0, "use_dump": True, "save_every_step": True,
                                    "consistency_check": False, "local_threads": 8}),
                      ("wendland", {"density_skf": 3, "intf_skf": 3, "artificial_viscosity_skf": 3,
                                    "average_velocity_skf": 3, "artificial_pressure_skf": 3}),
                      ("old_version", {"params_target_version_minor": 0, "params_target_version_patch": 0,
                                       "nwm_direction": 0}),
                      ("version_3_0_5", {"params_target_version_minor": 0, "params_target_version_patch": 5,
                                         "nwm_direction": 0})):
        c = cases.dam_break_2d(nx=40, ny=20)
        c.model = dict(c.model, **upd)
        out.append((name, c))
    return out


@pytest.mark.parametrize("name,case", _experiments(), ids=[n for n, _ in _experiments()])
def test_reference_loaders_and_binding_equal_the_library(tmp_path, name, case):
    from sph2d_gb300 import derive, load_params

    case.write_experiment(tmp_path)
    ref = _ref_load(tmp_path)
    mine = load_params(tmp_path)
    assert _diff(ref, mine) == []
    assert _diff(derive(ref, case.r), derive(mine, case.r)) == []


def test_reference_dam_break_experiment():
    from conftest import GOLDEN_CASE
    from sph2d_gb300 import load_params

    if not GOLDEN_CASE.is_dir():
        pytest.skip("reference sources not present on this machine")
    assert _diff(_ref_load(GOLDEN_CASE), load_params(GOLDEN_CASE)) == []
