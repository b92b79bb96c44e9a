"""Host side of the C ABI (no GPU): library loading and exports, the params
struct layout, experiment JSON loading with the reference's checks, the
derivations of fileInput(), and the CSV layer format."""

import ctypes as C
import json
import math

import numpy as np
import pytest


def test_library_exports_every_declared_symbol():
    from sph2d_gb300 import capi

    L = capi.lib()
    names = capi.declared_symbols()
    assert len(names) >= 25
    for name in names:
        assert hasattr(L, name), name
    assert L.rrsph_abi_version() == 1


def test_params_layout_matches_c():
    from sph2d_gb300 import capi

    L = capi.lib()
    assert L.rrsph_params_sizeof() == C.sizeof(capi.RrsphParams)
    for name, _ in capi.RrsphParams._fields_:
        off = C.c_size_t()
        assert L.rrsph_params_offsetof(name.encode(), C.byref(off)) == 0, name
        assert off.value == getattr(capi.RrsphParams, name).offset, name
    off = C.c_size_t()
    assert L.rrsph_params_offsetof(b"no_such_field", C.byref(off)) == capi.ERR_INVALID_ARGUMENT


def test_create_without_gpu_fails_loudly(monkeypatch):
    """Without a CUDA device the solver refuses to start (no CPU fallback)."""
    import torch

    from sph2d_gb300 import RrsphError, Solver, cases

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    case = cases.dam_break_2d(nx=10, ny=10)
    with pytest.raises(RrsphError) as e:
        Solver(case.params())
    assert e.value.code == 12


def _model(**kw):
    m = {"eos_sound_vel_method": 0, "eos_sound_vel_coef": 1.0, "save_time": 0.1, "boundary_treatment": 1,
         "simulation_time": 1.0, "visc": False, "dt_correction_method": 0, "dt": 1e-4}
    m.update(kw)
    return m


def _particle(**kw):
    p = {"x_mingeom": -1, "x_maxgeom": 2, "y_mingeom": -1, "y_maxgeom": 2, "delta": 0.01, "ntotal": 10,
         "nfluid": 8, "nvirt": 2}
    p.update(kw)
    return p


def test_json_defaults_and_mandatory_keys():
    from sph2d_gb300 import RrsphError, params_from_json

    p = params_from_json(_model(), _particle())
    # ModelParams member defaults (ModelParams.h) and ParticleParams defaults
    assert p.density_treatment == 1 and p.intf_sph_approximation == 2 and p.intf_skf == 1
    assert p.max_neighbours == 64 and p.consistency_treatment == 1 and p.rho0 == 1000
    assert p.nwm_particles_start == 10 and p.nwm_particles_end == 10 and p.dim == 2
    assert p.nwm_direction == 1  # backward compatibility for target versions < 3.1.4
    for key in ("eos_sound_vel_method", "save_time", "boundary_treatment", "simulation_time"):
        m = _model()
        del m[key]
        with pytest.raises(RrsphError, match=f"Mandatory param not specified: {key}"):
            params_from_json(m, _particle())
    for key in ("x_mingeom", "delta", "ntotal", "nvirt"):
        q = _particle()
        del q[key]
        with pytest.raises(RrsphError, match=f"Mandatory param not specified: {key}"):
            params_from_json(_model(), q)


def test_json_reference_checks():
    from sph2d_gb300 import RrsphError, params_from_json

    with pytest.raises(RrsphError, match="Not implemented: visc"):
        params_from_json(_model(visc=True), _particle())
    m = _model()
    del m["visc"]  # the ModelParams default is visc = true
    with pytest.raises(RrsphError, match="Not implemented: visc"):
        params_from_json(m, _particle())
    with pytest.raises(RrsphError, match="Need optional param: eos_sound_vel_coef"):
        params_from_json({k: v for k, v in _model().items() if k != "eos_sound_vel_coef"}, _particle())
    with pytest.raises(RrsphError, match="Need optional param: artificial_shear_visc"):
        params_from_json(_model(artificial_viscosity=True), _particle())
    with pytest.raises(RrsphError, match="Need optional param: dt"):
        params_from_json({k: v for k, v in _model().items() if k != "dt"}, _particle())
    with pytest.raises(RrsphError, match="Need optional param: nwm_wave_length"):
        params_from_json(_model(nwm=2), _particle())
    with pytest.raises(RrsphError, match="Invalid enum value: nwm"):
        params_from_json(_model(nwm=7), _particle())


def test_derivations_match_input_cpp():
    """fillInComputingParams/postFillInModelParams (Input.cpp:93-138)."""
    from sph2d_gb300 import derive, params_from_json

    p = params_from_json(_model(intf_hsml_coef=1.4, nwm=2, nwm_wave_length=3.0, nwm_wave_magnitude=0.02,
                                nwm_direction=1, dt_correction_method=1, CFL_coef=0.2, artificial_viscosity=True,
                                artificial_shear_visc=0.3, artificial_bulk_visc=0.0),
                         _particle(x_maxgeom=20.5, y_maxgeom=1.3, x_mingeom=-0.5, y_mingeom=-0.1, ntotal=1000,
                                   nfluid=900, nvirt=100, delta=0.005))
    r = np.zeros((1000, 2))
    r[:900, 1] = np.linspace(0.1, 0.6, 900)
    d = derive(p, r)
    h = 0.005 * 1.4
    assert d.hsml == pytest.approx(h)
    assert d.maxn == 1024
    assert d.mass == pytest.approx(1000 * 0.005 ** 2)
    assert d.cell_scale_k == 2.0
    assert d.depth == pytest.approx(0.5)  # find_depth over the fluid rows
    c = math.sqrt(200 * 9.81 * 0.5 * 1.0)
    assert d.eos_sound_vel == pytest.approx(c)
    assert d.dt == pytest.approx(0.2 * h / (c * (1 + 1.2 * 0.3)))
    k = 2 * math.pi / 3.0
    assert d.nwm_wave_number == pytest.approx(k)
    assert d.nwm_freq == pytest.approx(math.sqrt(k * 9.81 * math.tanh(k * 0.5)))
    # max_cells: next power of two above the Morton code of the far corner cell
    cx = int((20.5 + 0.5) / (2 * h))
    cy = int((1.3 + 0.1) / (2 * h))

    def split(x):
        out = 0
        for b in range(16):
            out |= ((x >> b) & 1) << (2 * b)
        return out

    mid = split(cx) | (split(cy) << 1)
    assert d.max_cells == 1 << (mid.bit_length())


def test_layer_round_trip_and_format(tmp_path):
    from sph2d_gb300 import cases, read_layer, write_layer

    case = cases.dam_break_2d(nx=8, ny=5)
    p = case.params()
    rho = case.rho
    pres = np.linspace(-5, 5, case.ntotal)
    path = tmp_path / "0.25.csv"
    write_layer(path, p, case.r, case.v, rho, pres, case.itype, dump=True)
    lines = path.read_text().splitlines()
    assert lines[0] == "x,y,itype,vx,vy,rho,p"
    # std::to_string formatting: %f with 6 decimals
    first = lines[1].split(",")
    assert first[0] == "%f" % case.r[0, 0] and first[2] == str(case.itype[0]) and first[5] == "%f" % rho[0]
    r2, v2, rho2, p2, it2 = read_layer(path, p)
    assert np.allclose(r2, case.r, atol=5e-7) and np.array_equal(it2, case.itype)
    assert np.allclose(rho2, rho, atol=5e-7) and np.allclose(p2, pres, atol=5e-7)
    # a data layer without velocity/pressure when the save switches are off
    q = p.copy()
    q.save_velocity = 0
    q.save_pressure = 0
    write_layer(tmp_path / "1.csv", q, case.r, case.v, rho, pres, case.itype, dump=False)
    assert (tmp_path / "1.csv").read_text().splitlines()[0] == "x,y,itype,rho"


def test_layer_row_count_mismatch_is_an_error(tmp_path):
    from sph2d_gb300 import RrsphError, cases, read_layer, write_layer

    case = cases.dam_break_2d(nx=8, ny=5)
    p = case.params()
    write_layer(tmp_path / "0.csv", p, case.r, case.v, case.rho, np.zeros(case.ntotal), case.itype)
    q = p.copy()
    q.ntotal = p.ntotal + 1
    with pytest.raises(RrsphError, match="dump corrupted"):
        read_layer(tmp_path / "0.csv", q)


def test_experiment_directory_round_trip(tmp_path):
    from sph2d_gb300 import cases, derive, load_params, read_layer

    case = cases.piston_flume_2d(nx=50, ny=10)
    case.write_experiment(tmp_path)
    p0 = load_params(tmp_path)
    r, v, rho, pres, itype = read_layer(tmp_path / "dump" / "0.csv", p0)
    p = derive(p0, r)
    q = case.params()
    for name in ("hsml", "mass", "max_cells", "dt", "nwm_freq", "nwm_wave_number", "eos_sound_vel"):
        assert getattr(p, name) == pytest.approx(getattr(q, name), rel=1e-12), name
    assert json.loads((tmp_path / "ModelParams.json").read_text())["nwm"] == 2


def test_layer_numbers_format_like_printf(tmp_path):
    """Layer values must print exactly as std::to_string (printf "%f")."""
    from sph2d_gb300 import cases, write_layer

    case = cases.dam_break_2d(nx=60, ny=60)
    p = case.params()
    n = case.ntotal
    rng = np.random.default_rng(3)
    specials = np.array([0.0078125, -0.0078125, 2.5e-7, 0.5e-6, 123456789.123456789, -1e-9, 1e15 + 0.5, 0.1, 0.3,
                         -0.0, 0.0, 0.9999995, 0.99999949999, 8.999999999999e12, 9.0e12, -9.0e12, 1e300, -1e-310,
                         5e-324, 2.0 ** -74, 4.5e15, np.inf, -np.inf])
    m = n - len(specials)
    # ties in millionths: odd multiples of 2^-7; random bit patterns over the exponents of
    # |v| in [2^-40, 2^50); plain normals over ten decades
    ties = (2 * rng.integers(0, 2**40, m // 3) + 1) / 128.0 * rng.choice([-1, 1], m // 3)
    bits = (rng.integers(0, 2**52, m // 3, dtype=np.int64) | (rng.integers(1023 - 40, 1023 + 50, m // 3) << 52))
    pats = bits.view(np.float64) * rng.choice([-1, 1], m // 3)
    rest = rng.normal(0, 10, m - 2 * (m // 3)) * 10.0 ** rng.integers(-8, 8, m - 2 * (m // 3))
    vals = np.concatenate([specials, ties, pats, rest])
    r = np.stack([vals, -vals[::-1]], axis=1)
    write_layer(tmp_path / "x.csv", p, r, r, vals, vals, case.itype, dump=True)
    lines = (tmp_path / "x.csv").read_text().splitlines()[1:]
    for i, line in enumerate(lines):
        f = line.split(",")
        assert f[0] == "%f" % r[i, 0] and f[1] == "%f" % r[i, 1], (i, f[:2], r[i])
        assert f[5] == "%f" % vals[i]


def test_empty_particle_set_is_an_error():
    """No particles: the derivations refuse the counts (the solver would have
    nothing to step), and so do counts with more fluid than particles."""
    from sph2d_gb300 import RrsphError, derive, params_from_json

    p = params_from_json(_model(), _particle(ntotal=0, nfluid=0, nvirt=0))
    with pytest.raises(RrsphError, match="bad particle counts"):
        derive(p, np.zeros((0, 2)))
    q = params_from_json(_model(), _particle(ntotal=10, nfluid=11, nvirt=0))
    with pytest.raises(RrsphError, match="bad particle counts"):
        derive(q, np.zeros((10, 2)))


def test_readme_c_usage_compiles(tmp_path):
    """The C usage in README.md compiles against include/rrsph_cuda.h."""
    import re
    import shutil
    import subprocess
    from pathlib import Path

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    root = Path(__file__).resolve().parent.parent
    block = re.search(r"```c\n(.*?)```", (root / "README.md").read_text(), re.S)
    assert block, "no C block in README.md"
    src = tmp_path / "usage.c"
    src.write_text(
        '#include <stdint.h>\n#include "rrsph_cuda.h"\n'
        "int main(void) {\n"
        "    static double r[2], v[2], rho[1], pres[1];\n"
        "    static int32_t itype[1];\n"
        + block.group(1)
        + "    return 0;\n}\n"
    )
    res = subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-c", str(src), "-I", str(root / "include"),
                          "-o", str(tmp_path / "usage.o")], capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
