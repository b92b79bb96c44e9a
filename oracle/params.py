"""Experiment parameters for the CPU oracle (TEST INFRASTRUCTURE).

A restatement, independent of the GPU library, of how the reference turns an
experiment's two JSON files and its first particle layer into the values the
step reads:

  ParticleParams loading   sources/RRSPH_PARAMS/src/ParticleParams.cpp:51-149
  ModelParams loading      sources/RRSPH_PARAMS/src/ModelParams.cpp:185-311,
                           defaults sources/RRSPH_PARAMS/include/ModelParams.h:11-78,
                           checks   sources/RRSPH_PARAMS/src/ModelParams.cpp:12-95,
                           apply    sources/RRSPH_PARAMS/src/ModelParams.cpp:110-173
                           (an optional without a value becomes T{} = 0)
  derived values           sources/RRSPH_COMMON/src/Input.cpp:17-138
  constants                sources/RRSPH_PARAMS/include/Params.h:176-193

The values are held in ``OracleParams``, a ctypes mirror of the C struct
``rrsph_params`` that the oracle's C code takes (declared in
include/rrsph_cuda.h, which this module reads to build the mirror). Nothing
here loads or imports the GPU library, so the benchmark's reference arm and
the fixture generators derive their parameters without it; the tests check
that this derivation gives the GPU library's values field for field.
"""

from __future__ import annotations

import ctypes as C
import math
import re
from pathlib import Path

import numpy as np

HEADER = Path(__file__).resolve().parent.parent / "include" / "rrsph_cuda.h"

_CTYPES = {"uint32_t": C.c_uint32, "uint64_t": C.c_uint64, "int32_t": C.c_int32, "double": C.c_double}


def _struct_fields(header: Path = HEADER):
    """Field list of ``typedef struct rrsph_params {...}`` in declaration order."""
    text = header.read_text()
    m = re.search(r"typedef struct rrsph_params \{(.*?)\} rrsph_params;", text, re.S)
    if not m:
        raise RuntimeError(f"rrsph_params not found in {header}")
    body = re.sub(r"/\*.*?\*/", "", m.group(1), flags=re.S)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        typ, _, names = decl.partition(" ")
        if typ not in _CTYPES:
            raise RuntimeError(f"rrsph_params: unexpected declaration {decl!r}")
        for name in names.split(","):
            fields.append((name.strip(), _CTYPES[typ]))
    return fields


class OracleParams(C.Structure):
    """ctypes mirror of ``rrsph_params`` (built from include/rrsph_cuda.h)."""

    _fields_ = _struct_fields()

    def copy(self) -> "OracleParams":
        q = OracleParams()
        C.memmove(C.addressof(q), C.addressof(self), C.sizeof(self))
        return q

    def as_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}


class ParamsError(RuntimeError):
    pass


def defaults() -> OracleParams:
    """ExperimentParams before loading (Params.h:8-196) with the ModelParams
    member initialisers (ModelParams.h:14-77) and the ParticleParams defaults
    (ParticleParams.h:13-28)."""
    p = OracleParams()
    p.struct_size = C.sizeof(OracleParams)
    p.dim = 2
    p.rho0 = 1000.0
    p.density_treatment = 1          # DENSITY_CONTINUITY
    p.density_skf = 1                # SKF_CUBIC
    p.intf_hsml_coef = 1.0
    p.intf_sph_approximation = 2
    p.intf_skf = 1
    p.artificial_pressure = 0
    p.artificial_pressure_skf = 1
    p.artificial_pressure_index = 4.0
    p.artificial_pressure_coef = 0.2
    p.artificial_viscosity = 0
    p.artificial_viscosity_skf = 1
    p.average_velocity = 0
    p.average_velocity_skf = 1
    p.use_crash_dump = 1
    p.consistency_check = 1
    p.consistency_treatment = 1      # CONSISTENCY_STOP
    p.nwm = 0
    p.dt_correction_method = 2       # DT_CORRECTION_DYNAMIC
    p.max_neighbours = 64
    p.save_velocity = 1
    p.save_pressure = 1
    p.save_density = 1
    p.cell_scale_k = 2.0             # the value countCells sees (Params.h)
    p.pi = 3.14159265358979323846
    p.g = 9.81
    p.type_boundary = -2
    p.type_non_existent = 0
    p.type_water = 2
    return p


def _version_before_3_1_4(js: dict) -> bool:
    """target < (3, 1, 4) by the reference's ParamsVersion::operator<
    (RRSPH_PARAMS/src/Version.h:17-21), which compares each component on its
    own: major <= 3 and minor <= 1 and patch < 4 (so 3.0.5 is not older)."""
    major, minor, patch = (int(js.get(f"params_target_version_{k}", 0)) for k in ("major", "minor", "patch"))
    return major <= 3 and minor <= 1 and patch < 4


def load(model: dict, particle: dict) -> OracleParams:
    """The two JSON objects of an experiment, loaded and checked as
    load_particle_params + load_model_params + apply_*_params do."""
    p = defaults()
    # ---- ParticleParams (ParticleParams.cpp:84-146)

    def mandatory(js, k):
        if k not in js:
            raise ParamsError(f"Mandatory param not specified: {k}")
        return js[k]

    p.dim = int(particle.get("dim", 2))
    for k in ("x_mingeom", "x_maxgeom", "y_mingeom", "y_maxgeom"):
        setattr(p, k, float(mandatory(particle, k)))
    if p.dim == 3:
        p.z_mingeom = float(mandatory(particle, "z_mingeom"))
        p.z_maxgeom = float(mandatory(particle, "z_maxgeom"))
    else:
        p.z_mingeom = p.z_maxgeom = 0.0
    p.delta = float(mandatory(particle, "delta"))
    for k in ("ntotal", "nfluid", "nvirt"):
        setattr(p, k, int(mandatory(particle, k)))
    p.rho0 = float(particle.get("rho0", 1000.0))
    p.nwm_particles_start = int(particle.get("nwm_particles_start", p.ntotal))
    p.nwm_particles_end = int(particle.get("nwm_particles_end", p.ntotal))
    p.depth = float(particle.get("depth", 0.0))   # optional; apply gives 0 when absent
    if p.dim not in (2, 3):
        raise ParamsError(f"invalid params.dim value: {p.dim}")

    # ---- ModelParams (ModelParams.cpp:185-311)
    js = dict(model)
    if _version_before_3_1_4(js):                 # backward_compatibility_model_params (:162-167)
        js["nwm_direction"] = 1
    u = lambda k, d: int(js[k]) if k in js else d          # noqa: E731
    f = lambda k, d: float(js[k]) if k in js else d        # noqa: E731
    p.density_treatment = u("density_treatment", p.density_treatment)
    density_normalization = u("density_normalization", 0)
    p.density_skf = u("density_skf", p.density_skf)
    p.density_delta_sph_coef = f("density_delta_sph_coef", 0.0)
    p.eos_sound_vel_method = int(mandatory(js, "eos_sound_vel_method"))
    p.eos_sound_vel = f("eos_sound_vel", 0.0)
    p.eos_sound_vel_coef = f("eos_sound_vel_coef", 0.0)
    p.intf_hsml_coef = f("intf_hsml_coef", p.intf_hsml_coef)
    p.intf_sph_approximation = u("intf_sph_approximation", p.intf_sph_approximation)
    p.intf_skf = u("intf_skf", p.intf_skf)
    p.artificial_pressure = u("artificial_pressure", 0)
    p.artificial_pressure_skf = u("artificial_pressure_skf", p.artificial_pressure_skf)
    p.artificial_pressure_index = f("artificial_pressure_index", p.artificial_pressure_index)
    p.artificial_pressure_coef = f("artificial_pressure_coef", p.artificial_pressure_coef)
    visc = u("visc", 1)
    p.artificial_viscosity = u("artificial_viscosity", 0)
    p.artificial_shear_visc = f("artificial_shear_visc", 0.0)
    p.artificial_bulk_visc = f("artificial_bulk_visc", 0.0)
    p.artificial_viscosity_skf = u("artificial_viscosity_skf", p.artificial_viscosity_skf)
    p.average_velocity = u("average_velocity", 0)
    p.average_velocity_coef = f("average_velocity_coef", 0.0)
    p.average_velocity_skf = u("average_velocity_skf", p.average_velocity_skf)
    p.save_every_step = u("save_every_step", 0)
    p.save_time = float(mandatory(js, "save_time"))
    p.dump_time = f("dump_time", 0.0)
    p.use_dump = u("use_dump", 0)
    p.use_crash_dump = u("use_crash_dump", p.use_crash_dump)
    p.consistency_check = u("consistency_check", p.consistency_check)
    p.consistency_treatment = u("consistency_treatment", p.consistency_treatment)
    p.boundary_treatment = int(mandatory(js, "boundary_treatment"))
    p.nwm = u("nwm", 0)
    p.nwm_time_start = f("nwm_time_start", 0.0)
    p.nwm_wave_length = f("nwm_wave_length", 0.0)
    p.nwm_wave_magnitude = f("nwm_wave_magnitude", 0.0)
    p.nwm_direction = u("nwm_direction", 0)
    p.nwm_phase = f("nwm_phase", 0.0)
    p.simulation_time = float(mandatory(js, "simulation_time"))
    p.dt_correction_method = u("dt_correction_method", p.dt_correction_method)
    p.dt = f("dt", 0.0)
    p.CFL_coef = f("CFL_coef", 0.0)
    p.max_neighbours = u("max_neighbours", p.max_neighbours)
    p.local_threads = u("local_threads", 0)
    p.save_velocity = u("save_velocity", 1)
    p.save_pressure = u("save_pressure", 1)
    p.save_density = u("save_density", 1)
    p.dt_dynamic_reduce = u("dt_dynamic_reduce", 0)   # this library's switch, no reference counterpart

    # check_optional_params (ModelParams.cpp:12-95)
    if visc:
        raise ParamsError("Not implemented: visc")
    if density_normalization:
        raise ParamsError("Not implemented: density_normalization")
    need = []
    if p.eos_sound_vel_method == 1:
        need.append("eos_sound_vel")
    elif p.eos_sound_vel_method == 0:
        need.append("eos_sound_vel_coef")
    else:
        raise ParamsError("Invalid enum value: eos_sound_vel_method")
    if p.density_treatment == 2:
        need.append("density_delta_sph_coef")
    if p.artificial_viscosity:
        need += ["artificial_shear_visc", "artificial_bulk_visc"]
    if p.average_velocity:
        need.append("average_velocity_coef")
    if p.use_dump:
        need.append("dump_time")
    if p.nwm in (2, 3):
        need += ["nwm_wave_length", "nwm_wave_magnitude", "nwm_direction"]
    elif p.nwm == 5:
        need.append("nwm_wave_magnitude")
    elif p.nwm not in (0, 4):
        raise ParamsError("Invalid enum value: nwm")
    if p.dt_correction_method == 0:
        need.append("dt")
    elif p.dt_correction_method in (1, 2):
        need.append("CFL_coef")
    else:
        raise ParamsError("Invalid enum value: dt_correction_method")
    for k in need:
        if k not in js:
            raise ParamsError(f"Need optional param: {k}")
    return p


def _intlog2(v: int) -> int:
    """intlog2 (RRSPH_COMMON/include/CommonIncl.h): the number of halvings to 1."""
    n = 0
    while v > 1:
        v >>= 1
        n += 1
    return n


def _split2(x: int) -> int:
    """Spreads the bits of x to the even positions (the 2D Morton encode of
    GridUtils.h:92-104)."""
    out = 0
    for b in range(16):
        out |= ((x >> b) & 1) << (2 * b)
    return out


def _split3(x: int) -> int:
    """Spreads the low 10 bits of x to every third position (GridUtils.h:50-64)."""
    out = 0
    for b in range(10):
        out |= ((x >> b) & 1) << (3 * b)
    return out


def _cell_coord(r: float, rmin: float, cell: float) -> int:
    """get_cell_coord_from_particle_coord (GridUtils.h:135-140): truncation of
    (r - rmin) / cell to an unsigned coordinate."""
    c = (r - rmin) / cell
    return int(c) if c > 0 else 0


_CELL_SCALE = {1: 2.0, 2: 3.0, 3: 2.0, 4: 2.0}   # get_cell_scale_k (Input.cpp:17-26)


def derive(p: OracleParams, r: np.ndarray | None) -> OracleParams:
    """fillInComputingParams + find_depth + postFillInModelParams
    (Input.cpp:77-138) on a copy of p; r holds the loaded positions."""
    q = p.copy()
    if q.dim not in (2, 3):
        raise ParamsError(f"invalid params.dim value: {q.dim}")
    # fillInComputingParams (Input.cpp:93-110)
    q.hsml = q.delta * q.intf_hsml_coef
    q.maxn = 1 << (1 + _intlog2(q.ntotal))
    # countCells (Input.cpp:45-75) runs while cell_scale_k still holds its
    # earlier value (2 unless set before)
    cell = q.cell_scale_k * q.hsml
    x_id = _cell_coord(q.x_maxgeom, q.x_mingeom, cell)
    y_id = _cell_coord(q.y_maxgeom, q.y_mingeom, cell)
    if q.dim == 3:
        z_id = _cell_coord(q.z_maxgeom, q.z_mingeom, cell)
        max_id = 1 << 10
        cid = _split3(x_id) | (_split3(y_id) << 1) | (_split3(z_id) << 2)
    else:
        z_id = 0
        max_id = 1 << 16
        cid = _split2(x_id) | (_split2(y_id) << 1)
    if x_id > max_id or y_id > max_id or z_id >= max_id:
        raise ParamsError(f"can't make grid with so many cells: ({x_id}/{max_id}; {y_id}/{max_id}; {z_id}/{max_id})")
    q.max_cells = 1 << (_intlog2(cid) + 1)
    m = 1.0
    for _ in range(q.dim):       # powun(delta, dim)
        m *= q.delta
    q.mass = q.rho0 * m
    ks = set()
    for skf in (q.artificial_pressure_skf, q.artificial_viscosity_skf, q.average_velocity_skf, q.intf_skf,
                q.density_skf):
        if skf not in _CELL_SCALE:
            raise ParamsError(f"get_cell_scale_k: unknown skf {skf}")
        ks.add(_CELL_SCALE[skf])
    if len(ks) != 1:
        raise ParamsError("selected incompatible skf")
    q.cell_scale_k = ks.pop()
    # find_depth (Input.cpp:77-91), only when no depth was given
    if q.depth == 0:
        if q.nfluid > 0 and r is None:
            raise ParamsError("positions needed to find the depth")
        ymin = float(np.finfo(np.float32).max)
        ymax = -ymin
        if q.nfluid > 0:
            ys = np.asarray(r, dtype=np.float64)[: q.nfluid, 1]
            ymax = max(float(ys.max()), ymax)
            ymin = min(float(ys.min()), ymin)
        q.depth = ymax - ymin
    # postFillInModelParams (Input.cpp:112-138)
    if q.eos_sound_vel_method == 0:
        q.eos_sound_vel = math.sqrt(200 * q.g * q.depth * q.eos_sound_vel_coef)
    if q.dt_correction_method == 1:
        q.dt = q.CFL_coef * q.hsml / (q.eos_sound_vel * (1 + 1.2 * q.artificial_shear_visc))
    if q.nwm in (2, 3):
        q.nwm_wave_number = 2.0 * q.pi / q.nwm_wave_length
        kd = q.nwm_wave_number * q.depth
        q.nwm_freq = math.sqrt(q.nwm_wave_number * q.g * math.tanh(kd))
        s = math.sinh(kd)
        q.nwm_piston_magnitude = q.nwm_wave_magnitude * 0.5 / (s * s) * (s * math.cosh(kd) + kd)
    if q.max_neighbours < 2:
        raise ParamsError("max_neighbours must be >= 2")
    return q


def case_params(case) -> OracleParams:
    """Parameters of a generated case (an object with ``model``, ``particle``
    and ``r``), derived here rather than by the GPU library."""
    return derive(load(case.model, case.particle), case.r)


def load_experiment(directory) -> OracleParams:
    """ModelParams.json + ParticleParams.json of an experiment directory (not derived)."""
    import json

    d = Path(directory)
    for name in ("ParticleParams.json", "ModelParams.json"):
        if not (d / name).exists():
            raise ParamsError(f"No params file provided: '{d / name}' expected")
    return load(json.loads((d / "ModelParams.json").read_text()), json.loads((d / "ParticleParams.json").read_text()))
