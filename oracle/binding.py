"""Python access to the CPU oracle (TEST INFRASTRUCTURE).

Two checkers live here:

- the C restatement of RRSPH_OMP's step in ``oracle/rrsph_oracle.c``
  (``oracle/liboracle.so``), usable wherever gcc is;
- the reference's own OMP compute core compiled from its sources by
  ``oracle/build_ref.sh`` (``oracle/_ref/rrsph_ref``), driven through files,
  available only where the reference sources were present at build time.

Only the tests, the smoke check and the benchmark's CPU-baseline leg use this
module; the GPU library never does.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

from .params import OracleParams

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_BIN = HERE / "_ref" / "rrsph_ref"

_lib = None
_dp = C.POINTER(C.c_double)
_u32p = C.POINTER(C.c_uint32)
_i32p = C.POINTER(C.c_int32)
_u64p = C.POINTER(C.c_uint64)
_pp = C.c_void_p


def _P(p) -> C.c_void_p:
    """Address of a params struct: an OracleParams or the GPU library's own
    ctypes mirror of the same C struct (the sizes are checked)."""
    if C.sizeof(p) != C.sizeof(OracleParams):
        raise TypeError(f"params struct of {C.sizeof(p)} bytes, expected {C.sizeof(OracleParams)}")
    return C.c_void_p(C.addressof(p))


def _d(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _u(a):
    return None if a is None else a.ctypes.data_as(_u32p)


def _i(a):
    return None if a is None else a.ctypes.data_as(_i32p)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} missing: run __graft_entry__.build()")
        L = C.CDLL(str(LIB_PATH))
        sigs = {
            "orc_kernel_factor": (C.c_double, [_pp, C.c_uint32]),
            "orc_kernel_w": (C.c_double, [_pp, C.c_double, C.c_uint32]),
            "orc_kernel_dwdr": (None, [_pp, C.c_double, _dp, C.c_uint32, _dp]),
            "orc_eos_c_sqr": (C.c_double, [_pp]),
            "orc_eos_c": (C.c_double, [_pp]),
            "orc_eos_p": (C.c_double, [_pp, C.c_double]),
            "orc_eos_rho": (C.c_double, [_pp, C.c_double]),
            "orc_morton2": (C.c_uint32, [C.c_uint32, C.c_uint32]),
            "orc_morton3": (C.c_uint32, [C.c_uint32, C.c_uint32, C.c_uint32]),
            "orc_morton2_decode": (None, [C.c_uint32, _u32p, _u32p]),
            "orc_morton3_decode": (None, [C.c_uint32, _u32p, _u32p, _u32p]),
            "orc_cell_idx": (C.c_uint32, [_pp, _dp]),
            "orc_neighbouring_cells": (None, [_pp, C.c_uint32, _u32p]),
            "orc_cell_keys": (C.c_int, [_pp, _dp, C.c_uint32, _u32p]),
            "orc_make_grid": (C.c_int, [_pp, _u32p, _u32p, _u32p]),
            "orc_find_neighbours": (C.c_int, [_pp, _dp, C.c_uint32, _i32p, _u32p, _u32p, _u32p, _u32p, C.c_uint32]),
            "orc_density_sum": (None, [_pp, _dp, C.c_uint32, _u32p, _u32p, C.c_uint32, _dp, _dp]),
            "orc_density_con": (None, [_pp, _dp, _dp, C.c_uint32, _dp, _u32p, _u32p, C.c_uint32, _dp, _dp]),
            "orc_forces": (None, [_pp, C.c_uint32, _i32p, _dp, _dp, C.c_uint32, _dp, _dp, _u32p, _u32p, C.c_uint32,
                                  _dp, _dp, _dp]),
            "orc_make_waves": (None, [_pp, _dp, _dp, C.c_uint32, _i32p, C.c_double]),
            "orc_run": (C.c_int, [_pp, _dp, _dp, C.c_uint32, _dp, _dp, _i32p, _dp, _dp, C.c_uint64, C.c_uint64, _dp,
                                  _u64p]),
            "orc_gauge": (C.c_double, [_pp, _dp, C.c_uint32, _i32p, C.c_double, C.c_double, C.c_int32]),
            "orc_piston_tangent_run": (C.c_int, [_pp, _dp, _dp, C.c_uint32, _dp, _dp, _i32p, _dp, C.c_uint64, _dp,
                                                 C.c_uint32, C.c_double, _dp, C.c_double, C.c_double, C.c_int32,
                                                 C.c_uint64, C.c_uint64, _dp, _dp, C.c_uint64,
                                                 C.POINTER(C.c_uint64)]),
            "orc_set_threads": (None, [C.c_int]),
            "orc_get_threads": (C.c_int, []),
        }
        for name, (res, args) in sigs.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def set_threads(n: int) -> None:
    lib().orc_set_threads(int(n))


def threads() -> int:
    return int(lib().orc_get_threads())


class OracleError(RuntimeError):
    pass


def _chk(rc):
    if rc != 0:
        raise OracleError(f"oracle status {rc}")


def grid(p, r: np.ndarray):
    r = np.ascontiguousarray(r, dtype=np.float64)
    n = int(p.ntotal)
    keys = np.zeros(n, dtype=np.uint32)
    g = np.zeros(n, dtype=np.uint32)
    cs = np.zeros(int(p.max_cells) + 1, dtype=np.uint32)
    _chk(lib().orc_cell_keys(_P(p), _d(r), r.shape[1], _u(keys)))
    _chk(lib().orc_make_grid(_P(p), _u(keys), _u(g), _u(cs)))
    return keys, g, cs


def neighbours(p, r, itype, max_per: int | None = None):
    """(counts, list[n, max_per], grid, cells_start) of find_neighbours."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    itype = np.ascontiguousarray(itype, dtype=np.int32)
    keys, g, cs = grid(p, r)
    n = int(p.ntotal)
    max_per = int(max_per or p.max_neighbours)
    counts = np.zeros(n, dtype=np.uint32)
    lst = np.zeros((n, max_per), dtype=np.uint32)
    _chk(lib().orc_find_neighbours(_P(p), _d(r), r.shape[1], _i(itype), _u(g), _u(cs), _u(counts), _u(lst),
                                   max_per))
    return counts, lst, keys, g, cs


def density(p, r, v, rho, itype):
    """density_sum (rho, p) or density_con (drho, p) by p.density_treatment."""
    r = np.ascontiguousarray(r, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    counts, lst, *_ = neighbours(p, r, itype)
    n = int(p.ntotal)
    out = np.zeros(n)
    pres = np.zeros(n)
    mp = lst.shape[1]
    if p.density_treatment == 0:
        lib().orc_density_sum(_P(p), _d(r), r.shape[1], _u(counts), _u(lst), mp, _d(out), _d(pres))
    else:
        lib().orc_density_con(_P(p), _d(r), _d(v), r.shape[1], _d(rho), _u(counts), _u(lst), mp, _d(out),
                              _d(pres))
    return out, pres


def forces(p, terms: int, r, v, rho, pres, itype):
    r = np.ascontiguousarray(r, dtype=np.float64)
    v = np.ascontiguousarray(v, dtype=np.float64)
    rho = np.ascontiguousarray(rho, dtype=np.float64)
    pres = np.ascontiguousarray(pres, dtype=np.float64)
    itype = np.ascontiguousarray(itype, dtype=np.int32)
    counts, lst, *_ = neighbours(p, r, itype)
    n, dim = int(p.ntotal), r.shape[1]
    a = np.zeros((n, dim))
    av = np.zeros((n, dim))
    mu = np.zeros(n)
    lib().orc_forces(_P(p), terms, _i(itype), _d(r), _d(v), dim, _d(rho), _d(pres), _u(counts), _u(lst),
                     lst.shape[1], _d(a), _d(av), _d(mu))
    return a, av, mu


def eos_p(p, rho) -> np.ndarray:
    return np.array([lib().orc_eos_p(_P(p), float(x)) for x in np.atleast_1d(rho)])


def run(p, r, v, rho, itype, nsteps: int, time: float = 0.0, pres=None, a=None, drho=None,
        itimestep: int = 0):
    """nsteps of the time loop; returns the state dict (r, v, rho, p, itype, a, drho, time, pairs:
    the directed pairs of the last step, pairs_each: of every step)."""
    q = p.copy()
    r = np.array(r, dtype=np.float64, order="C")
    v = np.array(v, dtype=np.float64, order="C")
    rho = np.array(rho, dtype=np.float64)
    itype = np.array(itype, dtype=np.int32)
    n, dim = r.shape
    pres = np.zeros(n) if pres is None else np.array(pres, dtype=np.float64)
    a = np.zeros((n, dim)) if a is None else np.array(a, dtype=np.float64, order="C")
    drho = np.zeros(n) if drho is None else np.array(drho, dtype=np.float64)
    t = C.c_double(time)
    pairs = np.zeros(max(int(nsteps), 1), dtype=np.uint64)
    _chk(lib().orc_run(_P(q), _d(r), _d(v), dim, _d(rho), _d(pres), _i(itype), _d(a), _d(drho), itimestep,
                       nsteps, C.byref(t), pairs.ctypes.data_as(_u64p)))
    return {"r": r, "v": v, "rho": rho, "p": pres, "itype": itype, "a": a, "drho": drho, "time": t.value,
            "pairs": int(pairs[nsteps - 1]) if nsteps else 0, "pairs_each": pairs[:nsteps]}


def piston_tangent_run(p, r, v, rho, itype, nsteps: int, omega: float, coef, gauge_x: float,
                       search_n: float = 3.0, gauge_type: int = 2, sample_from: int = 0, sample_every: int = 1,
                       time: float = 0.0):
    """Forward run with the Fourier piston X(t) = sum_k coef[k-1] sin(k omega t)
    and the forward-mode derivatives of the gauge series by the coefficients.
    Returns (gauges[ns], dgauges[ns, ncoef], state dict)."""
    q = p.copy()
    r = np.array(r, dtype=np.float64, order="C")
    v = np.array(v, dtype=np.float64, order="C")
    rho = np.array(rho, dtype=np.float64)
    itype = np.array(itype, dtype=np.int32)
    n, dim = r.shape
    coef = np.ascontiguousarray(coef, dtype=np.float64)
    pres = np.zeros(n)
    a = np.zeros((n, dim))
    cap = (nsteps - sample_from) // sample_every + 1 if nsteps >= sample_from else 0
    g = np.zeros(max(cap, 1))
    dg = np.zeros((max(cap, 1), coef.size))
    t = C.c_double(time)
    ns = C.c_uint64()
    _chk(lib().orc_piston_tangent_run(_P(q), _d(r), _d(v), dim, _d(rho), _d(pres), _i(itype), _d(a), nsteps,
                                      C.byref(t), coef.size, float(omega), _d(coef), float(gauge_x), float(search_n),
                                      int(gauge_type), sample_from, sample_every, _d(g), _d(dg), cap, C.byref(ns)))
    k = int(ns.value)
    return g[:k], dg[:k], {"r": r, "v": v, "rho": rho, "p": pres, "itype": itype, "a": a, "time": t.value}


def gauge(p, r, itype, x: float, search_n: float = 3.0, type_filter: int = 0) -> float:
    r = np.ascontiguousarray(r, dtype=np.float64)
    itype = np.ascontiguousarray(itype, dtype=np.int32)
    return float(lib().orc_gauge(_P(p), _d(r), r.shape[1], _i(itype), float(x), float(search_n),
                                 int(type_filter)))


# ----------------------------------------------------- reference core ------

def ref_available() -> bool:
    return REF_BIN.exists() and os.access(REF_BIN, os.X_OK)


_REF_KEYS = [
    "dim", "ntotal", "nfluid", "nvirt", "x_mingeom", "x_maxgeom", "y_mingeom", "y_maxgeom", "z_mingeom", "z_maxgeom",
    "delta", "rho0", "depth", "nwm_particles_start", "nwm_particles_end", "density_treatment", "density_skf",
    "density_delta_sph_coef", "eos_sound_vel_method", "eos_sound_vel", "eos_sound_vel_coef", "intf_hsml_coef",
    "intf_sph_approximation", "intf_skf", "artificial_pressure", "artificial_pressure_skf",
    "artificial_pressure_index", "artificial_pressure_coef", "artificial_viscosity", "artificial_shear_visc",
    "artificial_bulk_visc", "artificial_viscosity_skf", "average_velocity", "average_velocity_coef",
    "average_velocity_skf", "consistency_check", "consistency_treatment", "boundary_treatment", "nwm",
    "nwm_direction", "nwm_time_start", "nwm_wave_length", "nwm_wave_magnitude", "nwm_phase", "simulation_time",
    "dt_correction_method", "dt", "CFL_coef", "max_neighbours", "local_threads", "start_simulation_time", "hsml",
    "mass", "cell_scale_k", "maxn", "max_cells", "nwm_wave_number", "nwm_freq", "nwm_piston_magnitude",
]


def ref_run(p, mode: str, r, v, rho, itype, pres=None, threads: int = 0, timeout: float = 600,
            gauges=None):
    """Runs the reference's compute core (oracle/_ref/rrsph_ref) in a child
    process on this state. Returns a dict of the output arrays.

    For mode "run:N", ``gauges=(every, search_n, type_filter, xs)`` samples the
    WaterProfile elevation at the positions xs before the first step and after
    every ``every`` steps (result "gauges": samples x len(xs)); "pairs" holds the
    directed pairs of each step's find_neighbours."""
    if not ref_available():
        raise OracleError("reference core not built (oracle/_ref/rrsph_ref)")
    n, dim = int(p.ntotal), int(p.dim)
    with tempfile.TemporaryDirectory() as d:
        dd = Path(d)
        with open(dd / "params.txt", "w") as f:
            for k in _REF_KEYS:
                f.write(f"{k} {float(getattr(p, k))!r}\n")
        if gauges is not None:
            every, search_n, type_filter, xs = gauges
            with open(dd / "gauges.txt", "w") as f:
                f.write(f"{int(every)} {float(search_n)!r} {int(type_filter)}\n")
                f.write(" ".join(repr(float(x)) for x in xs) + "\n")
        np.ascontiguousarray(r, dtype=np.float64).tofile(dd / "r.f64")
        np.ascontiguousarray(v, dtype=np.float64).tofile(dd / "v.f64")
        np.ascontiguousarray(rho, dtype=np.float64).tofile(dd / "rho.f64")
        (np.zeros(n) if pres is None else np.ascontiguousarray(pres, dtype=np.float64)).tofile(dd / "p.f64")
        np.ascontiguousarray(itype, dtype=np.int32).tofile(dd / "itype.i32")
        res = subprocess.run([str(REF_BIN), d, mode, str(threads)], capture_output=True, text=True, timeout=timeout)
        if res.returncode != 0:
            raise OracleError(f"reference core failed ({res.returncode}): {res.stderr.strip()}")
        out = {}
        for f in dd.iterdir():
            name, _, ext = f.name.rpartition(".")
            if f.name in ("params.txt", "gauges.txt", "r.f64", "v.f64", "rho.f64", "p.f64", "itype.i32"):
                continue
            if ext == "u64":
                out[name] = np.fromfile(f, dtype=np.uint64)
            elif ext == "f64":
                out[name] = np.fromfile(f, dtype=np.float64)
            elif ext == "u32":
                out[name] = np.fromfile(f, dtype=np.uint32)
            elif ext == "i32":
                out[name] = np.fromfile(f, dtype=np.int32)
            elif ext == "txt":
                out[name] = {ln.split()[0]: float(ln.split()[1]) for ln in f.read_text().splitlines() if ln.strip()}
        for key in ("a", "av", "r_out", "v_out", "a_out"):
            if key in out:
                out[key] = out[key].reshape(n, dim)
        if "phase_ms" in out:  # per step: predict, grid_find, density, accel, whole
            out["phase_ms"] = out["phase_ms"].reshape(-1, 5)
        if gauges is not None and "gauges" in out:
            out["gauges"] = out["gauges"].reshape(-1, len(gauges[3]))
        return out
