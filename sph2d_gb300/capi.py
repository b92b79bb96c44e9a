"""ctypes binding of the C ABI in ``include/rrsph_cuda.h`` (librrsph_cuda.so).

The library is built in-tree (``sph2d_gb300/build.py``) and loaded from this
package directory only; there is no fallback implementation — if the shared
library is missing the import of :func:`lib` raises.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "librrsph_cuda.so"

# status codes (rrsph_cuda.h)
OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_CUDA = 2
ERR_OUT_OF_MEMORY = 3
ERR_NEIGHBOUR_OVERFLOW = 4
ERR_OUT_OF_DOMAIN = 5
ERR_NON_FINITE = 6
ERR_OUTSIDE_GEOMETRY = 7
ERR_UNSUPPORTED = 8
ERR_IO = 9
ERR_PARSE = 10
ERR_NEVER_ENDING = 11
ERR_NO_DEVICE = 12

FLAG_NEIGHBOUR_OVERFLOW = 0x1
FLAG_OUT_OF_DOMAIN = 0x2
FLAG_NON_FINITE = 0x4
FLAG_OUTSIDE_GEOMETRY = 0x8
FLAG_NEVER_ENDING = 0x10

PRECISION_FP64 = 0
PRECISION_MIXED = 1

TERM_GRAVITY = 0x1
TERM_EXTERNAL = 0x2
TERM_INTERNAL = 0x4
TERM_ART_VISC = 0x8
TERM_AVERAGE_VELOCITY = 0x10
TERM_ALL = 0x1F

SORT_NOALLOC_MAX_PAIRS = 1 << 20

u32, u64, i32, f64 = C.c_uint32, C.c_uint64, C.c_int32, C.c_double


class RrsphParams(C.Structure):
    """Mirror of ``rrsph_params`` (field order and types as declared in C)."""

    _fields_ = [
        ("struct_size", u32), ("dim", u32),
        ("ntotal", u64), ("nfluid", u64), ("nvirt", u64),
        ("x_mingeom", f64), ("x_maxgeom", f64), ("y_mingeom", f64), ("y_maxgeom", f64),
        ("z_mingeom", f64), ("z_maxgeom", f64),
        ("delta", f64), ("rho0", f64), ("depth", f64),
        ("nwm_particles_start", u64), ("nwm_particles_end", u64),
        ("density_treatment", u32), ("density_skf", u32),
        ("density_delta_sph_coef", f64),
        ("eos_sound_vel_method", u32), ("intf_sph_approximation", u32),
        ("eos_sound_vel", f64), ("eos_sound_vel_coef", f64),
        ("intf_hsml_coef", f64),
        ("intf_skf", u32), ("artificial_pressure", u32), ("artificial_pressure_skf", u32),
        ("artificial_viscosity", u32),
        ("artificial_pressure_index", f64), ("artificial_pressure_coef", f64),
        ("artificial_shear_visc", f64), ("artificial_bulk_visc", f64),
        ("artificial_viscosity_skf", u32), ("average_velocity", u32),
        ("average_velocity_coef", f64),
        ("average_velocity_skf", u32), ("consistency_check", u32),
        ("consistency_treatment", u32), ("boundary_treatment", u32),
        ("nwm", u32), ("nwm_direction", u32),
        ("nwm_time_start", f64), ("nwm_wave_length", f64), ("nwm_wave_magnitude", f64), ("nwm_phase", f64),
        ("simulation_time", f64),
        ("dt_correction_method", u32), ("dt_dynamic_reduce", u32),
        ("dt", f64), ("CFL_coef", f64),
        ("max_neighbours", u32), ("local_threads", u32),
        ("save_time", f64), ("dump_time", f64),
        ("use_dump", u32), ("save_every_step", u32),
        ("save_velocity", u32), ("save_pressure", u32),
        ("save_density", u32), ("use_crash_dump", u32),
        ("start_simulation_time", f64),
        ("hsml", f64), ("mass", f64), ("cell_scale_k", f64),
        ("maxn", u64), ("max_cells", u64),
        ("nwm_wave_number", f64), ("nwm_freq", f64), ("nwm_piston_magnitude", f64),
        ("pi", f64), ("g", f64),
        ("type_boundary", i32), ("type_non_existent", i32), ("type_water", i32),
        ("reserved0", u32),
    ]

    def to_dict(self) -> dict:
        return {name: getattr(self, name) for name, _ in self._fields_}

    def copy(self) -> "RrsphParams":
        out = RrsphParams()
        C.memmove(C.byref(out), C.byref(self), C.sizeof(self))
        return out


PISTON_FOURIER_MAX = 16


class RrsphAdjointConfig(C.Structure):
    """Mirror of rrsph_adjoint_config."""

    _fields_ = [
        ("struct_size", C.c_uint32),
        ("checkpoint_every", C.c_uint32),
        ("nsteps", C.c_uint64),
        ("gauge_x", C.c_double),
        ("gauge_search_n", C.c_double),
        ("gauge_type", C.c_int32),
        ("sample_every", C.c_uint32),
        ("sample_from", C.c_uint64),
    ]


class RrsphDiagnostics(C.Structure):
    """Mirror of rrsph_diagnostics."""

    _fields_ = [
        ("mass", C.c_double),
        ("kinetic", C.c_double),
        ("potential", C.c_double),
        ("internal", C.c_double),
        ("momentum", C.c_double * 3),
        ("mass_boundary", C.c_double),
        ("fluid", C.c_uint64),
        ("boundary", C.c_uint64),
    ]


class RrsphWaveMaker(C.Structure):
    """Mirror of rrsph_wave_maker."""

    _fields_ = [
        ("particles_start", C.c_uint64),
        ("particles_end", C.c_uint64),
        ("nwm", C.c_uint32),
        ("reserved", C.c_uint32),
        ("time_start", C.c_double),
        ("phase", C.c_double),
        ("wave_length", C.c_double),
        ("wave_magnitude", C.c_double),
        ("depth", C.c_double),
    ]


_lib = None

_P = C.POINTER
_dp = _P(C.c_double)
_u32p = _P(C.c_uint32)
_i32p = _P(C.c_int32)

_SIGS = {
    "rrsph_abi_version": (C.c_int, []),
    "rrsph_params_sizeof": (C.c_size_t, []),
    "rrsph_params_offsetof": (C.c_int, [C.c_char_p, _P(C.c_size_t)]),
    "rrsph_last_error": (C.c_char_p, []),
    "rrsph_params_defaults": (C.c_int, [_P(RrsphParams)]),
    "rrsph_experiment_load_params": (C.c_int, [C.c_char_p, _P(RrsphParams)]),
    "rrsph_params_derive": (C.c_int, [_P(RrsphParams), _dp, C.c_uint32]),
    "rrsph_layer_time_from_path": (C.c_int, [C.c_char_p, _dp]),
    "rrsph_layer_read": (C.c_int, [C.c_char_p, _P(RrsphParams), _dp, C.c_uint32, _dp, _dp, _dp, _i32p]),
    "rrsph_layer_write": (C.c_int, [C.c_char_p, _P(RrsphParams), _dp, C.c_uint32, _dp, _dp, _dp, _i32p, C.c_int]),
    "rrsph_create": (C.c_int, [_P(RrsphParams), C.c_int, _P(C.c_void_p)]),
    "rrsph_destroy": (None, [C.c_void_p]),
    "rrsph_get_stream": (C.c_int, [C.c_void_p, _P(C.c_void_p)]),
    "rrsph_upload": (C.c_int, [C.c_void_p, _dp, C.c_uint32, _dp, _dp, _dp, _i32p]),
    "rrsph_download": (C.c_int, [C.c_void_p, _dp, C.c_uint32, _dp, _dp, _dp, _i32p]),
    "rrsph_step": (C.c_int, [C.c_void_p, C.c_uint64, _dp]),
    "rrsph_step_async": (C.c_int, [C.c_void_p, C.c_uint64]),
    "rrsph_set_time": (C.c_int, [C.c_void_p, C.c_double]),
    "rrsph_sync": (C.c_int, [C.c_void_p, _dp]),
    "rrsph_run": (C.c_int, [C.c_void_p, C.c_char_p, _dp, C.c_uint64, _P(C.c_uint64)]),
    "rrsph_status": (C.c_int, [C.c_void_p, _u32p, C.c_int]),
    "rrsph_diagnostics_get": (C.c_int, [C.c_void_p, _P(RrsphDiagnostics)]),
    "rrsph_get_dt": (C.c_int, [C.c_void_p, _dp]),
    "rrsph_pair_count": (C.c_int, [C.c_void_p, _P(C.c_uint64), _P(C.c_uint64)]),
    "rrsph_step_host": (C.c_int, [C.c_void_p, C.c_uint64, _P(C.c_double), _dp, C.c_uint32, _dp, _dp, _dp, _i32p]),
    "rrsph_step_download": (C.c_int, [C.c_void_p, C.c_uint64, _P(C.c_double), _dp, C.c_uint32, _dp, _dp, _dp, _i32p]),
    "rrsph_last_report": (C.c_int, [C.c_void_p, _P(C.c_double), _P(C.c_uint32), _P(C.c_uint64), _P(C.c_uint64)]),
    "rrsph_grid_find": (C.c_int, [C.c_void_p, _u32p, _u32p, _u32p]),
    "rrsph_neighbours": (C.c_int, [C.c_void_p, _u32p, _u32p, C.c_uint32, _P(C.c_uint64)]),
    "rrsph_step_neighbours": (C.c_int, [C.c_void_p, _u32p, _u32p, C.c_uint32, _P(C.c_uint64)]),
    "rrsph_download_rates": (C.c_int, [C.c_void_p, _dp, C.c_uint32, _dp]),
    "rrsph_density": (C.c_int, [C.c_void_p, _dp, _dp]),
    "rrsph_forces": (C.c_int, [C.c_void_p, C.c_uint32, _dp, C.c_uint32, _dp, _dp]),
    "rrsph_phase_count": (C.c_int, [C.c_void_p, _P(C.c_int)]),
    "rrsph_phase_name": (C.c_char_p, [C.c_void_p, C.c_int]),
    "rrsph_set_phase_timing": (C.c_int, [C.c_void_p, C.c_int]),
    "rrsph_phase_times": (C.c_int, [C.c_void_p, _dp, C.c_int, _P(C.c_uint64), C.c_int]),
    "rrsph_kernel_launches": (C.c_int, [C.c_void_p, _P(C.c_uint64)]),
    "rrsph_sort_pairs_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                           C.c_void_p]),
    "rrsph_set_piston_fourier": (C.c_int, [C.c_void_p, C.c_uint32, C.c_double, _dp]),
    "rrsph_adjoint_forward": (C.c_int, [C.c_void_p, _P(RrsphAdjointConfig), _dp, _dp, C.c_uint64, _P(C.c_uint64)]),
    "rrsph_adjoint_reverse": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "rrsph_set_wave_makers": (C.c_int, [C.c_void_p, C.c_uint32, _P(RrsphWaveMaker)]),
    "rrsph_set_gather_threads": (C.c_int, [C.c_void_p, C.c_uint32, C.c_uint32]),
    "rrsph_autotune": (C.c_int, [C.c_void_p, C.c_uint32, _u32p]),
    "rrsph_autotune_skin": (C.c_int, [C.c_void_p, C.c_uint32, _P(C.c_double)]),
    "rrsph_set_neighbour_reuse": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "rrsph_neighbour_rebuilds": (C.c_int, [C.c_void_p, _P(C.c_uint64)]),
}


class RrsphError(RuntimeError):
    """A non-zero status of the C ABI, with the library's message."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


def lib() -> C.CDLL:
    """Loads librrsph_cuda.so from the package directory (raises if absent)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
            )
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        if L.rrsph_params_sizeof() != C.sizeof(RrsphParams):
            raise ImportError("rrsph_params layout mismatch between C and Python")
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != OK:
        raise RrsphError(code, lib().rrsph_last_error().decode(errors="replace"))


def declared_symbols(header: Path | None = None) -> list[str]:
    """Names of the functions declared in include/rrsph_cuda.h."""
    import re

    h = header or (Path(__file__).resolve().parent.parent / "include" / "rrsph_cuda.h")
    text = h.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rrsph_[a-z0-9_]+)\s*\(", text)))
