"""Python handle over the C ABI of the GPU step (``include/rrsph_cuda.h``).

Arrays are numpy float64 / int32 / uint32; positions and velocities are
``(ntotal, dim)`` particle-major (stride = dim) unless a stride is given.
Every call goes through librrsph_cuda.so; there is no other implementation.
"""

from __future__ import annotations

import ctypes as C
import json
import tempfile
from pathlib import Path

import numpy as np

from . import capi
from .capi import RrsphParams, check, lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _u32p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint32))


def _i32p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int32))


def default_params() -> RrsphParams:
    p = RrsphParams()
    check(lib().rrsph_params_defaults(C.byref(p)))
    return p


def load_params(experiment_dir: str | Path) -> RrsphParams:
    """ParticleParams.json + ModelParams.json of an experiment directory."""
    p = default_params()
    check(lib().rrsph_experiment_load_params(str(experiment_dir).encode(), C.byref(p)))
    return p


def params_from_json(model: dict, particle: dict) -> RrsphParams:
    """Parses the two JSON objects through the library's own loader."""
    with tempfile.TemporaryDirectory() as d:
        Path(d, "ModelParams.json").write_text(json.dumps(model, indent=2))
        Path(d, "ParticleParams.json").write_text(json.dumps(particle, indent=2))
        return load_params(d)


def derive(p: RrsphParams, r: np.ndarray | None) -> RrsphParams:
    """fillInComputingParams/postFillInModelParams on a copy of p."""
    q = p.copy()
    if r is not None:
        r = np.ascontiguousarray(r, dtype=np.float64)
        stride = r.shape[1]
    else:
        stride = q.dim
    check(lib().rrsph_params_derive(C.byref(q), _dp(r), stride))
    return q


def read_layer(path: str | Path, p: RrsphParams):
    n, dim = p.ntotal, p.dim
    r = np.zeros((n, dim))
    v = np.zeros((n, dim))
    rho = np.zeros(n)
    pres = np.zeros(n)
    itype = np.zeros(n, dtype=np.int32)
    check(lib().rrsph_layer_read(str(path).encode(), C.byref(p), _dp(r), dim, _dp(v), _dp(rho), _dp(pres), _i32p(itype)))
    return r, v, rho, pres, itype


def write_layer(path: str | Path, p: RrsphParams, r, v, rho, pres, itype, dump: bool = True) -> None:
    r = np.ascontiguousarray(r, dtype=np.float64)
    v = None if v is None else np.ascontiguousarray(v, dtype=np.float64)
    rho = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
    pres = None if pres is None else np.ascontiguousarray(pres, dtype=np.float64)
    itype = np.ascontiguousarray(itype, dtype=np.int32)
    check(lib().rrsph_layer_write(str(path).encode(), C.byref(p), _dp(r), r.shape[1], _dp(v), _dp(rho), _dp(pres),
                                  _i32p(itype), 1 if dump else 0))


class Solver:
    """One GPU solver handle (rrsph_create ... rrsph_destroy)."""

    def __init__(self, params: RrsphParams, precision: str = "fp64"):
        self.params = params.copy()
        self.precision = capi.PRECISION_MIXED if precision == "mixed" else capi.PRECISION_FP64
        h = C.c_void_p()
        check(lib().rrsph_create(C.byref(self.params), self.precision, C.byref(h)))
        self._h = h
        self.n = int(params.ntotal)
        self.dim = int(params.dim)

    # -- lifetime
    def close(self) -> None:
        if self._h:
            lib().rrsph_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        check(lib().rrsph_get_stream(self._h, C.byref(s)))
        return int(s.value or 0)

    # -- state
    def upload(self, r, v, rho, itype, pres=None) -> None:
        r = np.ascontiguousarray(r, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        rho = np.ascontiguousarray(rho, dtype=np.float64)
        itype = np.ascontiguousarray(itype, dtype=np.int32)
        pres = None if pres is None else np.ascontiguousarray(pres, dtype=np.float64)
        assert r.shape == (self.n, r.shape[1]) and r.shape[1] >= self.dim and v.shape == r.shape
        check(lib().rrsph_upload(self._h, _dp(r), r.shape[1], _dp(v), _dp(rho), _dp(pres), _i32p(itype)))

    def download(self) -> dict:
        r = np.zeros((self.n, self.dim))
        v = np.zeros((self.n, self.dim))
        rho = np.zeros(self.n)
        pres = np.zeros(self.n)
        itype = np.zeros(self.n, dtype=np.int32)
        check(lib().rrsph_download(self._h, _dp(r), self.dim, _dp(v), _dp(rho), _dp(pres), _i32p(itype)))
        return {"r": r, "v": v, "rho": rho, "p": pres, "itype": itype}

    def step_host(self, state: dict, nsteps: int = 1, time: float = 0.0) -> float:
        """rrsph_step_host on a host state dict (r, v, rho, itype; p written
        if present): upload, nsteps steps and download in one call, in place.
        The arrays must be C-contiguous float64 (itype int32) with r and v of
        shape (n, stride >= dim). Returns the time after the steps."""
        r, v, rho, itype = state["r"], state["v"], state["rho"], state["itype"]
        pres = state.get("p")
        for a in (r, v, rho) + (() if pres is None else (pres,)):
            assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
        assert itype.dtype == np.int32 and itype.flags["C_CONTIGUOUS"]
        assert r.shape == (self.n, r.shape[1]) and r.shape[1] >= self.dim and v.shape == r.shape
        t = C.c_double(time)
        check(lib().rrsph_step_host(self._h, nsteps, C.byref(t), _dp(r), r.shape[1], _dp(v), _dp(rho), _dp(pres),
                                    _i32p(itype)))
        return t.value

    def step_download(self, nsteps: int = 1, time: float = 0.0):
        """rrsph_step_download: nsteps steps and the download of the state in one
        call. Returns (time, state dict as download())."""
        r = np.zeros((self.n, self.dim))
        v = np.zeros((self.n, self.dim))
        rho = np.zeros(self.n)
        pres = np.zeros(self.n)
        itype = np.zeros(self.n, dtype=np.int32)
        t = C.c_double(time)
        check(lib().rrsph_step_download(self._h, nsteps, C.byref(t), _dp(r), self.dim, _dp(v), _dp(rho), _dp(pres),
                                        _i32p(itype)))
        return t.value, {"r": r, "v": v, "rho": rho, "p": pres, "itype": itype}

    def download_rates(self) -> dict:
        """Accelerations and drho of the last completed step (rrsph_download_rates)."""
        a = np.zeros((self.n, self.dim))
        drho = np.zeros(self.n)
        check(lib().rrsph_download_rates(self._h, _dp(a), self.dim, _dp(drho)))
        return {"a": a, "drho": drho}

    def step(self, nsteps: int, time: float = 0.0) -> float:
        t = C.c_double(time)
        check(lib().rrsph_step(self._h, nsteps, C.byref(t)))
        return t.value

    def run(self, experiment_dir, time: float = 0.0, max_steps: int = 2**63 - 1):
        """The loop with layer output (rrsph_run); returns (time, steps)."""
        t = C.c_double(time)
        n = C.c_uint64()
        check(lib().rrsph_run(self._h, str(experiment_dir).encode(), C.byref(t), max_steps, C.byref(n)))
        return t.value, int(n.value)

    def step_async(self, nsteps: int) -> None:
        check(lib().rrsph_step_async(self._h, nsteps))

    def set_time(self, time: float) -> None:
        check(lib().rrsph_set_time(self._h, time))

    def sync(self) -> float:
        t = C.c_double()
        check(lib().rrsph_sync(self._h, C.byref(t)))
        return t.value

    def status(self, clear: bool = False) -> int:
        f = C.c_uint32()
        check(lib().rrsph_status(self._h, C.byref(f), 1 if clear else 0))
        return f.value

    def diagnostics(self) -> dict:
        """The double-precision mass and energy checks of the current state
        (rrsph_diagnostics_get)."""
        d = capi.RrsphDiagnostics()
        check(lib().rrsph_diagnostics_get(self._h, C.byref(d)))
        return {"mass": d.mass, "kinetic": d.kinetic, "potential": d.potential, "internal": d.internal,
                "momentum": list(d.momentum), "mass_boundary": d.mass_boundary, "fluid": int(d.fluid),
                "boundary": int(d.boundary)}

    def pair_count(self):
        """(pairs of the last step, pairs summed since upload)."""
        a, b = C.c_uint64(), C.c_uint64()
        check(lib().rrsph_pair_count(self._h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def last_report(self) -> dict:
        """What the last step()/sync() read back (no device access): time,
        device flags, and the pair counts of pair_count() as of that call."""
        t, f, a, b = C.c_double(), C.c_uint32(), C.c_uint64(), C.c_uint64()
        check(lib().rrsph_last_report(self._h, C.byref(t), C.byref(f), C.byref(a), C.byref(b)))
        return {"time": t.value, "flags": int(f.value), "pairs_last": int(a.value), "pairs_total": int(b.value)}

    def dt(self) -> float:
        d = C.c_double()
        check(lib().rrsph_get_dt(self._h, C.byref(d)))
        return d.value

    # -- loop pieces
    def grid_find(self, with_cells_start: bool = True):
        keys = np.zeros(self.n, dtype=np.uint32)
        grid = np.zeros(self.n, dtype=np.uint32)
        cs = np.zeros(int(self.params.max_cells) + 1, dtype=np.uint32) if with_cells_start else None
        check(lib().rrsph_grid_find(self._h, _u32p(keys), _u32p(grid), _u32p(cs)))
        return keys, grid, cs

    def neighbours(self, max_per: int | None = None):
        max_per = int(max_per or self.params.max_neighbours)
        counts = np.zeros(self.n, dtype=np.uint32)
        lst = np.zeros(self.n * max_per, dtype=np.uint32)
        tot = C.c_uint64()
        check(lib().rrsph_neighbours(self._h, _u32p(counts), _u32p(lst), max_per, C.byref(tot)))
        return counts, lst.reshape(self.n, max_per), int(tot.value)

    def step_neighbours(self, max_per: int | None = None):
        """The pairs the last FP32-mixed reuse step's density pass used
        (rrsph_step_neighbours): counts, list[n, max_per] in the list's own
        order, total."""
        max_per = int(max_per or self.params.max_neighbours)
        counts = np.zeros(self.n, dtype=np.uint32)
        lst = np.zeros(self.n * max_per, dtype=np.uint32)
        tot = C.c_uint64()
        check(lib().rrsph_step_neighbours(self._h, _u32p(counts), _u32p(lst), max_per, C.byref(tot)))
        return counts, lst.reshape(self.n, max_per), int(tot.value)

    def density(self):
        out = np.zeros(self.n)
        pres = np.zeros(self.n)
        check(lib().rrsph_density(self._h, _dp(out), _dp(pres)))
        return out, pres

    def forces(self, terms: int = capi.TERM_ALL, with_av: bool = False):
        a = np.zeros((self.n, self.dim))
        av = np.zeros((self.n, self.dim)) if with_av else None
        mu = np.zeros(self.n)
        check(lib().rrsph_forces(self._h, terms, _dp(a), self.dim, _dp(av), _dp(mu)))
        return a, av, mu

    # -- ensembles and tuning
    def set_wave_makers(self, makers) -> None:
        """Pistons of a packed ensemble: dicts with particles_start, particles_end,
        nwm, time_start, phase, wave_length, wave_magnitude, depth."""
        arr = (capi.RrsphWaveMaker * max(len(makers), 1))()
        for i, m in enumerate(makers):
            for k, v in m.items():
                setattr(arr[i], k, v)
        check(lib().rrsph_set_wave_makers(self._h, len(makers), arr))

    def set_gather_threads(self, density: int, forces: int) -> None:
        check(lib().rrsph_set_gather_threads(self._h, density, forces))

    def autotune(self, steps: int = 5):
        """Picks the gather block sizes by timing; returns (density, forces) threads."""
        out = (C.c_uint32 * 2)()
        check(lib().rrsph_autotune(self._h, steps, out))
        return int(out[0]), int(out[1])

    def autotune_skin(self, steps: int = 30) -> float:
        """Picks the candidate lists' skin by timing `steps` steps per
        candidate (rebuilds included); returns it in units of hsml."""
        v = C.c_double()
        check(lib().rrsph_autotune_skin(self._h, steps, C.byref(v)))
        return float(v.value)

    def set_neighbour_reuse(self, enable: bool, skin_over_h: float = 0.0) -> None:
        """Candidate-list reuse of the FP32-mixed step (2D or 3D, summation or
        continuity density); skin_over_h 0 keeps the current skin (0.5 h in 2D,
        0.3 h in 3D by default). The next step rebuilds the grid and lists."""
        check(lib().rrsph_set_neighbour_reuse(self._h, 1 if enable else 0, float(skin_over_h)))

    def neighbour_rebuilds(self) -> int:
        v = C.c_uint64()
        check(lib().rrsph_neighbour_rebuilds(self._h, C.byref(v)))
        return int(v.value)

    # -- piston optimisation
    def set_piston_fourier(self, omega: float, coef) -> None:
        """Piston displacement X(t) = sum_k coef[k-1] sin(k omega t) (empty coef: the wave maker's own law)."""
        c = np.ascontiguousarray(coef, dtype=np.float64)
        self._fourier_n = int(c.size)
        check(lib().rrsph_set_piston_fourier(self._h, c.size, float(omega), _dp(c) if c.size else None))

    def adjoint_forward(self, nsteps: int, gauge_x: float, sample_from: int = 0, sample_every: int = 1,
                        checkpoint_every: int = 100, search_n: float = 3.0, gauge_type: int = 2,
                        time: float = 0.0):
        """Recorded FP64 forward run; returns (gauge series, time at the end)."""
        cfg = capi.RrsphAdjointConfig(C.sizeof(capi.RrsphAdjointConfig), checkpoint_every, nsteps, gauge_x, search_n,
                                      gauge_type, sample_every, sample_from)
        cap = (nsteps - sample_from) // sample_every + 1 if nsteps >= sample_from else 0
        g = np.zeros(max(cap, 1))
        t = C.c_double(time)
        ns = C.c_uint64()
        self._adj_steps = 0
        check(lib().rrsph_adjoint_forward(self._h, C.byref(cfg), C.byref(t), _dp(g), cap, C.byref(ns)))
        self._adj_steps = nsteps
        return g[: int(ns.value)], t.value

    def adjoint_reverse(self, dgauges):
        """(dL/dcoef of the Fourier piston, dL/d(piston vx) per step) for dL/dgauge."""
        dg = np.ascontiguousarray(dgauges, dtype=np.float64)
        dcoef = np.zeros(max(getattr(self, "_fourier_n", 0), 1))
        dvx = np.zeros(max(getattr(self, "_adj_steps", 0), 1))
        check(lib().rrsph_adjoint_reverse(self._h, _dp(dg), _dp(dcoef), _dp(dvx)))
        return dcoef[: getattr(self, "_fourier_n", 0)], dvx[: self._adj_steps]

    # -- timing
    def phase_names(self) -> list[str]:
        c = C.c_int()
        check(lib().rrsph_phase_count(self._h, C.byref(c)))
        return [lib().rrsph_phase_name(self._h, i).decode() for i in range(c.value)]

    def set_phase_timing(self, enable: bool) -> None:
        check(lib().rrsph_set_phase_timing(self._h, 1 if enable else 0))

    def phase_times(self, reset: bool = True):
        names = self.phase_names()
        ms = (C.c_double * len(names))()
        steps = C.c_uint64()
        check(lib().rrsph_phase_times(self._h, ms, len(names), C.byref(steps), 1 if reset else 0))
        return dict(zip(names, list(ms))), int(steps.value)

    def kernel_launches(self) -> int:
        c = C.c_uint64()
        check(lib().rrsph_kernel_launches(self._h, C.byref(c)))
        return int(c.value)
