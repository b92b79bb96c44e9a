"""Seeded synthetic experiments in the reference's experiment layout.

The reference builds experiments with Python scripts that write
ParticleParams.json, ModelParams.json and dump/0.csv
(tools/Scripts/Piston2DGenerator.py, DamBreakGenerator.py). These generators
produce the same files for the benchmark workloads; all randomness comes from
``numpy.random.default_rng(seed)``.

Layout choices (the workload descriptions leave them open):
- fluid particles come first (ids 0..nfluid-1), boundary particles after, as in
  the reference's generators (find_depth and the piston range rely on it);
- Lennard-Jones wall particles are laid at dx/2 spacing; the fluid lattice
  starts 2h from each wall, where the Lennard-Jones force of the reference
  (cutoff r0 = 2h, ExtForce.h:26) is zero, so the start is not an explosion;
- c0 = 10*sqrt(2*g*0.5) is expressed as eos_sound_vel_method 0 with
  eos_sound_vel_coef 1 and depth 0.5, which avoids the reference's method-1
  c/c^2 ambiguity (EOS.cpp:3-10);
- dt = 0.2*h/c0 with dt_correction_method 0;
- the dam break uses summation density: with continuity density this layout
  goes unstable after ~250 steps in the reference's own arithmetic (the
  oracle, bit-identical to the reference core, shows the same growth).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

G = 9.81
TYPE_BOUNDARY = -2
TYPE_WATER = 2


@dataclass
class Case:
    name: str
    model: dict
    particle: dict
    r: np.ndarray
    v: np.ndarray
    rho: np.ndarray
    itype: np.ndarray
    notes: dict = field(default_factory=dict)

    @property
    def ntotal(self) -> int:
        return int(self.r.shape[0])

    def params(self):
        """rrsph_params through the library's JSON loader and derivations."""
        from .solver import derive, params_from_json

        return derive(params_from_json(self.model, self.particle), self.r)

    def write_experiment(self, directory) -> None:
        """ModelParams.json, ParticleParams.json and dump/0.csv."""
        import json
        from pathlib import Path

        from .solver import write_layer

        d = Path(directory)
        (d / "dump").mkdir(parents=True, exist_ok=True)
        (d / "ModelParams.json").write_text(json.dumps(self.model, indent=2))
        (d / "ParticleParams.json").write_text(json.dumps(self.particle, indent=2))
        p = self.params()
        write_layer(d / "dump" / "0.csv", p, self.r, self.v, self.rho, np.zeros(self.ntotal), self.itype, dump=True)


def _hydrostatic_rho(y, surface, rho0, c2):
    B = c2 * rho0 / 7.0
    p = rho0 * G * np.maximum(surface - y, 0.0)
    return rho0 * np.power(1.0 + p / B, 1.0 / 7.0)


def _model_common(h_coef: float, dx: float, c0: float, density_treatment: int, simulation_time: float) -> dict:
    h = dx * h_coef
    return {
        "params_target_version_major": 3,
        "params_target_version_minor": 1,
        "params_target_version_patch": 4,
        "density_treatment": density_treatment,
        "density_skf": 1,
        "intf_skf": 1,
        "intf_sph_approximation": 2,
        "intf_hsml_coef": h_coef,
        "eos_sound_vel_method": 0,
        "eos_sound_vel_coef": 1.0,
        "artificial_viscosity": True,
        "artificial_shear_visc": 0.3,
        "artificial_bulk_visc": 0.0,
        "artificial_viscosity_skf": 1,
        "average_velocity": False,
        "visc": False,
        "boundary_treatment": 1,
        "dt_correction_method": 0,
        "dt": 0.2 * h / c0,
        "CFL_coef": 0.2,
        "max_neighbours": 64,
        "consistency_check": True,
        "consistency_treatment": 2,
        "save_time": 0.01,
        "dump_time": 0.1,
        "use_dump": False,
        "simulation_time": simulation_time,
        "nwm": 0,
    }


def _wall_line(x0, y0, x1, y1, step):
    n = int(math.floor(math.hypot(x1 - x0, y1 - y0) / step + 1e-9)) + 1
    t = np.arange(n) * step
    L = math.hypot(x1 - x0, y1 - y0)
    ux, uy = ((x1 - x0) / L, (y1 - y0) / L) if L > 0 else (0.0, 0.0)
    return np.stack([x0 + ux * t, y0 + uy * t], axis=1)


def dam_break_2d(seed: int = 1, nx: int = 100, ny: int = 50, dx: float = 0.01, tank=(3.2, 1.5),
                 steps: int = 2000, density_treatment: int = 0) -> Case:
    """2D dam break: tank 3.2 x 1.5 m, LJ walls at dx/2 on floor and side walls,
    water column nx*dx x ny*dx (1.0 x 0.5 m), h = 1.4 dx, alpha 0.3, beta 0,
    hydrostatic density, seeded +-1e-4 dx jitter."""
    rng = np.random.default_rng(seed)
    h = 1.4 * dx
    depth = 0.5
    c0 = 10.0 * math.sqrt(2.0 * G * depth)
    gap = 2.0 * h
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    fx = gap + ix.ravel() * dx
    fy = gap + iy.ravel() * dx
    fluid = np.stack([fx, fy], axis=1)
    fluid += rng.uniform(-1e-4 * dx, 1e-4 * dx, size=fluid.shape)
    surface = gap + (ny - 1) * dx
    L, H = tank
    wall = np.concatenate([
        _wall_line(0.0, 0.0, L, 0.0, dx / 2),                 # floor
        _wall_line(0.0, dx / 2, 0.0, H, dx / 2),              # left wall
        _wall_line(L, dx / 2, L, H, dx / 2),                  # right wall
    ])
    r = np.concatenate([fluid, wall])
    n_f, n_b = fluid.shape[0], wall.shape[0]
    itype = np.concatenate([np.full(n_f, TYPE_WATER), np.full(n_b, TYPE_BOUNDARY)]).astype(np.int32)
    rho = np.concatenate([_hydrostatic_rho(fluid[:, 1], surface, 1000.0, c0 * c0), np.full(n_b, 1000.0)])
    v = np.zeros_like(r)
    dt = 0.2 * h / c0
    model = _model_common(1.4, dx, c0, density_treatment, simulation_time=steps * dt)
    particle = {
        "params_target_version_major": 3, "params_target_version_minor": 1, "params_target_version_patch": 4,
        "dim": 2,
        "x_mingeom": -0.1, "x_maxgeom": L + 0.1, "y_mingeom": -0.1, "y_maxgeom": H + 0.1,
        "delta": dx, "rho0": 1000.0, "depth": depth,
        "ntotal": n_f + n_b, "nfluid": n_f, "nvirt": n_b,
    }
    return Case("dam_break_2d", model, particle, r, v, rho, itype,
                notes={"seed": seed, "nfluid": n_f, "nboundary": n_b, "steps": steps, "h": h, "c0": c0, "dt": dt,
                       "fluid_gap_to_walls": gap})


def piston_wave_number(period: float, depth: float) -> float:
    """k with sqrt(g k tanh(k d)) = 2 pi / period (the reference's dispersion, Input.cpp:125-137)."""
    omega = 2.0 * math.pi / period
    k = omega * omega / G
    for _ in range(100):
        f = G * k * math.tanh(k * depth) - omega * omega
        df = G * math.tanh(k * depth) + G * k * depth / math.cosh(k * depth) ** 2
        k -= f / df
    return k


def piston_flume_2d(seed: int = 7, nx: int = 4000, ny: int = 100, dx: float = 0.005, tank_height: float = 1.2,
                    amplitude: float = 0.05, period: float = 1.5, steps: int = 20000,
                    density_treatment: int = 0) -> Case:
    """2D piston wave flume: nx x ny fluid lattice (4000 x 100 = 400,000 at
    dx = 0.005: 20 m x 0.5 m), LJ floor / right wall / piston column at dx/2,
    piston displacement amplitude*sin(2 pi t / period), summation density."""
    rng = np.random.default_rng(seed)
    h = 1.4 * dx
    depth = ny * dx
    c0 = 10.0 * math.sqrt(2.0 * G * 0.5)
    gap = 2.0 * h
    length = gap + (nx - 1) * dx + gap
    ix, iy = np.meshgrid(np.arange(nx), np.arange(ny), indexing="ij")
    fluid = np.stack([gap + ix.ravel() * dx, gap + iy.ravel() * dx], axis=1)
    fluid += rng.uniform(-1e-4 * dx, 1e-4 * dx, size=fluid.shape)
    surface = gap + (ny - 1) * dx
    piston = _wall_line(0.0, 0.0, 0.0, tank_height, dx / 2)
    floor = _wall_line(dx / 2, 0.0, length, 0.0, dx / 2)
    right = _wall_line(length, dx / 2, length, tank_height, dx / 2)
    n_f = fluid.shape[0]
    r = np.concatenate([fluid, piston, floor, right])
    n_b = r.shape[0] - n_f
    itype = np.concatenate([np.full(n_f, TYPE_WATER), np.full(n_b, TYPE_BOUNDARY)]).astype(np.int32)
    rho = np.concatenate([_hydrostatic_rho(fluid[:, 1], surface, 1000.0, c0 * c0), np.full(n_b, 1000.0)])
    v = np.zeros_like(r)
    k = piston_wave_number(period, 0.5)
    kd = k * 0.5
    m1 = 2 * math.sinh(kd) ** 2 / (math.sinh(kd) * math.cosh(kd) + kd)
    dt = 0.2 * h / c0
    model = _model_common(1.4, dx, c0, density_treatment, simulation_time=steps * dt)
    model.update({
        "nwm": 2,
        "nwm_direction": 1,
        "nwm_time_start": 0.0,
        "nwm_phase": 0.0,
        "nwm_wave_length": 2.0 * math.pi / k,
        "nwm_wave_magnitude": 2.0 * amplitude * m1,
    })
    particle = {
        "params_target_version_major": 3, "params_target_version_minor": 1, "params_target_version_patch": 4,
        "dim": 2,
        "x_mingeom": -0.5, "x_maxgeom": length + 0.5, "y_mingeom": -0.1, "y_maxgeom": tank_height + 0.1,
        "delta": dx, "rho0": 1000.0, "depth": 0.5,
        "ntotal": n_f + n_b, "nfluid": n_f, "nvirt": n_b,
        "nwm_particles_start": n_f, "nwm_particles_end": n_f + piston.shape[0],
    }
    return Case("piston_flume_2d", model, particle, r, v, rho, itype,
                notes={"seed": seed, "nfluid": n_f, "nboundary": n_b, "steps": steps, "h": h, "c0": c0, "dt": dt,
                       "tank_length": length, "fluid_depth": depth, "piston_period": period,
                       "piston_amplitude": amplitude, "gauges_x": [2.0, 5.0, 10.0]})


def fourier_coefficients(seed: int, n: int = 8, lo: float = 0.005, hi: float = 0.03) -> np.ndarray:
    """Seeded amplitudes of the Fourier piston X(t) = sum_k c_k sin(k omega t)."""
    return np.random.default_rng(seed).uniform(lo, hi, size=n)


def adjoint_flume_2d(seed: int = 7, nx: int = 2000, ny: int = 100, dx: float = 0.005, coef_seed: int = 2,
                     target_seed: int = 3, ncoef: int = 8, period: float = 8.0, steps: int = 5000,
                     gauge_x: float = 0.3, window: float = 0.1, sample_every: int = 10) -> Case:
    """Piston flume for the adjoint: nx x ny fluid lattice (2000 x 100 =
    200,000 at dx = 0.005: 10 m x 0.5 m), the piston moving as the Fourier
    series X(t) = sum_k c_k sin(k omega t), omega = 2 pi / period, with c from
    ``coef_seed`` (amplitudes 0.005-0.03 m) and the target series from
    ``target_seed``. The loss is the mean squared gauge misfit at gauge_x over
    the last ``window`` seconds of ``steps`` steps, sampled every
    ``sample_every`` steps (5,000 steps are 0.22 s, so the gauge sits 0.3 m
    from the piston)."""
    case = piston_flume_2d(seed=seed, nx=nx, ny=ny, dx=dx, steps=steps)
    dt = case.notes["dt"]
    sample_from = max(0, steps - int(round(window / dt)))
    sample_from += (steps - sample_from) % sample_every  # the last sample is the last state
    case.name = "adjoint_flume_2d"
    case.notes.update({
        "omega": 2.0 * math.pi / period, "coef": fourier_coefficients(coef_seed, ncoef),
        "target_coef": fourier_coefficients(target_seed, ncoef), "coef_seed": coef_seed, "target_seed": target_seed,
        "piston_period": period, "gauge_x": gauge_x, "sample_from": sample_from, "sample_every": sample_every,
        "window": window,
    })
    return case


def ensemble_tanks(ntanks: int = 256, seed: int = 4, wave_seed: int = 5, n_lo: int = 2000, n_hi: int = 60000,
                   depth_lo: float = 0.2, depth_hi: float = 0.6, dx: float = 0.005, amp_lo: float = 0.01,
                   amp_hi: float = 0.05, period_lo: float = 1.0, period_hi: float = 2.0,
                   steps: int = 2000) -> list[Case]:
    """Independent 2D piston tanks: fluid counts log-uniform in [n_lo, n_hi]
    and depths uniform in [depth_lo, depth_hi] (seed), length = count dx^2 /
    depth; each piston with its own amplitude and period (wave_seed). Every
    tank shares c0, h and dt (the flume's); its piston law uses its own depth.
    Each case carries notes["wave_maker"] for rrsph_set_wave_makers."""
    rng = np.random.default_rng(seed)
    wrng = np.random.default_rng(wave_seed)
    counts = np.exp(rng.uniform(math.log(n_lo), math.log(n_hi), ntanks))
    depths = rng.uniform(depth_lo, depth_hi, ntanks)
    amps = wrng.uniform(amp_lo, amp_hi, ntanks)
    periods = wrng.uniform(period_lo, period_hi, ntanks)
    out = []
    for t in range(ntanks):
        ny = max(4, int(round(depths[t] / dx)))
        nx = max(4, int(round(counts[t] / ny)))
        c = piston_flume_2d(seed=seed * 100003 + t, nx=nx, ny=ny, dx=dx, tank_height=ny * dx + 0.3, steps=steps)
        d = ny * dx
        k = piston_wave_number(periods[t], d)
        kd = k * d
        m1 = 2 * math.sinh(kd) ** 2 / (math.sinh(kd) * math.cosh(kd) + kd)
        c.name = f"tank{t}"
        c.notes.update({"amplitude": float(amps[t]), "period": float(periods[t]), "water_depth": d})
        c.notes["wave_maker"] = {
            "particles_start": int(c.particle["nwm_particles_start"]),
            "particles_end": int(c.particle["nwm_particles_end"]),
            "nwm": 2, "time_start": 0.0, "phase": 0.0, "wave_length": 2.0 * math.pi / k,
            "wave_magnitude": 2.0 * float(amps[t]) * m1, "depth": d,
        }
        out.append(c)
    return out


def pack_tanks(tanks: list[Case], gap: float = 0.3) -> Case:
    """One particle set holding every tank, laid out in rows on a square-ish
    plane with `gap` between tanks (far beyond the 2h interaction range), for
    one solver over the whole ensemble. notes["wave_makers"] lists the pistons
    with global particle ranges; notes["offsets"] the (x, y) shift of each tank
    and notes["ranges"] its particle range."""
    foot = [(c.notes["tank_length"] + 2 * gap, c.particle["y_maxgeom"] - c.particle["y_mingeom"] + gap)
            for c in tanks]
    width = math.sqrt(sum(w * h for w, h in foot) * 1.3)
    offsets, x, y, row_h = [], 0.0, 0.0, 0.0
    for w, h in foot:
        if x > 0 and x + w > width:
            x, y, row_h = 0.0, y + row_h, 0.0
        offsets.append((x + gap, y))
        x += w
        row_h = max(row_h, h)
    rs, vs, rhos, its, makers, ranges = [], [], [], [], [], []
    base = 0
    for c, (ox, oy) in zip(tanks, offsets):
        rs.append(c.r + np.array([ox, oy]))
        vs.append(c.v)
        rhos.append(c.rho)
        its.append(c.itype)
        m = dict(c.notes["wave_maker"])
        m["particles_start"] += base
        m["particles_end"] += base
        makers.append(m)
        ranges.append((base, base + c.ntotal))
        base += c.ntotal
    r = np.concatenate(rs)
    model = dict(tanks[0].model)
    model["nwm"] = 0
    particle = dict(tanks[0].particle)
    particle.update({
        "x_mingeom": float(r[:, 0].min()) - 0.5, "x_maxgeom": float(r[:, 0].max()) + 0.5,
        "y_mingeom": float(r[:, 1].min()) - 0.1, "y_maxgeom": float(r[:, 1].max()) + 0.5,
        "ntotal": int(base), "nfluid": int(sum(c.notes["nfluid"] for c in tanks)),
        "nvirt": int(sum(c.notes["nboundary"] for c in tanks)),
        "nwm_particles_start": 0, "nwm_particles_end": 0,
    })
    return Case("ensemble_2d", model, particle, r, np.concatenate(vs), np.concatenate(rhos),
                np.concatenate(its).astype(np.int32),
                notes={"tanks": len(tanks), "wave_makers": makers, "offsets": offsets, "ranges": ranges,
                       "dt": tanks[0].notes["dt"], "nfluid": particle["nfluid"]})


def dam_break_3d(seed: int = 3, dx: float = 0.0026, tank=(1.6, 0.67, 0.6), block=(0.4, 0.67, 0.3),
                 steps: int = 5000, density_treatment: int = 1, max_neighbours: int = 400) -> Case:
    """3D dam break: fluid block inside a tank with LJ floor and walls at dx/2,
    h = 1.3 dx, seeded jitter. The fluid lattice is the block shrunk by 2h from
    each wall it touches."""
    rng = np.random.default_rng(seed)
    h = 1.3 * dx
    gap = 2.0 * h
    L, W, H = tank
    bl, bw, bh = block
    nx = int((bl - gap) / dx)
    ny = int((bh - gap) / dx)
    nz = int((min(bw, W) - 2 * gap) / dx) + 1
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    fluid = np.stack([gap + ix.ravel() * dx, gap + iy.ravel() * dx, gap + iz.ravel() * dx], axis=1)
    fluid += rng.uniform(-1e-4 * dx, 1e-4 * dx, size=fluid.shape)
    surface = gap + (ny - 1) * dx
    s = dx / 2
    ax_ = np.arange(0.0, L + 1e-9, s)
    az_ = np.arange(0.0, W + 1e-9, s)
    ay_ = np.arange(s, H + 1e-9, s)
    X, Z = np.meshgrid(ax_, az_, indexing="ij")
    floor = np.stack([X.ravel(), np.zeros(X.size), Z.ravel()], axis=1)
    Y, Z2 = np.meshgrid(ay_, az_, indexing="ij")
    left = np.stack([np.zeros(Y.size), Y.ravel(), Z2.ravel()], axis=1)
    right = np.stack([np.full(Y.size, L), Y.ravel(), Z2.ravel()], axis=1)
    X2, Y2 = np.meshgrid(ax_[1:-1], ay_, indexing="ij")
    front = np.stack([X2.ravel(), Y2.ravel(), np.zeros(X2.size)], axis=1)
    back = np.stack([X2.ravel(), Y2.ravel(), np.full(X2.size, W)], axis=1)
    wall = np.concatenate([floor, left, right, front, back])
    n_f, n_b = fluid.shape[0], wall.shape[0]
    r = np.concatenate([fluid, wall])
    depth = 0.5
    c0 = 10.0 * math.sqrt(2.0 * G * depth)
    itype = np.concatenate([np.full(n_f, TYPE_WATER), np.full(n_b, TYPE_BOUNDARY)]).astype(np.int32)
    rho = np.concatenate([_hydrostatic_rho(fluid[:, 1], surface, 1000.0, c0 * c0), np.full(n_b, 1000.0)])
    v = np.zeros_like(r)
    dt = 0.2 * h / c0
    model = _model_common(1.3, dx, c0, density_treatment, simulation_time=steps * dt)
    model["max_neighbours"] = max_neighbours
    particle = {
        "params_target_version_major": 3, "params_target_version_minor": 1, "params_target_version_patch": 4,
        "dim": 3,
        "x_mingeom": -0.05, "x_maxgeom": L + 0.05, "y_mingeom": -0.05, "y_maxgeom": H + 0.05,
        "z_mingeom": -0.05, "z_maxgeom": W + 0.05,
        "delta": dx, "rho0": 1000.0, "depth": depth,
        "ntotal": n_f + n_b, "nfluid": n_f, "nvirt": n_b,
    }
    return Case("dam_break_3d", model, particle, r, v, rho, itype,
                notes={"seed": seed, "nfluid": n_f, "nboundary": n_b, "steps": steps, "h": h, "c0": c0, "dt": dt,
                       "fluid_lattice": [nx, ny, nz]})
