"""Benchmark of the WCSPH step on one node.

Workload: the 2D piston wave flume — 4000 x 100 fluid lattice at dx = 0.005 m
(400,000 fluid particles, 20 m x 0.5 m of water) in a 1.2 m high tank with
Lennard-Jones floor, right wall and piston column at dx/2 (8,970 particles),
h = 1.4 dx, summation density, cubic spline, Tait EOS, Monaghan viscosity
(alpha 0.3), piston displacement 0.05 sin(2 pi t / 1.5 s), dt = 0.2 h / c0.
Inputs are seeded synthetic particles with those shapes (sph2d_gb300.cases).

One step is one pass of the loop body (predict, grid, density, forces,
piston, whole step). The headline is the FP32-mixed step; the plain FP64 GPU
step is timed beside it, and the mixed step's per-field error against the FP64
GPU step is reported.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: the step does not shard (one tank), so N ranks run N independent
replicas (weak scaling); value sums the ranks' pairs over the slowest rank's
time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "pair-interactions/s and ms/step: FP32-mixed vs FP64 GPU step at stated error"
UNIT = "pair-interactions/s"
L2_FLUSH_BYTES = 256 << 20  # larger than the 129 MB L2

# Algorithmic bytes of the dominant kernel, k_forces_verlet of the FP32-mixed
# 2D step with neighbour reuse (the force gather with the whole step and the
# next step's key pass fused in), by the per-particle figures of the scope
# table's roofline: force gather 64 B (read position, velocity, density,
# pressure, type; write a, drho), integrate + piston 96 B (read and write r, v
# in FP64, rho, a) and key pass 24 B (read r, write key and id): 184 B per
# particle. Neighbour data other threads also load are not algorithmic bytes.
FORCES_ALGORITHMIC_BYTES_PER_PARTICLE = 64 + 96 + 24
# What the kernel as built reads and writes once per particle and per pair
# (its own design's bytes, stated beside the algorithmic ones): per particle the
# gather reads id 4, position+type float4 16, velocity+pressure+density float4
# 16, (p, p/rho^2) float2 8, candidate and neighbour counts 4 + 4 and writes a.x,
# a.y doubles 16; the whole step reads r, v doubles 32, itype 4, key_of 4, build
# cell 4, build offset 8, build slot 4 and writes r, v 32, v_predict float2 8,
# cell offset float2 8, cell 4, key_of 4, sort key + id 8, the next step's
# position and velocity float4s 32 and one cell-table word 4; per pair one
# 4-byte word of this step's neighbour list.
FORCES_DESIGN_BYTES_PER_PARTICLE = (52 + 16) + (32 + 4 + 4 + 4 + 8 + 4) + (32 + 8 + 8 + 4 + 4 + 8 + 32 + 4)
FORCES_DESIGN_BYTES_PER_PAIR = 4
# Pair arithmetic of the FP32 pipe per directed pair: 16 flops for the density
# (distance, kernel, sum) and 52 for the forces (form-2 pressure term,
# artificial viscosity, Lennard-Jones amortised); the nominal FP32 (non-tensor)
# peak of the part is 152 SMs x 128 lanes x 2 flops x 2.07 GHz.
FLOPS_PER_PAIR = 16 + 52
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12
FORCES_FP64_BYTES_PER_PARTICLE_2D = 4 + 4 + 16 + 4 + 16 + 8 + 8 + 16


def workload_config(case, pairs_first: int, warmup: int, steps: int) -> dict:
    """The workload both arms run (the GPU arm and the reference's CPU code):
    the same seeded particles, parameters and step window."""
    return {
        "workload": "2D piston wave flume: 20 m x 0.5 m water (4000 x 100 at dx=0.005 m), 1.2 m tank, "
                    "LJ walls + piston at dx/2, summation density, piston 0.05*sin(2*pi*t/1.5 s)",
        "n_particles": int(case.ntotal),
        "n_fluid": int(case.notes["nfluid"]),
        "h": case.notes["h"],
        "dt": case.notes["dt"],
        "pairs_first_step": int(pairs_first),
        "window": f"steps {warmup + 1}-{warmup + steps} of the run from the seeded start "
                  f"(its start-up transient included)",
        "parallelism": "replicas",
    }


GPU_METHOD = {
    "precision": "mixed (f32 pairs, f64 state/integration)",
    "neighbour_search": "candidate lists within cutoff + 0.5 h, rebuilt when a particle has moved 0.25 h",
    "l2": "not flushed: the timed steps run back to back as the time loop runs them; one step reads and "
          "writes ~160 MB of particle state and neighbour lists (> 129 MB L2)",
}


def load_cases():
    """sph2d_gb300/cases.py (the seeded workload generators, numpy only) loaded
    as a plain module, without importing the sph2d_gb300 package or loading its
    library: the reference arm generates the same particles with it."""
    import importlib.util

    name = "rrsph_workload_cases"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, ROOT / "sph2d_gb300" / "cases.py")
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


# --------------------------------------------------------------- clocks ----

class ClockSampler:
    """nvidia-smi sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                rows.append((float(f[1]), float(f[2]), f))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for _, _, f in rows for n, v in zip(names, f[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------- GPU arm -------

def _time_steps(solver, flush, steps: int) -> float:
    """Device milliseconds of `steps` single-step graph launches, each after an
    L2 flush, timed with CUDA events on the solver's stream."""
    import torch

    ext = torch.cuda.ExternalStream(solver.stream)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    with torch.cuda.stream(ext):
        for k in range(steps):
            flush.add_(1)
            starts[k].record(ext)
            solver.step_async(1)
            ends[k].record(ext)
    solver.sync()
    return sum(s.elapsed_time(e) for s, e in zip(starts, ends))


def _loop_ms(solver, steps: int) -> float:
    """Device milliseconds per step of `steps` steps back to back (one graph
    launch each) between two CUDA events on the solver's stream, as the time
    loop runs them: no flush between steps, whose per-step data (~160 MB of
    particle state and neighbour lists on the flume) exceed the 129 MB L2."""
    import torch

    ext = torch.cuda.ExternalStream(solver.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(ext):
        e0.record(ext)
        solver.step_async(steps)
        e1.record(ext)
    solver.sync()
    return e0.elapsed_time(e1) / steps


def _phase_pass(solver, flush, steps: int):
    """Per-phase milliseconds per step (events between the kernels of each
    phase; direct launches). flush: a tensor written before every step (the
    L2 flushed), or None (steps back to back)."""
    import torch

    ext = torch.cuda.ExternalStream(solver.stream)
    solver.set_phase_timing(True)
    solver.phase_times(reset=True)
    for _ in range(steps):
        if flush is not None:
            with torch.cuda.stream(ext):
                flush.add_(1)
        solver.step_async(1)
    solver.sync()
    times, n = solver.phase_times(reset=True)
    solver.set_phase_timing(False)
    return {k: v / n for k, v in times.items()}


def _rel(a, b):
    nb = float(np.linalg.norm(b))
    return float(np.linalg.norm(a - b)) / (nb if nb > 0 else 1.0)


def aggregate_replicas(t_s: float, pairs: float, e2e_s: float, e2e_pairs: float, dist=None, device="cpu"):
    """Whole-job figures of N independent replicas (one per rank, weak
    scaling): the slowest rank's timed-region and e2e seconds, and the pairs
    summed over the ranks. One all-reduce of two doubles each way; with no
    process group (one rank) the inputs come back."""
    if dist is None or not dist.is_initialized():
        return t_s, float(pairs), e2e_s, float(e2e_pairs)
    import torch

    tt = torch.tensor([t_s, e2e_s], device=device, dtype=torch.float64)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    pp = torch.tensor([float(pairs), float(e2e_pairs)], device=device, dtype=torch.float64)
    dist.all_reduce(pp, op=dist.ReduceOp.SUM)
    return float(tt[0]), float(pp[0]), float(tt[1]), float(pp[1])


def run_gpu(args, rank: int, world: int, local_rank: int):
    import torch

    from sph2d_gb300 import Solver, cases

    torch.cuda.set_device(local_rank)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    case = cases.piston_flume_2d()
    p = case.params()
    flush = torch.zeros(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    peaks = {}
    pk = ROOT / "MEASURED_PEAKS.json"
    if pk.exists():
        peaks = json.loads(pk.read_text())
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    # ---- mixed step (headline)
    sm = Solver(p, "mixed")
    sm.upload(case.r, case.v, case.rho, case.itype)
    sm.set_time(0.0)
    sm.step_async(1)
    sm.sync()
    pairs_first = sm.pair_count()[0]  # the pairs of the seeded start, which both arms state
    sm.step_async(args.warmup - 1)
    sm.sync()
    clocks = ClockSampler(local_rank)
    diag0 = sm.diagnostics()
    launches0 = sm.kernel_launches()
    rebuilds0 = sm.neighbour_rebuilds()
    _, pairs0 = sm.pair_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    # clocks sampled from the start of the timed steps to the end of the e2e
    # loop (the K timed steps alone last ~K x 0.12 ms, shorter than the
    # sampling interval)
    clocks.start()
    ms_mixed = _loop_ms(sm, args.steps) * args.steps
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = sm.kernel_launches() - launches0
    rebuilds = sm.neighbour_rebuilds() - rebuilds0
    diag1 = sm.diagnostics()
    last_pairs, pairs1 = sm.pair_count()
    pairs_timed = pairs1 - pairs0
    # the same step, each after a 256 MiB write that flushes the L2 (stated beside)
    flushed_steps = min(args.steps, 50)
    _, f0 = sm.pair_count()
    flushed_ms = _time_steps(sm, flush, flushed_steps)
    _, f1 = sm.pair_count()
    phases_mixed = _phase_pass(sm, None, min(args.steps, 50))

    # ---- FP64 step beside it
    steps64 = max(3, min(args.steps, 30))
    s64 = Solver(p, "fp64")
    s64.upload(case.r, case.v, case.rho, case.itype)
    s64.set_time(0.0)
    s64.step_async(max(2, min(args.warmup, 3)))
    s64.sync()
    _, q0 = s64.pair_count()
    ms_fp64 = _loop_ms(s64, steps64) * steps64
    _, q1 = s64.pair_count()
    phases_fp64 = _phase_pass(s64, None, min(steps64, 10))

    # ---- error of the mixed step against the FP64 GPU step (same start, same
    # steps), every field the step writes: state r, v, rho, p and the rates a
    # (accelerations) and drho (zero here: summation density; the continuity
    # rate is stated on the dam break below)
    def _errors(nsteps):
        out = []
        for s in (sm, s64):
            s.upload(case.r, case.v, case.rho, case.itype)
            s.step(nsteps, 0.0)
            out.append({**s.download(), **s.download_rates()})
        a, b = out
        e = {k: _rel(a[k], b[k]) for k in ("r", "v", "rho", "p", "a")}
        e["drho"] = None
        return e

    err_steps = 50
    errors_1 = _errors(1)
    errors = _errors(err_steps)
    errors_cont = continuity_rate_error()

    # ---- end to end through the C ABI with pinned host buffers: each step is
    # one call of the drop-in boundary on host arrays (rrsph_step_host: upload
    # of the state, one step, download of the new state into the same arrays),
    # so the run advances and its list rebuilds fall inside the timed region
    # (as the reference's time_integration would run if called for one step at
    # a time: fresh work arrays at every call)
    pin = lambda x: torch.from_numpy(np.ascontiguousarray(x)).pin_memory().numpy()  # noqa: E731
    n = case.ntotal
    host = {"r": pin(case.r), "v": pin(case.v), "rho": pin(case.rho), "p": pin(np.zeros(n)),
            "itype": pin(case.itype)}
    import ctypes as C

    from sph2d_gb300 import capi

    L = capi.lib()
    dp = lambda x: x.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    ip = lambda x: x.ctypes.data_as(C.POINTER(C.c_int32))  # noqa: E731
    # the call's arguments, made once (the host arrays stay the same): the loop
    # times the C ABI call, not the building of ctypes pointers
    tt = C.c_double(0.0)
    pairs = C.c_uint64()  # the step's pairs, as the call read them back (no device access)
    step_args = (sm.handle, 1, C.byref(tt), dp(host["r"]), 2, dp(host["v"]), dp(host["rho"]), dp(host["p"]),
                 ip(host["itype"]))
    report_args = (sm.handle, None, None, C.byref(pairs), None)

    def e2e_step():
        # r, v, rho, itype in and out (rho read only with continuity density); p out only, as in the reference's
        # loop; the time carries over in tt
        rc = L.rrsph_step_host(*step_args)
        if rc:
            capi.check(rc)
        L.rrsph_last_report(*report_args)
        return pairs.value

    # 200 steps whatever K is (~85 ms): a stall of the host (the GPU machine's
    # cores are shared with other work) weighs little in the mean
    e2e_steps = 200
    for _ in range(max(3, args.warmup)):
        e2e_step()
    rb0 = sm.neighbour_rebuilds()
    itype0 = host["itype"].copy()
    torch.cuda.synchronize()
    e2e_pairs = 0
    e2e_each = []
    import gc

    gc.disable()  # no collector pause of this harness inside the timed loop
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ts = time.perf_counter()
        e2e_pairs += e2e_step()
        e2e_each.append(time.perf_counter() - ts)
    e2e_s = time.perf_counter() - t0
    gc.enable()
    e2e_rebuilds = sm.neighbour_rebuilds() - rb0
    types_changed = not np.array_equal(host["itype"], itype0)
    clocks_info = clocks.stop()
    if clocks_info is not None:
        clocks_info["window"] = "from the timed steps to the end of the e2e loop"
    # r, v, itype (and rho with continuity density: with summation density the step recomputes it)
    h2d = n * (2 * 8 + 2 * 8 + 4 + (8 if p.density_treatment else 0))
    # r, v, rho, p; itype only if a step changed a type (rrsph_step_host rewrites its page-locked
    # itype only then; a changed type stays changed, so the host array shows it)
    d2h = n * (2 * 8 + 2 * 8 + 8 + 8 + (4 if types_changed else 0))

    # ---- aggregate over the replicas (the slowest rank's time, the pairs of all ranks)
    t_s, tot_pairs, e2e_max, e2e_all = aggregate_replicas(ms_mixed / 1e3, pairs_timed, e2e_s, e2e_pairs, dist,
                                                          "cuda")
    e2e_rate = e2e_all / e2e_max
    value = tot_pairs / t_s

    fkey = "forces"
    f_ms = phases_mixed[fkey]
    bytes_launch = FORCES_ALGORITHMIC_BYTES_PER_PARTICLE * n
    achieved = bytes_launch / (f_ms * 1e-3) / 1e9
    design_bytes = FORCES_DESIGN_BYTES_PER_PARTICLE * n + FORCES_DESIGN_BYTES_PER_PAIR * last_pairs
    traffic = _profile_traffic()
    result = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms_mixed / args.steps,
        "l2_flushed": {"ms_per_step": flushed_ms / flushed_steps, "steps": flushed_steps,
                       "pair_interactions_per_s": (f1 - f0) / (flushed_ms / 1e3),
                       "note": "the steps after the timed ones, each after a 256 MiB device write that flushes the "
                               "L2, timed one step per pair of CUDA events"},
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32-pairs/f64-state",
        "data": "synthetic (seeded flume particles of the workload's shape)",
        "config": workload_config(case, pairs_first, args.warmup, args.steps),
        "method": GPU_METHOD,
        "pairs_last_timed_step": int(last_pairs),
        "fp64_step": {
            "ms_per_step": ms_fp64 / steps64,
            "pair_interactions_per_s": (q1 - q0) / (ms_fp64 / 1e3),
            "steps": steps64,
            "mixed_speedup": (ms_fp64 / steps64) / (ms_mixed / args.steps),
            "phases_ms_per_step": phases_fp64,
        },
        "error_vs_fp64_gpu": {"after_1_step": errors_1, f"after_{err_steps}_steps": errors,
                              "continuity_dam_break": errors_cont, "metric": "relative L2",
                              "note": "a = accelerations of the last step; drho is zero on the flume "
                                      "(summation density) and stated on the 2D dam break with continuity "
                                      "density and delta-SPH"},
        "phases_ms_per_step": phases_mixed,
        "roofline": {
            "bound": "hbm",
            "kernel": "k_forces_verlet (force gather + whole step)",
            "achieved": achieved,
            "peak": hbm_peak,
            "unit": "GB/s",
            "frac": achieved / hbm_peak,
            "peak_source": peak_src,
            "traffic": traffic,
            "algorithmic_bytes_per_launch": bytes_launch,
            "algorithmic_bytes_per_particle": FORCES_ALGORITHMIC_BYTES_PER_PARTICLE,
            "avg_launch_ms": f_ms,
            "design_bytes_per_launch": design_bytes,
            "design_gbs": design_bytes / (f_ms * 1e-3) / 1e9,
            "step_frac": 390 * n / (ms_mixed / args.steps * 1e-3) / 1e9 / hbm_peak,
            "note": "achieved = 184 B x particles (force 64 + integrate/piston 96 + key pass 24) / the launch's "
                    "CUDA-event time; design_gbs counts the kernel's own list words and next-step copies; "
                    "step_frac = 390 B x particles per step (the whole step's algorithmic bytes) / ms_per_step",
        },
        "fp32_pipe": {
            "flops_per_pair": FLOPS_PER_PAIR,
            "achieved_tflops": value * FLOPS_PER_PAIR / 1e12,
            "peak_tflops": FP32_PEAK_TFLOPS,
            "frac": value * FLOPS_PER_PAIR / 1e12 / FP32_PEAK_TFLOPS,
            "peak_source": "nominal",
            "note": "whole mixed step; the gathers are latency-bound on L1/L2 neighbour loads (ncu in profiles/)",
        },
        "e2e": {"value": e2e_rate, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "rebuilds": e2e_rebuilds,
                "ms_per_step_median": statistics.median(e2e_each) * 1e3, "ms_per_step_max": max(e2e_each) * 1e3,
                "path": "rrsph_step_host(1) per step on pinned host buffers (upload of r, v, itype: the "
                        "flume's summation density recomputes rho, which the call does not upload; one step; "
                        "download of r, v, rho, p into the same arrays, and itype when a step changed a type, "
                        "which the flume's does not; one wait), each step uploading the state the last one "
                        "returned"},
        "gpu_launches": launches,
        "checks": {
            "fluid_mass_exact": diag1["mass"] == diag0["mass"],
            "fluid_mass": diag1["mass"],
            "energy_before": {k: diag0[k] for k in ("kinetic", "potential", "internal")},
            "energy_after": {k: diag1[k] for k in ("kinetic", "potential", "internal")},
            "note": "rrsph_diagnostics_get before and after the timed steps (double, fixed-order sums)",
        },
        "neighbour_rebuilds": {"timed_steps": args.steps, "rebuilds": rebuilds,
                               "note": "grid + candidate lists rebuilt when a particle moved half the 0.5 h skin"},
        "clocks": clocks_info,
    }
    sm.close()
    s64.close()
    if rank == 0 and world == 1 and not args.no_ensemble:
        result["ensemble"] = ensemble_measure()
    if rank == 0 and world == 1 and not args.no_dam3d:
        result["dam_break_3d"] = dam3d_measure()
    if rank == 0 and world == 1 and not args.no_output:
        result["output_io"] = output_measure()
    if rank == 0 and world == 1 and not args.no_adjoint:
        result["adjoint"] = adjoint_measure(steps=args.adjoint_steps)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(case, p, steps=args.cpu_steps)
    if dist:
        dist.destroy_process_group()
    return result


def ensemble_measure(steps: int = 50, seq_steps: int = 10, ntanks: int = 256) -> dict:
    """Batched ensemble: every tank packed into one mixed-precision solver (one
    graph launch per step for all tanks, gather block sizes and the candidate
    lists' skin from the autotuners) against the same tanks stepped one after
    another, each in its own solver."""
    import torch

    from sph2d_gb300 import Solver, cases

    tanks = cases.ensemble_tanks(ntanks=ntanks)
    ens = cases.pack_tanks(tanks)
    p = ens.params()
    with Solver(p, "mixed") as s:
        s.upload(ens.r, ens.v, ens.rho, ens.itype)
        s.set_wave_makers(ens.notes["wave_makers"])
        s.set_time(0.0)
        s.step_async(3)
        s.sync()
        threads = s.autotune(steps=3)
        skin = s.autotune_skin(steps=30)
        s.step_async(3)
        s.sync()
        _, q0 = s.pair_count()
        ext = torch.cuda.ExternalStream(s.stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(ext)
        s.step_async(steps)
        e1.record(ext)
        s.sync()
        ms = e0.elapsed_time(e1)
        _, q1 = s.pair_count()
        launches = s.kernel_launches()
    seq_ms = 0.0
    seq_pairs = 0
    for c in tanks:
        with Solver(c.params(), "mixed") as s:
            s.upload(c.r, c.v, c.rho, c.itype)
            s.set_wave_makers([c.notes["wave_maker"]])
            s.set_time(0.0)
            s.step_async(5)
            s.sync()
            _, a0 = s.pair_count()
            ext = torch.cuda.ExternalStream(s.stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            s.step_async(seq_steps)
            e1.record(ext)
            s.sync()
            seq_ms += e0.elapsed_time(e1) / seq_steps
            _, a1 = s.pair_count()
            seq_pairs += (a1 - a0) / seq_steps
    batched_rate = (q1 - q0) / (ms / 1e3)
    seq_rate = seq_pairs / (seq_ms / 1e3)
    return {
        "workload": f"{ntanks} independent 2D piston tanks, fluid counts log-uniform 2,000-60,000 (seed 4), depths "
                    "0.2-0.6 m, length = count dx^2 / depth, dx 0.005 m, own piston amplitude 0.01-0.05 m and "
                    "period 1-2 s (seed 5); FP32-mixed step",
        "tanks": ntanks, "particles": ens.ntotal, "fluid_particles": int(ens.notes["nfluid"]),
        "batched": {"ms_per_step": ms / steps, "pair_interactions_per_s": batched_rate, "steps": steps,
                    "gather_threads": {"density": threads[0], "forces": threads[1]}, "skin_over_h": skin},
        "sequential": {"ms_per_step": seq_ms, "pair_interactions_per_s": seq_rate, "steps_per_tank": seq_steps},
        "speedup": seq_ms / (ms / steps),
        "launches_in_batched_region": launches,
    }


def output_measure(steps: int = 400, every: int = 100) -> dict:
    """The flume's FP32-mixed step with the reference's layer output
    (rrsph_run: a data layer every `every` steps, formatted by writer threads
    while the next steps run) against the same steps without output; wall
    time of the whole call, as a user sees it."""
    import shutil
    import tempfile

    import torch

    from sph2d_gb300 import Solver, cases

    case = cases.piston_flume_2d()
    p = case.params()
    p.save_time = every * p.dt
    p.simulation_time = steps * p.dt
    d = tempfile.mkdtemp(prefix="rrsph_run_")
    try:
        with Solver(p, "mixed") as s:
            s.upload(case.r, case.v, case.rho, case.itype)
            s.step(3, 0.0)  # graph capture and first build
            s.upload(case.r, case.v, case.rho, case.itype)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            _, n = s.run(d, 0.0)
            wall_out = time.perf_counter() - t0
            s.upload(case.r, case.v, case.rho, case.itype)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.step(n, 0.0)
            wall_plain = time.perf_counter() - t0
        layers = sorted((Path(d) / "data").glob("*.csv"))
        size = sum(f.stat().st_size for f in layers)
    finally:
        shutil.rmtree(d, ignore_errors=True)
    return {
        "workload": f"2D piston flume, {case.ntotal} particles, {n} steps, a data layer (CSV, 6 decimals) every {every} "
                    "steps as RRSPHOutput writes them",
        "with_output": {"ms_per_step": wall_out / n * 1e3, "layers": len(layers), "layer_bytes": size},
        "without_output": {"ms_per_step": wall_plain / n * 1e3},
        "timing": "wall clock of rrsph_run / rrsph_step over the whole call",
    }


def dam3d_measure(steps: int = 5, fp64_steps: int = 2) -> dict:
    """The 3D dam break at full size: the FP32-mixed step against the plain
    FP64 GPU step on the same uploaded state (each timed with CUDA events on its
    solver's stream over graph replays; the working set is gigabytes, far
    beyond the L2), and the mixed state's relative L2 error against the FP64
    step's after 1 and `steps` steps."""
    import torch

    from sph2d_gb300 import Solver, cases

    case = cases.dam_break_3d()
    p = case.params()
    out = {}
    states = {}
    for prec, n in (("mixed", steps), ("fp64", fp64_steps)):
        with Solver(p, prec) as s:
            s.upload(case.r, case.v, case.rho, case.itype)
            s.step(1, 0.0)
            states[(prec, 1)] = s.download()
            if prec == "mixed":
                s.step(steps - 1, 0.0)
                states[(prec, steps)] = s.download()
            s.upload(case.r, case.v, case.rho, case.itype)
            s.step_async(1)
            s.sync()
            _, q0 = s.pair_count()
            ext = torch.cuda.ExternalStream(s.stream)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(ext)
            s.step_async(n)
            e1.record(ext)
            s.sync()
            ms = e0.elapsed_time(e1) / n
            _, q1 = s.pair_count()
            out[prec] = {"ms_per_step": ms, "pair_interactions_per_s": (q1 - q0) / n / (ms / 1e3), "steps": n,
                         "pairs_per_step": (q1 - q0) / n}
    with Solver(p, "fp64") as s:  # the FP64 reference state after `steps` steps
        s.upload(case.r, case.v, case.rho, case.itype)
        s.step(steps, 0.0)
        states[("fp64", steps)] = s.download()
    err = {f"after_{k}_steps": {f: _rel(states[("mixed", k)][f], states[("fp64", k)][f]) for f in ("r", "v", "rho", "p")}
           for k in (1, steps)}
    return {
        "workload": f"3D dam break: tank 1.6 x 0.67 x 0.6 m, block 0.4 x 0.67 x 0.3 m at dx 2.6 mm, h 1.3 dx, "
                    f"LJ walls at dx/2, continuity density; {case.ntotal} particles ({int(case.notes['nfluid'])} fluid)",
        "mixed": out["mixed"], "fp64": out["fp64"],
        "mixed_speedup": out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"],
        "error_vs_fp64_gpu": dict(err, metric="relative L2"),
        "timing": "inputs larger than L2 (no flush)",
    }


def adjoint_measure(steps: int = 500, checkpoint_every: int = 100) -> dict:
    """Cost of d(gauge misfit)/d(piston Fourier coefficients) against a
    forward run: the 2D adjoint flume (2000 x 100 fluid at dx 0.005 m, 8
    Fourier coefficients), FP64."""
    import torch

    from sph2d_gb300 import Solver, cases

    case = cases.adjoint_flume_2d(steps=steps)
    p = case.params()
    om, coef = case.notes["omega"], case.notes["coef"]
    sf, se = case.notes["sample_from"], case.notes["sample_every"]
    with Solver(p, "fp64") as s:
        s.upload(case.r, case.v, case.rho, case.itype)
        s.set_piston_fourier(om, case.notes["target_coef"])
        target, _ = s.adjoint_forward(steps, case.notes["gauge_x"], sf, se, checkpoint_every)
        s.upload(case.r, case.v, case.rho, case.itype)
        s.set_piston_fourier(om, coef)
        s.step(5, 0.0)
        s.upload(case.r, case.v, case.rho, case.itype)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.step(steps, 0.0)
        fwd = time.perf_counter() - t0
        s.upload(case.r, case.v, case.rho, case.itype)
        t0 = time.perf_counter()
        g, _ = s.adjoint_forward(steps, case.notes["gauge_x"], sf, se, checkpoint_every)
        t1 = time.perf_counter()
        dcoef, _ = s.adjoint_reverse(2.0 * (g - target) / len(g))
        t2 = time.perf_counter()
    return {
        "workload": f"2D adjoint flume, {case.ntotal} particles (2000 x 100 fluid, 10 m x 0.5 m at dx 0.005 m), "
                    f"8 Fourier piston coefficients (seed 2, target seed 3), gauge x = {case.notes['gauge_x']} m, "
                    f"{len(g)} samples every {se} steps over the last {case.notes['window']} s; {steps} steps, "
                    f"checkpoints every {checkpoint_every}",
        "forward_s": fwd, "adjoint_forward_s": t1 - t0, "adjoint_reverse_s": t2 - t1,
        "gradient_cost_vs_forward": (t2 - t0) / fwd,
        "loss": float(np.mean((g - target) ** 2)), "dloss_dcoef": [float(x) for x in dcoef],
    }


def _profile_traffic():
    """DRAM bytes per launch of the force kernel from the committed ncu summary."""
    f = ROOT / "profiles" / "forces_reuse_flume.txt"
    if not f.exists():
        return None
    for line in f.read_text().splitlines():
        if line.startswith("traffic_bytes_per_launch_full_size:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ---------------------------------------------------------- CPU arms -------

def continuity_rate_error(steps: int = 1) -> dict:
    """Per-field error of the FP32-mixed step against the FP64 GPU step on the
    2D dam break with continuity density and delta-SPH (coefficient 0.1), after
    `steps` steps from the seeded start: r, v, rho, p, a and drho."""
    from sph2d_gb300 import Solver, cases

    case = cases.dam_break_2d(density_treatment=1)
    p = case.params()
    p.density_treatment = 2
    p.density_delta_sph_coef = 0.1
    out = []
    for prec in ("mixed", "fp64"):
        with Solver(p, prec) as s:
            s.upload(case.r, case.v, case.rho, case.itype)
            s.step(steps, 0.0)
            out.append({**s.download(), **s.download_rates()})
    a, b = out
    return {k: _rel(a[k], b[k]) for k in ("r", "v", "rho", "p", "a", "drho")}


REF_PHASES = ("predict", "grid_find", "density", "accel", "whole")


def reference_timing(case, p, warmup: int, steps: int, threads: int = 0) -> dict:
    """The reference's CPU implementation of the step on `threads` host threads
    (0: all cores), over `warmup` untimed and `steps` timed steps from the
    seeded start: the
    reference's own RRSPH_OMP compute core (oracle/_ref/rrsph_ref, built from
    its sources) where it was built, else the C restatement of it (oracle/).
    Time = the sum of the timed steps' wall times (no I/O)."""
    from oracle import binding as O

    threads = threads or os.cpu_count() or 1
    total = warmup + steps
    phases = None
    if O.ref_available():
        out = O.ref_run(p, f"run:{total}", case.r, case.v, case.rho, case.itype, threads=threads, timeout=3600)
        step_ms = out["step_ms"]
        pairs = out["pairs"].astype(np.int64)
        cores = int(out["timing"]["threads"])
        kind = "reference"
        what = "the reference's RRSPH_OMP compute core built from its sources (oracle/_ref/rrsph_ref)"
        if "phase_ms" in out:
            mean = out["phase_ms"][warmup:total].mean(axis=0)
            phases = dict(zip(REF_PHASES, (float(x) for x in mean)))
    else:
        O.set_threads(threads)
        res = O.run(p, case.r, case.v, case.rho, case.itype, nsteps=warmup) if warmup else None
        st = res or {"r": case.r, "v": case.v, "rho": case.rho, "itype": case.itype, "p": None, "a": None,
                     "drho": None, "time": 0.0, "pairs_each": np.zeros(0, dtype=np.uint64)}
        t0 = time.perf_counter()
        res2 = O.run(p, st["r"], st["v"], st["rho"], st["itype"], nsteps=steps, time=st["time"], pres=st["p"],
                     a=st["a"], drho=st["drho"], itimestep=warmup)
        wall_ms = (time.perf_counter() - t0) * 1e3
        pairs = np.concatenate([st["pairs_each"], res2["pairs_each"]]).astype(np.int64)
        step_ms = np.concatenate([np.zeros(warmup), np.full(steps, wall_ms / steps)])
        cores = O.threads()
        kind = "port"
        what = "the C restatement of RRSPH_OMP (oracle/rrsph_oracle.c, OpenMP)"
    t_ms = float(np.sum(step_ms[warmup:total]))
    timed_pairs = int(np.sum(pairs[warmup:total]))
    return {"kind": kind, "cores": cores, "ms_per_step": t_ms / steps, "value": timed_pairs / (t_ms / 1e3),
            "pairs_first": int(pairs[0]), "pairs_timed": timed_pairs, "phases_ms_per_step": phases,
            "sample": f"steps {warmup + 1}-{total} of the {case.ntotal}-particle flume from the seeded start on "
                      f"{cores} threads: {what}; directed pairs of those steps / the sum of their wall times"}


def cpu_baseline(case, p, steps: int, one_thread_steps: int = 2) -> dict:
    """The reference's CPU step beside the GPU arm: a bounded sample of the
    same workload (its first `steps` steps after one warm-up step) on all host
    cores, with its per-phase times, and a shorter sample on one thread."""
    r = reference_timing(case, p, 1, steps)
    out = {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": r["kind"], "sample": r["sample"],
           "ms_per_step": r["ms_per_step"], "phases_ms_per_step": r["phases_ms_per_step"]}
    if one_thread_steps > 0 and r["kind"] == "reference":
        r1 = reference_timing(case, p, 1, one_thread_steps, threads=1)
        out["one_thread"] = {"value": r1["value"], "ms_per_step": r1["ms_per_step"],
                             "phases_ms_per_step": r1["phases_ms_per_step"], "sample": r1["sample"]}
    return out


def run_reference(args, rank: int, world: int) -> dict | None:
    """The reference arm: the reference's CPU implementation of the step on the
    host cores, on the same workload and step window as the GPU arm. It loads
    neither the sph2d_gb300 package nor its library: the particles come from
    the workload generator loaded as a plain module, the parameters from the
    oracle's own restatement of the reference's loading (oracle/params.py)."""
    if rank != 0:
        return None
    from oracle import build as ob

    ob.build_all()
    from oracle import params as OP

    cases = load_cases()
    case = cases.piston_flume_2d()
    p = OP.case_params(case)
    r = reference_timing(case, p, args.warmup, args.steps)
    value = r["value"]
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded flume particles of the workload's shape)",
        "config": workload_config(case, r["pairs_first"], args.warmup, args.steps),
        "method": {"precision": "f64 (the reference's rr_float)", "neighbour_search": "grid + stencil every step",
                   "threads": r["cores"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": r["cores"], "kind": r["kind"], "sample": r["sample"],
                         "phases_ms_per_step": r["phases_ms_per_step"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-steps", type=int, default=50,
                    help="timed steps of the in-run CPU baseline (the reference's step on the host cores)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-ensemble", action="store_true", help="skip the 256-tank ensemble measurement")
    ap.add_argument("--no-dam3d", action="store_true", help="skip the 3D dam break measurement")
    ap.add_argument("--no-output", action="store_true", help="skip the run with layer output")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint cost measurement")
    ap.add_argument("--adjoint-steps", type=int, default=500)
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        ap.error("--warmup must be >= 3")
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", str(args.gpus)))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if "WORLD_SIZE" not in os.environ:
        world = 1 if args.gpus <= 1 else args.gpus
        if world > 1:
            raise SystemExit("for --gpus N > 1 launch with torch.distributed.run (one rank per GPU)")
    if args.impl == "reference":
        res = run_reference(args, rank, world)
    else:
        import __graft_entry__

        __graft_entry__.build()
        res = run_gpu(args, rank, world, local_rank)
    if rank == 0 and res is not None:
        print(json.dumps(res), flush=True)


if __name__ == "__main__":
    main()
