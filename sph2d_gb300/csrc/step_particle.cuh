// step_particle.cuh — the per-particle pieces of the time step that more than
// one kernel runs: the geometry test, the key pass, predict_half_step, the
// piston laws and the whole step of one particle. The whole-step kernel runs
// them over all particles; the fused force + whole-step gather of the mixed
// step with neighbour reuse runs them for the particle whose acceleration it
// has just summed.
#pragma once

#include "kernels.cuh"
#include "neighbour.cuh"

namespace rrsph {
namespace {

// predict_half_step (RRSPH_OMP/src/PredictHalfStep.cpp:4-23) fused with the
// key pass of make_grid (RRSPH_OMP/src/GridFind.cpp:55-75). Also clears the
// cell-table entries of the previous grid (key_of) so that the table needs no
// max_cells-sized reset.
// Cell key of particle i at (x, y, z) (GridFind.cpp:55-75); also clears the
// previous grid's cell-table entry of i and records the new key.
// Strictly inside the geometry box (WholeStep.cpp:4-17, ConsistencyCheck.cpp:162-218),
// the double compares done on the ordered bit patterns (a NaN is outside).
template <int DIM>
__device__ __forceinline__ bool in_geometry(const DevParams& P, double x, double y, double z) {
    const long long ox = dorder(x), oy = dorder(y);
    bool in = ox < P.oxmax && ox > P.oxmin && oy < P.oymax && oy > P.oymin && !dnan(x) && !dnan(y);
    if (DIM == 3) {
        const long long oz = dorder(z);
        in = in && oz < P.ozmax && oz > P.ozmin && !dnan(z);
    }
    return in;
}

// Compile-time variants of the per-particle kernels. A switch that is off in
// a variant leaves no instructions behind: the FP64 pipe (one lane per clock
// per SM on this part) also issues the predicated-off double instructions of
// small if-converted branches.
enum : int { kVarCont = 1, kVarRare = 2, kVarMixed = 4 };  // continuity, XSPH or dynamic dt, FP32-mixed
// M: 0 = FP64 step, 1 = FP32-mixed step, 2 = decided at run time from the state's buffers.

// Neighbour reuse, in the key pass of particle i: the next step's cell-order
// copies at the particle's slot of the last build, with (px, py, pz) its offset
// from the edge of its build cell (a step that rebuilds overwrites them in its
// new order). With continuity density V4.w is rho_predict and VD4 = (v,
// rho - rho0), as the reorder writes them.
template <int DIM>
__device__ __forceinline__ void reuse_copies(const DevParams& P, const State& S, const Sorted& G, uint32_t i,
                                             float px, float py, float pz) {
    const uint32_t k = S.slot[i];
    G.P4n[k] = make_float4(px, py, pz, __int_as_float(S.itype[i]));
    float4 v;
    if (DIM == 3) {
        v = S.vpf4[i];
        v.w = 0.0f;
    } else {
        const float2 v2 = S.vpf2[i];
        v = make_float4(v2.x, v2.y, 0.0f, 0.0f);  // .zw (summation): the density pass writes them
    }
    if (G.VD4n) {
        v.w = d2f(S.rho_pred[i]);
        G.VD4n[k] = vd4_of<DIM>(S.vx[i], S.vy[i], DIM == 3 ? S.vz[i] : 0.0, S.rho[i] - P.rho0);
    }
    G.V4n[k] = v;
}
// A particle that moved more than half the skin since the build asks for a
// rebuild (one atomic per warp).
__device__ __forceinline__ void reuse_check(const State& S, bool moved) {
    const unsigned am = __activemask();
    const unsigned who = __ballot_sync(am, moved);
    if (who && (threadIdx.x & 31) == (unsigned)(__ffs(am) - 1)) atomicOr(S.vl_rebuild, 1u);
}

template <int DIM, int M>
__device__ __forceinline__ void key_pass(const DevParams& P, const State& S, const Sorted& G, uint32_t i, double x,
                                         double y, double z, uint32_t* __restrict__ flags) {
    const CellSplit sx = cell_split(x, P.xmin, P.cell, P.inv_cell, P.mf.cell);
    const CellSplit sy = cell_split(y, P.ymin, P.cell, P.inv_cell, P.mf.cell);
    bool outside = sx.below || sy.below;
    uint64_t key;
    CellSplit sz{0, 0.0f, false};
    if (DIM == 3) {
        sz = cell_split(z, P.zmin, P.cell, P.inv_cell, P.mf.cell);
        outside = outside || sz.below;
        key = split3(sx.c) | (split3(sy.c) << 1) | (split3(sz.c) << 2);
    } else {
        key = split2(sx.c) | (split2(sy.c) << 1);
    }
    if (key >= P.max_cells || outside) {
        // cell_idx >= max_cells (GridFind.cpp:61-72); keep kernels in bounds
        if (P.consistency_check || key >= P.max_cells) atomicOr(flags, RRSPH_FLAG_OUT_OF_DOMAIN);
        if (key >= P.max_cells) key = P.max_cells - 1;
    }
    const uint32_t old = S.key_of[i];
    if (old < P.max_cells && !P.keep_cells) G.cell_start[old] = kEmpty;
    S.key_of[i] = (uint32_t)key;
    G.keys_in[i] = (uint32_t)key;
    G.ids_in[i] = i;
    if (M == 0 && !(DIM == 3 ? (void*)S.coff4 : (void*)S.coff2)) return;
    // offsets from the edge of the cell the key names: the Morton code keeps 16
    // bits per axis in 2D and 10 in 3D (GridUtils.h:50-64, 92-104). A cell
    // coordinate whose key lies in the grid fits in 32 bits, so the dropped bits
    // convert from 32 bits (a 64-bit integer conversion would take the FP64 pipe);
    // beyond that the key is out of the domain and the step fails.
    if (DIM == 2 && (M == 1 || S.coff2)) {
        const float ox = sx.off + (float)(uint32_t)(sx.c & ~0xFFFFull) * P.mf.cell;
        const float oy = sy.off + (float)(uint32_t)(sy.c & ~0xFFFFull) * P.mf.cell;
        S.coff2[i] = make_float2(ox, oy);
        if (S.cxy) {  // neighbour reuse: the current cell, and the displacement since the list build
            const uint32_t cx = (uint32_t)(sx.c & 0xFFFFu), cy = (uint32_t)(sy.c & 0xFFFFu);
            S.cxy[i] = cx | (cy << 16);
            const uint32_t b = S.bcxy[i];
            const float2 bo = S.boff[i];
            // offset from the edge of the cell the particle had at the build
            const float px = ox + (float)((int)cx - (int)(b & 0xFFFFu)) * P.mf.cell;
            const float py = oy + (float)((int)cy - (int)(b >> 16)) * P.mf.cell;
            reuse_copies<DIM>(P, S, G, i, px, py, 0.0f);
            const float dx = px - bo.x, dy = py - bo.y;
            reuse_check(S, !(dx * dx + dy * dy <= P.vl_half_skin2));
        }
    } else if (DIM == 3 && (M == 1 || S.coff4)) {
        const float ox = sx.off + (float)(uint32_t)(sx.c & ~0x3FFull) * P.mf.cell;
        const float oy = sy.off + (float)(uint32_t)(sy.c & ~0x3FFull) * P.mf.cell;
        const float oz = sz.off + (float)(uint32_t)(sz.c & ~0x3FFull) * P.mf.cell;
        S.coff4[i] = make_float4(ox, oy, oz, 0.0f);
        if (S.cxy) {
            const uint32_t cx = (uint32_t)(sx.c & 0x3FFu), cy = (uint32_t)(sy.c & 0x3FFu),
                           cz = (uint32_t)(sz.c & 0x3FFu);
            S.cxy[i] = cx | (cy << 10) | (cz << 20);
            const uint32_t b = S.bcxy[i];
            const float4 bo = S.boff4[i];
            const float px = ox + (float)((int)cx - (int)(b & 0x3FFu)) * P.mf.cell;
            const float py = oy + (float)((int)cy - (int)((b >> 10) & 0x3FFu)) * P.mf.cell;
            const float pz = oz + (float)((int)cz - (int)(b >> 20)) * P.mf.cell;
            reuse_copies<DIM>(P, S, G, i, px, py, pz);
            const float dx = px - bo.x, dy = py - bo.y, dz = pz - bo.z;
            reuse_check(S, !(dx * dx + dy * dy + dz * dz <= P.vl_half_skin2));
        }
    }
}

// predict_half_step (PredictHalfStep.cpp:4-23) of particle i with time step
// dt; the mixed step keeps v_predict in float only.
template <int DIM, int M, bool CONT>
__device__ __forceinline__ void predict(const DevParams& P, const State& S, uint32_t i, double vx, double vy,
                                        double vz, double rho, double dt, double ax, double ay, double az) {
    const bool mixed = M == 1 || (M == 2 && (DIM == 2 ? S.vpf2 != nullptr : S.vpf4 != nullptr));
    if (M != 0 && mixed) {  // v* = v + a dt/2 in float: the forces read it in float
        const float hf = d2f(dhalf(dt));
        if (DIM == 2) {
            S.vpf2[i] = make_float2(fmaf(d2f(ax), hf, d2f(vx)), fmaf(d2f(ay), hf, d2f(vy)));
        } else {
            S.vpf4[i] = make_float4(fmaf(d2f(ax), hf, d2f(vx)), fmaf(d2f(ay), hf, d2f(vy)),
                                    fmaf(d2f(az), hf, d2f(vz)), 0.0f);
        }
    } else if (M != 1) {  // the reference's v + (a dt) * 0.5
        S.vpx[i] = vx + __dmul_rn(ax, dt) * 0.5;
        S.vpy[i] = vy + __dmul_rn(ay, dt) * 0.5;
        if (DIM == 3) S.vpz[i] = vz + __dmul_rn(az, dt) * 0.5;
    }
    if (CONT) S.rho_pred[i] = rho + __dmul_rn(S.drho[i], dt) * 0.5;
}


// Piston velocity of dynamic_boundaries (RRSPH_OMP/src/WaveMaker.cpp:34-82)
// for one set of wave-maker parameters.
__device__ inline double piston_law_vx(int nwm, double phase, double freq, double H, double k, double depth,
                                double time_start, double time) {
    const double delta = phase - freq * time_start;
    const double omega = freq;
    const double kd = k * depth;
    const double sh = sinh(kd), ch = cosh(kd);
    const double m1 = 2 * (sh * sh) / (sh * ch + kd);
    const double S0 = H / m1;
    double vx = 0.5 * S0 * omega * cos(omega * time + delta);
    if (nwm == 3) {
        const double e2_1 = (H * H) / (32 * depth);
        const double e2_2 = 3 * ch / (sh * sh * sh) - 2 / m1;
        vx += 2 * omega * (e2_1 + e2_2) * cos(2 * omega * time + 2 * delta);
    }
    return vx;
}

// The params' piston, or X'(t) of the Fourier piston X(t) = sum_k c_k
// sin(k omega t) when one is set.
__device__ inline double piston_vx(const DevParams& P, double time) {
    if (P.fourier_n > 0) {
        double vx = 0;
        for (int k = 1; k <= P.fourier_n; k++) {
            const double phi = k * P.fourier_omega * cos(k * P.fourier_omega * time);
            vx += P.fourier_coef[k - 1] * phi;
        }
        return vx;
    }
    return piston_law_vx(P.nwm, P.nwm_phase, P.nwm_freq, P.nwm_H, P.nwm_k, P.depth, P.nwm_time_start, time);
}

// Piston velocity of nwm_solitary_rayleigh (WaveMaker.cpp:84-134).
__device__ inline double solitary_vx(const DevParams& P, double time) {
    const double H = P.nwm_H, h = P.depth, g = P.g;
    const double k = sqrt(3 * H / (4 * (h * h) * (H + h)));
    const double c = sqrt(g * (H + h));
    const double Tf = 2 / (k * c) * (3.8 + H / h);
    const double tau = k * c * (time - Tf);
    const double u = tanh(tau);
    const double top = k * H * (h + H - H * (u * u)) + 2 * k * ((H * u) * (H * u));
    const double b = k * (h + H - H * (u * u));
    const double dxdu = top / (b * b);
    const double th = tanh(tau);
    return dxdu * (1 - th * th) * (k * c);
}

// dt of the step: scal->dt, or update_dt (UpdateAcceleration.cpp:15-29) under
// DT_CORRECTION_DYNAMIC (with the step's maxima when dt_reduce is set). One
// thread (first) reports a never-ending dt.
template <bool RARE>
__device__ __forceinline__ double step_dt(const DevParams& P, const StepScalars* __restrict__ scal,
                                          uint32_t* __restrict__ flags, bool first) {
    double dt = scal->dt;
    if (RARE && P.dt_method == 2) {
        const double amax = P.dt_reduce ? __longlong_as_double((long long)scal->amax_bits) : 0.0;
        const double mumax = P.dt_reduce ? __longlong_as_double((long long)scal->mumax_bits) : 0.0;
        const double min_dt_a = sqrt(P.h / amax);
        const double min_dt_mu = P.h / (P.c_eos + mumax);
        dt = P.cfl * fmin(min_dt_a, min_dt_mu);
        if (dt <= P.never_ending_dt && first) atomicOr(flags, RRSPH_FLAG_NEVER_ENDING);
    }
    return dt;
}

// The next step's scalars (time += dt, step + 1, counters reset), by one thread.
__device__ __forceinline__ void advance_scalars(const DevParams& P, const StepScalars* __restrict__ scal,
                                                StepScalars* __restrict__ next, double dt) {
    const double time = scal->time;
    next->time = time + dt;
    next->dt = dt;
    next->step = scal->step + 1;
    next->amax_bits = 0;
    next->mumax_bits = 0;
    next->pairs = 0;
    next->nwm_off = scal->nwm_off || (P.nwm == 4 && time >= P.nwm_time_start) ? 1ull : 0ull;
    next->pairs_total = scal->pairs_total + scal->pairs;
}

// The per-particle part of k_whole: make_waves for particle i, whole_step,
// the boundary check and (next_keys) the next step's predictor + key pass,
// with the acceleration (ax, ay, az) of this step's force evaluation.
template <int DIM, int V>
__device__ __forceinline__ void whole_particle(const DevParams& P, const State& S, const Sorted& G, uint32_t i,
                                               double dt, const StepScalars* __restrict__ scal,
                                               uint32_t* __restrict__ flags, int next_keys, double ax, double ay,
                                               double az) {
    constexpr bool CONT = (V & kVarCont) != 0, RARE = (V & kVarRare) != 0;
    constexpr int M = (V & kVarMixed) ? 1 : 0;
    const double time = scal->time;
    const unsigned long long nwm_off = scal->nwm_off;
    const bool waves = P.nwm && !nwm_off && dorder(time) >= dorder(P.nwm_time_start);
    if (S.wave_tank) {  // a table of pistons (one per tank of an ensemble)
        const int32_t w = S.wave_tank[i];
        if (w >= 0) {
            const PistonLaw L = S.wave_law[w];
            if (time >= L.time_start) {
                const double vx = piston_law_vx(L.nwm, L.phase, L.freq, L.H, L.k, L.depth, L.time_start, time);
                S.rx[i] = S.rx[i] + vx * dt;
                S.vx[i] = vx;
            }
        }
    } else if (waves && P.nwm_valid && i >= P.nwm_start && i < P.nwm_end) {
        if (P.nwm == 2 || P.nwm == 3 || P.nwm == 5) {
            const double vx = P.nwm == 5 ? solitary_vx(P, time) : piston_vx(P, time);
            S.rx[i] = S.rx[i] + vx * dt;
            S.vx[i] = vx;
        } else if (P.nwm == 4) {
            S.itype[i] = P.type_non_existent;
            atomicOr(S.itype_changed, 1u);
        }
    }
    const double v_dt = scal->step ? dt : dhalf(dt);
    double rho = 0.0;
    if (CONT) {
        rho = S.rho[i] + S.drho[i] * v_dt;
        S.rho[i] = rho;
    }
    double x = S.rx[i], y = S.ry[i], z = DIM == 3 ? S.rz[i] : 0.0;
    double vx = S.vx[i], vy = S.vy[i], vz = DIM == 3 ? S.vz[i] : 0.0;
    bool in = true, in_known = false;  // the geometry test of the final position, once
    if (S.itype[i] > 0) {
        vx = vx + ax * v_dt;
        vy = vy + ay * v_dt;
        if (DIM == 3) vz = vz + az * v_dt;
        if (RARE && P.avg_vel) {
            vx += S.avx[i];
            vy += S.avy[i];
            if (DIM == 3) vz += S.avz[i];
        }
        S.vx[i] = vx;
        S.vy[i] = vy;
        if (DIM == 3) S.vz[i] = vz;
        const double nx = x + vx * dt, ny = y + vy * dt, nz = DIM == 3 ? z + vz * dt : 0.0;
        bool move = true;
        if (P.consistency_treatment == 2 || P.consistency_check) {
            in = in_geometry<DIM>(P, nx, ny, nz);
            in_known = true;
            if (P.consistency_treatment == 2 && !in) {  // CONSISTENCY_FIX (WholeStep.cpp:47-54)
                move = false;
                in_known = false;
                S.itype[i] = P.type_non_existent;
                atomicOr(S.itype_changed, 1u);
            }
        }
        if (move) {
            x = nx; y = ny; z = nz;
            S.rx[i] = x;
            S.ry[i] = y;
            if (DIM == 3) S.rz[i] = z;
        }
    }
    if (P.consistency_check) {  // check_particles_are_within_boundaries (ConsistencyCheck.cpp:147-218)
        if (!in_known) in = in_geometry<DIM>(P, x, y, z);
        if (!in) atomicOr(flags, RRSPH_FLAG_OUTSIDE_GEOMETRY);
    }
    if (next_keys) {
        // the next step's predict_half_step and cell keys, from the state just written
        predict<DIM, M, CONT>(P, S, i, vx, vy, vz, rho, dt, ax, ay, az);
        key_pass<DIM, M>(P, S, G, i, x, y, z, flags);
    }
}

}  // namespace
}  // namespace rrsph
