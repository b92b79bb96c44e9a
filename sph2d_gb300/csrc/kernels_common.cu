// kernels_common.cu — per-particle kernels of the step that are not pair
// gathers: predict + cell keys, reorder + cell table, whole step + piston,
// and the grid/neighbour exports used by parity checks.
#include "kernels.cuh"
#include "neighbour.cuh"

namespace rrsph {

namespace {

inline unsigned blocks_for(uint32_t n, int threads) { return (n + threads - 1) / threads; }

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
    if (old < P.max_cells) G.cell_start[old] = kEmpty;
    S.key_of[i] = (uint32_t)key;
    G.keys_in[i] = (uint32_t)key;
    G.ids_in[i] = i;
    if (M == 0) return;
    // offsets from the edge of the cell the key names: the Morton code keeps 16
    // bits per axis in 2D and 10 in 3D (GridUtils.h:50-64, 92-104)
    if (DIM == 2 && (M == 1 || S.coff2)) {
        const float ox = sx.off + (float)(sx.c & ~0xFFFFull) * P.mf.cell;
        const float oy = sy.off + (float)(sy.c & ~0xFFFFull) * P.mf.cell;
        S.coff2[i] = make_float2(ox, oy);
        if (S.cxy) {  // neighbour reuse: the current cell, and the displacement since the list build
            const uint32_t cx = (uint32_t)(sx.c & 0xFFFFu), cy = (uint32_t)(sy.c & 0xFFFFu);
            S.cxy[i] = cx | (cy << 16);
            const uint32_t b = S.bcxy[i];
            const float2 bo = S.boff[i];
            // offset from the edge of the cell the particle had at the build
            const float px = ox + (float)((int)cx - (int)(b & 0xFFFFu)) * P.mf.cell;
            const float py = oy + (float)((int)cy - (int)(b >> 16)) * P.mf.cell;
            // the next step's cell-order copies, at the particle's slot of the build
            // (a step that rebuilds overwrites them in its new order)
            const uint32_t k = S.slot[i];
            G.P4[k] = make_float4(px, py, 0.0f, __int_as_float(S.itype[i]));
            const float2 v = S.vpf2[i];
            G.V4[k] = make_float4(v.x, v.y, 0.0f, 0.0f);  // .zw: the density pass writes them
            const float dx = px - bo.x, dy = py - bo.y;
            const bool moved = !(dx * dx + dy * dy <= P.vl_half_skin2);
            const unsigned am = __activemask();
            const unsigned who = __ballot_sync(am, moved);
            if (who && (threadIdx.x & 31) == (unsigned)(__ffs(am) - 1)) atomicOr(S.vl_rebuild, 1u);
        }
    } else if (DIM == 3 && (M == 1 || S.coff4)) {
        const float ox = sx.off + (float)(sx.c & ~0x3FFull) * P.mf.cell;
        const float oy = sy.off + (float)(sy.c & ~0x3FFull) * P.mf.cell;
        const float oz = sz.off + (float)(sz.c & ~0x3FFull) * P.mf.cell;
        S.coff4[i] = make_float4(ox, oy, oz, 0.0f);
    }
}

// predict_half_step (PredictHalfStep.cpp:4-23) of particle i with time step
// dt; the mixed step keeps v_predict in float only.
template <int DIM, int M, bool CONT>
__device__ __forceinline__ void predict(const DevParams& P, const State& S, uint32_t i, double vx, double vy,
                                        double vz, double rho, double dt) {
    const bool mixed = M == 1 || (M == 2 && (DIM == 2 ? S.vpf2 != nullptr : S.vpf4 != nullptr));
    if (M != 0 && mixed) {  // v* = v + a dt/2 in float: the forces read it in float
        const float hf = d2f(dhalf(dt));
        if (DIM == 2) {
            S.vpf2[i] = make_float2(fmaf(d2f(S.ax[i]), hf, d2f(vx)), fmaf(d2f(S.ay[i]), hf, d2f(vy)));
        } else {
            S.vpf4[i] = make_float4(fmaf(d2f(S.ax[i]), hf, d2f(vx)), fmaf(d2f(S.ay[i]), hf, d2f(vy)),
                                    fmaf(d2f(S.az[i]), hf, d2f(vz)), 0.0f);
        }
    } else if (M != 1) {  // the reference's v + (a dt) * 0.5
        S.vpx[i] = vx + __dmul_rn(S.ax[i], dt) * 0.5;
        S.vpy[i] = vy + __dmul_rn(S.ay[i], dt) * 0.5;
        if (DIM == 3) S.vpz[i] = vz + __dmul_rn(S.az[i], dt) * 0.5;
    }
    if (CONT) S.rho_pred[i] = rho + __dmul_rn(S.drho[i], dt) * 0.5;
}

template <int DIM>
__global__ void k_keys(DevParams P, State S, Sorted G, const StepScalars* __restrict__ scal, int do_predict,
                       uint32_t* __restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    if (do_predict) {
        if (P.density_treatment)
            predict<DIM, 2, true>(P, S, i, S.vx[i], S.vy[i], DIM == 3 ? S.vz[i] : 0.0, S.rho[i], scal->dt);
        else
            predict<DIM, 2, false>(P, S, i, S.vx[i], S.vy[i], DIM == 3 ? S.vz[i] : 0.0, 0.0, scal->dt);
    }
    key_pass<DIM, 2>(P, S, G, i, S.rx[i], S.ry[i], DIM == 3 ? S.rz[i] : 0.0, flags);
}

// Gathers the state into cell order and records each cell's [start, end) in
// the sorted arrays (the cells_start table of make_grid, GridFind.cpp:77-87).
// R: 0 = FP64 gathers; 1 = the mixed loop with summation density; 2 = the
// mixed loop with continuity density; 3 = mixed, outside the loop (the
// velocities, density and pressure given by F, double copies for exports).
template <int DIM, int R>
__global__ void k_reorder(DevParams P, State S, Sorted G, GatherSrc F) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const uint32_t key = G.key[k];
    const uint32_t id = G.id[k];
    if (k == 0 || G.key[k - 1] != key) G.cell_start[key] = k;
    if (k == P.n - 1 || G.key[k + 1] != key) G.cell_end[key] = k + 1;
    const int32_t t = S.itype[id];
    if (R == 0 || R == 3) {  // double copies: the FP64 gathers and the grid/neighbour exports
        G.rx[k] = S.rx[id];
        G.ry[k] = S.ry[id];
        if (DIM == 3) G.rz[k] = S.rz[id];
        G.itype[k] = t;
    }
    if (R == 0) {
        G.vx[k] = F.vx[id];
        G.vy[k] = F.vy[id];
        if (DIM == 3) G.vz[k] = F.vz[id];
        G.rho[k] = F.rho[id];
        if (F.p) G.p[k] = F.p[id];
        if (P.density_treatment != 0) {
            G.vdx[k] = S.vx[id];
            G.vdy[k] = S.vy[id];
            if (DIM == 3) G.vdz[k] = S.vz[id];
            G.rhod[k] = S.rho[id];
        }
        return;
    }
    // FP32-mixed: cell-relative offsets the key pass computed from the same positions
    float ox, oy, oz = 0.0f;
    if (DIM == 2) {
        const float2 o = S.coff2[id];
        ox = o.x;
        oy = o.y;
    } else {
        const float4 o = S.coff4[id];
        ox = o.x;
        oy = o.y;
        oz = o.z;
    }
    G.P4[k] = make_float4(ox, oy, oz, __int_as_float(t));
    float fvx, fvy, fvz = 0.0f, frho = 0.0f;  // the loop's summation density writes .w itself
    if (R != 3) {  // v_predict in float from the predictor
        if (DIM == 2) {
            const float2 v = S.vpf2[id];
            fvx = v.x;
            fvy = v.y;
        } else {
            const float4 v = S.vpf4[id];
            fvx = v.x;
            fvy = v.y;
            fvz = v.z;
        }
        if (R == 2) frho = d2f(F.rho[id]);
    } else {
        fvx = d2f(F.vx[id]);
        fvy = d2f(F.vy[id]);
        if (DIM == 3) fvz = d2f(F.vz[id]);
        frho = d2f(F.rho[id]);
        if (F.p) G.PR[k] = make_float2(d2f(F.p[id]), d2f(F.p[id] / (F.rho[id] * F.rho[id])));
    }
    G.V4[k] = make_float4(fvx, fvy, fvz, frho);
    if (R == 2 || (R == 3 && P.density_treatment != 0))  // rho - rho0 keeps rho_i - rho_j accurate in float
        G.VD4[k] = make_float4(d2f(S.vx[id]), d2f(S.vy[id]), DIM == 3 ? d2f(S.vz[id]) : 0.0f,
                               d2f(S.rho[id] - P.rho0));
}

// Piston velocity of dynamic_boundaries (RRSPH_OMP/src/WaveMaker.cpp:34-82)
// for one set of wave-maker parameters.
__device__ double piston_law_vx(int nwm, double phase, double freq, double H, double k, double depth,
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
__device__ double piston_vx(const DevParams& P, double time) {
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
__device__ double solitary_vx(const DevParams& P, double time) {
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

// make_waves (WaveMaker.cpp:4-32, piston call enabled) + whole_step
// (RRSPH_OMP/src/WholeStep.cpp:19-62) + the per-step boundary check of
// RRSPHOutput::update_step (RRSPH_COMMON/src/Output.cpp:395-416). Thread 0
// advances the step scalars into scal_next (time += dt, step + 1).
template <int DIM, int V>
__global__ void k_whole(DevParams P, State S, Sorted G, const StepScalars* __restrict__ scal,
                        StepScalars* __restrict__ next, uint32_t* __restrict__ flags, int next_keys) {
    constexpr bool CONT = (V & kVarCont) != 0, RARE = (V & kVarRare) != 0;
    constexpr int M = (V & kVarMixed) ? 1 : 0;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // update_dt (UpdateAcceleration.cpp:15-29) under DT_CORRECTION_DYNAMIC
    double dt = scal->dt;
    if (RARE && P.dt_method == 2) {
        const double amax = P.dt_reduce ? __longlong_as_double((long long)scal->amax_bits) : 0.0;
        const double mumax = P.dt_reduce ? __longlong_as_double((long long)scal->mumax_bits) : 0.0;
        const double min_dt_a = sqrt(P.h / amax);
        const double min_dt_mu = P.h / (P.c_eos + mumax);
        dt = P.cfl * fmin(min_dt_a, min_dt_mu);
        if (dt <= P.never_ending_dt && i == 0) atomicOr(flags, RRSPH_FLAG_NEVER_ENDING);
    }
    const double time = scal->time;
    const unsigned long long nwm_off = scal->nwm_off;
    if (i == 0) {
        next->time = time + dt;
        next->dt = dt;
        next->step = scal->step + 1;
        next->amax_bits = 0;
        next->mumax_bits = 0;
        next->pairs = 0;
        next->nwm_off = nwm_off || (P.nwm == 4 && time >= P.nwm_time_start) ? 1ull : 0ull;
        next->pairs_total = scal->pairs_total + scal->pairs;
    }
    if (i >= P.n) return;
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
        vx = vx + S.ax[i] * v_dt;
        vy = vy + S.ay[i] * v_dt;
        if (DIM == 3) vz = vz + S.az[i] * v_dt;
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
        predict<DIM, M, CONT>(P, S, i, vx, vy, vz, rho, dt);
        key_pass<DIM, M>(P, S, G, i, x, y, z, flags);
    }
}

// cells_start[c] = lower bound of c in the sorted keys, c in [0, max_cells].
__global__ void k_cells_start(DevParams P, const uint32_t* __restrict__ key, uint32_t* __restrict__ out) {
    const uint64_t c = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c > P.max_cells) return;
    uint32_t lo = 0, hi = P.n;
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if ((uint64_t)key[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    out[c] = lo;
}

// find_neighbours (GridFind.cpp:112-189) as an explicit list per particle id,
// in the reference's order. For parity checks only; the step never stores it.
template <int DIM>
__global__ void k_neighbour_list(DevParams P, Sorted G, uint32_t* __restrict__ counts, uint32_t* __restrict__ list,
                                 uint32_t max_per, uint32_t* __restrict__ flags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const uint32_t j = G.id[k];
    uint32_t cnt = 0;
    bool over = false;
    if (G.itype[k] != P.type_non_existent) {
        const double xj = G.rx[k], yj = G.ry[k], zj = DIM == 3 ? G.rz[k] : 0.0;
        for_neighbour_cells<DIM>(P, G.key[k], [&](uint32_t c, int, int, int) {
            const uint32_t s = G.cell_start[c];
            if (s == kEmpty) return;
            const uint32_t e = G.cell_end[c];
            for (uint32_t i = s; i < e; i++) {
                if (i == k || G.itype[i] == P.type_non_existent) continue;
                const double d2 = exact_dist2<DIM>(__dsub_rn(G.rx[i], xj), __dsub_rn(G.ry[i], yj),
                                                   DIM == 3 ? __dsub_rn(G.rz[i], zj) : 0.0);
                if (d2 < P.cut2) {
                    if (cnt < max_per) list[(size_t)j * max_per + cnt] = G.id[i];
                    else over = true;
                    cnt++;
                }
            }
        });
    }
    counts[j] = cnt;
    if (over) atomicOr(flags, RRSPH_FLAG_NEIGHBOUR_OVERFLOW);
}

template <int DIM>
__global__ void k_unpack(DevParams P, State S, const double* __restrict__ r, const double* __restrict__ v,
                         uint32_t stride) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const size_t b = (size_t)i * stride;
    S.rx[i] = r[b];
    S.ry[i] = r[b + 1];
    S.vx[i] = v[b];
    S.vy[i] = v[b + 1];
    if (DIM == 3) {
        S.rz[i] = r[b + 2];
        S.vz[i] = v[b + 2];
    }
}

template <int DIM>
__global__ void k_pack(DevParams P, State S, double* __restrict__ r, double* __restrict__ v, uint32_t stride) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const size_t b = (size_t)i * stride;
    if (r) {
        r[b] = S.rx[i];
        r[b + 1] = S.ry[i];
        if (DIM == 3) r[b + 2] = S.rz[i];
    }
    if (v) {
        v[b] = S.vx[i];
        v[b + 1] = S.vy[i];
        if (DIM == 3) v[b + 2] = S.vz[i];
    }
}

}  // namespace

template <int DIM>
void launch_keys(const DevParams& P, const State& S, Sorted& G, StepScalars* scal, int predict, uint32_t* flags,
                 cudaStream_t st) {
    k_keys<DIM><<<blocks_for(P.n, 256), 256, 0, st>>>(P, S, G, scal, predict, flags);
}
template <int DIM>
void launch_reorder(const DevParams& P, const State& S, const Sorted& G, GatherSrc fsrc, int mixed, cudaStream_t st) {
    const unsigned b = blocks_for(P.n, 256);
    if (!mixed) k_reorder<DIM, 0><<<b, 256, 0, st>>>(P, S, G, fsrc);
    else if (!fsrc.loop) k_reorder<DIM, 3><<<b, 256, 0, st>>>(P, S, G, fsrc);
    else if (P.density_treatment == 0) k_reorder<DIM, 1><<<b, 256, 0, st>>>(P, S, G, fsrc);
    else k_reorder<DIM, 2><<<b, 256, 0, st>>>(P, S, G, fsrc);
}
template <int DIM>
void launch_whole_step(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal_cur,
                       StepScalars* scal_next, uint32_t* flags, int next_keys, cudaStream_t st) {
    const int v = (P.density_treatment != 0 ? kVarCont : 0) | (P.avg_vel || P.dt_method == 2 ? kVarRare : 0) |
                  ((DIM == 2 ? S.vpf2 != nullptr : S.vpf4 != nullptr) ? kVarMixed : 0);
    const unsigned b = blocks_for(P.n, 256);
    switch (v) {
#define RRSPH_WHOLE(V) \
    case V: k_whole<DIM, V><<<b, 256, 0, st>>>(P, S, G, scal_cur, scal_next, flags, next_keys); break;
        RRSPH_WHOLE(0) RRSPH_WHOLE(1) RRSPH_WHOLE(2) RRSPH_WHOLE(3)
        RRSPH_WHOLE(4) RRSPH_WHOLE(5) RRSPH_WHOLE(6) RRSPH_WHOLE(7)
#undef RRSPH_WHOLE
    }
}
void launch_cells_start(const DevParams& P, const Sorted& G, uint32_t* out, cudaStream_t st) {
    const uint64_t m = (uint64_t)P.max_cells + 1;
    k_cells_start<<<(unsigned)((m + 255) / 256), 256, 0, st>>>(P, G.key, out);
}
template <int DIM>
void launch_neighbour_list(const DevParams& P, const Sorted& G, uint32_t* counts, uint32_t* list, uint32_t max_per,
                           uint32_t* flags, cudaStream_t st) {
    k_neighbour_list<DIM><<<blocks_for(P.n, 128), 128, 0, st>>>(P, G, counts, list, max_per, flags);
}
template <int DIM>
void launch_unpack(const DevParams& P, State S, const double* r, const double* v, uint32_t stride, cudaStream_t st) {
    k_unpack<DIM><<<blocks_for(P.n, 256), 256, 0, st>>>(P, S, r, v, stride);
}
template <int DIM>
void launch_pack(const DevParams& P, State S, double* r, double* v, uint32_t stride, cudaStream_t st) {
    k_pack<DIM><<<blocks_for(P.n, 256), 256, 0, st>>>(P, S, r, v, stride);
}

#define RRSPH_INSTANTIATE(D)                                                                                     \
    template void launch_keys<D>(const DevParams&, const State&, Sorted&, StepScalars*, int, uint32_t*,        \
                                 cudaStream_t);                                                                \
    template void launch_reorder<D>(const DevParams&, const State&, const Sorted&, GatherSrc, int, cudaStream_t); \
    template void launch_whole_step<D>(const DevParams&, const State&, const Sorted&, StepScalars*,            \
                                       StepScalars*, uint32_t*, int, cudaStream_t);                            \
    template void launch_neighbour_list<D>(const DevParams&, const Sorted&, uint32_t*, uint32_t*, uint32_t,    \
                                           uint32_t*, cudaStream_t);                                           \
    template void launch_unpack<D>(const DevParams&, State, const double*, const double*, uint32_t, cudaStream_t); \
    template void launch_pack<D>(const DevParams&, State, double*, double*, uint32_t, cudaStream_t);
RRSPH_INSTANTIATE(2)
RRSPH_INSTANTIATE(3)
#undef RRSPH_INSTANTIATE

}  // namespace rrsph
