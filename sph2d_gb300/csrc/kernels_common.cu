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
template <int DIM>
__device__ __forceinline__ void key_pass(const DevParams& P, const State& S, const Sorted& G, uint32_t i, double x,
                                         double y, double z, uint32_t* __restrict__ flags) {
    bool outside = !(x >= P.xmin) || !(y >= P.ymin);
    const uint64_t cx = cell_coord_fast(x, P.xmin, P.cell, P.inv_cell);
    const uint64_t cy = cell_coord_fast(y, P.ymin, P.cell, P.inv_cell);
    uint64_t key;
    if (DIM == 3) {
        outside = outside || !(z >= P.zmin);
        const uint64_t cz = cell_coord_fast(z, P.zmin, P.cell, P.inv_cell);
        key = split3(cx) | (split3(cy) << 1) | (split3(cz) << 2);
    } else {
        key = split2(cx) | (split2(cy) << 1);
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
}

// predict_half_step (PredictHalfStep.cpp:4-23) of particle i with time step dt.
template <int DIM>
__device__ __forceinline__ void predict(const DevParams& P, const State& S, uint32_t i, double vx, double vy,
                                        double vz, double rho, double dt) {
    S.vpx[i] = vx + S.ax[i] * dt * 0.5;
    S.vpy[i] = vy + S.ay[i] * dt * 0.5;
    if (DIM == 3) S.vpz[i] = vz + S.az[i] * dt * 0.5;
    if (P.density_treatment != 0) S.rho_pred[i] = rho + S.drho[i] * dt * 0.5;
}

template <int DIM>
__global__ void k_keys(DevParams P, State S, Sorted G, const StepScalars* __restrict__ scal, int do_predict,
                       uint32_t* __restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    if (do_predict)
        predict<DIM>(P, S, i, S.vx[i], S.vy[i], DIM == 3 ? S.vz[i] : 0.0, P.density_treatment ? S.rho[i] : 0.0,
                     scal->dt);
    key_pass<DIM>(P, S, G, i, S.rx[i], S.ry[i], DIM == 3 ? S.rz[i] : 0.0, flags);
}

// Gathers the state into cell order and records each cell's [start, end) in
// the sorted arrays (the cells_start table of make_grid, GridFind.cpp:77-87).
template <int DIM>
__global__ void k_reorder(DevParams P, State S, Sorted G, GatherSrc F, int mixed) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const uint32_t key = G.key[k];
    const uint32_t id = G.id[k];
    if (k == 0 || G.key[k - 1] != key) G.cell_start[key] = k;
    if (k == P.n - 1 || G.key[k + 1] != key) G.cell_end[key] = k + 1;
    const double x = S.rx[id], y = S.ry[id], z = DIM == 3 ? S.rz[id] : 0.0;
    const int32_t t = S.itype[id];
    G.rx[k] = x;
    G.ry[k] = y;
    if (DIM == 3) G.rz[k] = z;
    G.itype[k] = t;
    const double fvx = F.vx[id], fvy = F.vy[id], fvz = DIM == 3 ? F.vz[id] : 0.0;
    const double frho = F.rho[id];
    const bool cont = P.density_treatment != 0;
    if (!mixed) {
        G.vx[k] = fvx;
        G.vy[k] = fvy;
        if (DIM == 3) G.vz[k] = fvz;
        G.rho[k] = frho;
        if (F.p) G.p[k] = F.p[id];
        if (cont) {
            G.vdx[k] = S.vx[id];
            G.vdy[k] = S.vy[id];
            if (DIM == 3) G.vdz[k] = S.vz[id];
            G.rhod[k] = S.rho[id];
        }
    } else {
        uint64_t cx, cy, cz;
        decode_key<DIM>(key, cx, cy, cz);
        const float ox = (float)(x - (P.xmin + (double)cx * P.cell));
        const float oy = (float)(y - (P.ymin + (double)cy * P.cell));
        const float oz = DIM == 3 ? (float)(z - (P.zmin + (double)cz * P.cell)) : 0.0f;
        G.P4[k] = make_float4(ox, oy, oz, __int_as_float(t));
        G.V4[k] = make_float4((float)fvx, (float)fvy, (float)fvz, (float)frho);
        if (F.p) G.PR[k] = make_float2((float)F.p[id], (float)(F.p[id] / (frho * frho)));
        if (cont)  // the density deviation keeps rho_i - rho_j accurate in float
            G.VD4[k] = make_float4((float)S.vx[id], (float)S.vy[id], DIM == 3 ? (float)S.vz[id] : 0.0f,
                                   (float)(S.rho[id] - P.rho0));
    }
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
template <int DIM>
__global__ void k_whole(DevParams P, State S, Sorted G, const StepScalars* __restrict__ scal,
                        StepScalars* __restrict__ next, uint32_t* __restrict__ flags, int next_keys) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // update_dt (UpdateAcceleration.cpp:15-29) under DT_CORRECTION_DYNAMIC
    double dt = scal->dt;
    if (P.dt_method == 2) {
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
    const bool waves = P.nwm && !nwm_off && time >= P.nwm_time_start;
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
    const double v_dt = scal->step ? dt : dt * 0.5;
    double rho = 0.0;
    if (P.density_treatment != 0) {
        rho = S.rho[i] + S.drho[i] * v_dt;
        S.rho[i] = rho;
    }
    double x = S.rx[i], y = S.ry[i], z = DIM == 3 ? S.rz[i] : 0.0;
    double vx = S.vx[i], vy = S.vy[i], vz = DIM == 3 ? S.vz[i] : 0.0;
    if (S.itype[i] > 0) {
        vx = vx + S.ax[i] * v_dt;
        vy = vy + S.ay[i] * v_dt;
        if (DIM == 3) vz = vz + S.az[i] * v_dt;
        if (P.avg_vel) {
            vx += S.avx[i];
            vy += S.avy[i];
            if (DIM == 3) vz += S.avz[i];
        }
        S.vx[i] = vx;
        S.vy[i] = vy;
        if (DIM == 3) S.vz[i] = vz;
        const double nx = x + vx * dt, ny = y + vy * dt, nz = DIM == 3 ? z + vz * dt : 0.0;
        bool move = true;
        if (P.consistency_treatment == 2) {  // CONSISTENCY_FIX (WholeStep.cpp:47-54)
            bool in = nx < P.xmax && nx > P.xmin && ny < P.ymax && ny > P.ymin;
            if (DIM == 3) in = in && nz < P.zmax && nz > P.zmin;
            if (!in) {
                move = false;
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
        bool in = x < P.xmax && x > P.xmin && y < P.ymax && y > P.ymin;
        if (DIM == 3) in = in && z < P.zmax && z > P.zmin;
        if (!in) atomicOr(flags, RRSPH_FLAG_OUTSIDE_GEOMETRY);
    }
    if (next_keys) {
        // the next step's predict_half_step and cell keys, from the state just written
        predict<DIM>(P, S, i, vx, vy, vz, rho, dt);
        key_pass<DIM>(P, S, G, i, x, y, z, flags);
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
    k_reorder<DIM><<<blocks_for(P.n, 256), 256, 0, st>>>(P, S, G, fsrc, mixed);
}
template <int DIM>
void launch_whole_step(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal_cur,
                       StepScalars* scal_next, uint32_t* flags, int next_keys, cudaStream_t st) {
    k_whole<DIM><<<blocks_for(P.n, 256), 256, 0, st>>>(P, S, G, scal_cur, scal_next, flags, next_keys);
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
