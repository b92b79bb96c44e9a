// kernels_common.cu — per-particle kernels of the step that are not pair
// gathers: predict + cell keys, reorder + cell table, whole step + piston,
// and the grid/neighbour exports used by parity checks.
#include "kernels.cuh"
#include "neighbour.cuh"
#include "step_particle.cuh"

namespace rrsph {

namespace {

inline unsigned blocks_for(uint32_t n, int threads) { return (n + threads - 1) / threads; }

template <int DIM>
__global__ void k_keys(DevParams P, State S, Sorted G, const StepScalars* __restrict__ scal, int do_predict,
                       uint32_t* __restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    if (do_predict) {
        if (P.density_treatment)
            predict<DIM, 2, true>(P, S, i, S.vx[i], S.vy[i], DIM == 3 ? S.vz[i] : 0.0, S.rho[i], scal->dt, S.ax[i],
                                  S.ay[i], DIM == 3 ? S.az[i] : 0.0);
        else
            predict<DIM, 2, false>(P, S, i, S.vx[i], S.vy[i], DIM == 3 ? S.vz[i] : 0.0, 0.0, scal->dt, S.ax[i],
                                   S.ay[i], DIM == 3 ? S.az[i] : 0.0);
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
        if (G.P4) {  // the cell-relative float offsets of the FP64 density pass's first test
            const float4 o = DIM == 3 ? S.coff4[id] : make_float4(S.coff2[id].x, S.coff2[id].y, 0.0f, 0.0f);
            G.P4[k] = make_float4(o.x, o.y, o.z, __int_as_float(t));
        }
        G.vx[k] = F.vx[id];
        G.vy[k] = F.vy[id];
        if (DIM == 3) G.vz[k] = F.vz[id];
        G.rho[k] = F.rho[id];
        if (F.p) {  // a given pressure (rrsph_forces): p / rho^2 as the density pass writes it
            G.p[k] = F.p[id];
            G.pr2[k] = F.p[id] / (F.rho[id] * F.rho[id]);
        }
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
        G.VD4[k] = vd4_of<DIM>(S.vx[id], S.vy[id], DIM == 3 ? S.vz[id] : 0.0, S.rho[id] - P.rho0);
}

// make_waves (WaveMaker.cpp:4-32, piston call enabled) + whole_step
// (RRSPH_OMP/src/WholeStep.cpp:19-62) + the per-step boundary check of
// RRSPHOutput::update_step (RRSPH_COMMON/src/Output.cpp:395-416). Thread 0
// advances the step scalars into scal_next (time += dt, step + 1).
template <int DIM, int V>
__global__ void k_whole(DevParams P, State S, Sorted G, const StepScalars* __restrict__ scal,
                        StepScalars* __restrict__ next, uint32_t* __restrict__ flags, int next_keys) {
    constexpr bool RARE = (V & kVarRare) != 0;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const double dt = step_dt<RARE>(P, scal, flags, i == 0);
    if (i == 0) advance_scalars(P, scal, next, dt);
    if (i >= P.n) return;
    whole_particle<DIM, V>(P, S, G, i, dt, scal, flags, next_keys, S.ax[i], S.ay[i], DIM == 3 ? S.az[i] : 0.0);
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

// A coordinate triple (x, y[, z]) of a strided host array: 16-byte loads and
// stores where the layout allows (stride 2 in 2D, stride 4 in 3D, 16-byte
// aligned), since partial-line accesses over the host link are slow. A
// stride-4 store also writes 0 into the pad.
template <int DIM>
__device__ __forceinline__ void host_read3(const double* __restrict__ a, size_t b, bool vec, double& x, double& y,
                                           double& z) {
    if (vec) {
        const double2 q = *reinterpret_cast<const double2*>(a + b);
        x = q.x;
        y = q.y;
        if (DIM == 3) z = *(a + b + 2);
    } else {
        x = a[b];
        y = a[b + 1];
        if (DIM == 3) z = a[b + 2];
    }
}
template <int DIM>
__device__ __forceinline__ void host_write3(double* __restrict__ a, size_t b, bool vec, double x, double y,
                                            double z) {
    if (vec) {
        reinterpret_cast<double2*>(a + b)[0] = make_double2(x, y);
        if (DIM == 3) reinterpret_cast<double2*>(a + b)[1] = make_double2(z, 0.0);
    } else {
        a[b] = x;
        a[b + 1] = y;
        if (DIM == 3) a[b + 2] = z;
    }
}

// rrsph_upload from host arrays the device can address (page-locked host
// memory): the state straight from the caller's arrays over the host link, the
// fresh work arrays of time_integration (TimeIntegration.cpp:35-50) zeroed,
// (thread 0) the step scalars of step 0, then the first step's predict + key
// pass of k_keys (zero acceleration, dt of step 0) while the link is still
// busy. The neighbour-list check of an upload runs before this kernel: its
// key pass may raise the rebuild flag, which the check resets. rho may be
// null with summation density, whose step recomputes it before any read.
template <int DIM>
__global__ void k_upload_direct(DevParams P, State S, Sorted G, const double* __restrict__ r,
                                const double* __restrict__ v, const double* __restrict__ rho,
                                const double* __restrict__ p, const int32_t* __restrict__ itype, uint32_t stride,
                                int vec, StepScalars* __restrict__ scal, double dt, uint32_t* __restrict__ flags) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) {
        *scal = StepScalars{};
        scal->dt = dt;
        *S.itype_changed = 0u;  // the uploaded types are the reference
    }
    if (i >= P.n) return;
    const size_t b = (size_t)i * stride;
    double x, y, z = 0.0;
    host_read3<DIM>(r, b, vec, x, y, z);
    S.rx[i] = x;
    S.ry[i] = y;
    if (DIM == 3) S.rz[i] = z;
    host_read3<DIM>(v, b, vec, x, y, z);
    S.vx[i] = x;
    S.vy[i] = y;
    if (DIM == 3) {
        S.vz[i] = z;
        S.az[i] = 0.0;
    }
    const double rh = rho ? rho[i] : P.rho0;  // no rho: summation density, which the step recomputes
    S.rho[i] = rh;
    S.p[i] = p ? p[i] : 0.0;
    S.itype[i] = itype[i];
    S.ax[i] = 0.0;
    S.ay[i] = 0.0;
    if (S.avx) {
        S.avx[i] = 0.0;
        S.avy[i] = 0.0;
        if (DIM == 3) S.avz[i] = 0.0;
    }
    S.drho[i] = 0.0;
    const double vx = S.vx[i], vy = S.vy[i], vz = DIM == 3 ? S.vz[i] : 0.0;
    if (P.density_treatment) predict<DIM, 2, true>(P, S, i, vx, vy, vz, rh, dt, 0.0, 0.0, 0.0);
    else predict<DIM, 2, false>(P, S, i, vx, vy, vz, 0.0, dt, 0.0, 0.0, 0.0);
    key_pass<DIM, 2>(P, S, G, i, S.rx[i], S.ry[i], DIM == 3 ? S.rz[i] : 0.0, flags);
}

// Global checks in double (rrsph_diagnostics): per fluid particle (itype > 0)
// its mass, kinetic energy m|v|^2/2, potential energy m g y, the internal
// energy m e(rho) of the Tait EOS p = B((rho/rho0)^7 - 1) — e(rho) the
// integral of p/rho^2 from rho0, written with x = rho/rho0, t = x - 1 as
// (B/rho0) t^2 (6 + 5x + 4x^2 + 3x^3 + 2x^4 + x^5) / (6x), free of
// cancellation — and its momentum; per boundary particle (itype < 0) its mass.
// Each block reduces a fixed set of particles in a fixed order and a second
// kernel sums the blocks in a fixed order, so the result is the same every run.
constexpr int kDiagQ = 10;  // mass, kinetic, potential, internal, px, py, pz, boundary mass, fluid, boundary
constexpr int kDiagThreads = 256;

template <int DIM>
__global__ void __launch_bounds__(kDiagThreads) k_diag_blocks(DevParams P, State S, double* __restrict__ part) {
    __shared__ double sh[kDiagQ][kDiagThreads];
    double q[kDiagQ] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (uint32_t i = blockIdx.x * kDiagThreads + threadIdx.x; i < P.n; i += gridDim.x * kDiagThreads) {
        const int32_t t = S.itype[i];
        if (t > 0) {
            const double vx = S.vx[i], vy = S.vy[i], vz = DIM == 3 ? S.vz[i] : 0.0;
            const double x = S.rho[i] / P.rho0, tt = x - 1.0;
            const double poly = 6.0 + x * (5.0 + x * (4.0 + x * (3.0 + x * (2.0 + x))));
            q[0] += P.mass;
            q[1] += 0.5 * P.mass * (vx * vx + vy * vy + vz * vz);
            q[2] += P.mass * P.g * S.ry[i];
            q[3] += P.mass * (P.B / P.rho0) * (tt * tt) * poly / (6.0 * x);
            q[4] += P.mass * vx;
            q[5] += P.mass * vy;
            q[6] += P.mass * vz;
            q[8] += 1.0;
        } else if (t < 0) {
            q[7] += P.mass;
            q[9] += 1.0;
        }
    }
#pragma unroll
    for (int j = 0; j < kDiagQ; j++) sh[j][threadIdx.x] = q[j];
    __syncthreads();
    for (int w = kDiagThreads / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w)
#pragma unroll
            for (int j = 0; j < kDiagQ; j++) sh[j][threadIdx.x] += sh[j][threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x < kDiagQ) part[(size_t)blockIdx.x * kDiagQ + threadIdx.x] = sh[threadIdx.x][0];
}
__global__ void __launch_bounds__(kDiagThreads) k_diag_sum(const double* __restrict__ part, int blocks,
                                                           double* __restrict__ out) {
    __shared__ double sh[kDiagThreads];
    for (int j = 0; j < kDiagQ; j++) {
        double v = 0.0;
        for (int b = threadIdx.x; b < blocks; b += kDiagThreads) v += part[(size_t)b * kDiagQ + j];
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int w = kDiagThreads / 2; w > 0; w >>= 1) {
            if ((int)threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[j] = sh[0];
        __syncthreads();
    }
}

// rrsph_step's bookkeeping as kernels on the stream (no copy-engine round
// trips): the time of the next step (and cleared status flags) before the
// steps, the time and flags after them into a host mailbox.
__global__ void k_set_time(StepScalars* __restrict__ scal, double time, uint32_t* __restrict__ flags) {
    scal->time = time;
    if (flags) *flags = 0u;
}
__global__ void k_report(const StepScalars* __restrict__ scal, const StepScalars* __restrict__ last,
                         const uint32_t* __restrict__ flags, HostReport* __restrict__ out) {
    out->time = scal->time;
    out->flags = *flags;
    out->pairs_last = last ? last->pairs : 0ull;
    out->pairs_total = scal->pairs_total;
}

// rrsph_download into host arrays the device can address: one pass writing
// the requested arrays (null: skipped) over the host link; itype only if
// itype_if (when given) is non-zero.
template <int DIM>
__global__ void k_download_direct(DevParams P, State S, double* __restrict__ r, double* __restrict__ v,
                                  double* __restrict__ rho, double* __restrict__ p, int32_t* __restrict__ itype,
                                  uint32_t stride, int vec, const uint32_t* __restrict__ itype_if) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const size_t b = (size_t)i * stride;
    if (r) host_write3<DIM>(r, b, vec, S.rx[i], S.ry[i], DIM == 3 ? S.rz[i] : 0.0);
    if (v) host_write3<DIM>(v, b, vec, S.vx[i], S.vy[i], DIM == 3 ? S.vz[i] : 0.0);
    if (rho) rho[i] = S.rho[i];
    if (p) p[i] = S.p[i];
    if (itype && (!itype_if || *itype_if)) itype[i] = S.itype[i];
}

}  // namespace

// 16-byte accesses for strided coordinate arrays where the layout allows.
inline int vec_layout(int dim, uint32_t stride, const void* a, const void* b) {
    const bool al = (reinterpret_cast<uintptr_t>(a) % 16 == 0) && (reinterpret_cast<uintptr_t>(b) % 16 == 0);
    return al && ((dim == 2 && stride == 2) || (dim == 3 && stride == 4)) ? 1 : 0;
}

template <int DIM>
void launch_diagnostics(const DevParams& P, const State& S, double* part, int blocks, double* out, cudaStream_t st) {
    k_diag_blocks<DIM><<<blocks, kDiagThreads, 0, st>>>(P, S, part);
    k_diag_sum<<<1, kDiagThreads, 0, st>>>(part, blocks, out);
}

void launch_set_time(StepScalars* scal, double time, uint32_t* flags, cudaStream_t st) {
    k_set_time<<<1, 1, 0, st>>>(scal, time, flags);
}
void launch_report(const StepScalars* scal, const StepScalars* last, const uint32_t* flags, HostReport* out,
                   cudaStream_t st) {
    k_report<<<1, 1, 0, st>>>(scal, last, flags, out);
}

template <int DIM>
void launch_upload_direct(const DevParams& P, const State& S, const Sorted& G, const double* r, const double* v,
                          const double* rho, const double* p, const int32_t* itype, uint32_t stride,
                          StepScalars* scal, double dt, uint32_t* flags, cudaStream_t st) {
    k_upload_direct<DIM><<<blocks_for(P.n, 256), 256, 0, st>>>(P, S, G, r, v, rho, p, itype, stride,
                                                               vec_layout(DIM, stride, r, v), scal, dt, flags);
}
template <int DIM>
void launch_download_direct(const DevParams& P, const State& S, double* r, double* v, double* rho, double* p,
                            int32_t* itype, uint32_t stride, cudaStream_t st, const uint32_t* itype_if) {
    k_download_direct<DIM><<<blocks_for(P.n, 256), 256, 0, st>>>(P, S, r, v, rho, p, itype, stride,
                                                                 vec_layout(DIM, stride, r, v), itype_if);
}

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
    template void launch_pack<D>(const DevParams&, State, double*, double*, uint32_t, cudaStream_t);         \
    template void launch_diagnostics<D>(const DevParams&, const State&, double*, int, double*, cudaStream_t);  \
    template void launch_upload_direct<D>(const DevParams&, const State&, const Sorted&, const double*,        \
                                          const double*, const double*, const double*, const int32_t*,         \
                                          uint32_t, StepScalars*, double, uint32_t*, cudaStream_t);            \
    template void launch_download_direct<D>(const DevParams&, const State&, double*, double*, double*, double*, \
                                            int32_t*, uint32_t, cudaStream_t, const uint32_t*);
RRSPH_INSTANTIATE(2)
RRSPH_INSTANTIATE(3)
#undef RRSPH_INSTANTIATE

}  // namespace rrsph
