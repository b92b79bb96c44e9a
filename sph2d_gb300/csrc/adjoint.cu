// adjoint.cu — the Fourier piston and the reverse (adjoint) sweep of the FP64
// loop: d(gauge series)ᵀ·w / d(piston coefficients) for the method set of the
// piston flume (2D, summation density, cubic spline, pressure form 1/2,
// Monaghan viscosity, Lennard-Jones boundary, constant dt).
//
// Forward step n (TimeIntegration.cpp:60-100, the piston call enabled), state
// S^n = (r, v, a_prev, itype):
//   v*   = v + a_prev dt/2                         predict_half_step
//   rho  = m W0 + sum_i m W(|r_j - r_i|), p = EOS   density_sum (Density.h:25-61)
//   a_j  = g + sum_i [e S - LJ],  e = r_i - r_j,    update_acceleration
//          S = m sc (PF + Pi), dW/dr = e sc
//   piston: r.x += vx dt, v.x = vx                 dynamic_boundaries
//   fluid:  v += a v_dt, r += v dt                 whole_step
// Its adjoint runs backwards through the same pieces. The pair part uses the
// symmetry of each pair's contribution: with Λ = λa_j − λa_i the pair adds
// ℓ = (Λ·e) S − (Λ_LJ·e) fl to Σ_j λa_j·a_j, the same scalar seen from j or
// from i, so every particle gathers ∂ℓ/∂(its own r, v*, rho, p) over its
// neighbours and no pair result is scattered (no atomics). The density part is
// ℓ_rho = (λrho_j + λrho_i) m W(|e|), gathered the same way. The neighbour
// pairs of step n are the forward step's own: its sorted grid (keys, ids) and
// the neighbour masks its density pass recorded are kept for every step of the
// segment being reversed.
//
// Checkpointing: the forward run stores S^n every K steps; the reverse sweep
// takes the segments last to first, recomputes the K states of a segment from
// its checkpoint with the forward step itself (bitwise the same states), and
// runs the K reverse steps of the segment.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "../host/error.hpp"
#include "kernels.cuh"
#include "neighbour.cuh"
#include "sort.cuh"
#include "solver_impl.cuh"

using rrsph::set_error;

namespace rrsph {

constexpr int kAdjThreads = 128;

// One stored state per slot: fields are [slots][n].
struct Snap {
    double *rx, *ry, *vx, *vy, *ax, *ay;
    int32_t* itype;
};
struct SnapView {
    const double *rx, *ry, *vx, *vy, *ax, *ay;
    const int32_t* itype;
};

// Adjoint arrays of one reverse step: in_* are the adjoints of S^{n+1} (id
// order), out_* those of S^n; la_*, lrho and pr2 are in cell order.
struct AdjBuf {
    const double *in_rx, *in_ry, *in_vx, *in_vy, *in_ax, *in_ay;
    double *out_rx, *out_ry, *out_vx, *out_vy, *out_ax, *out_ay;
    double *la_x, *la_y;  // λa of step n (cell order)
    double* lrho;         // total λrho (cell order)
    double* pr2;          // p / rho^2 (cell order)
    double* gvx;          // dL/d(piston vx) per piston particle (id order)
};

namespace {

// cubic spline (SmoothingKernel.h:42-56): sc with dW/dr = e*sc, and
// sc1d = (dsc/ddist)/dist; inv_d = 1/dist.
__device__ __forceinline__ void cubic_sc(const DevParams& P, double q, double inv_d, double& sc, double& sc1d) {
    const double f = P.kf[1];
    const double ih = P.inv_h;
    if (q <= 1.0) {
        sc = f * ih * ih * (-2.0 + 1.5 * q);
        sc1d = 1.5 * f * ih * ih * ih * inv_d;
    } else if (q <= 2.0) {
        const double t = 2.0 - q;
        sc = -0.5 * f * ih * t * t * inv_d;
        sc1d = 0.5 * f * ih * (2.0 * t * ih * inv_d * inv_d + t * t * inv_d * inv_d * inv_d);
    } else {
        sc = 0.0;
        sc1d = 0.0;
    }
}

__device__ __forceinline__ double eos_dp(const DevParams& P, double rho) {
    const double x = rho / P.rho0;
    const double x2 = x * x;
    return 7.0 * P.B / P.rho0 * (x2 * x2 * x2);
}

// ---------------------------------------------------------------- gauges --
// maxInLayer (tools/WaterProfile/include/HeightTesting.h:25-54): largest y > 0
// of the selected particles; then the smallest id that attains it.
__global__ void k_gauge_max(uint32_t n, const double* __restrict__ rx, const double* __restrict__ ry,
                            const int32_t* __restrict__ itype, double xg, double radius, int32_t type,
                            unsigned long long* __restrict__ best) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long b = 0;
    if (i < n && (type == 0 || itype[i] == type)) {
        const double y = ry[i];
        if (fabs(rx[i] - xg) < radius && y > 0.0) b = (unsigned long long)__double_as_longlong(y);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_down_sync(0xFFFFFFFFu, b, o);
        b = t > b ? t : b;
    }
    if ((threadIdx.x & 31) == 0 && b) atomicMax(best, b);
}
__global__ void k_gauge_arg(uint32_t n, const double* __restrict__ rx, const double* __restrict__ ry,
                            const int32_t* __restrict__ itype, double xg, double radius, int32_t type,
                            const unsigned long long* __restrict__ best, uint32_t* __restrict__ id) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || !(type == 0 || itype[i] == type)) return;
    const double y = ry[i];
    if (fabs(rx[i] - xg) < radius && y > 0.0 && (unsigned long long)__double_as_longlong(y) == *best)
        atomicMin(id, i);
}

// -------------------------------------------------------- reverse step ----
// Cell-order copies of step n's forward quantities (the grid of r^n), and the
// adjoint of whole_step and the piston: from the adjoints of S^{n+1} to those
// before the step's updates, and λa of step n in cell order.
__global__ void k_adj_reorder(DevParams P, Sorted G, SnapView sn, const double* __restrict__ rho_n, AdjBuf A,
                              double dt, double v_dt, int piston) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const uint32_t key = G.key[k];
    const uint32_t id = G.id[k];
    if (k == 0 || G.key[k - 1] != key) G.cell_start[key] = k;
    if (k == P.n - 1 || G.key[k + 1] != key) G.cell_end[key] = k + 1;
    const int32_t t = sn.itype[id];
    const double rho = rho_n[id];
    const double p = eos_p(P, rho);
    G.rx[k] = sn.rx[id];
    G.ry[k] = sn.ry[id];
    G.vx[k] = sn.vx[id] + sn.ax[id] * dt * 0.5;
    G.vy[k] = sn.vy[id] + sn.ay[id] * dt * 0.5;
    G.rho[k] = rho;
    G.p[k] = p;
    G.itype[k] = t;
    A.pr2[k] = p / (rho * rho);
    double lrx = A.in_rx[id], lry = A.in_ry[id], lvx = A.in_vx[id], lvy = A.in_vy[id];
    double lax = A.in_ax[id], lay = A.in_ay[id];
    if (t > 0) {  // v' = v + a v_dt, r' = r + v' dt
        const double mx = lvx + dt * lrx, my = lvy + dt * lry;
        lvx = mx;
        lvy = my;
        lax += v_dt * mx;
        lay += v_dt * my;
    }
    if (piston && id >= P.nwm_start && id < P.nwm_end) {  // r.x += vx dt, v.x = vx
        A.gvx[id] = lrx * dt + lvx;
        lvx = 0.0;
    }
    A.out_rx[id] = lrx;
    A.out_ry[id] = lry;
    A.out_vx[id] = lvx;
    A.out_vy[id] = lvy;
    A.la_x[k] = lax;
    A.la_y[k] = lay;
}

// Adjoint of update_acceleration: per particle j the gather of ∂ℓ/∂r_j,
// ∂ℓ/∂v*_j, ∂ℓ/∂rho_j and ∂ℓ/∂p_j over its neighbours; v* = v + a_prev dt/2
// passes λv* to λv and λa_prev; λrho collects the EOS chain rule.
__global__ void __launch_bounds__(kAdjThreads) k_adj_forces(DevParams P, Sorted G, AdjBuf A, double dt) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const uint32_t id = G.id[k];
    const int32_t tj = G.itype[k];
    double grx = 0, gry = 0, gvx = 0, gvy = 0, grho = 0, gp = 0;
    const double rhoj = G.rho[k];
    if (tj != P.type_non_existent) {
        const double xj = G.rx[k], yj = G.ry[k];
        const double vxj = G.vx[k], vyj = G.vy[k];
        const double pj = G.p[k], pr2j = A.pr2[k];
        const double laxj = A.la_x[k], layj = A.la_y[k];
        const double m = P.mass;
        const double ac = P.av_alpha * P.c_av;
        const bool form1 = P.intf_form == 1;
        // the forward step's neighbours, recorded by its density pass, as one flat
        // sequence over the stencil cells (cells of more than 32 particles searched
        // in place with the forward's test), the lanes of a warp together
        const uint32_t* const masks = G.nbmask + k;  // [c * n]: this particle's bits of stencil cell c
        const uint32_t over = masks[(size_t)9 * P.n];
        const Stencil<2> st(P, G.key[k]);
        int c = -1;
        uint32_t bits = 0, base = 0, next = 0, end = 0;
        for (;;) {
            if (bits == 0 && next == end) {
                for (c++; c < 9; c++) {
                    uint32_t cell;
                    int sx, sy, sz;
                    if (!st.cell(c, cell, sx, sy, sz)) continue;
                    const uint32_t s = G.cell_start[cell];
                    if (s == kEmpty) continue;
                    if ((over >> c) & 1u) {
                        next = s;
                        end = G.cell_end[cell];
                        break;
                    }
                    bits = masks[(size_t)c * P.n];
                    base = s;
                    if (bits) break;
                }
                if (c >= 9) break;
            }
            uint32_t i;
            bool known;
            if (bits) {
                i = base + (uint32_t)(__ffs(bits) - 1);
                bits &= bits - 1;
                known = true;
            } else {
                i = next++;
                known = false;
            }
            const int32_t ti = G.itype[i];
            const double ex = __dsub_rn(G.rx[i], xj), ey = __dsub_rn(G.ry[i], yj);
            const double s2 = exact_dist2<2>(ex, ey, 0.0);
            if (!known && !(i != k && ti != P.type_non_existent && s2 < P.cut2)) continue;
            const double inv_d = rsqrt(s2);
            const double q = s2 * inv_d * P.inv_h;
            double sc, sc1d;
            cubic_sc(P, q, inv_d, sc, sc1d);
            const double lx = laxj - A.la_x[i], ly = layj - A.la_y[i];
            const double le = lx * ex + ly * ey;
            const double rhoi = G.rho[i];
            double PF, PFr, PFp;  // PF, dPF/drho_j, dPF/dp_j
            if (form1) {
                const double inv = 1.0 / (rhoj * rhoi);
                PF = (pj + G.p[i]) * inv;
                PFr = -PF / rhoj;
                PFp = inv;
            } else {
                PF = A.pr2[i] + pr2j;
                PFr = -2.0 * pr2j / rhoj;
                PFp = 1.0 / (rhoj * rhoj);
            }
            double Pi = 0, Pimu = 0, coefE, coefDv = 0, inv_rbar = 0;
            const double dvx = vxj - G.vx[i], dvy = vyj - G.vy[i];
            const double vr = -(dvx * ex + dvy * ey);
            if (P.art_visc && vr < 0) {
                const double den = 1.0 / (s2 + P.etq_h2);
                const double mu = P.h * vr * den;
                inv_rbar = 2.0 / (rhoi + rhoj);
                Pi = (P.av_beta * mu - ac) * mu * inv_rbar;
                Pimu = (2.0 * P.av_beta * mu - ac) * inv_rbar;
                coefDv = -m * sc * Pimu * P.h * den;
                coefE = m * (sc1d * (PF + Pi) - 2.0 * sc * Pimu * P.h * vr * den * den);
            } else {
                coefE = m * sc1d * PF;
            }
            const double S = m * sc * (PF + Pi);
            // ∂ℓ/∂e = Λ S + (Λ·e) ∂S/∂e; r_j enters e with a minus sign
            grx -= lx * S + le * (coefE * ex + coefDv * dvx);
            gry -= ly * S + le * (coefE * ey + coefDv * dvy);
            gvx += le * coefDv * ex;
            gvy += le * coefDv * ey;
            const double msc = m * sc * le;
            grho += msc * (PFr - 0.5 * Pi * inv_rbar);
            gp += msc * PFp;
            if (P.repulsive && s2 * inv_d < P.lj_rr0) {
                const bool sj = tj > 0 && ti < 0, si = ti > 0 && tj < 0;
                if (sj || si) {
                    const double Lx = sj ? laxj : -A.la_x[i], Ly = sj ? layj : -A.la_y[i];
                    const double rn = P.lj_rr0 * inv_d;
                    const double rn2 = rn * rn, rn4 = rn2 * rn2, rn12 = rn4 * rn4 * rn4;
                    const double inv_s = inv_d * inv_d;
                    const double fl = P.lj_D * (rn12 - rn4) * inv_s;
                    const double fls = P.lj_D * (-7.0 * rn12 + 3.0 * rn4) * inv_s * inv_s;
                    const double LE = Lx * ex + Ly * ey;
                    grx += Lx * fl + 2.0 * LE * fls * ex;
                    gry += Ly * fl + 2.0 * LE * fls * ey;
                }
            }
        }
    }
    A.out_rx[id] += grx;
    A.out_ry[id] += gry;
    A.out_vx[id] += gvx;
    A.out_vy[id] += gvy;
    A.out_ax[id] = gvx * dt * 0.5;
    A.out_ay[id] = gvy * dt * 0.5;
    A.lrho[k] = grho + eos_dp(P, rhoj) * gp;
}

// Adjoint of density_sum: λr_j -= Σ_i (λrho_j + λrho_i) m sc e.
__global__ void __launch_bounds__(kAdjThreads) k_adj_density(DevParams P, Sorted G, AdjBuf A) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    if (G.itype[k] == P.type_non_existent) return;
    const uint32_t id = G.id[k];
    const double xj = G.rx[k], yj = G.ry[k];
    const double lj = A.lrho[k];
    double grx = 0, gry = 0;
    const Stencil<2> st(P, G.key[k]);
    // the neighbours the force adjoint recorded, as one flat sequence (cells of
    // more than 32 particles searched in place), the lanes of a warp together
    const uint32_t* const masks = G.nbmask + k;
    const uint32_t over = masks[(size_t)9 * P.n];
    int c = -1;
    uint32_t bits = 0, base = 0, next = 0, end = 0;
    for (;;) {
        if (bits == 0 && next == end) {
            for (c++; c < 9; c++) {
                uint32_t cell;
                int sx, sy, sz;
                if (!st.cell(c, cell, sx, sy, sz)) continue;
                const uint32_t s = G.cell_start[cell];
                if (s == kEmpty) continue;
                if ((over >> c) & 1u) {
                    next = s;
                    end = G.cell_end[cell];
                    break;
                }
                bits = masks[(size_t)c * P.n];
                base = s;
                if (bits) break;
            }
            if (c >= 9) break;
        }
        uint32_t i;
        bool known;
        if (bits) {
            i = base + (uint32_t)(__ffs(bits) - 1);
            bits &= bits - 1;
            known = true;
        } else {
            i = next++;
            known = false;
        }
        const double ex = __dsub_rn(G.rx[i], xj), ey = __dsub_rn(G.ry[i], yj);
        const double s2 = exact_dist2<2>(ex, ey, 0.0);
        if (!known && !(i != k && G.itype[i] != P.type_non_existent && s2 < P.cut2)) continue;
        const double inv_d = rsqrt(s2);
        double sc, sc1d;
        cubic_sc(P, s2 * inv_d * P.inv_h, inv_d, sc, sc1d);
        const double cf = (lj + A.lrho[i]) * P.mass * sc;
        grx -= cf * ex;
        gry -= cf * ey;
    }
    A.out_rx[id] += grx;
    A.out_ry[id] += gry;
}

// Σ dL/d(piston vx) over the piston particles, in a fixed order.
__global__ void k_adj_piston_sum(const double* __restrict__ gvx, uint32_t start, uint32_t end,
                                 double* __restrict__ out) {
    __shared__ double part[256];
    double s = 0;
    for (uint32_t i = start + threadIdx.x; i < end; i += blockDim.x) s += gvx[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] += part[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = part[0];
}

__global__ void k_adj_seed(double* __restrict__ lry, uint32_t id, double value) { lry[id] += value; }

}  // namespace
}  // namespace rrsph

namespace rrsph_impl {

// A forward run kept for the reverse sweep.
struct AdjointRun {
    rrsph_adjoint_config cfg{};
    uint64_t N = 0, K = 0, nck = 0, nsamples = 0;
    uint64_t index0 = 0;  // solver step_index at the first step
    uint64_t step0 = 0;   // itimestep of the first step
    double dt = 0;
    std::vector<double> times;  // t_n, n = 0..N
    std::vector<void*> allocs;
    rrsph::Snap ck{}, seg{};
    rrsph::StepScalars* ck_scal = nullptr;  // [nck]
    double* seg_rho = nullptr;
    // the segment's forward grids: sorted keys and ids, and the neighbour masks
    // of each step's density pass ([K][n], [K][n], [K][10][n])
    uint32_t *seg_key = nullptr, *seg_id = nullptr, *seg_mask = nullptr;
    double* lam[2][6] = {};
    double *la_x = nullptr, *la_y = nullptr, *lrho = nullptr, *pr2 = nullptr, *gvx = nullptr;
    double* g_steps = nullptr;
    double *end_rho = nullptr, *end_p = nullptr;  // density and pressure at the end of the forward run
    unsigned long long* gauge_best = nullptr;
    uint32_t* gauge_id = nullptr;
    std::vector<double> gauges;
    std::vector<uint32_t> gauge_ids;
    int fourier_n = 0;
    double fourier_omega = 0;
    double fourier_coef[16] = {};
    bool valid = false;
};

void adjoint_release(rrsph_solver* s) {
    if (!s->adj) return;
    for (void* p : s->adj->allocs)
        if (p) cudaFree(p);
    delete s->adj;
    s->adj = nullptr;
}

}  // namespace rrsph_impl

namespace {

using rrsph_impl::AdjointRun;

#define ADJ_TRY(call)                                                                                        \
    do {                                                                                                     \
        cudaError_t err_ = (call);                                                                           \
        if (err_ != cudaSuccess)                                                                             \
            return set_error(err_ == cudaErrorMemoryAllocation ? RRSPH_ERR_OUT_OF_MEMORY : RRSPH_ERR_CUDA,   \
                             std::string(#call) + ": " + cudaGetErrorString(err_));                          \
    } while (0)

template <typename T>
int adj_alloc(AdjointRun* run, T** ptr, size_t count) {
    void* p = nullptr;
    ADJ_TRY(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
    run->allocs.push_back(p);
    *ptr = static_cast<T*>(p);
    return RRSPH_OK;
}

int alloc_snap(AdjointRun* run, rrsph::Snap& sn, size_t slots, size_t n) {
    int rc;
    double** f[6] = {&sn.rx, &sn.ry, &sn.vx, &sn.vy, &sn.ax, &sn.ay};
    for (auto* p : f)
        if ((rc = adj_alloc(run, p, slots * n)) != 0) return rc;
    return adj_alloc(run, &sn.itype, slots * n);
}

// Copies between the solver's state and a snapshot slot.
int snap_copy(rrsph_solver* s, const rrsph::Snap& sn, size_t slot, bool to_solver) {
    const size_t n = s->P.n;
    double* sf[6] = {s->S.rx, s->S.ry, s->S.vx, s->S.vy, s->S.ax, s->S.ay};
    double* kf[6] = {sn.rx, sn.ry, sn.vx, sn.vy, sn.ax, sn.ay};
    for (int f = 0; f < 6; f++) {
        double* slotp = kf[f] + slot * n;
        ADJ_TRY(cudaMemcpyAsync(to_solver ? sf[f] : slotp, to_solver ? slotp : sf[f], n * sizeof(double),
                                cudaMemcpyDeviceToDevice, s->stream));
    }
    int32_t* it = sn.itype + slot * n;
    ADJ_TRY(cudaMemcpyAsync(to_solver ? s->S.itype : it, to_solver ? it : s->S.itype, n * sizeof(int32_t),
                            cudaMemcpyDeviceToDevice, s->stream));
    return RRSPH_OK;
}

int checkpoint_save(rrsph_solver* s, AdjointRun* run, size_t slot) {
    int rc = snap_copy(s, run->ck, slot, false);
    if (rc) return rc;
    const int par = (int)(s->step_index & 1);
    ADJ_TRY(cudaMemcpyAsync(run->ck_scal + slot, s->scal + par, sizeof(rrsph::StepScalars), cudaMemcpyDeviceToDevice,
                            s->stream));
    return RRSPH_OK;
}

int checkpoint_restore(rrsph_solver* s, AdjointRun* run, size_t slot, uint64_t m) {
    int rc = snap_copy(s, run->ck, slot, true);
    if (rc) return rc;
    s->step_index = run->index0 + m;
    s->keys_ready = false;  // the next step runs predict + keys on the restored state
    const int par = (int)(s->step_index & 1);
    ADJ_TRY(cudaMemcpyAsync(s->scal + par, run->ck_scal + slot, sizeof(rrsph::StepScalars), cudaMemcpyDeviceToDevice,
                            s->stream));
    return RRSPH_OK;
}

bool piston_active(const rrsph_solver* s, double t) {
    const auto& P = s->P;
    return (P.nwm == 2 || P.nwm == 3 || P.nwm == 5) && P.nwm_valid && t >= P.nwm_time_start;
}

int check_method(const rrsph_solver* s) {
    const auto& P = s->P;
    if (s->precision != RRSPH_PRECISION_FP64) return set_error(RRSPH_ERR_UNSUPPORTED, "adjoint: needs an FP64 solver");
    if (s->dim != 2) return set_error(RRSPH_ERR_UNSUPPORTED, "adjoint: 2D only");
    if (P.density_treatment != 0) return set_error(RRSPH_ERR_UNSUPPORTED, "adjoint: summation density only");
    if (P.density_skf != 1 || P.intf_skf != 1 || (P.art_visc && P.av_skf != 1))
        return set_error(RRSPH_ERR_UNSUPPORTED, "adjoint: cubic spline kernel only");
    if (P.art_pressure || P.avg_vel)
        return set_error(RRSPH_ERR_UNSUPPORTED, "adjoint: artificial pressure and XSPH are not supported");
    if (P.dt_method == 2) return set_error(RRSPH_ERR_UNSUPPORTED, "adjoint: constant dt only");
    if (P.nwm == 4) return set_error(RRSPH_ERR_UNSUPPORTED, "adjoint: the wall-disappear wave maker is not supported");
    return RRSPH_OK;
}

int sample_index(const AdjointRun* run, uint64_t m, uint64_t* s) {
    const auto& c = run->cfg;
    if (m < c.sample_from || (m - c.sample_from) % c.sample_every) return 0;
    *s = (m - c.sample_from) / c.sample_every;
    return 1;
}

void enqueue_gauge(rrsph_solver* s, AdjointRun* run, uint64_t si) {
    const auto& c = run->cfg;
    const uint32_t n = s->P.n;
    const unsigned blocks = (n + 255) / 256;
    const double radius = c.gauge_search_n * s->params.hsml;
    rrsph::k_gauge_max<<<blocks, 256, 0, s->stream>>>(n, s->S.rx, s->S.ry, s->S.itype, c.gauge_x, radius,
                                                       c.gauge_type, run->gauge_best + si);
    rrsph::k_gauge_arg<<<blocks, 256, 0, s->stream>>>(n, s->S.rx, s->S.ry, s->S.itype, c.gauge_x, radius,
                                                       c.gauge_type, run->gauge_best + si, run->gauge_id + si);
    s->launches += 2;
}

int sync_and_check(rrsph_solver* s, const char* fn) {
    ADJ_TRY(cudaMemcpyAsync(s->h_flags, s->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost, s->stream));
    ADJ_TRY(cudaStreamSynchronize(s->stream));
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(RRSPH_ERR_CUDA, std::string(fn) + ": " + cudaGetErrorString(e));
    return rrsph_impl::flags_status(s, *s->h_flags);
}

// One reverse step n on the states of segment slot j.
void enqueue_reverse_step(rrsph_solver* s, AdjointRun* run, uint64_t m, size_t j, int cur) {
    const size_t n = s->P.n;
    cudaStream_t st = s->stream;
    rrsph::SnapView sv{run->seg.rx + j * n, run->seg.ry + j * n, run->seg.vx + j * n, run->seg.vy + j * n,
                       run->seg.ax + j * n, run->seg.ay + j * n, run->seg.itype + j * n};
    // the forward step's grid and neighbour masks (recorded in the recompute);
    // the cell table is rebuilt from the recorded keys, from empty
    rrsph::Sorted G = s->G;
    G.key = run->seg_key + j * n;
    G.id = run->seg_id + j * n;
    G.nbmask = run->seg_mask + j * 10 * n;
    rrsph::launch_clear_cells(G.cell_start, s->P.max_cells, st);
    const int nxt = cur ^ 1;
    rrsph::AdjBuf A{run->lam[cur][0], run->lam[cur][1], run->lam[cur][2], run->lam[cur][3], run->lam[cur][4],
                    run->lam[cur][5], run->lam[nxt][0], run->lam[nxt][1], run->lam[nxt][2], run->lam[nxt][3],
                    run->lam[nxt][4], run->lam[nxt][5], run->la_x, run->la_y, run->lrho, run->pr2, run->gvx};
    const double t = run->times[m];
    const int piston = piston_active(s, t) ? 1 : 0;
    const double v_dt = (run->step0 + m) ? run->dt : run->dt * 0.5;
    const unsigned blocks = (unsigned)((n + 255) / 256);
    const unsigned gblocks = (unsigned)((n + rrsph::kAdjThreads - 1) / rrsph::kAdjThreads);
    rrsph::k_adj_reorder<<<blocks, 256, 0, st>>>(s->P, G, sv, run->seg_rho + j * n, A, run->dt, v_dt, piston);
    rrsph::k_adj_forces<<<gblocks, rrsph::kAdjThreads, 0, st>>>(s->P, G, A, run->dt);
    rrsph::k_adj_density<<<gblocks, rrsph::kAdjThreads, 0, st>>>(s->P, G, A);
    s->launches += 4;
    if (piston) {
        rrsph::k_adj_piston_sum<<<1, 256, 0, st>>>(run->gvx, s->P.nwm_start, s->P.nwm_end, run->g_steps + m);
        s->launches++;
    }
}

void enqueue_seed(rrsph_solver* s, AdjointRun* run, uint64_t m, int cur, const double* dgauges) {
    uint64_t si;
    if (!sample_index(run, m, &si)) return;
    const uint32_t id = run->gauge_ids[si];
    if (id == 0xFFFFFFFFu || dgauges[si] == 0.0) return;
    rrsph::k_adj_seed<<<1, 1, 0, s->stream>>>(run->lam[cur][1], id, dgauges[si]);
    s->launches++;
}

}  // namespace

extern "C" int rrsph_set_piston_fourier(rrsph_solver* s, uint32_t ncoef, double omega, const double* coef) {
    if (!s) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_set_piston_fourier: null solver");
    if (ncoef > RRSPH_PISTON_FOURIER_MAX || (ncoef && !coef) || !std::isfinite(omega))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_set_piston_fourier: bad coefficients");
    if (ncoef && s->P.nwm != 2) return set_error(RRSPH_ERR_UNSUPPORTED, "rrsph_set_piston_fourier: needs nwm == 2");
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(RRSPH_ERR_CUDA, "rrsph_set_piston_fourier: device");
    // the step graphs hold the parameters by value
    cudaStreamSynchronize(s->stream);
    rrsph_impl::destroy_step_graphs(s);
    s->P.fourier_n = (int)ncoef;
    s->P.fourier_omega = ncoef ? omega : 0.0;
    for (int k = 0; k < RRSPH_PISTON_FOURIER_MAX; k++) s->P.fourier_coef[k] = k < (int)ncoef ? coef[k] : 0.0;
    return RRSPH_OK;
}

extern "C" int rrsph_adjoint_forward(rrsph_solver* s, const rrsph_adjoint_config* cfg, double* time_io,
                                     double* gauges, uint64_t max_samples, uint64_t* nsamples) {
    if (!s || !cfg || !time_io) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_adjoint_forward: null argument");
    if (cfg->struct_size != sizeof(rrsph_adjoint_config))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_adjoint_forward: cfg->struct_size mismatch");
    if (cfg->nsteps == 0 || cfg->checkpoint_every == 0 || cfg->sample_every == 0 || !(cfg->gauge_search_n > 0))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_adjoint_forward: nsteps, checkpoint_every, sample_every "
                                                     "and gauge_search_n must be positive");
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(RRSPH_ERR_CUDA, "rrsph_adjoint_forward: device");
    int rc = check_method(s);
    if (rc) return rc;
    rrsph_impl::adjoint_release(s);
    AdjointRun* run = new AdjointRun();
    s->adj = run;
    run->cfg = *cfg;
    run->N = cfg->nsteps;
    run->K = std::min<uint64_t>(cfg->checkpoint_every, run->N);
    run->nck = (run->N + run->K - 1) / run->K + 1;  // multiples of K below N, and N
    run->nsamples = run->N >= cfg->sample_from ? (run->N - cfg->sample_from) / cfg->sample_every + 1 : 0;
    run->fourier_n = s->P.fourier_n;
    run->fourier_omega = s->P.fourier_omega;
    std::memcpy(run->fourier_coef, s->P.fourier_coef, sizeof(run->fourier_coef));
    const size_t n = s->P.n;
    if ((rc = alloc_snap(run, run->ck, run->nck, n)) != 0 || (rc = alloc_snap(run, run->seg, run->K, n)) != 0 ||
        (rc = adj_alloc(run, &run->ck_scal, run->nck)) != 0 || (rc = adj_alloc(run, &run->seg_rho, run->K * n)) != 0 ||
        (rc = adj_alloc(run, &run->seg_key, run->K * n)) != 0 || (rc = adj_alloc(run, &run->seg_id, run->K * n)) != 0 ||
        (rc = adj_alloc(run, &run->seg_mask, run->K * 10 * n)) != 0)
        return rc;
    for (auto& set : run->lam)
        for (auto& p : set)
            if ((rc = adj_alloc(run, &p, n)) != 0) return rc;
    if ((rc = adj_alloc(run, &run->la_x, n)) != 0 || (rc = adj_alloc(run, &run->la_y, n)) != 0 ||
        (rc = adj_alloc(run, &run->lrho, n)) != 0 || (rc = adj_alloc(run, &run->pr2, n)) != 0 ||
        (rc = adj_alloc(run, &run->gvx, n)) != 0 || (rc = adj_alloc(run, &run->g_steps, run->N)) != 0 ||
        (rc = adj_alloc(run, &run->end_rho, n)) != 0 || (rc = adj_alloc(run, &run->end_p, n)) != 0 ||
        (rc = adj_alloc(run, &run->gauge_best, run->nsamples)) != 0 ||
        (rc = adj_alloc(run, &run->gauge_id, run->nsamples)) != 0)
        return rc;
    cudaStream_t st = s->stream;
    ADJ_TRY(cudaMemsetAsync(run->gauge_best, 0, std::max<uint64_t>(run->nsamples, 1) * sizeof(unsigned long long), st));
    ADJ_TRY(cudaMemsetAsync(run->gauge_id, 0xFF, std::max<uint64_t>(run->nsamples, 1) * sizeof(uint32_t), st));
    if ((rc = rrsph_set_time(s, *time_io)) != 0) return rc;
    ADJ_TRY(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), st));
    {   // the step counter and dt the run starts with
        const int par = (int)(s->step_index & 1);
        ADJ_TRY(cudaMemcpyAsync(s->h_scal, s->scal + par, sizeof(rrsph::StepScalars), cudaMemcpyDeviceToHost, st));
        ADJ_TRY(cudaStreamSynchronize(st));
        run->step0 = s->h_scal->step;
        run->dt = s->h_scal->dt;
    }
    run->index0 = s->step_index;
    run->times.resize(run->N + 1);
    run->times[0] = *time_io;
    for (uint64_t m = 0; m < run->N; m++) run->times[m + 1] = run->times[m] + run->dt;

    // the smallest sampled state index after m
    auto next_sample = [cfg](uint64_t m) -> uint64_t {
        if (m + 1 <= cfg->sample_from) return cfg->sample_from;
        const uint64_t rel = m + 1 - cfg->sample_from;
        return cfg->sample_from + ((rel + cfg->sample_every - 1) / cfg->sample_every) * cfg->sample_every;
    };
    uint64_t m = 0, si;
    if ((rc = checkpoint_save(s, run, 0)) != 0) return rc;
    if (sample_index(run, 0, &si)) enqueue_gauge(s, run, si);
    while (m < run->N) {
        const uint64_t next = std::min({(m / run->K + 1) * run->K, next_sample(m), run->N});
        if ((rc = rrsph_step_async(s, next - m)) != 0) return rc;
        m = next;
        if (m % run->K == 0 && m < run->N && (rc = checkpoint_save(s, run, m / run->K)) != 0) return rc;
        if (sample_index(run, m, &si)) enqueue_gauge(s, run, si);
    }
    if ((rc = checkpoint_save(s, run, run->nck - 1)) != 0) return rc;
    ADJ_TRY(cudaMemcpyAsync(run->end_rho, s->S.rho, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ADJ_TRY(cudaMemcpyAsync(run->end_p, s->S.p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    if ((rc = sync_and_check(s, "rrsph_adjoint_forward")) != 0) return rc;
    std::vector<unsigned long long> best(run->nsamples);
    run->gauge_ids.assign(run->nsamples, 0xFFFFFFFFu);
    if (run->nsamples) {
        ADJ_TRY(cudaMemcpy(best.data(), run->gauge_best, run->nsamples * sizeof(unsigned long long),
                           cudaMemcpyDeviceToHost));
        ADJ_TRY(cudaMemcpy(run->gauge_ids.data(), run->gauge_id, run->nsamples * sizeof(uint32_t),
                           cudaMemcpyDeviceToHost));
    }
    run->gauges.resize(run->nsamples);
    for (uint64_t k = 0; k < run->nsamples; k++) {
        double g;
        std::memcpy(&g, &best[k], sizeof(g));
        run->gauges[k] = g;
        if (gauges && k < max_samples) gauges[k] = g;
    }
    if (nsamples) *nsamples = run->nsamples;
    *time_io = run->times[run->N];
    run->valid = true;
    return RRSPH_OK;
}

extern "C" int rrsph_adjoint_reverse(rrsph_solver* s, const double* dgauges, double* dcoef, double* dpiston_vx) {
    if (!s) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_adjoint_reverse: null solver");
    AdjointRun* run = s->adj;
    if (!run || !run->valid)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_adjoint_reverse: no recorded forward run");
    if (run->nsamples && !dgauges) return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_adjoint_reverse: null dgauges");
    if (run->fourier_n != s->P.fourier_n || run->fourier_omega != s->P.fourier_omega ||
        std::memcmp(run->fourier_coef, s->P.fourier_coef, sizeof(run->fourier_coef)) != 0)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_adjoint_reverse: the piston changed since the forward run");
    if (cudaSetDevice(s->device) != cudaSuccess) return set_error(RRSPH_ERR_CUDA, "rrsph_adjoint_reverse: device");
    cudaStream_t st = s->stream;
    const size_t n = s->P.n;
    int rc;
    for (auto& set : run->lam)
        for (double* p : set) ADJ_TRY(cudaMemsetAsync(p, 0, n * sizeof(double), st));
    ADJ_TRY(cudaMemsetAsync(run->g_steps, 0, run->N * sizeof(double), st));
    ADJ_TRY(cudaMemsetAsync(s->flags, 0, sizeof(uint32_t), st));
    int cur = 0;
    enqueue_seed(s, run, run->N, cur, dgauges);
    const uint64_t nseg = run->nck - 1;
    for (uint64_t c = nseg; c-- > 0;) {
        const uint64_t m0 = c * run->K, m1 = std::min(m0 + run->K, run->N);
        if ((rc = checkpoint_restore(s, run, c, m0)) != 0) return rc;
        for (uint64_t m = m0; m < m1; m++) {  // recompute the segment's states and densities
            if ((rc = snap_copy(s, run->seg, m - m0, false)) != 0) return rc;
            if ((rc = rrsph_step_async(s, 1)) != 0) return rc;
            ADJ_TRY(cudaMemcpyAsync(run->seg_rho + (m - m0) * n, s->S.rho, n * sizeof(double),
                                    cudaMemcpyDeviceToDevice, st));
            ADJ_TRY(cudaMemcpyAsync(run->seg_key + (m - m0) * n, s->G.key, n * sizeof(uint32_t),
                                    cudaMemcpyDeviceToDevice, st));
            ADJ_TRY(cudaMemcpyAsync(run->seg_id + (m - m0) * n, s->G.id, n * sizeof(uint32_t),
                                    cudaMemcpyDeviceToDevice, st));
            ADJ_TRY(cudaMemcpyAsync(run->seg_mask + (m - m0) * 10 * n, s->G.nbmask, 10 * n * sizeof(uint32_t),
                                    cudaMemcpyDeviceToDevice, st));
        }
        for (uint64_t m = m1; m-- > m0;) {
            enqueue_reverse_step(s, run, m, m - m0, cur);
            cur ^= 1;
            enqueue_seed(s, run, m, cur, dgauges);
        }
        // the forward steps' key passes clear only the cells they filled: leave
        // no cell of the reversed grids behind
        rrsph::launch_clear_cells(s->G.cell_start, s->P.max_cells, st);
        s->launches++;
    }
    if ((rc = checkpoint_restore(s, run, run->nck - 1, run->N)) != 0) return rc;
    ADJ_TRY(cudaMemcpyAsync(s->S.rho, run->end_rho, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    ADJ_TRY(cudaMemcpyAsync(s->S.p, run->end_p, n * sizeof(double), cudaMemcpyDeviceToDevice, st));
    std::vector<double> g(run->N);
    ADJ_TRY(cudaMemcpyAsync(g.data(), run->g_steps, run->N * sizeof(double), cudaMemcpyDeviceToHost, st));
    if ((rc = sync_and_check(s, "rrsph_adjoint_reverse")) != 0) return rc;
    if (dpiston_vx) std::memcpy(dpiston_vx, g.data(), run->N * sizeof(double));
    if (dcoef) {
        for (int k = 1; k <= run->fourier_n; k++) {
            double acc = 0;
            for (uint64_t m = 0; m < run->N; m++)
                acc += g[m] * (k * run->fourier_omega * std::cos(k * run->fourier_omega * run->times[m]));
            dcoef[k - 1] = acc;
        }
    }
    return RRSPH_OK;
}
