// kernels_mixed.cu — the density and force gathers of the FP32-mixed step.
//
// Pair arithmetic is float32 on cell-relative coordinates: the reorder stores
// each particle's offset from the corner of its own cell (computed in double),
// and a pair's separation is (offset_i + cell displacement) - offset_j, which
// keeps ~1e-7 relative accuracy of h anywhere in the domain. Pairs whose float
// distance lies within a guard band of the cutoff are re-tested with the
// reference's double arithmetic, so the neighbour set equals the FP64 one.
// Sums are accumulated per neighbour cell in float and Kahan-compensated across
// cells; the per-particle EOS and all state updates stay in double.
//
// One thread per particle in cell order. The 3^dim stencil is a runtime loop
// (a single copy of the pair body keeps the kernel in the instruction cache);
// reciprocals and square roots use the fast MUFU forms (<= 2 ulp).
#include "kernels.cuh"
#include "neighbour.cuh"
#include "step_particle.cuh"

namespace rrsph {

namespace {

constexpr int kVlBatch = 4;       // list entries the reuse density gather loads together (one uint4)
constexpr int kVlForceBatch = 2;  // neighbours the reuse force gather loads together

struct Kahan {
    float s, c;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return f2d(s) - f2d(c); }
};

// W(q) of smoothing kernel skf (SmoothingKernel.h:20-252), float.
__device__ __forceinline__ float kernel_wf(int skf, float f, float q) {
    switch (skf) {
    case 2: return f * __expf(-q * q);
    case 3: {
        if (q <= 2.0f) {
            const float t = 1.0f - 0.5f * q;
            const float t2 = t * t;
            return f * (t2 * t2) * (2.0f * q + 1.0f);
        }
        return 0.0f;
    }
    case 4: {
        if (q <= 2.0f) { const float t = 2.0f - q; return f * (t * t * t); }
        return 0.0f;
    }
    default:
        if (q <= 1.0f) return f * ((2.0f / 3.0f - q * q) + q * q * q * 0.5f);
        if (q <= 2.0f) { const float t = 2.0f - q; return f * ((1.0f / 6.0f) * (t * t * t)); }
        return 0.0f;
    }
}

// dW/dr = diff * scale with diff = r_i - r_j (SmoothingKernel.h:42-274), float.
__device__ __forceinline__ float kernel_dwdr_scalef(int skf, float f, float q, float inv_dist, float inv_h) {
    switch (skf) {
    case 2: return inv_h * inv_h * (-2.0f) * (f * __expf(-q * q));
    case 3: {
        if (q < 1.e-6f || !(q < 2.0f)) return 0.0f;
        const float t = 1.0f - 0.5f * q;
        const float t3 = t * t * t;
        return inv_h * inv_dist * f * 2.0f * (t3 * t - (2.0f * q + 1.0f) * t3);
    }
    case 4: {
        if (q < 2.0f) { const float t = 2.0f - q; return inv_h * inv_dist * f * (-3.0f * t * t); }
        return 0.0f;
    }
    default:
        if (q <= 1.0f) return inv_h * inv_h * f * (-2.0f + 1.5f * q);
        if (q <= 2.0f) { const float t = 2.0f - q; return -(inv_h * inv_dist) * f * (t * t * 0.5f); }
        return 0.0f;
    }
}

// Cutoff test: float test outside the guard band, the reference's double test inside it.
// The guard band is rare, so its double positions come from the id-order state.
template <int DIM>
__device__ __forceinline__ bool within_cutoff(const DevParams& P, const State& S, const Sorted& G, uint32_t i,
                                              uint32_t k, float d2) {
    if (d2 >= P.mf.cut2_hi) return false;
    if (d2 < P.mf.cut2_lo) return true;
    const uint32_t a = G.id[i], b = G.id[k];
    const double dx = __dsub_rn(S.rx[a], S.rx[b]), dy = __dsub_rn(S.ry[a], S.ry[b]);
    const double dz = DIM == 3 ? __dsub_rn(S.rz[a], S.rz[b]) : 0.0;
    return exact_dist2<DIM>(dx, dy, dz) < P.cut2;
}

__device__ __forceinline__ void warp_sum_add(unsigned long long* dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}
__device__ __forceinline__ void warp_max_bits(unsigned long long* dst, double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xFFFFFFFFu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0) atomicMax(dst, dbits(v));
}

// eos_art_p (EOS.cpp:31-34) in float on the density deviation d = rho - rho0:
// (rho/rho0)^7 - 1 = t (1 + x + ... + x^6) with t = d/rho0, x = 1 + t, which
// has no cancellation, so p keeps float accuracy relative to itself.
__device__ __forceinline__ float eos_pf(const MixedF& M, float d) {
    const float t = d * M.inv_rho0;
    const float x = 1.0f + t;
    const float sum = 1.0f + x * (1.0f + x * (1.0f + x * (1.0f + x * (1.0f + x * (1.0f + x)))));
    return M.B * t * sum;
}

// density_sum / density_con (Density.h:25-114) + EOS. SKF: 1 = cubic only
// (every kernel choice cubic), 0 = any kernel (runtime switch).
template <int DIM, int SKF>
__global__ void __launch_bounds__(kMaxGatherThreads) k_density_mixed(DevParams P, State S, Sorted G,
                                                                  StepScalars* __restrict__ scal,
                                                                  uint32_t* __restrict__ flags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    uint32_t cnt = 0;
    if (active) {
        const MixedF& M = P.mf;
        const uint32_t id = G.id[k];
        const bool cont = P.density_treatment != 0;
        const bool delta = P.density_treatment == 2;
        const float4 pj = G.P4[k];
        const int32_t tj = __float_as_int(pj.w);
        float4 vdj = make_float4(0, 0, 0, 0);
        if (cont) vdj = G.VD4[k];
        const int skf = SKF ? SKF : P.density_skf;
        const float f = M.kf[skf];
        Kahan acc{0.0f, 0.0f};
        const bool masks = DIM == 2 && G.nbmask != nullptr;
        uint32_t over = 0;
        // 2D: the neighbour masks of the 9 cells, kept in registers and stored
        // together at the end so the stores stay coalesced
        uint32_t m0 = 0, m1 = 0, m2 = 0, m3 = 0, m4 = 0, m5 = 0, m6 = 0, m7 = 0, m8 = 0;
        constexpr int NC = DIM == 3 ? 27 : 9;
        if (tj != P.type_non_existent) {
            const Stencil<DIM> st(P, G.key[k]);
#pragma unroll 1
            for (int c = 0; c < NC; c++) {
                uint32_t cell;
                int sx, sy, sz;
                if (!st.cell(c, cell, sx, sy, sz)) continue;
                const uint32_t s = G.cell_start[cell];
                if (s == kEmpty) continue;
                const uint32_t e = G.cell_end[cell];
                if (e - s > 32) over |= 1u << c;
                const float shx = (float)sx * M.cell - pj.x;
                const float shy = (float)sy * M.cell - pj.y;
                const float shz = DIM == 3 ? (float)sz * M.cell - pj.z : 0.0f;
                float part = 0.0f;
                uint32_t bits = 0;
                for (uint32_t i = s; i < e; i++) {
                    if (i == k) continue;
                    const float4 pi = G.P4[i];
                    if (__float_as_int(pi.w) == P.type_non_existent) continue;
                    const float dx = pi.x + shx, dy = pi.y + shy, dz = DIM == 3 ? pi.z + shz : 0.0f;
                    const float d2 = DIM == 3 ? dx * dx + dy * dy + dz * dz : dx * dx + dy * dy;
                    if (!within_cutoff<DIM>(P, S, G, i, k, d2)) continue;
                    cnt++;
                    if (i - s < 32) bits |= 1u << (i - s);
                    const float inv_dist = rsqrtf(d2);
                    const float q = d2 * inv_dist * M.inv_h;
                    if (!cont) {
                        part += kernel_wf(skf, f, q);
                    } else {
                        const float sc = kernel_dwdr_scalef(skf, f, q, inv_dist, M.inv_h);
                        const float4 vdi = G.VD4[i];
                        float vcc = (vdi.x - vdj.x) * dx + (vdi.y - vdj.y) * dy;
                        if (DIM == 3) vcc += (vdi.z - vdj.z) * dz;
                        float term = vcc * sc;
                        if (delta) {
                            // r_factor = dot(r_j - r_i, diff * sc) / |diff|^2 = -sc;
                            // rho_factor = (rho_i - rho_j) / rho_i on the deviations from rho0
                            const float rho_factor = __fdividef(vdi.w - vdj.w, M.rho0 + vdi.w);
                            term += 2.0f * M.dhc * (rho_factor * -sc);
                        }
                        part += term;
                    }
                }
                if (masks) {
                    switch (c) {
                    case 0: m0 = bits; break;
                    case 1: m1 = bits; break;
                    case 2: m2 = bits; break;
                    case 3: m3 = bits; break;
                    case 4: m4 = bits; break;
                    case 5: m5 = bits; break;
                    case 6: m6 = bits; break;
                    case 7: m7 = bits; break;
                    default: m8 = bits; break;
                    }
                }
                acc.add(M.mass * part);
            }
        }
        if (masks) {
            const size_t n = P.n;
            G.nbmask[k] = m0;
            G.nbmask[n + k] = m1;
            G.nbmask[2 * n + k] = m2;
            G.nbmask[3 * n + k] = m3;
            G.nbmask[4 * n + k] = m4;
            G.nbmask[5 * n + k] = m5;
            G.nbmask[6 * n + k] = m6;
            G.nbmask[7 * n + k] = m7;
            G.nbmask[8 * n + k] = m8;
            G.nbmask[9 * n + k] = over;
        }
        if (cnt > P.max_nb - 1) atomicOr(flags, RRSPH_FLAG_NEIGHBOUR_OVERFLOW);
        if (!cont) {
            // rho - rho0 = sum - (rho0 - m W(0)): the two are within a factor of two,
            // so the float difference is exact; the Kahan and rounding residuals follow
            const float d = ((acc.s - M.rho0_minus_w0_hi) - acc.c) - M.rho0_minus_w0_lo;
            const float rho = M.rho0 + d;
            const float pr = eos_pf(M, d);
            G.V4[k].w = rho;
            G.PR[k] = make_float2(pr, pr * __frcp_rn(rho * rho));
            S.rho[id] = P.rho0 + f2d(d);
            S.p[id] = f2d(pr);
        } else {
            const float d = (float)(S.rho[id] - P.rho0);
            const float pr = eos_pf(M, d);
            const float rf = G.V4[k].w;  // rho_predict, the density of the forces
            G.PR[k] = make_float2(pr, pr * __frcp_rn(rf * rf));
            S.p[id] = pr;
            S.drho[id] = acc.value();
        }
    }
    warp_sum_add(&scal->pairs, cnt);
}

// One pair's contribution to particle j's acceleration (and XSPH velocity):
// update_acceleration's inner loop (UpdateAcceleration.cpp:66-97).
template <int DIM, int SKF>
struct ForceAcc {
    // Lennard-Jones repulsion of a boundary neighbour (ExtForce.h), over |diff|.
    static __device__ __forceinline__ float lj_coef(const MixedF& M, float inv_dist) {
        const float rn = M.lj_rr0 * inv_dist;
        const float rn2 = rn * rn, rn4 = rn2 * rn2, rn8 = rn4 * rn4;
        return M.lj_D * (rn8 * rn4 - rn4) * (inv_dist * inv_dist);
    }
    const DevParams& P;
    const Sorted& G;
    float4 vj;
    float2 prj;
    float rhoj;
    bool ext, intf, visc, avel, form1;
    int intf_skf, av_skf;
    float cax, cay, caz, cvx, cvy, cvz, arvmu;

    __device__ __forceinline__ void pair(uint32_t i, float dx, float dy, float dz, float d2, int32_t ti) {
        pair_with(G.V4[i], G.PR[i], dx, dy, dz, d2, ti);
    }
    // The same with neighbour i's velocity + density (vi) and pressure pair (pri) given.
    __device__ __forceinline__ void pair_with(const float4 vi, const float2 pri, float dx, float dy, float dz,
                                              float d2, int32_t ti) {
        const MixedF& M = P.mf;
        const float inv_dist = rsqrtf(d2);
        const float dist = d2 * inv_dist;
        const float q = dist * M.inv_h;
        float m = 0.0f;  // coefficient of diff (= r_i - r_j) in this pair's acceleration
        if (ext && ti < 0 && dist < M.lj_rr0) m -= lj_coef(M, inv_dist);
        const float rhoi = vi.w;
        const float sc = kernel_dwdr_scalef(intf_skf, M.kf[intf_skf], q, inv_dist, M.inv_h);
        if (intf) {
            float pf = form1 ? __fdividef(prj.x + pri.x, rhoj * rhoi) : (pri.y + prj.y);
            if (P.art_pressure && (pri.x < 0 || prj.x < 0)) {
                const float w = kernel_wf(P.ap_skf, M.kf[P.ap_skf], q);
                const float api = pri.x < 0 ? (-M.ap_coef * pri.y) : 0.0f;
                const float apj = prj.x < 0 ? (-M.ap_coef * prj.y) : 0.0f;
                pf += (api + apj) * __powf(w * M.ap_inv_wdelta, M.ap_index);
            }
            m += sc * pf * M.mass;
        }
        if (visc) {
            // approaching pairs only (vr < 0); evaluated by every lane and masked,
            // so the lanes of a warp stay together
            float vr = -((vj.x - vi.x) * dx + (vj.y - vi.y) * dy);
            if (DIM == 3) vr -= (vj.z - vi.z) * dz;
            const float mu = fminf(__fdividef(M.h * vr, d2 + M.etq_h2), 0.0f);
            arvmu = fmaxf(arvmu, -mu);
            const float piv = __fdividef((M.av_beta * mu - M.av_alpha_c) * mu, 0.5f * (rhoi + rhoj));
            const float sca = (SKF || av_skf == intf_skf)
                                  ? sc
                                  : kernel_dwdr_scalef(av_skf, M.kf[av_skf], q, inv_dist, M.inv_h);
            m += sca * piv * M.mass;
        }
        cax += dx * m;
        cay += dy * m;
        if (DIM == 3) caz += dz * m;
        if (avel && ti > 0) {
            const int sk = SKF ? SKF : P.avel_skf;
            const float w = kernel_wf(sk, M.kf[sk], q);
            const float mv = __fdividef(M.mass * w * M.avel_coef2, rhoi + rhoj);
            cvx += (vi.x - vj.x) * mv;
            cvy += (vi.y - vj.y) * mv;
            if (DIM == 3) cvz += (vi.z - vj.z) * mv;
        }
    }
    // pair_with for the common method set, 2D: pressure form 2, Monaghan
    // viscosity, cubic kernel, no artificial pressure or XSPH; vi.z holds the
    // neighbour's p/rho^2. The same arithmetic as pair_with with those switches.
    __device__ __forceinline__ void pair_std(const float4 vi, float dx, float dy, float d2, int32_t ti) {
        const MixedF& M = P.mf;
        const float inv_dist = rsqrtf(d2);
        const float dist = d2 * inv_dist;
        const float q = dist * M.inv_h;
        float m = 0.0f;
        if (ext && ti < 0 && dist < M.lj_rr0) m -= lj_coef(M, inv_dist);
        const float rhoi = vi.w;
        const float sc = kernel_dwdr_scalef(1, M.kf[1], q, inv_dist, M.inv_h);
        m += sc * (vi.z + prj.y) * M.mass;
        const float vr = -((vj.x - vi.x) * dx + (vj.y - vi.y) * dy);
        const float mu = fminf(__fdividef(M.h * vr, d2 + M.etq_h2), 0.0f);
        arvmu = fmaxf(arvmu, -mu);
        const float piv = __fdividef((M.av_beta * mu - M.av_alpha_c) * mu, 0.5f * (rhoi + rhoj));
        m += sc * piv * M.mass;
        cax += dx * m;
        cay += dy * m;
    }
};

// update_acceleration (UpdateAcceleration.cpp:33-125) with the external
// (Lennard-Jones), internal (pressure), artificial-viscosity and XSPH terms.
// MASKS: iterate the neighbour bits the density pass recorded (2D) instead of
// searching the stencil cells again.
template <int DIM, int SKF, bool MASKS>
__global__ void __launch_bounds__(kMaxGatherThreads) k_forces_mixed(DevParams P, State S, Sorted G, uint32_t terms,
                                                                 StepScalars* __restrict__ scal,
                                                                 uint32_t* __restrict__ flags, int write_mu) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    double amag = 0, arvmu_d = 0;
    if (active) {
        const MixedF& M = P.mf;
        const uint32_t id = G.id[k];
        const float4 pj4 = G.P4[k];
        const int32_t tj = __float_as_int(pj4.w);
        ForceAcc<DIM, SKF> F{P, G, G.V4[k], G.PR[k], 0.0f, false, false, false, false, false, 0, 0,
                             0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        F.rhoj = F.vj.w;
        F.ext = (terms & RRSPH_TERM_EXTERNAL) && P.repulsive && tj > 0;
        F.intf = terms & RRSPH_TERM_INTERNAL;
        F.visc = (terms & RRSPH_TERM_ART_VISC) && P.art_visc;
        F.avel = (terms & RRSPH_TERM_AVERAGE_VELOCITY) && P.avg_vel;
        F.form1 = P.intf_form == 1;
        F.intf_skf = SKF ? SKF : P.intf_skf;
        F.av_skf = SKF ? SKF : P.av_skf;
        Kahan ax{0, 0}, ay{0, 0}, az{0, 0};
        Kahan avx{0, 0}, avy{0, 0}, avz{0, 0};
        if (tj != P.type_non_existent && MASKS) {
            // the pairs recorded by the density pass, as one flat sequence over the
            // stencil cells so that the warp runs the pair body together
            const Stencil<DIM> st(P, G.key[k]);
            const uint32_t over = G.nbmask[(size_t)9 * P.n + k];
            int c = -1;
            uint32_t bits = 0, s = 0;
            float shx = 0.0f, shy = 0.0f;
            for (;;) {
                if (bits == 0) {
                    if (c >= 0) {
                        ax.add(F.cax);
                        ay.add(F.cay);
                        if (F.avel) {
                            avx.add(F.cvx);
                            avy.add(F.cvy);
                        }
                        F.cax = F.cay = F.cvx = F.cvy = 0.0f;
                    }
                    for (c++; c < 9; c++) {
                        if (over & (1u << c)) continue;
                        const uint32_t bb = G.nbmask[(size_t)c * P.n + k];
                        if (!bb) continue;
                        uint32_t cell;
                        int sx, sy, sz;
                        st.cell(c, cell, sx, sy, sz);
                        s = G.cell_start[cell];
                        shx = (float)sx * M.cell - pj4.x;
                        shy = (float)sy * M.cell - pj4.y;
                        bits = bb;
                        break;
                    }
                    if (c >= 9) break;
                }
                const uint32_t b = __ffs(bits) - 1;
                bits &= bits - 1;
                const uint32_t i = s + b;
                const float4 pi4 = G.P4[i];
                const float dx = pi4.x + shx, dy = pi4.y + shy;
                F.pair(i, dx, dy, 0.0f, dx * dx + dy * dy, __float_as_int(pi4.w));
            }
            // cells with more than 32 particles: search them
            for (uint32_t rest = over; rest; rest &= rest - 1) {
                const int cc = __ffs(rest) - 1;
                uint32_t cell;
                int sx, sy, sz;
                if (!st.cell(cc, cell, sx, sy, sz)) continue;
                const uint32_t s0 = G.cell_start[cell];
                if (s0 == kEmpty) continue;
                const uint32_t e0 = G.cell_end[cell];
                const float hx = (float)sx * M.cell - pj4.x;
                const float hy = (float)sy * M.cell - pj4.y;
                F.cax = F.cay = F.cvx = F.cvy = 0.0f;
                for (uint32_t i = s0; i < e0; i++) {
                    if (i == k) continue;
                    const float4 pi4 = G.P4[i];
                    const int32_t ti = __float_as_int(pi4.w);
                    if (ti == P.type_non_existent) continue;
                    const float dx = pi4.x + hx, dy = pi4.y + hy;
                    const float d2 = dx * dx + dy * dy;
                    if (!within_cutoff<DIM>(P, S, G, i, k, d2)) continue;
                    F.pair(i, dx, dy, 0.0f, d2, ti);
                }
                ax.add(F.cax);
                ay.add(F.cay);
                if (F.avel) {
                    avx.add(F.cvx);
                    avy.add(F.cvy);
                }
            }
        } else if (tj != P.type_non_existent) {
            const Stencil<DIM> st(P, G.key[k]);
            constexpr int NC = DIM == 3 ? 27 : 9;
#pragma unroll 1
            for (int c = 0; c < NC; c++) {
                uint32_t cell;
                int sx, sy, sz;
                if (!st.cell(c, cell, sx, sy, sz)) continue;
                const uint32_t s = G.cell_start[cell];
                if (s == kEmpty) continue;
                const uint32_t e = G.cell_end[cell];
                const float shx = (float)sx * M.cell - pj4.x;
                const float shy = (float)sy * M.cell - pj4.y;
                const float shz = DIM == 3 ? (float)sz * M.cell - pj4.z : 0.0f;
                F.cax = F.cay = F.caz = F.cvx = F.cvy = F.cvz = 0.0f;
                for (uint32_t i = s; i < e; i++) {
                    if (i == k) continue;
                    const float4 pi4 = G.P4[i];
                    const int32_t ti = __float_as_int(pi4.w);
                    if (ti == P.type_non_existent) continue;
                    const float dx = pi4.x + shx, dy = pi4.y + shy, dz = DIM == 3 ? pi4.z + shz : 0.0f;
                    const float d2 = DIM == 3 ? dx * dx + dy * dy + dz * dz : dx * dx + dy * dy;
                    if (!within_cutoff<DIM>(P, S, G, i, k, d2)) continue;
                    F.pair(i, dx, dy, dz, d2, ti);
                }
                ax.add(F.cax);
                ay.add(F.cay);
                if (DIM == 3) az.add(F.caz);
                if (F.avel) {
                    avx.add(F.cvx);
                    avy.add(F.cvy);
                    if (DIM == 3) avz.add(F.cvz);
                }
            }
        }
        const double g = (terms & RRSPH_TERM_GRAVITY) ? P.g : 0.0;
        const double axd = ax.value(), ayd = ay.value() - g, azd = DIM == 3 ? az.value() : 0.0;
        S.ax[id] = axd;
        S.ay[id] = ayd;
        if (DIM == 3) S.az[id] = azd;
        if (F.avel) {
            S.avx[id] = avx.value();
            S.avy[id] = avy.value();
            if (DIM == 3) S.avz[id] = avz.value();
        }
        arvmu_d = F.arvmu;
        if (write_mu) S.mu[id] = arvmu_d;
        if (P.dt_reduce) amag = sqrt(axd * axd + ayd * ayd + azd * azd);
    }
    if (P.dt_method == 2 && P.dt_reduce) {
        warp_max_bits(&scal->amax_bits, amag);
        warp_max_bits(&scal->mumax_bits, arvmu_d);
    }
}

// ------------------------------------------------------- neighbour reuse --
// 2D FP32-mixed step with summation density. A particle's candidate list
// holds the particles within cutoff + skin of it when the grid was last built;
// while no particle has moved more than skin/2 since then, every pair within
// the cutoff is in the lists, and each step tests the list instead of the 9
// stencil cells (the pair set is the reference's: the same cutoff test). Each
// particle's build cell stays its reference cell for the cell-relative
// offsets until the next build.

__global__ void k_vl_decide(cudaGraphConditionalHandle h, const uint32_t* __restrict__ rebuild) {
    cudaGraphSetConditional(h, *rebuild ? 1u : 0u);
}
__global__ void k_vl_reset(uint32_t* __restrict__ rebuild, uint32_t* __restrict__ gone,
                           unsigned long long* __restrict__ builds) {
    *rebuild = 0u;
    *gone = 0u;
    *builds += 1ull;
}
// After an upload: a flag raised by the key pass that ran for the replaced
// positions is dropped (the next key pass checks the uploaded ones), unless no
// list exists yet (all bits set) or the last build left out a non-existent
// particle or overflowed a list.
__global__ void k_vl_upload_check(uint32_t* __restrict__ rebuild, const uint32_t* __restrict__ gone) {
    if (*rebuild != 0xFFFFFFFFu) *rebuild = *gone ? 1u : 0u;
}

// After this step's grid (sort + reorder): each particle's candidates, four
// entries gathered in registers and stored as one uint4 into the group's slab
// (the lanes of a warp store neighbouring uint4s). The cell equals the cutoff,
// so a candidate within cutoff + skin can lie two cells away: a particle within
// one skin of a cell edge also searches the cells beyond that edge.
__global__ void __launch_bounds__(kMaxGatherThreads) k_vl_build(DevParams P, State S, Sorted G) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.n) return;
    const MixedF& M = P.mf;
    const uint32_t id = G.id[k], key = G.key[k];
    const float4 pj = G.P4[k];
    const uint32_t cx = second_bits(key), cy = second_bits(key >> 1);
    S.bcxy[id] = cx | (cy << 16);
    S.slot[id] = k;
    S.boff[id] = make_float2(pj.x, pj.y);
    uint4* const slab = reinterpret_cast<uint4*>(G.vlist) + k;  // group g at slab[g * n]
    uint4 buf = make_uint4(kVlNone, kVlNone, kVlNone, kVlNone);
    uint32_t nl = 0;
    if (__float_as_int(pj.w) == P.type_non_existent) atomicOr(S.vl_gone, 1u);
    if (__float_as_int(pj.w) != P.type_non_existent) {
        const float edge = P.vl_skin_edge;
        const int x0 = (pj.x < edge && cx >= 2) ? -2 : (cx >= 1 ? -1 : 0);
        const int x1 = (pj.x > M.cell - edge && cx + 2 <= kMaxCellCoord2) ? 2 : (cx + 1 <= kMaxCellCoord2 ? 1 : 0);
        const int y0 = (pj.y < edge && cy >= 2) ? -2 : (cy >= 1 ? -1 : 0);
        const int y1 = (pj.y > M.cell - edge && cy + 2 <= kMaxCellCoord2) ? 2 : (cy + 1 <= kMaxCellCoord2 ? 1 : 0);
#pragma unroll 1
        for (int dx = x0; dx <= x1; dx++) {
#pragma unroll 1
            for (int dy = y0; dy <= y1; dy++) {
                const uint32_t cell = split2_32(cx + dx) | (split2_32(cy + dy) << 1);
                if (cell >= P.max_cells) continue;
                const uint32_t s = G.cell_start[cell];
                if (s == kEmpty) continue;
                const uint32_t e = G.cell_end[cell];
                const float shx = (float)dx * M.cell - pj.x;
                const float shy = (float)dy * M.cell - pj.y;
                const uint32_t code = (uint32_t)((dx + 2) * 5 + (dy + 2)) << 27;
                for (uint32_t i = s; i < e; i++) {
                    if (i == k) continue;
                    const float4 pi = G.P4[i];
                    if (__float_as_int(pi.w) == P.type_non_existent) continue;  // stays non-existent
                    const float ddx = pi.x + shx, ddy = pi.y + shy;
                    if (ddx * ddx + ddy * ddy < P.vl_cut2) {
                        if (nl < (uint32_t)kVerletCap) {
                            const uint32_t v = i | code, slot = nl & 3u;
                            buf.x = slot == 0 ? v : buf.x;
                            buf.y = slot == 1 ? v : buf.y;
                            buf.z = slot == 2 ? v : buf.z;
                            buf.w = slot == 3 ? v : buf.w;
                            if (slot == 3) {
                                slab[(size_t)(nl >> 2) * P.n] = buf;
                                buf = make_uint4(kVlNone, kVlNone, kVlNone, kVlNone);
                            }
                        }
                        nl++;
                    }
                }
            }
        }
    }
    if (nl < (uint32_t)kVerletCap && (nl & 3u)) slab[(size_t)(nl >> 2) * P.n] = buf;  // the padded last group
    G.vcount[k] = nl <= (uint32_t)kVerletCap ? nl : kListOver;
    if (nl > (uint32_t)kVerletCap) {  // its search needs a fresh grid each step
        atomicOr(S.vl_rebuild, 1u);
        atomicOr(S.vl_gone, 2u);
    }
}

// Stencil offset of a list entry's 5-bit cell code (dx + 2) * 5 + (dy + 2):
// cx = dx + 2, cy = dy + 2 (c / 5 as (c * 13) >> 6, exact for c < 32).
__device__ __forceinline__ void vl_code_xy(uint32_t en, uint32_t& cx, uint32_t& cy) {
    const uint32_t c = en >> 27;
    cx = (c * 13u) >> 6;
    cy = c - 5u * cx;
}

// The cubic W(q) of kernel_wf as selects: every lane runs the same instructions.
__device__ __forceinline__ float cubic_wf_sel(float f, float q) {
    const float t = 2.0f - q;
    const float w1 = f * ((2.0f / 3.0f - q * q) + q * q * q * 0.5f);
    const float w2 = f * ((1.0f / 6.0f) * (t * t * t));
    return q <= 1.0f ? w1 : (q <= 2.0f ? w2 : 0.0f);
}

// density_sum (Density.h:25-61) + EOS over the candidate list: the entries
// within the cutoff are this step's neighbours (written to nlist for the force
// pass). A particle whose list overflowed searches the stencil cells
// (the grid is rebuilt every step while one does).
template <int SKF>
__global__ void __launch_bounds__(kMaxGatherThreads) k_density_verlet(DevParams P, State S, Sorted G,
                                                                     StepScalars* __restrict__ scal,
                                                                     uint32_t* __restrict__ flags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    uint32_t cnt = 0;
    if (active) {
        const MixedF& M = P.mf;
        const uint32_t id = G.id[k];
        const float4 pj = G.P4[k];
        const int32_t tj = __float_as_int(pj.w);
        const int skf = SKF ? SKF : P.density_skf;
        const float f = M.kf[skf];
        Kahan acc{0.0f, 0.0f};
        uint32_t* const nslab = G.nlist + (size_t)k * 4;  // neighbour e at nslab[(e / 4) * 4n + e % 4]
        if (tj != P.type_non_existent) {
            const uint32_t vc = G.vcount[k];
            if (vc != kListOver) {
                const uint4* slab = reinterpret_cast<const uint4*>(G.vlist) + k;  // group g at slab[g * n]
                // shift of stencil offset (cx, cy) = (cx - 2, cy - 2) cells, relative to this particle
                const float bx = -2.0f * M.cell - pj.x, by = -2.0f * M.cell - pj.y;
                // groups of four entries (one load, the next group's issued before this
                // one's particles are loaded), then their particles, loaded together;
                // the body has no branch but the rare guard-band test, and each group's
                // sum is added with compensation
                // (list words are read once a step: streaming loads keep L1 for the neighbours' data)
                uint4 w = vc ? __ldcs(slab) : make_uint4(kVlNone, kVlNone, kVlNone, kVlNone);
                for (uint32_t e0 = 0; e0 < vc; e0 += kVlBatch) {
                    const uint4 wn = e0 + kVlBatch < vc ? __ldcs(slab + (size_t)((e0 >> 2) + 1) * P.n) : w;
                    const uint32_t en[kVlBatch] = {w.x, w.y, w.z, w.w};
                    float4 pb[kVlBatch];
#pragma unroll
                    for (int j = 0; j < kVlBatch; j++)
                        pb[j] = en[j] != kVlNone ? G.P4[en[j] & 0x07FFFFFFu] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    float part = 0.0f;
#pragma unroll
                    for (int j = 0; j < kVlBatch; j++) {
                        uint32_t cx, cy;
                        vl_code_xy(en[j], cx, cy);
                        const float dx = pb[j].x + fmaf((float)cx, M.cell, bx);
                        const float dy = pb[j].y + fmaf((float)cy, M.cell, by);
                        const float d2 = dx * dx + dy * dy;
                        bool in = en[j] != kVlNone && __float_as_int(pb[j].w) != P.type_non_existent &&
                                  d2 < M.cut2_hi;
                        if (in && !(d2 < M.cut2_lo)) in = within_cutoff<2>(P, S, G, en[j] & 0x07FFFFFFu, k, d2);
                        const float q = d2 * rsqrtf(d2) * M.inv_h;
                        const float wv = SKF == 1 ? cubic_wf_sel(f, q) : kernel_wf(skf, f, q);
                        part += in ? wv : 0.0f;
                        if (in) nslab[(size_t)(cnt >> 2) * 4 * P.n + (cnt & 3u)] = en[j];
                        cnt += in;
                    }
                    acc.add(M.mass * part);
                    w = wn;
                }
            } else {
                const Stencil<2> st(P, G.key[k]);
#pragma unroll 1
                for (int c = 0; c < 9; c++) {
                    uint32_t cell;
                    int sx, sy, sz;
                    if (!st.cell(c, cell, sx, sy, sz)) continue;
                    const uint32_t s = G.cell_start[cell];
                    if (s == kEmpty) continue;
                    const uint32_t e = G.cell_end[cell];
                    const float shx = (float)sx * M.cell - pj.x;
                    const float shy = (float)sy * M.cell - pj.y;
                    float part = 0.0f;
                    for (uint32_t i = s; i < e; i++) {
                        if (i == k) continue;
                        const float4 pi = G.P4[i];
                        if (__float_as_int(pi.w) == P.type_non_existent) continue;
                        const float dx = pi.x + shx, dy = pi.y + shy;
                        const float d2 = dx * dx + dy * dy;
                        if (!within_cutoff<2>(P, S, G, i, k, d2)) continue;
                        // this step's neighbour list too (the grid is this step's: code of (sx, sy))
                        if (cnt < (uint32_t)kVerletCap)
                            nslab[(size_t)(cnt >> 2) * 4 * P.n + (cnt & 3u)] =
                                i | ((uint32_t)((sx + 2) * 5 + (sy + 2)) << 27);
                        cnt++;
                        part += kernel_wf(skf, f, d2 * rsqrtf(d2) * M.inv_h);
                    }
                    acc.add(M.mass * part);
                }
            }
        }
        G.ncount[k] = cnt < (uint32_t)kVerletCap ? cnt : (uint32_t)kVerletCap;
        if (cnt > P.max_nb - 1) atomicOr(flags, RRSPH_FLAG_NEIGHBOUR_OVERFLOW);
        const float d = ((acc.s - M.rho0_minus_w0_hi) - acc.c) - M.rho0_minus_w0_lo;
        const float rho = M.rho0 + d;
        const float pr = eos_pf(M, d);
        const float2 prr = make_float2(pr, pr * __frcp_rn(rho * rho));
        // V4.zw = (the pressure the force pass reads of a neighbour: p with form 1, else p/rho^2, rho)
        reinterpret_cast<float2*>(G.V4 + k)[1] = make_float2(P.intf_form == 1 ? prr.x : prr.y, rho);
        G.PR[k] = prr;
        S.rho[id] = P.rho0 + f2d(d);
        S.p[id] = f2d(pr);
    }
    warp_sum_add(&scal->pairs, cnt);
}

// update_acceleration over this step's neighbours: the list the density pass
// wrote (or the stencil search for an overflowed list). A neighbour's pressure
// comes with its velocity and density (V4.z). STD: the common method set of
// ForceAcc::pair_std, fixed at compile time. At most 64 registers (4 blocks of
// 256 threads per SM): the gather hides its L1/L2 latency with warps.
// WV != 0: the whole step follows in the same thread (whole_particle with
// variant WV, thread 0 advancing the scalars into next): it reads nothing that
// another thread's whole step writes, because this step's copies (P4, V4) are
// not the ones the key pass writes (P4n, V4n), and the list of every particle
// is complete (the density pass wrote the neighbours of overflowed lists too,
// which needs at most kVerletCap neighbours per particle).
template <int SKF, bool STD, int WV>
__global__ void __launch_bounds__(kMaxGatherThreads, 4) k_forces_verlet(DevParams P, State S, Sorted G,
                                                                    StepScalars* __restrict__ scal,
                                                                    StepScalars* __restrict__ next,
                                                                    uint32_t* __restrict__ flags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    double amag = 0, arvmu_d = 0;
    if (active) {
        const MixedF& M = P.mf;
        const uint32_t id = G.id[k];
        const float4 pj4 = G.P4[k];
        const int32_t tj = __float_as_int(pj4.w);
        ForceAcc<2, SKF> F{P, G, G.V4[k], G.PR[k], 0.0f, false, false, false, false, false, 0, 0,
                           0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        F.rhoj = F.vj.w;
        F.ext = P.repulsive && tj > 0;
        F.intf = true;
        F.visc = P.art_visc;
        F.avel = P.avg_vel;
        F.form1 = P.intf_form == 1;
        F.intf_skf = SKF ? SKF : P.intf_skf;
        F.av_skf = SKF ? SKF : P.av_skf;
        Kahan ax{0, 0}, ay{0, 0};
        Kahan avx{0, 0}, avy{0, 0};
        if (tj != P.type_non_existent) {
            const uint32_t vc = G.vcount[k];
            if (WV != 0 || vc != kListOver) {
                // this step's neighbours, four list words per load (the lanes of a
                // warp load neighbouring uint4s), their data two at a time
                const uint32_t nc = G.ncount[k];
                const uint4* nslab = reinterpret_cast<const uint4*>(G.nlist) + k;  // group g at nslab[g * n]
                const float bx = -2.0f * M.cell - pj4.x, by = -2.0f * M.cell - pj4.y;
                for (uint32_t e0 = 0; e0 < nc; e0 += 4) {
                    const uint4 w = __ldcs(nslab + (size_t)(e0 >> 2) * P.n);  // streaming, as in the density pass
                    const uint32_t eg[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                    for (int h = 0; h < 4; h += kVlForceBatch) {
                        uint32_t en[kVlForceBatch];
                        float4 pb[kVlForceBatch], vb[kVlForceBatch];
#pragma unroll
                        for (int j = 0; j < kVlForceBatch; j++) en[j] = e0 + h + j < nc ? eg[h + j] : kVlNone;
#pragma unroll
                        for (int j = 0; j < kVlForceBatch; j++) {
                            if (en[j] == kVlNone) continue;
                            const uint32_t i = en[j] & 0x07FFFFFFu;
                            pb[j] = G.P4[i];
                            vb[j] = G.V4[i];
                        }
                        // each pair's terms are added with compensation (no per-cell
                        // partial sums, whose flushes would split the warp)
#pragma unroll
                        for (int j = 0; j < kVlForceBatch; j++) {
                            if (en[j] == kVlNone) continue;
                            uint32_t cx, cy;
                            vl_code_xy(en[j], cx, cy);
                            const float dx = pb[j].x + fmaf((float)cx, M.cell, bx);
                            const float dy = pb[j].y + fmaf((float)cy, M.cell, by);
                            F.cax = F.cay = F.cvx = F.cvy = 0.0f;
                            if (STD) {
                                F.pair_std(vb[j], dx, dy, dx * dx + dy * dy, __float_as_int(pb[j].w));
                            } else {
                                const float z = vb[j].z;  // p (form 1) or p/rho^2, as the density pass wrote it
                                const float2 pri = F.form1 ? make_float2(z, z * __frcp_rn(vb[j].w * vb[j].w))
                                                           : make_float2(z, z);
                                F.pair_with(vb[j], pri, dx, dy, 0.0f, dx * dx + dy * dy, __float_as_int(pb[j].w));
                            }
                            ax.add(F.cax);
                            ay.add(F.cay);
                            if (!STD && F.avel) {
                                avx.add(F.cvx);
                                avy.add(F.cvy);
                            }
                        }
                    }
                }
            } else {
                const Stencil<2> st(P, G.key[k]);
#pragma unroll 1
                for (int c = 0; c < 9; c++) {
                    uint32_t cell;
                    int sx, sy, sz;
                    if (!st.cell(c, cell, sx, sy, sz)) continue;
                    const uint32_t s = G.cell_start[cell];
                    if (s == kEmpty) continue;
                    const uint32_t e = G.cell_end[cell];
                    const float shx = (float)sx * M.cell - pj4.x;
                    const float shy = (float)sy * M.cell - pj4.y;
                    F.cax = F.cay = F.cvx = F.cvy = 0.0f;
                    for (uint32_t i = s; i < e; i++) {
                        if (i == k) continue;
                        const float4 pi4 = G.P4[i];
                        const int32_t ti = __float_as_int(pi4.w);
                        if (ti == P.type_non_existent) continue;
                        const float dx = pi4.x + shx, dy = pi4.y + shy;
                        const float d2 = dx * dx + dy * dy;
                        if (!within_cutoff<2>(P, S, G, i, k, d2)) continue;
                        F.pair(i, dx, dy, 0.0f, d2, ti);
                    }
                    ax.add(F.cax);
                    ay.add(F.cay);
                    if (F.avel) {
                        avx.add(F.cvx);
                        avy.add(F.cvy);
                    }
                }
            }
        }
        const double axd = ax.value(), ayd = ay.value() - P.g;
        S.ax[id] = axd;
        S.ay[id] = ayd;
        if (F.avel) {
            S.avx[id] = avx.value();
            S.avy[id] = avy.value();
        }
        arvmu_d = F.arvmu;
        if (P.dt_reduce) amag = sqrt(axd * axd + ayd * ayd);
        if (WV != 0) {
            const double dt = step_dt<(WV & kVarRare) != 0>(P, scal, flags, k == 0);
            if (k == 0) advance_scalars(P, scal, next, dt);
            whole_particle<2, WV>(P, S, G, id, dt, scal, flags, 1, axd, ayd, 0.0);
        }
    }
    if (P.dt_method == 2 && P.dt_reduce) {
        warp_max_bits(&scal->amax_bits, amag);
        warp_max_bits(&scal->mumax_bits, arvmu_d);
    }
}

}  // namespace

void launch_verlet_decide(cudaGraphConditionalHandle h, const uint32_t* rebuild, cudaStream_t st) {
    k_vl_decide<<<1, 1, 0, st>>>(h, rebuild);
}
void launch_verlet_reset(uint32_t* rebuild, uint32_t* gone, unsigned long long* builds, cudaStream_t st) {
    k_vl_reset<<<1, 1, 0, st>>>(rebuild, gone, builds);
}
void launch_verlet_upload_check(uint32_t* rebuild, const uint32_t* gone, cudaStream_t st) {
    k_vl_upload_check<<<1, 1, 0, st>>>(rebuild, gone);
}
void launch_verlet_build(const DevParams& P, const State& S, const Sorted& G, cudaStream_t st) {
    constexpr int kBuildThreads = 128;
    k_vl_build<<<(P.n + kBuildThreads - 1) / kBuildThreads, kBuildThreads, 0, st>>>(P, S, G);
}
void launch_density_verlet(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal, uint32_t* flags,
                           cudaStream_t st, int threads) {
    const unsigned blocks = (P.n + threads - 1) / threads;
    if (P.all_cubic) k_density_verlet<1><<<blocks, threads, 0, st>>>(P, S, G, scal, flags);
    else k_density_verlet<0><<<blocks, threads, 0, st>>>(P, S, G, scal, flags);
}
void launch_forces_verlet(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal,
                          StepScalars* scal_next, uint32_t* flags, cudaStream_t st, int threads, int whole) {
    const unsigned blocks = (P.n + threads - 1) / threads;
    const bool std_terms = P.all_cubic && P.intf_form != 1 && P.art_visc && !P.art_pressure && !P.avg_vel;
    const int wv = whole ? (kVarMixed | (P.avg_vel || P.dt_method == 2 ? kVarRare : 0)) : 0;
#define RRSPH_FV(SKF, STD)                                                                                      \
    do {                                                                                                        \
        if (wv == 0) k_forces_verlet<SKF, STD, 0><<<blocks, threads, 0, st>>>(P, S, G, scal, scal_next, flags);  \
        else if (wv == kVarMixed)                                                                               \
            k_forces_verlet<SKF, STD, kVarMixed><<<blocks, threads, 0, st>>>(P, S, G, scal, scal_next, flags);  \
        else k_forces_verlet<SKF, STD, kVarMixed | kVarRare><<<blocks, threads, 0, st>>>(P, S, G, scal, scal_next, \
                                                                                          flags);               \
    } while (0)
    if (std_terms) RRSPH_FV(1, true);
    else if (P.all_cubic) RRSPH_FV(1, false);
    else RRSPH_FV(0, false);
#undef RRSPH_FV
}

template <int DIM>
void launch_density_mixed(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal, uint32_t* flags,
                          cudaStream_t st, int threads) {
    const unsigned blocks = (P.n + threads - 1) / threads;
    if (P.all_cubic) k_density_mixed<DIM, 1><<<blocks, threads, 0, st>>>(P, S, G, scal, flags);
    else k_density_mixed<DIM, 0><<<blocks, threads, 0, st>>>(P, S, G, scal, flags);
}
template <int DIM>
void launch_forces_mixed(const DevParams& P, const State& S, const Sorted& G, uint32_t terms, StepScalars* scal,
                         uint32_t* flags, int write_mu, int use_masks, cudaStream_t st, int threads) {
    const unsigned blocks = (P.n + threads - 1) / threads;
    const bool m = DIM == 2 && use_masks && G.nbmask != nullptr;
    if (P.all_cubic) {
        if (m) k_forces_mixed<DIM, 1, true><<<blocks, threads, 0, st>>>(P, S, G, terms, scal, flags, write_mu);
        else k_forces_mixed<DIM, 1, false><<<blocks, threads, 0, st>>>(P, S, G, terms, scal, flags, write_mu);
    } else {
        if (m) k_forces_mixed<DIM, 0, true><<<blocks, threads, 0, st>>>(P, S, G, terms, scal, flags, write_mu);
        else k_forces_mixed<DIM, 0, false><<<blocks, threads, 0, st>>>(P, S, G, terms, scal, flags, write_mu);
    }
}

template void launch_density_mixed<2>(const DevParams&, const State&, const Sorted&, StepScalars*, uint32_t*,
                                      cudaStream_t, int);
template void launch_density_mixed<3>(const DevParams&, const State&, const Sorted&, StepScalars*, uint32_t*,
                                      cudaStream_t, int);
template void launch_forces_mixed<2>(const DevParams&, const State&, const Sorted&, uint32_t, StepScalars*, uint32_t*,
                                     int, int, cudaStream_t, int);
template void launch_forces_mixed<3>(const DevParams&, const State&, const Sorted&, uint32_t, StepScalars*, uint32_t*,
                                     int, int, cudaStream_t, int);

}  // namespace rrsph
