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
#include "mixed_common.cuh"

namespace rrsph {

namespace {

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
                            const float rho_factor = __fdividef(vd4_drho<DIM>(vdi, vdj), M.rho0 + vdi.w);
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

}  // namespace

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
