// kernels_fp64.cu — the density and force gathers in double precision (the
// plain FP64 step). One thread per particle in cell order; the neighbours of a
// particle are the particles of the 3^dim cells around its cell that pass the
// reference's cutoff test, visited in the reference's order (cells x-major,
// ids ascending inside a cell), so the sums run in the same order as RRSPH_OMP.
// The density pass records them per stencil cell as bit masks for the force
// pass, and both walk a particle's pairs as one flat sequence across the cells
// so that the lanes of a warp run the double pair body together: a warp's FP64
// instruction costs the pipe the same time whatever lanes are active.
#include <type_traits>

#include "kernels.cuh"
#include "neighbour.cuh"

namespace rrsph {

namespace {

__device__ __forceinline__ void warp_sum_add(unsigned long long* dst, unsigned long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd(dst, v);
}
__device__ __forceinline__ void warp_max_bits(unsigned long long* dst, double v) {
    // non-negative doubles order like their bit patterns
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xFFFFFFFFu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0) atomicMax(dst, dbits(v));
}

// The neighbour masks of the FP64 gathers: a bit per particle of a stencil
// cell, 32-bit in 2D and 64-bit in 3D (a 3D cell near a wall holds up to ~40
// particles); a cell with more is searched in place.
template <int DIM>
struct NbMask {
    using T = typename std::conditional<DIM == 3, unsigned long long, uint32_t>::type;
    static constexpr uint32_t bits = DIM == 3 ? 64 : 32;
    static __device__ __forceinline__ T* at(const Sorted& G, uint32_t k) { return reinterpret_cast<T*>(G.nbmask) + k; }
    static __device__ __forceinline__ uint32_t lowest(T m) {
        return DIM == 3 ? (uint32_t)(__ffsll((long long)m) - 1) : (uint32_t)(__ffs((int)m) - 1);
    }
};

// density_sum (RRSPH_COMMON/include/Density.h:25-61) and density_con
// (Density.h:63-114, delta-SPH when density_treatment == 2), EOS p (EOS.cpp:31-34).
template <int DIM>
__global__ void __launch_bounds__(kMaxGatherThreads) k_density(DevParams P, State S, Sorted G,
                                                            StepScalars* __restrict__ scal,
                                                            uint32_t* __restrict__ flags) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    uint32_t cnt = 0;
    if (active) {
        const uint32_t id = G.id[k];
        const bool cont = P.density_treatment != 0;
        const double xj = G.rx[k], yj = G.ry[k], zj = DIM == 3 ? G.rz[k] : 0.0;
        double vxj = 0, vyj = 0, vzj = 0, rhoj = 0;
        if (cont) {
            vxj = G.vdx[k];
            vyj = G.vdy[k];
            if (DIM == 3) vzj = G.vdz[k];
            rhoj = G.rhod[k];
        }
        const int skf = P.density_skf;
        const double f = P.kf[skf];
        double acc = cont ? 0.0 : P.mass * P.w0_density;
        if (G.itype[k] != P.type_non_existent) {
            const Stencil<DIM> st(P, G.key[k]);
            constexpr int NC = DIM == 3 ? 27 : 9;
            using Mask = typename NbMask<DIM>::T;
            Mask* const masks = NbMask<DIM>::at(G, k);  // [c * n]: this particle's bits of stencil cell c
            const float4 pj4 = G.P4[k];
            const float cellf = P.mf.cell, cut2_hi = P.mf.cut2_hi;
            // 1. The float test on the cell-relative offsets: a particle beyond the
            // cutoff's upper guard band is beyond the cutoff in double too; the
            // others are candidates (bit b of cell c: particle cell_start + b). A cell
            // of more particles than a mask has bits is searched in place below. The
            // warp goes through the cells together, so the mask stores are coalesced.
            uint32_t over = 0;
#pragma unroll 1
            for (int c = 0; c < NC; c++) {
                Mask cand = 0;
                uint32_t cell;
                int sx, sy, sz;
                const uint32_t s = st.cell(c, cell, sx, sy, sz) ? G.cell_start[cell] : kEmpty;
                const uint32_t e = s != kEmpty ? G.cell_end[cell] : s;
                if (e - s > NbMask<DIM>::bits) {
                    over |= 1u << c;
                } else {
                    const float shx = (float)sx * cellf - pj4.x, shy = (float)sy * cellf - pj4.y;
                    const float shz = DIM == 3 ? (float)sz * cellf - pj4.z : 0.0f;
                    for (uint32_t i = s; i < e; i++) {
                        const float4 pi4 = G.P4[i];
                        const float fx = pi4.x + shx, fy = pi4.y + shy, fz = DIM == 3 ? pi4.z + shz : 0.0f;
                        const bool cnd = i != k && __float_as_int(pi4.w) != P.type_non_existent &&
                                         fx * fx + fy * fy + fz * fz < cut2_hi;
                        cand |= (Mask)(cnd ? 1u : 0u) << (i - s);
                    }
                }
                masks[(size_t)c * P.n] = cand;
            }
            masks[(size_t)NC * P.n] = (Mask)over;
            // 2. The candidates in the search's order (cells in stencil order, ids
            // ascending) as one flat sequence, so the lanes of a warp run the double
            // test and terms together (a warp's FP64 instruction costs the pipe the
            // same time whatever lanes are active). A cell's neighbours replace its
            // candidates in the masks the force pass reads.
            int c = -1;
            Mask bits = 0, kept = 0;     // candidates left in a masked cell, and its neighbours
            uint32_t base = 0;
            uint32_t next = 0, end = 0;  // or the range of a searched cell left
            bool masked = false;
            for (;;) {
                if (bits == 0 && next == end) {
                    if (masked) masks[(size_t)c * P.n] = kept;
                    masked = false;
                    for (c++; c < NC; c++) {
                        uint32_t cell;
                        int sx, sy, sz;
                        if ((over >> c) & 1u) {  // a valid, non-empty cell
                            st.cell(c, cell, sx, sy, sz);
                            next = G.cell_start[cell];
                            end = G.cell_end[cell];
                            break;
                        }
                        bits = masks[(size_t)c * P.n];
                        if (bits) {
                            st.cell(c, cell, sx, sy, sz);
                            base = G.cell_start[cell];
                            kept = 0;
                            masked = true;
                            break;
                        }
                    }
                    if (c >= NC) break;
                }
                uint32_t i, b = 0;
                bool searched;
                if (bits) {
                    b = NbMask<DIM>::lowest(bits);
                    i = base + b;
                    bits &= bits - 1;
                    searched = false;
                } else {
                    i = next++;
                    searched = true;
                }
                const double dx = __dsub_rn(G.rx[i], xj), dy = __dsub_rn(G.ry[i], yj);
                const double dz = DIM == 3 ? __dsub_rn(G.rz[i], zj) : 0.0;
                const double d2 = exact_dist2<DIM>(dx, dy, dz);
                if (!(d2 < P.cut2)) continue;
                if (searched && (i == k || G.itype[i] == P.type_non_existent)) continue;
                cnt++;
                kept |= (Mask)(searched ? 0u : 1u) << b;
                const double dist = sqrt(d2);
                const double q = dist * P.inv_h;
                if (!cont) {
                    acc += P.mass * kernel_w(skf, f, q);
                } else {
                    // diff = r_i - r_j; dwdr = diff * s
                    const double sc = kernel_dwdr_scale(skf, f, q, dist, P.inv_h);
                    const double gx = dx * sc, gy = dy * sc, gz = dz * sc;
                    double vcc = (G.vdx[i] - vxj) * gx + (G.vdy[i] - vyj) * gy;
                    if (DIM == 3) vcc += (G.vdz[i] - vzj) * gz;
                    acc += P.mass * vcc;
                    if (P.density_treatment == 2) {
                        // r_ab = r_j - r_i = -diff
                        double rd = -(dx * gx + dy * gy);
                        if (DIM == 3) rd -= dz * gz;
                        const double r_factor = rd / d2;
                        const double rhoi = G.rhod[i];
                        const double rho_factor = (rhoi - rhoj) / rhoi;
                        acc += 2 * P.delta_sph_dhc * (rho_factor * r_factor) * P.mass;
                    }
                }
            }
        }
        if (cnt > P.max_nb - 1) atomicOr(flags, RRSPH_FLAG_NEIGHBOUR_OVERFLOW);
        if (!cont) {
            const double pj = eos_p(P, acc);
            G.rho[k] = acc;
            G.p[k] = pj;
            G.pr2[k] = pj / (acc * acc);
            S.rho[id] = acc;
            S.p[id] = pj;
        } else {
            const double pj = eos_p(P, rhoj);
            const double rf = G.rho[k];  // the density the forces use (rho_predict)
            G.p[k] = pj;
            G.pr2[k] = pj / (rf * rf);
            S.p[id] = pj;
            S.drho[id] = acc;
        }
    }
    warp_sum_add(&scal->pairs, cnt);
}

// update_acceleration (RRSPH_OMP/src/UpdateAcceleration.cpp:33-125) with
// external_force_part (ExtForce.h:15-60), find_internal_changes_part
// (InternalForce.h:24-141), artificial_viscosity_part (ArtificialViscosity.h:29-65)
// and average_velocity_part (AverageVelocity.h:20-37).
template <int DIM>
__global__ void __launch_bounds__(kMaxGatherThreads) k_forces(DevParams P, State S, Sorted G, uint32_t terms,
                                                           StepScalars* __restrict__ scal,
                                                           uint32_t* __restrict__ flags, int write_mu,
                                                           int use_masks) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = k < P.n;
    double amag = 0, arvmu = 0;
    if (active) {
        const uint32_t id = G.id[k];
        const double xj = G.rx[k], yj = G.ry[k], zj = DIM == 3 ? G.rz[k] : 0.0;
        const double vxj = G.vx[k], vyj = G.vy[k], vzj = DIM == 3 ? G.vz[k] : 0.0;
        const double rhoj = G.rho[k], pj = G.p[k];
        const int32_t tj = G.itype[k];
        double ax = 0, ay = (terms & RRSPH_TERM_GRAVITY) ? -P.g : 0.0, az = 0;
        double avx = 0, avy = 0, avz = 0;
        const bool ext = (terms & RRSPH_TERM_EXTERNAL) && P.repulsive && tj > 0;
        const bool intf = terms & RRSPH_TERM_INTERNAL;
        const bool visc = (terms & RRSPH_TERM_ART_VISC) && P.art_visc;
        const bool avel = (terms & RRSPH_TERM_AVERAGE_VELOCITY) && P.avg_vel;
        const double pj_r2 = pj / (rhoj * rhoj);
        // the viscosity's kernel gradient is the pressure term's when both use one kernel
        const bool same_skf = P.av_skf == P.intf_skf;
        // the terms of one neighbour i (separation dx = r_i - r_j, d2 = |dx|^2)
        auto pair = [&](uint32_t i, int32_t ti, double dx, double dy, double dz, double d2) {
            const double dist = sqrt(d2);
            const double q = dist * P.inv_h;
            if (ext && ti < 0 && dist < P.lj_rr0) {
                const double rn = P.lj_rr0 / dist;
                const double rn2 = rn * rn, rn4 = rn2 * rn2, rn8 = rn4 * rn4;
                const double fl = P.lj_D * (rn8 * rn4 - rn4) / d2;
                ax -= dx * fl;
                ay -= dy * fl;
                if (DIM == 3) az -= dz * fl;
            }
            const double rhoi = G.rho[i];
            double sc_intf = 0.0;
            if (intf) {
                const double pi = G.p[i];
                const double sc = kernel_dwdr_scale(P.intf_skf, P.kf[P.intf_skf], q, dist, P.inv_h);
                sc_intf = sc;
                // p_i / rho_i^2: the density pass computed it per particle from the same values
                double pf = P.intf_form == 1 ? (pj + pi) / (rhoj * rhoi) : (G.pr2[i] + pj_r2);
                if (P.art_pressure && (pi < 0 || pj < 0)) {
                    const double w = kernel_w(P.ap_skf, P.kf[P.ap_skf], q);
                    const double api = pi < 0 ? (-P.ap_coef * pi / (rhoi * rhoi)) : 0.0;
                    const double apj = pj < 0 ? (-P.ap_coef * pj / (rhoj * rhoj)) : 0.0;
                    pf += (api + apj) * pow(w / P.ap_wdelta, P.ap_index);
                }
                const double m = sc * pf * P.mass;
                ax += dx * m;
                ay += dy * m;
                if (DIM == 3) az += dz * m;
            }
            if (visc || avel) {
                const double vxi = G.vx[i], vyi = G.vy[i], vzi = DIM == 3 ? G.vz[i] : 0.0;
                if (visc) {
                    // dv = v_j - v_i, dr = r_j - r_i = -diff
                    double vr = -((vxj - vxi) * dx + (vyj - vyi) * dy);
                    if (DIM == 3) vr -= (vzj - vzi) * dz;
                    if (vr < 0) {
                        const double mu = P.h * vr / (d2 + P.etq_h2);
                        arvmu = fmax(arvmu, fabs(mu));
                        const double rho_ij = 0.5 * (rhoi + rhoj);
                        const double piv = (P.av_beta * mu - P.av_alpha * P.c_av) * mu / rho_ij;
                        const double sc = intf && same_skf ? sc_intf
                                                           : kernel_dwdr_scale(P.av_skf, P.kf[P.av_skf], q, dist, P.inv_h);
                        const double m = sc * piv * P.mass;
                        ax += dx * m;
                        ay += dy * m;
                        if (DIM == 3) az += dz * m;
                    }
                }
                if (avel && ti > 0) {
                    const double w = kernel_w(P.avel_skf, P.kf[P.avel_skf], q);
                    const double m = P.mass / (rhoi + rhoj) * w * 2 * P.avg_vel_coef;
                    avx += (vxi - vxj) * m;
                    avy += (vyi - vyj) * m;
                    if (DIM == 3) avz += (vzi - vzj) * m;
                }
            }
        };
        if (tj != P.type_non_existent) {
            const Stencil<DIM> st(P, G.key[k]);
            constexpr int NC = DIM == 3 ? 27 : 9;
            using Mask = typename NbMask<DIM>::T;
            const Mask* const masks = use_masks ? NbMask<DIM>::at(G, k) : nullptr;
            const uint32_t over = masks ? (uint32_t)masks[(size_t)NC * P.n] : 0xFFFFFFFFu;
            // One flat sequence over the stencil cells: each iteration takes this
            // particle's next candidate (the next neighbour the density pass recorded
            // in a cell, or the next particle of a cell searched in place: more
            // particles than a mask has bits, or no masks), so the lanes of a warp run the double pair
            // body together (a warp's FP64 instruction costs the pipe the same time
            // whatever lanes are active). The order is the search's: cells in
            // stencil order, ids ascending.
            int c = -1;
            Mask bits = 0;                // the recorded neighbours of the current cell
            uint32_t base = 0;
            uint32_t next = 0, end = 0;   // or the range left to search
            for (;;) {
                if (bits == 0 && next == end) {
                    for (c++; c < NC; c++) {
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
                    if (c >= NC) break;
                }
                uint32_t i;
                bool known;
                if (bits) {
                    i = base + NbMask<DIM>::lowest(bits);
                    bits &= bits - 1;
                    known = true;
                } else {
                    i = next++;
                    known = false;
                }
                const int32_t ti = G.itype[i];
                const double dx = __dsub_rn(G.rx[i], xj), dy = __dsub_rn(G.ry[i], yj);
                const double dz = DIM == 3 ? __dsub_rn(G.rz[i], zj) : 0.0;
                const double d2 = exact_dist2<DIM>(dx, dy, dz);
                if (known || (i != k && ti != P.type_non_existent && d2 < P.cut2)) pair(i, ti, dx, dy, dz, d2);
            }
        }
        S.ax[id] = ax;
        S.ay[id] = ay;
        if (DIM == 3) S.az[id] = az;
        if (avel) {
            S.avx[id] = avx;
            S.avy[id] = avy;
            if (DIM == 3) S.avz[id] = avz;
        }
        if (write_mu) S.mu[id] = arvmu;
        amag = sqrt(ax * ax + ay * ay + az * az);
    }
    if (P.dt_method == 2 && P.dt_reduce) {
        warp_max_bits(&scal->amax_bits, amag);
        warp_max_bits(&scal->mumax_bits, arvmu);
    }
}

}  // namespace

template <int DIM>
void launch_density_fp64(const DevParams& P, const State& S, const Sorted& G, StepScalars* scal, uint32_t* flags,
                         cudaStream_t st, int threads) {
    k_density<DIM><<<(P.n + threads - 1) / threads, threads, 0, st>>>(P, S, G, scal, flags);
}
template <int DIM>
void launch_forces_fp64(const DevParams& P, const State& S, const Sorted& G, uint32_t terms, StepScalars* scal,
                        uint32_t* flags, int write_mu, cudaStream_t st, int threads, int use_masks) {
    k_forces<DIM><<<(P.n + threads - 1) / threads, threads, 0, st>>>(P, S, G, terms, scal, flags, write_mu,
                                                                    use_masks && G.nbmask ? 1 : 0);
}

template void launch_density_fp64<2>(const DevParams&, const State&, const Sorted&, StepScalars*, uint32_t*,
                                     cudaStream_t, int);
template void launch_density_fp64<3>(const DevParams&, const State&, const Sorted&, StepScalars*, uint32_t*,
                                     cudaStream_t, int);
template void launch_forces_fp64<2>(const DevParams&, const State&, const Sorted&, uint32_t, StepScalars*, uint32_t*,
                                    int, cudaStream_t, int, int);
template void launch_forces_fp64<3>(const DevParams&, const State&, const Sorted&, uint32_t, StepScalars*, uint32_t*,
                                    int, cudaStream_t, int, int);

}  // namespace rrsph
