// mixed_common.cuh — the float pair arithmetic shared by the FP32-mixed
// gathers (kernels_mixed.cu: stencil search; kernels_reuse.cu: neighbour
// lists): compensated sums, the smoothing kernels, the cutoff test with its
// double guard band, warp reductions, the EOS and one pair's force terms.
#pragma once

#include "kernels.cuh"
#include "neighbour.cuh"

namespace rrsph {
namespace {

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

// The cubic dW/dr scale of kernel_dwdr_scalef as selects (both branches of the
// spline evaluated, no divergence between the lanes of a warp).
__device__ __forceinline__ float cubic_dwdr_sel(float f, float q, float inv_dist, float inv_h) {
    const float t = 2.0f - q;
    const float s1 = inv_h * inv_h * f * (-2.0f + 1.5f * q);
    const float s2 = -(inv_h * inv_dist) * f * (t * t * 0.5f);
    return q <= 1.0f ? s1 : (q <= 2.0f ? s2 : 0.0f);
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
        const float sc = cubic_dwdr_sel(M.kf[1], q, inv_dist, M.inv_h);
        m += sc * (vi.z + prj.y) * M.mass;
        const float vr = -((vj.x - vi.x) * dx + (vj.y - vi.y) * dy);
        const float mu = fminf(__fdividef(M.h * vr, d2 + M.etq_h2), 0.0f);
        arvmu = fmaxf(arvmu, -mu);
        const float piv = __fdividef((M.av_beta * mu - M.av_alpha_c) * mu, 0.5f * (rhoi + rhoj));
        m += sc * piv * M.mass;
        cax += dx * m;
        cay += dy * m;
    }
    // pair_with for the common method set, 3D (the same switches as pair_std);
    // the neighbour's p/rho^2 comes from its pressure pair (pri.y).
    __device__ __forceinline__ void pair_std3(const float4 vi, const float2 pri, float dx, float dy, float dz,
                                              float d2, int32_t ti) {
        const MixedF& M = P.mf;
        const float inv_dist = rsqrtf(d2);
        const float dist = d2 * inv_dist;
        const float q = dist * M.inv_h;
        float m = 0.0f;
        if (ext && ti < 0 && dist < M.lj_rr0) m -= lj_coef(M, inv_dist);
        const float rhoi = vi.w;
        const float sc = cubic_dwdr_sel(M.kf[1], q, inv_dist, M.inv_h);
        m += sc * (pri.y + prj.y) * M.mass;
        const float vr = -((vj.x - vi.x) * dx + (vj.y - vi.y) * dy + (vj.z - vi.z) * dz);
        const float mu = fminf(__fdividef(M.h * vr, d2 + M.etq_h2), 0.0f);
        arvmu = fmaxf(arvmu, -mu);
        const float piv = __fdividef((M.av_beta * mu - M.av_alpha_c) * mu, 0.5f * (rhoi + rhoj));
        m += sc * piv * M.mass;
        cax += dx * m;
        cay += dy * m;
        caz += dz * m;
    }
};

}  // namespace
}  // namespace rrsph
