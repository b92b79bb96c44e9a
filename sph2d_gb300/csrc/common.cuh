// common.cuh — device-side definitions shared by the WCSPH kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/rrsph_cuda.h"

namespace rrsph {

constexpr uint32_t kInvalidCell = 0xFFFFFFFFu;      // GRID_INVALID_CELL (GridUtils.h:8)
constexpr uint32_t kMaxCellCoord2 = (1u << 16) - 1; // GRID_MAX_CELL_COORD2 (GridUtils.h:9)
constexpr uint32_t kEmpty = 0xFFFFFFFFu;            // empty cell-table entry

// Float constants of the FP32-mixed gathers, precomputed on the host.
struct MixedF {
    float cell, h, inv_h, mass, rho0;
    float cut2_lo, cut2_hi;     // guard band around the cutoff: pairs inside it are re-tested in double
    float kf[5];                // kernel factors by skf
    float w0_density;           // mass * W(0)
    float rho0_minus_w0_hi, rho0_minus_w0_lo;  // rho0 - mass*W(0) as an unevaluated float sum
    float B, inv_rho0;          // EOS constants
    float lj_rr0, lj_D, etq_h2;
    float av_alpha_c, av_beta;  // alpha * c, beta
    float ap_coef, ap_index, ap_inv_wdelta;
    float avel_coef2;           // 2 * average_velocity_coef
    float dhc;                  // delta-SPH: coef * h * c
};

// Everything a kernel needs from rrsph_params, precomputed on the host.
struct DevParams {
    int dim;
    uint32_t n;             // ntotal
    uint32_t nfluid;
    uint32_t max_cells;     // Morton key bound (power of two)
    uint32_t max_nb;        // max_neighbours: the reference stores at most max_nb - 1
    int type_non_existent;
    double xmin, ymin, zmin, xmax, ymax, zmax;
    long long oxmin, oymin, ozmin, oxmax, oymax, ozmax;  // dorder() of the bounds
    double cell;            // cell_scale_k * hsml (grid_cell_size)
    double inv_cell;
    double cut2;            // sqr(grid_cell_size()) computed as the reference does
    double h, inv_h, mass, g, rho0;
    double B;               // EOS: c^2 rho0 / 7
    double c_eos;           // eos_art_c()
    double c_av;            // params.eos_sound_vel used by the artificial viscosity
    double etq_h2;          // sqr(hsml * 0.1f)
    double w0_density;      // smoothing_kernel_w(0, density_skf)
    double kf[5];           // kernel factors by skf (index 1..4)
    int density_skf, intf_skf, av_skf, avel_skf, ap_skf;
    int density_treatment;  // 0 sum, 1 con, 2 con + delta
    double delta_sph_dhc;   // density_delta_sph_coef * hsml * eos_art_c()
    int intf_form;          // 1 or 2
    int art_pressure;
    double ap_index, ap_coef, ap_wdelta;  // wdelta = smoothing_kernel_w(delta, ap_skf)
    int art_visc;
    double av_alpha, av_beta;
    int avg_vel;
    double avg_vel_coef;
    int repulsive;          // boundary_treatment == SBT_REPULSIVE
    double lj_rr0, lj_D;
    int consistency_check, consistency_treatment;
    // piston / wave maker
    int nwm;
    uint32_t nwm_start, nwm_end;
    int nwm_valid;
    double nwm_time_start, nwm_phase, nwm_freq, nwm_H, nwm_k, depth;
    // Fourier piston (rrsph_set_piston_fourier): X(t) = sum_k fourier_coef[k-1] sin(k omega t)
    int fourier_n;          // 0: the wave maker's own law
    double fourier_omega;
    double fourier_coef[16];
    // dt control
    int dt_method;          // 0 const, 1 CFL const, 2 dynamic
    int dt_reduce;          // 1: true max reduction
    double cfl, never_ending_dt;
    int all_cubic;          // every smoothing kernel choice is the cubic spline
    // neighbour reuse (mixed step): list cutoff (cell + skin)^2, (skin / 2)^2, and
    // the distance from a cell edge within which the list looks two cells away
    float vl_cut2, vl_half_skin2, vl_skin_edge;
    // 1: the key pass leaves the cell table of the last list build in place
    // (the cell-tile density pass reads it on reuse steps); each rebuild then
    // clears the table wholesale before the reorder writes the new one
    int keep_cells;
    MixedF mf;
};

// One piston of a wave-maker table (rrsph_set_wave_makers): the law of
// dynamic_boundaries (WaveMaker.cpp:34-82) with its own parameters.
struct PistonLaw {
    int nwm;  // 2: first order, 3: second order
    double time_start, phase, freq, H, k, depth;
};

// Per-step scalars kept on the device (double-buffered by step parity so a
// captured step graph can advance them without host involvement).
struct StepScalars {
    double time;
    double dt;
    unsigned long long step;   // itimestep of the reference loop
    unsigned long long amax_bits;  // max |a| over particles (as ordered bits)
    unsigned long long mumax_bits; // max arvmu
    unsigned long long pairs;      // directed pairs found by the density gather of this step
    unsigned long long nwm_off;    // 1 once a one-shot wave maker (wall disappear) has fired
    unsigned long long pairs_total;  // pairs summed over the steps since upload
};

// ------------------------------------------- FP64-free double handling --
// The FP64 pipe is the scarce one on this part (one lane per clock per SM), so
// compares, halvings and conversions of doubles that need no FP64 arithmetic
// are done on their bit patterns with integer operations.

// Integer image of a double that orders like the double (IEEE total order with
// -0 mapped to +0, so equal zeros stay equal). NaNs are excluded by callers.
__host__ __device__ inline long long dorder(double v) {
    long long b;
#ifdef __CUDA_ARCH__
    b = __double_as_longlong(v);
#else
    __builtin_memcpy(&b, &v, sizeof(b));
#endif
    if (b == (long long)0x8000000000000000ull) b = 0;
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFll);
}
__device__ __forceinline__ bool dnan(double v) {
    return ((unsigned long long)__double_as_longlong(v) & 0x7FFFFFFFFFFFFFFFull) > 0x7FF0000000000000ull;
}
// v / 2, exactly, for a normal v whose half is normal; otherwise the multiply.
__device__ __forceinline__ double dhalf(double v) {
    const long long b = __double_as_longlong(v);
    const long long e = (b >> 52) & 0x7FF;
    if (e > 1 && e < 0x7FF) return __longlong_as_double(b - (1ll << 52));
    return v * 0.5;
}
// Round-to-nearest-even double -> float (bit-identical to the conversion
// instruction) for results in the normal float range; the rest converts in hardware.
__device__ __forceinline__ float d2f(double v) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(v);
    const unsigned int e = (unsigned int)(b >> 52) & 0x7FFu;
    if (e >= 1023u - 126u && e <= 1023u + 127u) {
        const unsigned int sign = (unsigned int)(b >> 32) & 0x80000000u;
        const unsigned int mf = (unsigned int)((b >> 29) & 0x7FFFFFu);
        const unsigned int rem = (unsigned int)(b & 0x1FFFFFFFu);
        unsigned int r = ((e - 1023u + 127u) << 23) | mf;
        if (rem > 0x10000000u || (rem == 0x10000000u && (mf & 1u))) r += 1;  // a carry moves to the next binade or to inf
        return __uint_as_float(sign | r);
    }
    return (float)v;
}
// Exact float -> double for normal floats; the rest converts in hardware.
__device__ __forceinline__ double f2d(float f) {
    const unsigned int b = __float_as_uint(f);
    const unsigned int e = (b >> 23) & 0xFFu;
    if (e != 0u && e != 0xFFu) {
        const unsigned long long r = ((unsigned long long)(b & 0x80000000u) << 32) |
                                     ((unsigned long long)(e - 127u + 1023u) << 52) |
                                     ((unsigned long long)(b & 0x7FFFFFu) << 29);
        return __longlong_as_double((long long)r);
    }
    return (double)f;
}

// The float copy of (v, rho - rho0) that density_con reads of a neighbour. In
// 2D the unused z carries the low part of rho - rho0 (the double minus its
// float), so that rho_i - rho_j keeps ~1e-7 of the difference itself: the
// deviations are ~5 at half a metre of water and differ by ~0.1 between
// neighbours, so one float each would leave ~3e-6 of the difference.
template <int DIM>
__device__ __forceinline__ float4 vd4_of(double vx, double vy, double vz, double drho0) {
    const float hi = d2f(drho0);
    return make_float4(d2f(vx), d2f(vy), DIM == 3 ? d2f(vz) : d2f(drho0 - f2d(hi)), hi);
}
// rho_i - rho_j from two such copies.
template <int DIM>
__device__ __forceinline__ float vd4_drho(float4 vdi, float4 vdj) {
    return DIM == 3 ? vdi.w - vdj.w : (vdi.w - vdj.w) + (vdi.z - vdj.z);
}

// ---------------------------------------------------------------- Morton --
// GridUtils.h:50-64 and 92-104, computed in 64-bit like rr_uint.
__host__ __device__ inline uint64_t split2(uint64_t x) {
    x = (x | x << 16) & 0x0000FFFFull;
    x = (x | x << 8) & 0x00FF00FFull;
    x = (x | x << 4) & 0x0F0F0F0Full;
    x = (x | x << 2) & 0x33333333ull;
    x = (x | x << 1) & 0x55555555ull;
    return x;
}
__host__ __device__ inline uint64_t split3(uint64_t a) {
    uint64_t x = a & 0x000003ffull;
    x = (x | x << 16) & 0x30000ffull;
    x = (x | x << 8) & 0x0300f00full;
    x = (x | x << 4) & 0x30c30c3ull;
    x = (x | x << 2) & 0x9249249ull;
    return x;
}
__host__ __device__ inline uint32_t second_bits(uint32_t m) { // GridUtils.h:107-114
    uint32_t x = m & 0x55555555u;
    x = (x ^ (x >> 1)) & 0x33333333u;
    x = (x ^ (x >> 2)) & 0x0F0F0F0Fu;
    x = (x ^ (x >> 4)) & 0x00FF00FFu;
    x = (x ^ (x >> 8)) & 0x0000FFFFu;
    return x;
}
__host__ __device__ inline uint32_t third_bits(uint32_t m) { // GridUtils.h:67-74
    uint32_t x = m & 0x9249249u;
    x = (x ^ (x >> 2)) & 0x30c30c3u;
    x = (x ^ (x >> 4)) & 0x0300f00fu;
    x = (x ^ (x >> 8)) & 0x30000ffu;
    x = (x ^ (x >> 16)) & 0x000003ffu;
    return x;
}

// get_cell_coord_from_particle_coord (GridUtils.h:135-137): truncation of
// (r - r_min) / cell. A negative quotient (outside the geometry) maps to 0 and
// is reported through the out-of-domain flag by the key pass.
__device__ inline uint64_t cell_coord(double r, double rmin, double cell) {
    const double c = __ddiv_rn(__dsub_rn(r, rmin), cell);
    if (!(c >= 0.0)) return 0;
    if (c >= 18446744073709551615.0) return ~0ull;
    return (uint64_t)c;
}

// Cell coordinate of r (the truncation above) and r's offset from that
// cell's lower edge, from one double subtract and one multiply. The FP64 pipe
// is the scarce one, so the integer part and the fraction of
// q = (r - rmin) * (1/cell) are read from q's bits with integer operations.
// q is within 2 ulp of the exact quotient, so where 2^-30 <= q < 2^21 and q's
// fraction is more than 2^-30 from an integer its truncation is the
// quotient's; every other case (outside the geometry, near a cell edge, not
// finite) takes the exact division. below: r < rmin or r is NaN.
struct CellSplit {
    uint64_t c;
    float off;   // r - (rmin + c cell), in float
    bool below;
};
__device__ inline CellSplit cell_split(double r, double rmin, double cell, double inv_cell, float cellf) {
    const double q = __dmul_rn(__dsub_rn(r, rmin), inv_cell);
    const long long bits = __double_as_longlong(q);
    if (bits > 0) {
        const int e = (int)(bits >> 52) - 1023;
        const unsigned long long m = ((unsigned long long)bits & 0xFFFFFFFFFFFFFull) | (1ull << 52);
        if (e >= 0 && e <= 20) {
            const int F = 52 - e;
            const unsigned long long frac = m & ((1ull << F) - 1);
            const unsigned long long top = frac >> (F - 30);
            if (top != 0 && top != (1ull << 30) - 1) {
                const float f = (float)(uint32_t)(frac >> (F - 24)) * 5.9604644775390625e-8f;  // * 2^-24
                return {m >> F, f * cellf, false};
            }
        } else if (e < 0 && e >= -30 && !(e == -1 && (m >> 23) == (1ull << 30) - 1)) {
            return {0, (float)q * cellf, false};
        }
    }
    const uint64_t c = cell_coord(r, rmin, cell);
    return {c, (float)(r - (rmin + (double)c * cell)), !(r >= rmin)};
}

// Neighbour-cell coordinate steps (GridUtils.h:158-163).
__device__ inline uint64_t step_coord(uint64_t c, int d) {
    if (d < 0) return c == 0 ? (uint64_t)kInvalidCell : c - 1;
    if (d > 0) return c == kMaxCellCoord2 ? (uint64_t)kInvalidCell : c + 1;
    return c;
}

// ------------------------------------------------------ smoothing kernels --
// SmoothingKernel.h:20-274 with q = dist * (1/h). `f` is the factor of skf.
__device__ inline double kernel_w(int skf, double f, double q) {
    switch (skf) {
    case 2: return f * exp(-q * q);
    case 3: {
        if (q <= 2.0) {
            const double t = 1.0 - 0.5 * q;
            const double t2 = t * t;
            return f * (t2 * t2) * (2.0 * q + 1.0);
        }
        return 0.0;
    }
    case 4: {
        if (q <= 2.0) { const double t = 2.0 - q; return f * (t * t * t); }
        return 0.0;
    }
    default:
        if (q <= 1.0) return f * (2.0 / 3.0 - q * q + q * q * q * 0.5);
        if (q <= 2.0) { const double t = 2.0 - q; return f * (1.0 / 6.0 * (t * t * t)); }
        return 0.0;
    }
}

// Scalar s such that dW/dr = diff * s (diff = r_i - r_j, |diff| = dist).
__device__ inline double kernel_dwdr_scale(int skf, double f, double q, double dist, double inv_h) {
    switch (skf) {
    case 2: return inv_h * inv_h * (-2.0) * (f * exp(-q * q));
    case 3: {
        if (q < (double)1.e-6f || !(q < 2.0)) return 0.0;
        const double t = 1.0 - 0.5 * q;
        const double t3 = t * t * t;
        return inv_h / dist * f * 2.0 * (t3 * t - (2.0 * q + 1.0) * t3);
    }
    case 4: {
        if (q < 2.0) { const double t = 2.0 - q; return inv_h / dist * f * (-3.0 * t * t); }
        return 0.0;
    }
    default:
        if (q <= 1.0) return inv_h * inv_h * f * (-2.0 + 1.5 * q);
        if (q <= 2.0) { const double t = 2.0 - q; return -(inv_h / dist) * f * (t * t * 0.5); }
        return 0.0;
    }
}

// eos_art_p (EOS.cpp:31-34)
__device__ inline double eos_p(const DevParams& P, double rho) {
    const double x = rho / P.rho0;
    const double x2 = x * x;
    const double x4 = x2 * x2;
    return P.B * (x4 * x2 * x - 1.0);
}

// Ordered-bits encoding of non-negative doubles for atomicMax.
__device__ inline unsigned long long dbits(double v) { return (unsigned long long)__double_as_longlong(v); }

}  // namespace rrsph
