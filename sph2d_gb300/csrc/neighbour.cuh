// neighbour.cuh — the 3^dim cell stencil of the grid search.
#pragma once

#include "common.cuh"

namespace rrsph {

// get_cell_coord2/3 (GridUtils.h:152-157): Morton decode of a cell key.
template <int DIM>
__device__ inline void decode_key(uint32_t key, uint64_t& x, uint64_t& y, uint64_t& z) {
    if (DIM == 3) {
        x = third_bits(key);
        y = third_bits(key >> 1);
        z = third_bits(key >> 2);
    } else {
        x = second_bits(key);
        y = second_bits(key >> 1);
        z = 0;
    }
}

// Visits the neighbouring cells of `key` in the order of get_neighbouring_cells2/3
// (GridUtils.h:190-250): x outer, then y, then z; an invalid coordinate drops
// the cell. f(cell, sx, sy, sz) gets each cell key below max_cells and the
// signed displacement of that cell's coordinates from the centre cell (which
// is not +-1 where the reference's Morton encoding wraps a 3D coordinate).
template <int DIM, class F>
__device__ __forceinline__ void for_neighbour_cells(const DevParams& P, uint32_t key, F&& f) {
    uint64_t cx, cy, cz;
    decode_key<DIM>(key, cx, cy, cz);
    const uint64_t mask = DIM == 3 ? 0x3FFull : 0xFFFFull;
#pragma unroll
    for (int dx = -1; dx <= 1; dx++) {
        const uint64_t x = step_coord(cx, dx);
        if (x == kInvalidCell) continue;
#pragma unroll
        for (int dy = -1; dy <= 1; dy++) {
            const uint64_t y = step_coord(cy, dy);
            if (y == kInvalidCell) continue;
            if (DIM == 3) {
#pragma unroll
                for (int dz = -1; dz <= 1; dz++) {
                    const uint64_t z = step_coord(cz, dz);
                    if (z == kInvalidCell) continue;
                    const uint64_t c = split3(x) | (split3(y) << 1) | (split3(z) << 2);
                    if (c < P.max_cells)
                        f((uint32_t)c, (int)((int64_t)(x & mask) - (int64_t)cx),
                          (int)((int64_t)(y & mask) - (int64_t)cy), (int)((int64_t)(z & mask) - (int64_t)cz));
                }
            } else {
                const uint64_t c = split2(x) | (split2(y) << 1);
                if (c < P.max_cells)
                    f((uint32_t)c, (int)((int64_t)(x & mask) - (int64_t)cx),
                      (int)((int64_t)(y & mask) - (int64_t)cy), 0);
            }
        }
    }
}

// 32-bit Morton splits. For coordinates below 2^16 (2D) / any coordinate
// (3D, masked to 10 bits) they equal the reference's 64-bit split2/split3.
__device__ __forceinline__ uint32_t split2_32(uint32_t x) {
    x &= 0x0000FFFFu;
    x = (x | x << 8) & 0x00FF00FFu;
    x = (x | x << 4) & 0x0F0F0F0Fu;
    x = (x | x << 2) & 0x33333333u;
    x = (x | x << 1) & 0x55555555u;
    return x;
}
__device__ __forceinline__ uint32_t split3_32(uint32_t a) {
    uint32_t x = a & 0x000003ffu;
    x = (x | x << 16) & 0x30000ffu;
    x = (x | x << 8) & 0x0300f00fu;
    x = (x | x << 4) & 0x30c30c3u;
    x = (x | x << 2) & 0x9249249u;
    return x;
}

// The 3^dim cell stencil of one particle's cell, in the order of
// get_neighbouring_cells2/3 (GridUtils.h:190-250): x outer, then y, then z.
// Each axis keeps its three Morton-split coordinates (offsets -1, 0, +1),
// their validity (dec_cell_coord / inc_cell_coord, GridUtils.h:158-163) and
// their displacement from the centre (not +-1 where the reference's 10-bit
// 3D split wraps coordinate 1024 to 0).
template <int DIM>
struct Stencil {
    uint32_t mx[3], my[3], mz[3];
    int sx[3], sy[3], sz[3];
    uint32_t valid;  // bit 3*axis + offset
    uint32_t max_cells;

    __device__ __forceinline__ void axis(uint32_t c, int ax, uint32_t* m, int* s) {
        const uint32_t mask = DIM == 3 ? 0x3FFu : 0xFFFFu;
        // offset -1
        if (c != 0) {
            valid |= 1u << (3 * ax);
            m[0] = DIM == 3 ? split3_32(c - 1) : split2_32(c - 1);
            s[0] = -1;
        }
        valid |= 1u << (3 * ax + 1);
        m[1] = DIM == 3 ? split3_32(c) : split2_32(c);
        s[1] = 0;
        if (c != kMaxCellCoord2) {
            valid |= 1u << (3 * ax + 2);
            m[2] = DIM == 3 ? split3_32(c + 1) : split2_32(c + 1);
            s[2] = (int)((c + 1) & mask) - (int)c;
        }
    }

    __device__ __forceinline__ Stencil(const DevParams& P, uint32_t key) : valid(0), max_cells(P.max_cells) {
        uint32_t cx, cy, cz;
        if (DIM == 3) {
            cx = third_bits(key);
            cy = third_bits(key >> 1);
            cz = third_bits(key >> 2);
        } else {
            cx = second_bits(key);
            cy = second_bits(key >> 1);
            cz = 0;
        }
#pragma unroll
        for (int i = 0; i < 3; i++) { mx[i] = my[i] = mz[i] = 0; sx[i] = sy[i] = sz[i] = 0; }
        axis(cx, 0, mx, sx);
        axis(cy, 1, my, sy);
        if (DIM == 3) axis(cz, 2, mz, sz);
    }

    static __device__ __forceinline__ uint32_t pick(int i, const uint32_t* v) { return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]); }
    static __device__ __forceinline__ int pick(int i, const int* v) { return i == 0 ? v[0] : (i == 1 ? v[1] : v[2]); }

    // Coordinate offsets of stencil cell c (as cell() returns them).
    __device__ __forceinline__ void offsets(int c, int& dx, int& dy, int& dz) const {
        int a, b, d;
        if (DIM == 3) {
            a = c / 9;
            b = (c / 3) % 3;
            d = c % 3;
        } else {
            a = c / 3;
            b = c % 3;
            d = 1;
        }
        dx = pick(a, sx);
        dy = pick(b, sy);
        dz = DIM == 3 ? pick(d, sz) : 0;
    }

    // Cell c of the stencil (c in [0, 3^DIM)); false when the reference marks
    // it invalid or its key is >= max_cells.
    __device__ __forceinline__ bool cell(int c, uint32_t& key, int& dx, int& dy, int& dz) const {
        int a, b, d;
        if (DIM == 3) {
            a = c / 9;
            b = (c / 3) % 3;
            d = c % 3;
        } else {
            a = c / 3;
            b = c % 3;
            d = 1;
        }
        const uint32_t need = (1u << a) | (1u << (3 + b)) | (DIM == 3 ? (1u << (6 + d)) : 0u);
        if ((valid & need) != need) return false;
        key = pick(a, mx) | (pick(b, my) << 1);
        if (DIM == 3) key |= pick(d, mz) << 2;
        if (key >= max_cells) return false;
        dx = pick(a, sx);
        dy = pick(b, sy);
        dz = DIM == 3 ? pick(d, sz) : 0;
        return true;
    }
};

// The reference's cutoff test dist^2 < (cell_scale_k*h)^2 (GridFind.cpp:143-146)
// in double without contraction, so the pair set matches bit for bit.
template <int DIM>
__device__ __forceinline__ double exact_dist2(double dx, double dy, double dz) {
    double s = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (DIM == 3) s = __dadd_rn(s, __dmul_rn(dz, dz));
    return s;
}

}  // namespace rrsph
