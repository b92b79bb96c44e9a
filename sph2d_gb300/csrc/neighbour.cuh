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

// The c-th cell (c in [0, 3^DIM)) of the stencil of the cell at (cx, cy, cz),
// in the order of get_neighbouring_cells2/3 (x outer, then y, then z). Returns
// false when the reference marks the cell invalid or its key is >= max_cells.
// (sx, sy, sz) is the displacement of the cell's coordinates from the centre.
template <int DIM>
__device__ __forceinline__ bool stencil_cell(const DevParams& P, uint64_t cx, uint64_t cy, uint64_t cz, int c,
                                             uint32_t& cell, int& sx, int& sy, int& sz) {
    int dx, dy, dz;
    if (DIM == 3) {
        dx = c / 9 - 1;
        dy = (c / 3) % 3 - 1;
        dz = c % 3 - 1;
    } else {
        dx = c / 3 - 1;
        dy = c % 3 - 1;
        dz = 0;
    }
    const uint64_t x = step_coord(cx, dx), y = step_coord(cy, dy);
    if (x == kInvalidCell || y == kInvalidCell) return false;
    uint64_t key;
    const uint64_t mask = DIM == 3 ? 0x3FFull : 0xFFFFull;
    if (DIM == 3) {
        const uint64_t z = step_coord(cz, dz);
        if (z == kInvalidCell) return false;
        key = split3(x) | (split3(y) << 1) | (split3(z) << 2);
        sz = (int)((int64_t)(z & mask) - (int64_t)cz);
    } else {
        key = split2(x) | (split2(y) << 1);
        sz = 0;
    }
    if (key >= P.max_cells) return false;
    cell = (uint32_t)key;
    sx = (int)((int64_t)(x & mask) - (int64_t)cx);
    sy = (int)((int64_t)(y & mask) - (int64_t)cy);
    return true;
}

// The reference's cutoff test dist^2 < (cell_scale_k*h)^2 (GridFind.cpp:143-146)
// in double without contraction, so the pair set matches bit for bit.
template <int DIM>
__device__ __forceinline__ double exact_dist2(double dx, double dy, double dz) {
    double s = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
    if (DIM == 3) s = __dadd_rn(s, __dmul_rn(dz, dz));
    return s;
}

}  // namespace rrsph
