// sort.cu — stable LSD radix sort of (cell key, particle id) pairs.
//
// Replaces the reference's serial counting sort over max_cells
// (sources/RRSPH_OMP/src/GridFind.cpp:47-88) and the OpenCL bitonic sort
// (sources/RRSPH_CL/cl/GridFind.cl:73-93, power-of-two sizes only): any n,
// stable, so that ids stay ascending within a cell exactly as after the
// reference's reverse scatter.
//
// One 8-bit digit per pass, three kernels per pass, no inter-block waiting:
//   1. k_tile_hist:   digit counts of each 1024-key tile        -> counts[d][tile]
//   2. k_digit_scan:  one warp per digit scans its row over tiles (exclusive)
//                     and records the digit total
//   3. k_scatter:     each tile ranks its keys stably (warp match + per-warp
//                     counts, in (warp, round, lane) = input order) and writes
//                     them to total-prefix[d] + tile-prefix[d][tile] + rank.
#include "sort.cuh"

namespace rrsph {

namespace {

constexpr int kWarps = kSortThreads / 32;

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__global__ void __launch_bounds__(kSortThreads) k_tile_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                            uint32_t tiles, uint32_t* __restrict__ counts) {
    __shared__ uint32_t h[kRadix];
    for (int d = threadIdx.x; d < kRadix; d += kSortThreads) h[d] = 0;
    __syncthreads();
    const uint32_t base = blockIdx.x * (uint32_t)kSortTile;
    const uint32_t lane = threadIdx.x & 31;
#pragma unroll
    for (int r = 0; r < kSortItems; r++) {
        const uint32_t idx = base + r * kSortThreads + threadIdx.x;
        const bool valid = idx < n;
        const uint32_t d = valid ? ((keys[idx] >> shift) & (kRadix - 1)) : kRadix;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        // one shared-memory add per distinct digit in the warp
        if (valid && (__ffs(peers) - 1) == (int)lane) atomicAdd(&h[d], __popc(peers));
    }
    __syncthreads();
    for (int d = threadIdx.x; d < kRadix; d += kSortThreads) counts[(size_t)d * tiles + blockIdx.x] = h[d];
}

// counts[d][t] -> exclusive prefix over t; totals[d] = row sum.
__global__ void k_digit_scan(uint32_t* __restrict__ counts, uint32_t tiles, uint32_t* __restrict__ totals) {
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t lane = threadIdx.x & 31;
    if (warp >= kRadix) return;
    uint32_t* row = counts + (size_t)warp * tiles;
    uint32_t carry = 0;
    for (uint32_t t0 = 0; t0 < tiles; t0 += 32) {
        const uint32_t t = t0 + lane;
        const uint32_t v = t < tiles ? row[t] : 0;
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if ((int)lane >= o) incl += x;
        }
        if (t < tiles) row[t] = carry + incl - v;
        carry += __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    if (lane == 0) totals[warp] = carry;
}

// Stable scatter of one tile. Each warp owns 256 consecutive keys of the tile
// (kSortItems rounds of 32), so the tile's input order is (warp, round, lane):
// a key's rank is the count of equal digits before it in its warp (per-warp
// running counts, updated by one leader per digit group and round), plus the
// counts of that digit in the warps before it, plus the digit's start for
// this tile. Three block barriers per tile.
__global__ void __launch_bounds__(kSortThreads) k_scatter(const uint32_t* __restrict__ keys_in,
                                                          const uint32_t* __restrict__ vals_in,
                                                          uint32_t* __restrict__ keys_out,
                                                          uint32_t* __restrict__ vals_out, uint32_t n, int shift,
                                                          uint32_t tiles, const uint32_t* __restrict__ prefix,
                                                          const uint32_t* __restrict__ totals) {
    __shared__ uint32_t base_of[kRadix];                // output start of each digit for this tile
    __shared__ uint16_t wcnt[kWarps][kRadix];           // per-warp digit counts, then per-warp offsets
    __shared__ uint32_t scan_tmp[kWarps];

    const int tid = threadIdx.x;
    const uint32_t warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < kWarps * kRadix / 2; i += kSortThreads) reinterpret_cast<uint32_t*>(&wcnt[0][0])[i] = 0;
    // exclusive scan of the 256 digit totals (kSortThreads == kRadix)
    {
        const uint32_t v = totals[tid];
        uint32_t incl = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if ((int)lane >= o) incl += x;
        }
        if (lane == 31) scan_tmp[warp] = incl;
        __syncthreads();
        uint32_t warp_off = 0;
        for (uint32_t w = 0; w < warp; w++) warp_off += scan_tmp[w];
        base_of[tid] = warp_off + incl - v + prefix[(size_t)tid * tiles + blockIdx.x];
    }
    uint32_t key[kSortItems], val[kSortItems], rank[kSortItems];
    const uint32_t wbase = blockIdx.x * (uint32_t)kSortTile + warp * (kSortItems * 32);
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int r = 0; r < kSortItems; r++) {
        const uint32_t idx = wbase + r * 32 + lane;
        const bool valid = idx < n;
        key[r] = valid ? keys_in[idx] : 0u;
        val[r] = valid ? vals_in[idx] : 0u;
        const uint32_t d = valid ? ((key[r] >> shift) & (kRadix - 1)) : kRadix;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t cur = valid ? wcnt[warp][d] : 0u;
        __syncwarp();
        if (valid && (__ffs(peers) - 1) == (int)lane) wcnt[warp][d] = (uint16_t)(cur + __popc(peers));
        __syncwarp();
        rank[r] = valid ? cur + __popc(peers & lt) : 0xFFFFFFFFu;
    }
    __syncthreads();
    {   // per digit: counts of the warps -> exclusive offsets over warps
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kWarps; w++) {
            const uint32_t c = wcnt[w][tid];
            wcnt[w][tid] = (uint16_t)run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < kSortItems; r++) {
        if (rank[r] == 0xFFFFFFFFu) continue;
        const uint32_t d = (key[r] >> shift) & (kRadix - 1);
        const uint32_t pos = base_of[d] + wcnt[warp][d] + rank[r];
        keys_out[pos] = key[r];
        vals_out[pos] = val[r];
    }
}

}  // namespace

void radix_sort_pairs_into(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                           uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t* counts, uint32_t n, int bits,
                           cudaStream_t stream, unsigned long long* launches) {
    if (n == 0) return;
    const uint32_t tiles = sort_tiles(n);
    uint32_t* totals = counts + (size_t)kRadix * tiles;
    const int passes = (bits + 7) / 8;
    const uint32_t *ki = keys_in, *vi = vals_in;
    for (int pass = 0; pass < passes; pass++) {
        // the last pass must land in the output, so targets alternate backwards from it
        const bool to_out = ((passes - 1 - pass) % 2) == 0;
        uint32_t* ko = to_out ? keys_out : keys_tmp;
        uint32_t* vo = to_out ? vals_out : vals_tmp;
        const int shift = pass * 8;
        k_tile_hist<<<tiles, kSortThreads, 0, stream>>>(ki, n, shift, tiles, counts);
        k_digit_scan<<<kRadix * 32 / 256, 256, 0, stream>>>(counts, tiles, totals);
        k_scatter<<<tiles, kSortThreads, 0, stream>>>(ki, vi, ko, vo, n, shift, tiles, counts, totals);
        if (launches) *launches += 3;
        ki = ko;
        vi = vo;
    }
}

}  // namespace rrsph
