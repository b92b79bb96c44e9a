// sort.cuh — stable LSD radix sort of (32-bit cell key, 32-bit particle id) pairs.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace rrsph {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 4;
constexpr int kSortTile = kSortThreads * kSortItems;  // keys per tile
constexpr int kRadix = 256;                           // 8-bit digits

inline uint32_t sort_tiles(uint32_t n) { return (n + kSortTile - 1) / kSortTile; }
// Scratch words the sort needs for n keys: per-tile digit counts + digit totals.
inline size_t sort_scratch_words(uint32_t n) { return (size_t)kRadix * sort_tiles(n) + kRadix; }

// Sorts n pairs by the low `bits` bits of the keys, stably (equal keys keep
// their input order): reads keys_in/vals_in (not modified), leaves the result
// in keys_out/vals_out, and uses keys_tmp/vals_tmp (n words each) and counts
// (sort_scratch_words(n) words) as working memory. Launches 3 kernels per
// 8-bit digit on `stream`; adds them to *launches.
void radix_sort_pairs_into(const uint32_t* keys_in, const uint32_t* vals_in, uint32_t* keys_out, uint32_t* vals_out,
                           uint32_t* keys_tmp, uint32_t* vals_tmp, uint32_t* counts, uint32_t n, int bits,
                           cudaStream_t stream, unsigned long long* launches);

}  // namespace rrsph
