// sort_noalloc.cu — the grid's (cell key, particle id) radix sort for callers
// that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code whose device memory is owned by
// another framework's pool, or a step loop that must not allocate because an
// allocation can block the device or fail part-way through a run. This entry
// point takes device pointers to the caller's inputs and outputs and keeps its
// own working memory in a fixed array compiled into the library, so it
// allocates nothing.
//
// The array holds one spare key/id buffer pair for the ping-pong passes plus
// the per-tile digit counts, sized for RRSPH_SORT_NOALLOC_MAX_PAIRS pairs
// (about 9.4 MB). Every GPU that loads this library holds it until the process
// exits. Nothing in it needs clearing between calls: every pass rewrites the
// counts it reads. All calls on a device share it, so calls that can overlap on
// the GPU race; the caller orders them (one stream, or events).
#include <cstdint>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/rrsph_cuda.h"
#include "../host/error.hpp"
#include "sort.cuh"

namespace {

constexpr uint32_t kMaxPairs = RRSPH_SORT_NOALLOC_MAX_PAIRS;
constexpr size_t kTilesMax = (kMaxPairs + rrsph::kSortTile - 1) / rrsph::kSortTile;
constexpr size_t kCountWords = (size_t)rrsph::kRadix * kTilesMax + rrsph::kRadix;
constexpr size_t kScratchWords = 2 * (size_t)kMaxPairs + kCountWords;

// Working memory of rrsph_sort_pairs_noalloc. In host code this name is only a
// host-side stand-in; the device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) uint32_t g_sort_scratch[kScratchWords];

constexpr int kMaxDevices = 256;
std::mutex g_mutex;
uint32_t* g_scratch_addr[kMaxDevices] = {};

// Device address of g_sort_scratch on the current device, looked up once per
// device (with that device current) and kept for the life of the process: a
// cudaDeviceReset of that device invalidates it, so the entry point must not
// be used on a device after a reset.
int scratch_address(uint32_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return rrsph::set_error(RRSPH_ERR_CUDA, std::string("rrsph_sort_pairs_noalloc: cudaGetDevice: ") +
                                                   cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices)
        return rrsph::set_error(RRSPH_ERR_UNSUPPORTED, "rrsph_sort_pairs_noalloc: device index out of range");
    std::lock_guard<std::mutex> lock(g_mutex);
    if (!g_scratch_addr[dev]) {
        void* ptr = nullptr;
        e = cudaGetSymbolAddress(&ptr, g_sort_scratch);
        if (e != cudaSuccess || !ptr)
            return rrsph::set_error(RRSPH_ERR_CUDA, std::string("rrsph_sort_pairs_noalloc: cudaGetSymbolAddress: ") +
                                                       cudaGetErrorString(e));
        g_scratch_addr[dev] = static_cast<uint32_t*>(ptr);
    }
    *out = g_scratch_addr[dev];
    return RRSPH_OK;
}

// Whether [a, a + n) and [b, b + n) (32-bit words) share a word.
bool overlaps(const void* a, const void* b, uint32_t n) {
    const uintptr_t x = reinterpret_cast<uintptr_t>(a), y = reinterpret_cast<uintptr_t>(b);
    const uintptr_t len = (uintptr_t)n * sizeof(uint32_t);
    return x < y + len && y < x + len;
}

}  // namespace

extern "C" int rrsph_sort_pairs_noalloc(const uint32_t* keys_in, const uint32_t* ids_in, uint32_t* keys_out,
                                        uint32_t* ids_out, uint32_t n, uint32_t key_bits, void* stream) {
    using rrsph::set_error;
    if (n > kMaxPairs)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT,
                         "rrsph_sort_pairs_noalloc: n = " + std::to_string(n) + " exceeds the maximum of " +
                             std::to_string(kMaxPairs) + " pairs (the size of its fixed working memory)");
    if (key_bits < 1 || key_bits > 32)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_sort_pairs_noalloc: key_bits must be in [1, 32]");
    if (n == 0) return RRSPH_OK;
    if (!keys_in || !ids_in || !keys_out || !ids_out)
        return set_error(RRSPH_ERR_INVALID_ARGUMENT, "rrsph_sort_pairs_noalloc: null pointer");
    // the passes write an output while other blocks still read the inputs, and
    // the two outputs alternate with the working array
    if (overlaps(keys_out, keys_in, n) || overlaps(keys_out, ids_in, n) || overlaps(ids_out, keys_in, n) ||
        overlaps(ids_out, ids_in, n) || overlaps(keys_out, ids_out, n))
        return set_error(RRSPH_ERR_INVALID_ARGUMENT,
                         "rrsph_sort_pairs_noalloc: the output buffers must not overlap the inputs or each other");
    uint32_t* base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    // an error left by the caller's earlier work is reported, not cleared: its
    // owner's own check still sees it
    cudaError_t e = cudaPeekAtLastError();
    if (e != cudaSuccess)
        return set_error(RRSPH_ERR_CUDA, std::string("rrsph_sort_pairs_noalloc: an earlier CUDA error is pending: ") +
                                             cudaGetErrorString(e));
    rrsph::radix_sort_pairs_into(keys_in, ids_in, keys_out, ids_out, base, base + kMaxPairs, base + 2 * (size_t)kMaxPairs,
                                 n, (int)key_bits, static_cast<cudaStream_t>(stream), nullptr);
    e = cudaGetLastError();  // this call's own launches
    if (e != cudaSuccess)
        return set_error(RRSPH_ERR_CUDA, std::string("rrsph_sort_pairs_noalloc: launch: ") + cudaGetErrorString(e));
    return RRSPH_OK;
}
