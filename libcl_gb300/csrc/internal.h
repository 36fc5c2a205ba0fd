// internal.h -- declarations shared by the library's translation units (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/gbsph.h"

namespace gbsph {

// Bits of the per-handle device error word (uint32 in device memory). Kernels set bits
// with atomicOr and keep going (or return); the host reads the word in *_sync_status.
enum : uint32_t {
    DEV_ERR_LOOKBACK_TIMEOUT = 1u,  // decoupled look-back spin hit its limit
    DEV_ERR_MBAR_TIMEOUT = 2u,      // bulk-copy mbarrier wait hit its limit
    DEV_ERR_KEY_RANGE = 4u,         // a key fell outside its cell table
    DEV_ERR_CAPACITY = 8u,          // a fixed-capacity list overflowed
    DEV_ERR_GRID_TIMEOUT = 16u      // a persistent kernel's grid-wide barrier wait hit its limit
};

int dev_err_to_status(uint32_t bits);

// Logging through the optional sink set by gbsph_set_logger.
void log_msg(int level, const std::string& msg);

// Records `msg` as the handle's last error, logs it, returns `status`.
int fail(std::string* last_error, int status, const std::string& msg);

// Wraps a CUDA call: on failure records the error string and returns GBSPH_ERR_CUDA.
#define GBSPH_CUDA_TRY(last_error_ptr, expr)                                              \
    do {                                                                                  \
        cudaError_t _e = (expr);                                                          \
        if (_e != cudaSuccess)                                                            \
            return ::gbsph::fail((last_error_ptr), GBSPH_ERR_CUDA,                        \
                                 std::string(#expr) + ": " + cudaGetErrorString(_e));     \
    } while (0)

// --------------------------------------------------------------------------------------
// One-sweep LSD radix sort (radix_sort.cu).
//
// Scratch layout (device, zeroed by onesweep_prepare before every sort):
//   [0, 4096)       uint32 hist[4][256]   global digit counts of every pass
//   [4096, 4112)    uint32 tile_counter[4]
//   [4112, 4352)    uint32 user counters (fluid: brick count, work counters)
//   [4352, ...)     uint32 status[passes][tiles][256]  look-back words
// --------------------------------------------------------------------------------------
constexpr int SORT_RADIX_BITS = 8;
constexpr int SORT_RADIX = 1 << SORT_RADIX_BITS;
constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 16;                              // keys per thread in the largest tile
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;        // largest tile (4096 keys)
constexpr int SORT_MIN_TILE = SORT_THREADS * 4;             // smallest tile (1024 keys): sizes the look-back words
constexpr int SORT_MAX_PASSES = 4;
constexpr size_t SORT_HEADER_BYTES = 4352;
constexpr size_t SORT_USER_COUNTER_OFFSET = 4112;  // 60 uint32 free for callers
constexpr uint32_t SORT_MAX_KEYS = (1u << 30) - 1u;

// Passes of a sort on bits [start_bit, end_bit) with `digit`-bit digits (1 to 8).
__host__ __device__ inline int sort_passes(int start_bit, int end_bit, int digit = SORT_RADIX_BITS) {
    return (end_bit - start_bit + digit - 1) / digit;
}
__host__ __device__ inline uint32_t sort_tiles(uint32_t n, uint32_t tile = SORT_MIN_TILE) { return (n + tile - 1) / tile; }
// Keys per thread of a pass over n keys: small sorts use small tiles (more tiles in flight,
// shorter per-tile latency), large ones the largest tile (fewer look-back steps).
inline int sort_items_for(uint32_t n) { return n <= (1u << 21) ? 8 : 16; }
size_t onesweep_scratch_bytes(uint32_t n, int passes);

// Optional gather fused into the last pass: dst[k][dest] = src[k][value] for k < n_gather.
struct SortGather {
    const float4* src[2] = {nullptr, nullptr};
    float4* dst[2] = {nullptr, nullptr};
    int n_gather = 0;
};

struct OnesweepArgs {
    const uint32_t* keys_in = nullptr;
    const uint32_t* vals_in = nullptr;  // nullptr: values are 0..n-1
    uint32_t* keys_out = nullptr;        // final sorted keys
    uint32_t* vals_out = nullptr;        // final sorted values
    uint32_t* tmp_keys[2] = {nullptr, nullptr};  // ping-pong for intermediate passes
    uint32_t* tmp_vals[2] = {nullptr, nullptr};
    uint32_t n = 0;
    int start_bit = 0, end_bit = 32;
    void* scratch = nullptr;
    uint32_t* err = nullptr;
    SortGather gather;
    cudaEvent_t before_last = nullptr;  // if set: the last pass waits for it (its gather's inputs)
    int digit_bits = SORT_RADIX_BITS;   // bits per pass (1 to 8, at most SORT_MAX_PASSES passes)
    int items = 0;                      // keys per thread of a tile (8 or 16); 0: by key count
};

// Zeroes the scratch header and the look-back words.
cudaError_t onesweep_prepare(void* scratch, uint32_t n, int passes, cudaStream_t s);
// Zeroes only the tile counters and look-back words (keeps the histogram), so that the
// passes can be re-run on the same keys.
cudaError_t onesweep_reset_progress(void* scratch, uint32_t n, int passes, cudaStream_t s);
// Histogram of every pass's digit (not needed when the caller's kernel filled hist).
cudaError_t onesweep_histogram(const uint32_t* keys, uint32_t n, int start_bit, int end_bit,
                               void* scratch, cudaStream_t s);
// The passes. keys_in may alias tmp_keys[1] (never keys_out unless passes are even...);
// the caller guarantees keys_in/keys_out/tmp buffers do not overlap one pass's in/out.
cudaError_t onesweep_passes(const OnesweepArgs& a, cudaStream_t s);

// fill + clFindBounds into two uint32 tables (radix_sort.cu).
cudaError_t cell_bounds_launch(const uint32_t* sorted_keys, uint32_t n, uint32_t* cell_start,
                               uint32_t* cell_end, uint32_t n_cells, uint32_t* err,
                               cudaStream_t s);

int num_sms();

}  // namespace gbsph
