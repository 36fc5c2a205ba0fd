// radix_sort.cu -- stable LSD radix sort of (uint32 key, uint32 value) pairs for sm_103a.
//
// Replaces libCL's oclRadixSort (libCL/sort/oclRadixSort.cpp:62-144,
// libCL/sort/oclRadixSort.cl:20-222): same contract (stable sort on key bits
// [start_bit, end_bit), in place, counts must match, bit range a multiple of 4), different
// algorithm. The reference runs 4-bit passes of four kernels each, with single-thread serial
// prefix sums. Here every 8-bit digit is one "one-sweep" pass:
//   * one histogram kernel counts the digits of every pass in a single read of the keys;
//   * each pass kernel takes a tile of 4096 keys (tile id from an atomic counter, so tiles
//     are started in order and the look-back always waits on running CTAs), ranks keys
//     inside each warp with warp ballots (peers of the same digit = AND of 8 ballots),
//     combines the warps' counts, publishes the tile's per-digit count, and finds the
//     exclusive prefix over earlier tiles by decoupled look-back on 32-bit status words
//     (2 flag bits + 30 count bits). The look-back spin is bounded: on timeout the kernel
//     sets an error bit, publishes anyway (so later tiles never hang) and finishes.
//   * keys are scattered through shared memory so each digit's run is written contiguously.
// The last pass can gather float4 payloads by the sorted value (the fluid's reorder stage).
#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>

#include "device.cuh"
#include "grid_sync.cuh"
#include "internal.h"
#include "onesweep.cuh"

namespace gbsph {
namespace {

__global__ void __launch_bounds__(512) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n,
                                                   int start_bit, int end_bit,
                                                   uint32_t* __restrict__ hist) {
    __shared__ uint32_t s_h[SORT_MAX_PASSES * SORT_RADIX];
    for (int i = threadIdx.x; i < SORT_MAX_PASSES * SORT_RADIX; i += blockDim.x) s_h[i] = 0;
    __syncthreads();
    const int passes = sort_passes(start_bit, end_bit);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = __ldg(keys + i);
        for (int p = 0; p < passes; ++p) {
            const int shift = start_bit + p * SORT_RADIX_BITS;
            const int bits = min(SORT_RADIX_BITS, end_bit - shift);
            atomicAdd(&s_h[p * SORT_RADIX + ((k >> shift) & ((1u << bits) - 1u))], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * SORT_RADIX; i += blockDim.x)
        if (s_h[i]) atomicAdd(&hist[i], s_h[i]);
}

// Resident CTAs per SM the register budget is set for: shared memory caps a 4096-key tile at
// five (42 KB each), a 2048-key tile fits six at 40 registers without spills.
constexpr int onesweep_min_blocks(int items) { return items == 16 ? 5 : 6; }

template <bool IOTA, int NGATHER, int ITEMS>
__global__ void __launch_bounds__(SORT_THREADS, onesweep_min_blocks(ITEMS)) k_onesweep(
    const uint32_t* __restrict__ keys_in, const uint32_t* __restrict__ vals_in,
    uint32_t* __restrict__ keys_out, uint32_t* __restrict__ vals_out, uint32_t n, int shift,
    int bits, int pass, uint32_t tiles, uint32_t* __restrict__ scratch, uint32_t* err,
    SortGather gather) {
    __shared__ __align__(16) uint32_t s_w[onesweep_smem_words(ITEMS)];
    const OnesweepSmem sm = onesweep_smem<ITEMS>(s_w);
    if (!onesweep_tile<IOTA, NGATHER, ITEMS>(sm, keys_in, vals_in, keys_out, vals_out, n, shift, bits, pass, tiles,
                                             scratch, err, gather)) {
        // counter not reset since the last sort: refuse rather than overrun
        if (threadIdx.x == 0) atomicOr(err, DEV_ERR_CAPACITY);
    }
}

__global__ void k_cell_bounds(const uint32_t* __restrict__ keys, uint32_t n,
                              uint32_t* __restrict__ cs, uint32_t* __restrict__ ce,
                              uint32_t n_cells, uint32_t* err) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t k = keys[i];
    if (k >= n_cells) {
        atomicOr(err, DEV_ERR_KEY_RANGE);
        return;
    }
    if (i == 0) {
        cs[k] = 0;
    } else {
        const uint32_t prev = keys[i - 1];
        if (prev != k) {
            cs[k] = i;
            if (prev < n_cells) ce[prev] = i;
        }
    }
    if (i == n - 1) ce[k] = n;
}

template <bool IOTA, int ITEMS>
cudaError_t launch_pass_items(int ngather, const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                              uint32_t* vout, uint32_t n, int shift, int bits, int pass, uint32_t* scratch,
                              uint32_t* err, const SortGather& g, cudaStream_t s) {
    const uint32_t tiles = sort_tiles(n, SORT_THREADS * ITEMS);
    if (ngather == 2)
        k_onesweep<IOTA, 2, ITEMS><<<tiles, SORT_THREADS, 0, s>>>(kin, vin, kout, vout, n, shift, bits, pass, tiles, scratch, err, g);
    else if (ngather == 1)
        k_onesweep<IOTA, 1, ITEMS><<<tiles, SORT_THREADS, 0, s>>>(kin, vin, kout, vout, n, shift, bits, pass, tiles, scratch, err, g);
    else
        k_onesweep<IOTA, 0, ITEMS><<<tiles, SORT_THREADS, 0, s>>>(kin, vin, kout, vout, n, shift, bits, pass, tiles, scratch, err, g);
    return cudaGetLastError();
}

template <bool IOTA>
cudaError_t launch_pass(int ngather, const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                        uint32_t* vout, uint32_t n, int shift, int bits, int pass, uint32_t* scratch,
                        uint32_t* err, const SortGather& g, cudaStream_t s, int items) {
    if (items == 8)
        return launch_pass_items<IOTA, 8>(ngather, kin, vin, kout, vout, n, shift, bits, pass, scratch, err, g, s);
    return launch_pass_items<IOTA, 16>(ngather, kin, vin, kout, vout, n, shift, bits, pass, scratch, err, g, s);
}

// A wait on an mbarrier that expects 16 bytes no copy will deliver: the bounded wait gives up
// and sets DEV_ERR_MBAR_TIMEOUT (failure-detection self-test).
__global__ void k_selftest_mbar(uint32_t* err) {
    __shared__ __align__(8) uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        mbar_arrive_expect_tx(&bar, 16u);
        if (!mbar_wait_bounded(&bar, 0)) atomicOr(err, DEV_ERR_MBAR_TIMEOUT);
    }
}

// Two CTAs at a grid barrier that waits for three: the bounded wait gives up, sets
// DEV_ERR_GRID_TIMEOUT and the abort flag, and both CTAs leave (failure-detection self-test
// of the persistent batch step's barrier).
__global__ void k_selftest_grid(uint32_t* words, uint32_t* err) {
    __shared__ uint32_t s_flag;
    GridSync gs{words, err, 0u, gridDim.x + 1u};
    gs.sync(&s_flag);
}

}  // namespace

int selftest_grid_timeout(cudaStream_t s) {
    uint32_t* words = nullptr;
    if (cudaMalloc(&words, 256) != cudaSuccess) {
        cudaGetLastError();
        return GBSPH_ERR_OUT_OF_MEMORY;
    }
    int rc = GBSPH_OK;
    uint32_t bits = 0;
    uint32_t* err = words + 32;
    if (cudaMemsetAsync(words, 0, 256, s) != cudaSuccess) {
        rc = GBSPH_ERR_CUDA;
    } else {
        k_selftest_grid<<<2, 64, 0, s>>>(words, err);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess ||
            cudaMemcpy(&bits, err, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = GBSPH_ERR_CUDA;
        else
            rc = (bits & DEV_ERR_GRID_TIMEOUT) ? GBSPH_ERR_DEVICE_TIMEOUT : GBSPH_OK;
    }
    cudaFree(words);
    return rc;
}

int selftest_mbarrier_timeout(cudaStream_t s) {
    uint32_t* err = nullptr;
    if (cudaMalloc(&err, 4) != cudaSuccess) {
        cudaGetLastError();
        return GBSPH_ERR_OUT_OF_MEMORY;
    }
    int rc = GBSPH_OK;
    uint32_t bits = 0;
    if (cudaMemsetAsync(err, 0, 4, s) != cudaSuccess) {
        rc = GBSPH_ERR_CUDA;
    } else {
        k_selftest_mbar<<<1, 32, 0, s>>>(err);
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess ||
            cudaMemcpy(&bits, err, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = GBSPH_ERR_CUDA;
        else
            rc = (bits & DEV_ERR_MBAR_TIMEOUT) ? GBSPH_ERR_DEVICE_TIMEOUT : GBSPH_OK;
    }
    cudaFree(err);
    return rc;
}

size_t onesweep_scratch_bytes(uint32_t n, int passes) {
    return SORT_HEADER_BYTES + (size_t)std::max(passes, 1) * sort_tiles(std::max(n, 1u)) * SORT_RADIX * 4;
}

cudaError_t onesweep_prepare(void* scratch, uint32_t n, int passes, cudaStream_t s) {
    return cudaMemsetAsync(scratch, 0, onesweep_scratch_bytes(n, passes), s);
}

cudaError_t onesweep_reset_progress(void* scratch, uint32_t n, int passes, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync((char*)scratch + 4096, 0, 16, s);
    if (e != cudaSuccess) return e;
    return cudaMemsetAsync((char*)scratch + SORT_HEADER_BYTES, 0,
                           onesweep_scratch_bytes(n, passes) - SORT_HEADER_BYTES, s);
}

cudaError_t onesweep_histogram(const uint32_t* keys, uint32_t n, int start_bit, int end_bit,
                               void* scratch, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const int threads = 512;
    int blocks = (int)std::min<uint64_t>(((uint64_t)n + threads * 8 - 1) / (threads * 8), (uint64_t)num_sms() * 4);
    blocks = std::max(blocks, 1);
    k_sort_hist<<<blocks, threads, 0, s>>>(keys, n, start_bit, end_bit, (uint32_t*)scratch);
    return cudaGetLastError();
}

cudaError_t onesweep_passes(const OnesweepArgs& a, cudaStream_t s) {
    const int digit = a.digit_bits;
    if (digit < 1 || digit > SORT_RADIX_BITS) return cudaErrorInvalidValue;
    const int P = sort_passes(a.start_bit, a.end_bit, digit);
    if (a.n == 0 || P == 0) return cudaSuccess;
    if (P > SORT_MAX_PASSES) return cudaErrorInvalidValue;
    const int items = a.items ? a.items : sort_items_for(a.n);
    if (items != 8 && items != 16) return cudaErrorInvalidValue;
    const uint32_t* kin = a.keys_in;
    const uint32_t* vin = a.vals_in;
    for (int p = 0; p < P; ++p) {
        const bool last = p == P - 1;
        uint32_t* kout = last ? a.keys_out : a.tmp_keys[p & 1];
        uint32_t* vout = last ? a.vals_out : a.tmp_vals[p & 1];
        const int shift = a.start_bit + p * digit;
        const int bits = std::min(digit, a.end_bit - shift);
        const int ng = last ? a.gather.n_gather : 0;
        if (last && a.before_last) {
            cudaError_t e = cudaStreamWaitEvent(s, a.before_last, 0);
            if (e != cudaSuccess) return e;
        }
        cudaError_t e = (vin == nullptr)
            ? launch_pass<true>(ng, kin, nullptr, kout, vout, a.n, shift, bits, p, (uint32_t*)a.scratch, a.err, a.gather, s, items)
            : launch_pass<false>(ng, kin, vin, kout, vout, a.n, shift, bits, p, (uint32_t*)a.scratch, a.err, a.gather, s, items);
        if (e != cudaSuccess) return e;
        kin = kout;
        vin = vout;
    }
    return cudaSuccess;
}

cudaError_t cell_bounds_launch(const uint32_t* sorted_keys, uint32_t n, uint32_t* cell_start,
                               uint32_t* cell_end, uint32_t n_cells, uint32_t* err,
                               cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(cell_start, 0xFF, (size_t)n_cells * 4, s);
    if (e != cudaSuccess) return e;
    e = cudaMemsetAsync(cell_end, 0xFF, (size_t)n_cells * 4, s);
    if (e != cudaSuccess || n == 0) return e;
    k_cell_bounds<<<(n + 255) / 256, 256, 0, s>>>(sorted_keys, n, cell_start, cell_end, n_cells, err);
    return cudaGetLastError();
}

}  // namespace gbsph

// ------------------------------------------------------------------------------------------
// C ABI: the oclRadixSort replacement.
// ------------------------------------------------------------------------------------------
struct gbsph_radix_sort_s {
    int device = 0;
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    uint32_t* tmp = nullptr;  // 4 arrays of tmp_cap: keys0, vals0, keys1, vals1
    size_t tmp_cap = 0;
    uint32_t* err = nullptr;
    std::string last_error;
};

using namespace gbsph;

namespace {

int fit_scratch(gbsph_radix_sort_s* h, size_t bytes) {
    if (h->scratch_bytes >= bytes) return GBSPH_OK;
    if (h->scratch) cudaFree(h->scratch);
    h->scratch = nullptr;
    h->scratch_bytes = 0;
    if (cudaMalloc(&h->scratch, bytes) != cudaSuccess)
        return fail(&h->last_error, GBSPH_ERR_OUT_OF_MEMORY, "radix sort: scratch allocation failed");
    h->scratch_bytes = bytes;
    return GBSPH_OK;
}

int fit_tmp(gbsph_radix_sort_s* h, size_t n) {
    if (h->tmp_cap >= n) return GBSPH_OK;
    if (h->tmp) cudaFree(h->tmp);
    h->tmp = nullptr;
    h->tmp_cap = 0;
    if (cudaMalloc(&h->tmp, 4 * n * sizeof(uint32_t)) != cudaSuccess)
        return fail(&h->last_error, GBSPH_ERR_OUT_OF_MEMORY, "radix sort: temporary allocation failed");
    h->tmp_cap = n;
    return GBSPH_OK;
}

}  // namespace

extern "C" {

GBSPH_API int gbsph_radix_sort_create(gbsph_radix_sort_t* out) {
    if (!out) return GBSPH_ERR_ARGUMENT;
    *out = nullptr;
    auto* h = new gbsph_radix_sort_s();
    if (cudaGetDevice(&h->device) != cudaSuccess || cudaMalloc(&h->err, 256) != cudaSuccess ||
        cudaMemset(h->err, 0, 256) != cudaSuccess) {
        cudaGetLastError();
        if (h->err) cudaFree(h->err);
        delete h;
        return GBSPH_ERR_CUDA;
    }
    *out = h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_radix_sort_destroy(gbsph_radix_sort_t h) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    cudaSetDevice(h->device);
    if (h->scratch) cudaFree(h->scratch);
    if (h->tmp) cudaFree(h->tmp);
    if (h->err) cudaFree(h->err);
    delete h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_radix_sort_compute(gbsph_radix_sort_t h, uint32_t* keys, uint32_t* values,
                                       size_t n_keys, size_t n_values, int start_bit,
                                       int end_bit, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    // Checks in the reference's order (libCL/sort/oclRadixSort.cpp:64-80).
    if (n_keys != n_values)
        return fail(&h->last_error, GBSPH_ERR_SIZE_MISMATCH,
                    "key and value arrays are of different size (" + std::to_string(n_keys) + "," +
                        std::to_string(n_values) + ")");
    if (n_keys > SORT_MAX_KEYS - SORT_TILE)
        return fail(&h->last_error, GBSPH_ERR_TOO_LARGE,
                    "maximum sortable array size = " + std::to_string(SORT_MAX_KEYS - SORT_TILE));
    if (start_bit < 0 || end_bit > 32 || end_bit < start_bit || (end_bit - start_bit) % 4 != 0)
        return fail(&h->last_error, GBSPH_ERR_BIT_RANGE,
                    "end bit(" + std::to_string(end_bit) + ") - start bit(" + std::to_string(start_bit) +
                        ") must be divisible by 4");
    if (n_keys == 0 || start_bit == end_bit) return GBSPH_OK;
    if (!keys || !values) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null key or value pointer");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    const uint32_t n = (uint32_t)n_keys;
    const int P = sort_passes(start_bit, end_bit);
    int rc = fit_scratch(h, onesweep_scratch_bytes(n, P));
    if (rc) return rc;
    rc = fit_tmp(h, n);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    GBSPH_CUDA_TRY(&h->last_error, onesweep_prepare(h->scratch, n, P, s));
    GBSPH_CUDA_TRY(&h->last_error, onesweep_histogram(keys, n, start_bit, end_bit, h->scratch, s));
    OnesweepArgs a;
    a.keys_in = keys;
    a.vals_in = values;
    a.tmp_keys[0] = h->tmp;
    a.tmp_vals[0] = h->tmp + h->tmp_cap;
    a.tmp_keys[1] = h->tmp + 2 * h->tmp_cap;
    a.tmp_vals[1] = h->tmp + 3 * h->tmp_cap;
    a.n = n;
    a.start_bit = start_bit;
    a.end_bit = end_bit;
    a.scratch = h->scratch;
    a.err = h->err;
    if (P == 1) {  // single pass cannot be in place: sort into tmp, copy back
        a.keys_out = a.tmp_keys[0];
        a.vals_out = a.tmp_vals[0];
        GBSPH_CUDA_TRY(&h->last_error, onesweep_passes(a, s));
        GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(keys, a.keys_out, n * 4ull, cudaMemcpyDeviceToDevice, s));
        GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(values, a.vals_out, n * 4ull, cudaMemcpyDeviceToDevice, s));
    } else {  // keys -> T0 -> T1 -> ... -> keys: the input is free after pass 0
        a.keys_out = keys;
        a.vals_out = values;
        GBSPH_CUDA_TRY(&h->last_error, onesweep_passes(a, s));
    }
    return GBSPH_OK;
}

GBSPH_API int gbsph_radix_sort_cell_bounds(gbsph_radix_sort_t h, const uint32_t* sorted_keys,
                                           size_t n, uint32_t* cell_start, uint32_t* cell_end,
                                           size_t n_cells, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!cell_start || !cell_end || (n && !sorted_keys))
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null pointer");
    if (n > 0xFFFFFFFEull || n_cells > 0xFFFFFFFFull)
        return fail(&h->last_error, GBSPH_ERR_TOO_LARGE, "cell bounds: n or n_cells too large");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cell_bounds_launch(sorted_keys, (uint32_t)n, cell_start, cell_end,
                                                      (uint32_t)n_cells, h->err, (cudaStream_t)stream));
    return GBSPH_OK;
}

GBSPH_API int gbsph_radix_sort_sync_status(gbsph_radix_sort_t h, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t bits = 0;
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpy(&bits, h->err, 4, cudaMemcpyDeviceToHost));
    if (bits) {
        GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->err, 0, 4));
        return fail(&h->last_error, dev_err_to_status(bits),
                    "device error word 0x" + std::to_string(bits));
    }
    return GBSPH_OK;
}

int selftest_noalloc_timeout(cudaStream_t s);  // below, beside the static scratch array

GBSPH_API int gbsph_selftest_bounded_wait(int which, void* stream) {
    if (which < 0 || which > 3) return GBSPH_ERR_ARGUMENT;
    cudaStream_t s = (cudaStream_t)stream;
    if (which == 1) return selftest_mbarrier_timeout(s);
    if (which == 3) return selftest_grid_timeout(s);
    if (which == 2) return selftest_noalloc_timeout(s);
    // Two tiles of 2048 keys; the pass's tile counter starts at 1, so tile 0 never runs, the
    // CTA that draws tile 1 looks back at tile 0's unwritten status until its bound expires,
    // and the CTA that draws tile 2 finds no tile (a capacity error). The outputs stay inside
    // the buffers: with an all-zero histogram every destination is a tile-local position.
    constexpr int ITEMS = 8;
    const uint32_t n = 2 * SORT_THREADS * ITEMS, tiles = 2;
    const size_t scratch_bytes = SORT_HEADER_BYTES + (size_t)tiles * SORT_RADIX * 4;
    char* block = nullptr;
    const size_t bytes = scratch_bytes + 4 * (size_t)n * 4 + 256;
    if (cudaMalloc(&block, bytes) != cudaSuccess) {
        cudaGetLastError();
        return GBSPH_ERR_OUT_OF_MEMORY;
    }
    int rc = GBSPH_OK;
    uint32_t* scratch = (uint32_t*)block;
    uint32_t* keys = (uint32_t*)(block + scratch_bytes);
    uint32_t* kout = keys + n;
    uint32_t* vout = kout + n;
    uint32_t* err = vout + n;
    const uint32_t one = 1;
    SortGather g{};
    if (cudaMemsetAsync(block, 0, bytes, s) != cudaSuccess ||
        cudaMemcpyAsync(scratch + 4096 / 4, &one, 4, cudaMemcpyHostToDevice, s) != cudaSuccess) {
        rc = GBSPH_ERR_CUDA;
    } else {
        k_onesweep<true, 0, ITEMS><<<tiles, SORT_THREADS, 0, s>>>(keys, nullptr, kout, vout, n, 0, 8, 0, tiles, scratch,
                                                                  err, g);
        uint32_t bits = 0;
        if (cudaGetLastError() != cudaSuccess || cudaStreamSynchronize(s) != cudaSuccess ||
            cudaMemcpy(&bits, err, 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = GBSPH_ERR_CUDA;
        else
            rc = (bits & DEV_ERR_LOOKBACK_TIMEOUT) ? GBSPH_ERR_DEVICE_TIMEOUT : GBSPH_OK;
    }
    cudaFree(block);
    return rc;
}

GBSPH_API const char* gbsph_radix_sort_last_error(gbsph_radix_sort_t h) {
    return h ? h->last_error.c_str() : "null handle";
}

}  // extern "C"

// ------------------------------------------------------------------------------------------
// Allocation-free variant of gbsph_radix_sort_compute.
//
// Some callers cannot call cudaMalloc: code that runs while a host framework owns all device
// memory through its own fixed-budget allocator, real-time loops where cudaMalloc/cudaFree
// would stall on an implicit device synchronisation, and plugins that must not change the
// device's memory footprint after start-up. gbsph_radix_sort_noalloc serves them: its
// scratch (histograms, tile counters, look-back words and the two ping-pong key/value pairs)
// lives in the file-scope device array below, which every GPU that loads this library holds
// until the process exits. The array's host-side name is only a stand-in for the symbol, so
// its device address is looked up per device with cudaGetSymbolAddress.
// ------------------------------------------------------------------------------------------
namespace {

constexpr uint32_t NOALLOC_MAX_KEYS = 262144;  // 2^18 pairs
constexpr size_t NOALLOC_STATUS_BYTES = (size_t)SORT_MAX_PASSES * ((NOALLOC_MAX_KEYS + SORT_MIN_TILE - 1) / SORT_MIN_TILE) * SORT_RADIX * 4;
constexpr size_t NOALLOC_ERR_OFFSET = SORT_HEADER_BYTES + NOALLOC_STATUS_BYTES;  // one uint32 (256 B slot)
constexpr size_t NOALLOC_TMP_OFFSET = NOALLOC_ERR_OFFSET + 256;
constexpr size_t NOALLOC_BYTES = NOALLOC_TMP_OFFSET + 4ull * NOALLOC_MAX_KEYS * sizeof(uint32_t);  // ~5 MB
static_assert(SORT_HEADER_BYTES % 256 == 0 && NOALLOC_ERR_OFFSET % 256 == 0, "256-byte aligned regions");

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mutex;
void* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of g_noalloc_scratch on the current device, looked up once per device (the
// first call on a device does the lookup; a cudaDeviceReset later in the process would leave
// the stored address stale, so the no-alloc entry points do not support one).
cudaError_t noalloc_scratch(int device, void** out) {
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_ptr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[device] = p;
    }
    *out = g_noalloc_ptr[device];
    return cudaSuccess;
}

// The current device's scratch address (looked up on first use), or a status code.
int noalloc_base(char** base) {
    int device = 0;
    GBSPH_CUDA_TRY(nullptr, cudaGetDevice(&device));
    if (device < 0 || device >= NOALLOC_MAX_DEVICES)
        return fail(nullptr, GBSPH_ERR_ARGUMENT, "noalloc sort: device ordinal too large");
    void* p = nullptr;
    GBSPH_CUDA_TRY(nullptr, noalloc_scratch(device, &p));
    *base = (char*)p;
    return GBSPH_OK;
}

}  // namespace

// gbsph_selftest_bounded_wait(2): selftest (0)'s timed-out pass run inside the static scratch
// array (two 2048-key tiles whose keys, outputs, histogram and look-back words all lie in the
// array), recording the timeout in the array's error word, where
// gbsph_radix_sort_noalloc_status finds it. Asynchronous on `s`; allocates nothing.
int selftest_noalloc_timeout(cudaStream_t s) {
    char* b = nullptr;
    int rc = noalloc_base(&b);
    if (rc) return rc;
    constexpr int ITEMS = 8;
    const uint32_t n = 2 * SORT_THREADS * ITEMS, tiles = 2;
    static_assert(2 * SORT_THREADS * 8 * 3 <= 4 * NOALLOC_MAX_KEYS, "selftest keys fit the array");
    uint32_t* scratch = (uint32_t*)b;
    uint32_t* keys = (uint32_t*)(b + NOALLOC_TMP_OFFSET);
    uint32_t* kout = keys + n;
    uint32_t* vout = kout + n;
    uint32_t* err = (uint32_t*)(b + NOALLOC_ERR_OFFSET);
    static const uint32_t one = 1;
    SortGather g{};
    GBSPH_CUDA_TRY(nullptr, cudaMemsetAsync(b, 0, SORT_HEADER_BYTES + (size_t)tiles * SORT_RADIX * 4, s));
    GBSPH_CUDA_TRY(nullptr, cudaMemsetAsync(keys, 0, 3ull * n * 4, s));
    GBSPH_CUDA_TRY(nullptr, cudaMemcpyAsync(scratch + 4096 / 4, &one, 4, cudaMemcpyHostToDevice, s));
    k_onesweep<true, 0, ITEMS><<<tiles, SORT_THREADS, 0, s>>>(keys, nullptr, kout, vout, n, 0, 8, 0, tiles, scratch, err,
                                                              g);
    GBSPH_CUDA_TRY(nullptr, cudaGetLastError());
    return GBSPH_OK;
}

extern "C" {

// Same contract as gbsph_radix_sort_compute (stable LSD sort of (key, value) pairs on key
// bits [start_bit, end_bit), in place, on `stream`), but no device memory is allocated:
// * n_keys may not exceed 262,144 (GBSPH_ERR_TOO_LARGE otherwise);
// * the first call on a device looks up the scratch array's device address, so make that
//   first call before any stream capture begins;
// * every call on a device shares the one scratch array and the call clears it with
//   cudaMemsetAsync on `stream`; calls that overlap on the GPU (different streams without
//   ordering between them) race on it and must not be issued;
// * a device-side fault of the sort (a look-back wait that ran out, a tile-capacity error)
//   leaves the output undefined and sets a bit in the array's error word, which stays set
//   across calls until gbsph_radix_sort_noalloc_status reads and clears it.
GBSPH_API int gbsph_radix_sort_noalloc(uint32_t* keys, uint32_t* values, size_t n_keys, size_t n_values,
                                       int start_bit, int end_bit, void* stream) {
    if (n_keys != n_values) return fail(nullptr, GBSPH_ERR_SIZE_MISMATCH, "noalloc sort: key and value counts differ");
    if (n_keys > NOALLOC_MAX_KEYS)
        return fail(nullptr, GBSPH_ERR_TOO_LARGE,
                    "noalloc sort: " + std::to_string(n_keys) + " pairs exceed its limit of " +
                        std::to_string(NOALLOC_MAX_KEYS));
    if (start_bit < 0 || end_bit > 32 || end_bit < start_bit || (end_bit - start_bit) % 4 != 0)
        return fail(nullptr, GBSPH_ERR_BIT_RANGE, "noalloc sort: bit range must be a multiple of 4 within [0, 32]");
    if (n_keys == 0 || start_bit == end_bit) return GBSPH_OK;
    if (!keys || !values) return fail(nullptr, GBSPH_ERR_ARGUMENT, "noalloc sort: null key or value pointer");
    char* b = nullptr;
    int rc = noalloc_base(&b);
    if (rc) return rc;
    const uint32_t n = (uint32_t)n_keys;
    const int P = sort_passes(start_bit, end_bit);
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* err = (uint32_t*)(b + NOALLOC_ERR_OFFSET);
    uint32_t* tmp = (uint32_t*)(b + NOALLOC_TMP_OFFSET);
    GBSPH_CUDA_TRY(nullptr, onesweep_prepare(b, n, P, s));  // histogram, counters, look-back words
    GBSPH_CUDA_TRY(nullptr, onesweep_histogram(keys, n, start_bit, end_bit, b, s));
    OnesweepArgs a;
    a.keys_in = keys;
    a.vals_in = values;
    a.tmp_keys[0] = tmp;
    a.tmp_vals[0] = tmp + NOALLOC_MAX_KEYS;
    a.tmp_keys[1] = tmp + 2 * NOALLOC_MAX_KEYS;
    a.tmp_vals[1] = tmp + 3 * NOALLOC_MAX_KEYS;
    a.n = n;
    a.start_bit = start_bit;
    a.end_bit = end_bit;
    a.scratch = b;
    a.err = err;
    if (P == 1) {
        a.keys_out = a.tmp_keys[0];
        a.vals_out = a.tmp_vals[0];
        GBSPH_CUDA_TRY(nullptr, onesweep_passes(a, s));
        GBSPH_CUDA_TRY(nullptr, cudaMemcpyAsync(keys, a.keys_out, n * 4ull, cudaMemcpyDeviceToDevice, s));
        GBSPH_CUDA_TRY(nullptr, cudaMemcpyAsync(values, a.vals_out, n * 4ull, cudaMemcpyDeviceToDevice, s));
    } else {
        a.keys_out = keys;
        a.vals_out = values;
        GBSPH_CUDA_TRY(nullptr, onesweep_passes(a, s));
    }
    return GBSPH_OK;
}

// Synchronises `stream`, then reads the static array's error word: GBSPH_OK when no no-alloc
// sort on this device has recorded a device-side fault since the last read, else the fault's
// status (GBSPH_ERR_DEVICE_TIMEOUT for a look-back wait that ran out, GBSPH_ERR_STATE for a
// tile-capacity error), after which the word is cleared. Allocates nothing; like the sort, the
// first call on a device looks up the array's address.
GBSPH_API int gbsph_radix_sort_noalloc_status(void* stream) {
    char* b = nullptr;
    int rc = noalloc_base(&b);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* err = (uint32_t*)(b + NOALLOC_ERR_OFFSET);
    GBSPH_CUDA_TRY(nullptr, cudaStreamSynchronize(s));
    uint32_t bits = 0;
    GBSPH_CUDA_TRY(nullptr, cudaMemcpy(&bits, err, 4, cudaMemcpyDeviceToHost));
    if (!bits) return GBSPH_OK;
    GBSPH_CUDA_TRY(nullptr, cudaMemsetAsync(err, 0, 4, s));
    GBSPH_CUDA_TRY(nullptr, cudaStreamSynchronize(s));
    return fail(nullptr, dev_err_to_status(bits), "noalloc sort: device error word 0x" + std::to_string(bits));
}

}  // extern "C"
