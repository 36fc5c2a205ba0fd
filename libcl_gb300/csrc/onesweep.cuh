// onesweep.cuh -- one tile of a one-sweep radix-sort pass, as a device function shared by the
// sort's pass kernel (radix_sort.cu, one tile per CTA) and the batched step's persistent
// kernel (batch3d.cu, CTAs loop over tiles). The algorithm is described in radix_sort.cu.
#pragma once

#include "device.cuh"
#include "internal.h"

namespace gbsph {

constexpr uint32_t FLAG_AGG = 1u << 30;
constexpr uint32_t FLAG_PREFIX = 2u << 30;
constexpr uint32_t COUNT_MASK = (1u << 30) - 1u;
constexpr int SORT_WARPS = SORT_THREADS / 32;

static_assert(SORT_THREADS == SORT_RADIX, "one thread per digit in the per-digit phases");

// Exclusive scan of one value per thread over a 256-thread block. `s_tmp` holds 8 words.
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* s_tmp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_tmp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = lane < SORT_WARPS ? s_tmp[lane] : 0u;
        uint32_t incl = w;
#pragma unroll
        for (int o = 1; o < SORT_WARPS; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane < SORT_WARPS) s_tmp[lane] = incl - w;
    }
    __syncthreads();
    uint32_t r = x - v + s_tmp[warp];
    __syncthreads();  // s_tmp may be reused by the caller
    return r;
}

// Shared memory of one tile (ITEMS keys per thread): the keys and values of the tile, the
// per-warp digit counts, the digits' output bases, scan scratch and the tile id.
struct OnesweepSmem {
    uint32_t* keys;   // [SORT_THREADS * ITEMS]
    uint32_t* vals;   // [SORT_THREADS * ITEMS]
    uint32_t* whist;  // [SORT_WARPS * SORT_RADIX]
    uint32_t* base;   // [SORT_RADIX]
    uint32_t* tmp;    // [SORT_WARPS]
    uint32_t* tile;   // [1]
};

__host__ __device__ constexpr size_t onesweep_smem_words(int items) {
    return (size_t)2 * SORT_THREADS * items + SORT_WARPS * SORT_RADIX + SORT_RADIX + SORT_WARPS + 4;
}

// Carves an OnesweepSmem out of `w` (onesweep_smem_words(ITEMS) words, 16-byte aligned).
template <int ITEMS>
__device__ __forceinline__ OnesweepSmem onesweep_smem(uint32_t* w) {
    OnesweepSmem sm;
    sm.keys = w;
    sm.vals = w + SORT_THREADS * ITEMS;
    sm.whist = sm.vals + SORT_THREADS * ITEMS;
    sm.base = sm.whist + SORT_WARPS * SORT_RADIX;
    sm.tmp = sm.base + SORT_RADIX;
    sm.tile = sm.tmp + SORT_WARPS;
    return sm;
}

// Takes the pass's next tile (an atomic counter in the scratch) and sorts it into place;
// returns false, without touching anything, when every tile of the pass has been taken.
// The digit is `bits` (1..8) wide. COH: keys, values and histogram were written earlier in
// the same launch (a persistent kernel's previous phase), so they are read through L2 only.
template <bool IOTA, int NGATHER, int ITEMS, bool COH = false>
__device__ __forceinline__ bool onesweep_tile(const OnesweepSmem& sm, const uint32_t* __restrict__ keys_in,
                                              const uint32_t* __restrict__ vals_in, uint32_t* __restrict__ keys_out,
                                              uint32_t* __restrict__ vals_out, uint32_t n, int shift, int bits,
                                              int pass, uint32_t tiles, uint32_t* __restrict__ scratch, uint32_t* err,
                                              const SortGather& gather) {
    static_assert(ITEMS % 2 == 0, "ranks are packed two per register");
    constexpr int TILE = SORT_THREADS * ITEMS;
    uint32_t* s_keys = sm.keys;
    uint32_t* s_vals = sm.vals;
    uint32_t* s_whist = sm.whist;
    uint32_t* s_base = sm.base;
    uint32_t* s_tmp = sm.tmp;

    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t* hist = scratch + pass * SORT_RADIX;
    uint32_t* counter = scratch + 4096 / 4 + pass;
    uint32_t* status = scratch + SORT_HEADER_BYTES / 4 + (size_t)pass * tiles * SORT_RADIX;

    if (t == 0) *sm.tile = atomicAdd(counter, 1u);
    for (int i = t; i < SORT_WARPS * SORT_RADIX; i += SORT_THREADS) s_whist[i] = 0;
    __syncthreads();
    const uint32_t tile = *sm.tile;
    if (tile >= tiles) return false;  // every tile of the pass is taken
    const uint32_t base = tile * TILE;
    const uint32_t mask = (1u << bits) - 1u;

    // Load: warp-striped, so item order inside the tile is (warp, i, lane) == index order.
    // The keys wait in the value half of the tile buffer (each warp its own slice) until the
    // scatter, which keeps the register count low enough for five CTAs per SM.
    uint32_t* stash = s_vals + warp * 32 * ITEMS + lane;
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const uint32_t idx = base + (uint32_t)(warp * 32 * ITEMS + i * 32 + lane);
        stash[i * 32] = idx < n ? ld_phase<COH>(keys_in + idx) : 0xFFFFFFFFu;  // padding sorts last in the top digit
    }
    __syncwarp();

    // Rank within the warp: peers of equal digit = AND over the digit's bits of the ballot or
    // its complement (digits narrower than 8 bits have zero high bits, whose ballots are
    // empty and leave the mask alone). All peers read the warp's digit counter, then the
    // lowest peer advances it. Ranks are < 2^16 and stored two per register.
    uint32_t* wh = s_whist + warp * SORT_RADIX;
    const uint32_t lt = lanemask_lt();
    uint32_t r[ITEMS / 2];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const uint32_t d = (stash[i * 32] >> shift) & mask;
        uint32_t peers = 0xffffffffu;
#pragma unroll
        for (int b = 0; b < SORT_RADIX_BITS; ++b) {
            const uint32_t bit = (d >> b) & 1u;
            peers &= __ballot_sync(0xffffffffu, bit) ^ (bit - 1u);
        }
        const uint32_t old = wh[d];
        __syncwarp();
        if ((uint32_t)lane == __ffs(peers) - 1u) wh[d] = old + __popc(peers);
        const uint32_t rank = old + __popc(peers & lt);
        r[i >> 1] = (i & 1) ? (r[i >> 1] | rank << 16) : rank;
        __syncwarp();
    }
    __syncthreads();

    // Thread t owns digit t: tile count, then each warp's start of digit t inside the tile
    // (tile-local start + the counts of the warps before it).
    uint32_t cnt = 0;
#pragma unroll
    for (int w = 0; w < SORT_WARPS; ++w) {
        const uint32_t c = s_whist[w * SORT_RADIX + t];
        s_whist[w * SORT_RADIX + t] = cnt;
        cnt += c;
    }
    const uint32_t tstart = block_exclusive_scan(cnt, s_tmp);
#pragma unroll
    for (int w = 0; w < SORT_WARPS; ++w) s_whist[w * SORT_RADIX + t] += tstart;
    const uint32_t goff = block_exclusive_scan(ld_phase<COH>(hist + t), s_tmp);

    // Decoupled look-back for digit t.
    uint32_t excl = 0;
    if (tile == 0) {
        st_relaxed_gpu(&status[t], FLAG_PREFIX | cnt);
    } else {
        st_relaxed_gpu(&status[(size_t)tile * SORT_RADIX + t], FLAG_AGG | cnt);
        int pred = (int)tile - 1;
        WaitBudget budget;
        while (pred >= 0) {
            const uint32_t s = ld_relaxed_gpu(&status[(size_t)pred * SORT_RADIX + t]);
            if ((s & ~COUNT_MASK) == 0u) {
                if (budget.expired()) {
                    atomicOr(err, DEV_ERR_LOOKBACK_TIMEOUT);
                    break;
                }
                continue;
            }
            excl += s & COUNT_MASK;
            if (s & FLAG_PREFIX) break;
            --pred;
        }
        st_relaxed_gpu(&status[(size_t)tile * SORT_RADIX + t], FLAG_PREFIX | ((excl + cnt) & COUNT_MASK));
    }
    s_base[t] = goff + excl - tstart;
    uint32_t k[ITEMS];
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) k[i] = stash[i * 32];
    __syncthreads();

    // Tile-local sorted order in shared memory; values are read here, after the ranking.
#pragma unroll
    for (int i = 0; i < ITEMS; ++i) {
        const uint32_t idx = base + (uint32_t)(warp * 32 * ITEMS + i * 32 + lane);
        const uint32_t pos = s_whist[warp * SORT_RADIX + ((k[i] >> shift) & mask)] + ((r[i >> 1] >> (16 * (i & 1))) & 0xffffu);
        s_keys[pos] = k[i];
        s_vals[pos] = IOTA ? idx : (idx < n ? ld_phase<COH>(vals_in + idx) : 0u);
    }
    __syncthreads();

    // Each digit's run goes to one contiguous range of the output.
    const uint32_t valid = min((uint32_t)TILE, n - base);
#pragma unroll 4
    for (int i = 0; i < ITEMS; ++i) {
        const uint32_t j = (uint32_t)(i * SORT_THREADS + t);
        if (j < valid) {
            const uint32_t key = s_keys[j], val = s_vals[j];
            const uint32_t dst = s_base[(key >> shift) & mask] + j;
            if (dst >= n) {  // histogram inconsistent with the keys (misuse): never write out of range
                atomicOr(err, DEV_ERR_KEY_RANGE);
                continue;
            }
            keys_out[dst] = key;
            vals_out[dst] = val;
            if (NGATHER > 0) gather.dst[0][dst] = __ldg(gather.src[0] + val);
            if (NGATHER > 1) gather.dst[1][dst] = __ldg(gather.src[1] + val);
        }
    }
    __syncthreads();  // the tile buffers are free for the caller's next tile
    return true;
}

}  // namespace gbsph
