// grid_sync.cuh -- bounded grid-wide barrier for persistent (cooperative) kernels.
#pragma once

#include "device.cuh"
#include "internal.h"

namespace gbsph {

// Grid-wide barrier of a cooperative launch (every CTA resident). It uses three words of
// device memory, zeroed before the launch: arrivals (counting up over the launch), the number
// of the last barrier that every CTA reached, and an abort flag. Thread 0 of each CTA arrives
// and waits; the other threads wait at the CTA barrier behind it. The wait is bounded: a CTA
// that gives up sets DEV_ERR_GRID_TIMEOUT and the abort flag, and every CTA that gives up or
// sees the flag gets false and is expected to leave the kernel, so the others leave at their
// next barrier.
//
// Memory: thread 0's fences around the arrival make the CTA's writes before the barrier
// visible to every CTA after it (plain loads; loads of lines an earlier phase may have left
// in L1 or the read-only cache go through ld_phase<true>). The proxy fences order the writes
// with bulk copies (async proxy) that read them after the barrier.
struct GridSync {
    uint32_t* w;     // [0] arrivals, [1] barriers completed, [2] abort flag
    uint32_t* err;   // device error word
    uint32_t epoch;  // barriers this CTA has passed
    uint32_t ctas;   // CTAs that arrive at each barrier (gridDim.x)

    __device__ __forceinline__ bool sync(uint32_t* s_flag) {
        fence_proxy_async_global();  // this thread's writes, before bulk copies read them
        __syncthreads();
        const uint32_t target = ++epoch;
        if (threadIdx.x == 0) {
            bool ok = true;
            __threadfence();
            const uint32_t arrived = atomicAdd(w, 1u) + 1u;
            if (arrived == target * ctas) {
                st_release_gpu(w + 1, target);
            } else {
                WaitBudget budget;
                while (ld_acquire_gpu(w + 1) < target) {
                    if (ld_relaxed_gpu(w + 2)) {
                        ok = false;
                        break;
                    }
                    if (budget.expired()) {
                        atomicOr(err, DEV_ERR_GRID_TIMEOUT);
                        atomicExch(w + 2, 1u);
                        ok = false;
                        break;
                    }
                }
            }
            __threadfence();
            fence_proxy_async_global();  // bulk copies issued after the barrier see the writes
            if (ld_relaxed_gpu(w + 2)) ok = false;
            *s_flag = ok ? 1u : 0u;
        }
        __syncthreads();
        return *s_flag != 0u;
    }

    // One thread: make every CTA leave at its next barrier.
    __device__ __forceinline__ void abort() { atomicExch(w + 2, 1u); }
};

}  // namespace gbsph
