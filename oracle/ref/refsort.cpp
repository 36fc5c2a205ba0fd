// refsort.cpp -- the reference's radix sort kernels (libCL/sort/oclRadixSort.cl, compiled
// unchanged apart from oracle/ref/rewrite.py's edits) driven as oclRadixSort::compute
// drives them (libCL/sort/oclRadixSort.cpp:62-144).
//
// TEST INFRASTRUCTURE ONLY: the checker of the oracle's restated sort and the reference
// arm's CPU sort. Nothing in the product library links it.
#include <cmath>
#include <cstdint>
#include <vector>

#include "clshim.h"

namespace clc {
namespace ksort {
#include "oclRadixSort.cl.inc"
}  // namespace ksort
}  // namespace clc

namespace {
const int kBits = 4;             // CBITS, libCL/sort/oclRadixSort.cpp:18
const size_t kBlockSize = 256;   // BLOCK_SIZE, :19 (cBlockSize, the local size)
const size_t kMaxArraySize = kBlockSize * kBlockSize * kBlockSize * 4 / (1 << kBits);  // :24
}  // namespace

extern "C" {

// oclRadixSort::compute(dev, key, val, startBit, endBit) on host arrays, in place.
// Returns 0, or the reference's refusals: -3 (n >= cMaxArraySize, :70-74), -4 (bit range
// not a multiple of 4, :76-80). n == 0 sorts nothing.
int clref_radix_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int startBit, int endBit) {
    using namespace clc;
    if (n >= kMaxArraySize) return -3;
    if ((endBit - startBit) % kBits != 0) return -4;
    if (n == 0) return 0;
    // :82-96 (fit() grows the reference's buffers to these sizes; the block sum stays at
    // cBlockSize entries).
    const size_t blocks = (size_t)std::ceil((float)n / kBlockSize);
    std::vector<uint> tempKey(n), tempVal(n);
    std::vector<uint4> blockScan4(blocks * (1 << kBits) / 4, uint4(0u));
    std::vector<uint> blockOffset(blocks * (1 << kBits), 0u), blockSum(kBlockSize, 0u);
    uint* blockScan = (uint*)blockScan4.data();
    const size_t globalSize = blocks * kBlockSize;
    const uint scanCount = (uint)(blocks * (1 << kBits) / 4);
    const size_t scanSize = (size_t)std::ceil((float)scanCount / kBlockSize) * kBlockSize;
    const uint size = n;
    for (int j = startBit; j < endBit; j += kBits) {  // :98-142
        const uint bit = (uint)j;
        run_groups_coro(globalSize, kBlockSize, [&] {
            return ksort::clBlockSort(keys, tempKey.data(), vals, tempVal.data(), bit, blockScan, blockOffset.data(),
                                      size);
        });
        run_groups_coro(scanSize, kBlockSize,
                        [&] { return ksort::clBlockScan(blockScan4.data(), blockSum.data(), scanCount); });
        run_groups_coro(scanSize, kBlockSize,
                        [&] { return ksort::clBlockPrefix(blockScan4.data(), blockSum.data(), scanCount); });
        run_groups_coro(globalSize, kBlockSize, [&] {
            return ksort::clReorder(tempKey.data(), keys, tempVal.data(), vals, blockScan, blockOffset.data(), bit,
                                    size);
        });
    }
    return 0;
}

// The shim's pow convention (clc::POW_INTEGER_CUBE or clc::POW_LIBM) for later launches.
void clref_set_pow_mode(int mode) { clc::set_pow_mode(mode); }

// Host threads the work-groups of a launch run on (OpenMP); returns the count in use.
int clref_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
    return omp_get_max_threads();
#else
    (void)n;
    return 1;
#endif
}

}  // extern "C"
