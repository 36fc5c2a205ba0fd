// refbvh.cpp -- the reference's BVH build kernels (libCL/geom/oclBvhTrimesh.cl and
// libCL/geom/oclBvhLines.cl, compiled unchanged apart from oracle/ref/rewrite.py's edits)
// driven as oclBvhTrimesh::compute (libCL/geom/oclBvhTrimesh.cpp:53-162) and
// oclBvhLines::compute (libCL/geom/oclBvhLines.cpp:48-116) drive them, with the reference's
// own radix sort (refsort.cpp) for the Morton keys.
//
// TEST INFRASTRUCTURE ONLY: the checker of the oracle's restated BVH builds. Nothing in the
// product library links it.
//
// Launch forms: clAABB as the reference enqueues it (work-groups of 32); every other kernel
// with a local size of 1 (the reference passes NULL). The launches run their work-items in
// order on the calling thread: clAABB's work-groups meet through a spin lock and
// clComputeAABBs's work-items through atomic flags, and in-order execution is one of the
// schedules the reference allows for both.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "clshim.h"

namespace clc {
namespace kbvh {
#include "oclBvhTrimesh.cl.inc"
}  // namespace kbvh
namespace kbvhl {
#include "oclBvhLines.cl.inc"
}  // namespace kbvhl
}  // namespace clc

static_assert(sizeof(clc::kbvh::BVHNode) == 48, "BVHNode of libCL/geom/oclBvhTrimesh.cl");
static_assert(sizeof(clc::kbvhl::BVHNode) == 32, "BVHNode of libCL/geom/oclBvhLines.cl");

extern "C" int clref_radix_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int startBit, int endBit);

namespace {
// Morton keys that repeat make the reference's clLinkNodes race (two nodes claim one child):
// the drivers refuse such inputs instead of running clComputeAABBs's fixed-depth descent
// over a structure that is not a tree.
bool keys_distinct(const std::vector<uint32_t>& k) {
    for (size_t i = 1; i < k.size(); i++)
        if (k[i] == k[i - 1]) return false;
    return true;
}
}  // namespace

extern "C" {

// oclBvhTrimesh::compute over n triangles. vertex: float4[nv]; index: uint32[3 n]; box:
// float[8] in/out (bfAABB's bbMin xyzw, bbMax xyzw; the reference keeps the buffer across
// builds); nodes: 48-byte BVHNode[2n - 1] out; root: in/out (mRootNode); sorted_keys /
// sorted_vals: uint32[n] out. Returns 0, -1 for n < 2, the sort's refusal (-3), or -5 if two
// Morton keys are equal.
int clref_bvh_build(const float* vertex, uint32_t nv, const uint32_t* index, uint32_t n, float* box, void* nodes,
                    uint32_t* root, uint32_t* sorted_keys, uint32_t* sorted_vals) {
    using namespace clc;
    if (n < 2 || nv == 0) return -1;
    std::vector<float4> vtx(nv);
    std::memcpy(vtx.data(), vertex, 16 * (size_t)nv);
    std::vector<uint> idx(index, index + 3 * (size_t)n);
    kbvh::AABB aabb;
    std::memset(&aabb, 0, sizeof(aabb));
    std::memcpy(&aabb.bbMin, box, 16);
    std::memcpy(&aabb.bbMax, box + 4, 16);
    // :74-91: ceil(ceil(V / 8) / 32) * 32 work-items in groups of cWarpSize
    const size_t batch = (size_t)(std::ceil(std::ceil(nv / 8.0) / 32) * 32);
    const int size = (int)nv;
    run_groups_coro<false>(batch, 32, [&] { return kbvh::clAABB(vtx.data(), &aabb, size); });
    // :94-103
    std::vector<uint> key(n), val(n);
    run_groups<false>(n, 1, [&] { kbvh::clMorton(idx.data(), vtx.data(), key.data(), val.data(), &aabb); });
    // :105-111
    const int rc = clref_radix_sort(key.data(), val.data(), n, 0, 32);
    if (rc) return rc;
    if (!keys_distinct(key)) return -5;
    // :113-145
    std::vector<kbvh::BVHNode> bvh(2 * (size_t)n - 1);
    std::memset(bvh.data(), 0, bvh.size() * sizeof(kbvh::BVHNode));
    uint r = *root;
    run_groups<false>(n - 1, 1, [&] { kbvh::clCreateNodes(key.data(), val.data(), bvh.data()); });
    run_groups<false>(n - 1, 1, [&] { kbvh::clLinkNodes(key.data(), bvh.data(), &r); });
    run_groups<false>(n, 1, [&] { kbvh::clCreateLeaves(val.data(), bvh.data()); });
    run_groups<false>(n, 1, [&] {
        kbvh::clComputeAABBs(idx.data(), vtx.data(), bvh.data(), reinterpret_cast<int*>(&r));
    });
    std::memcpy(nodes, bvh.data(), bvh.size() * sizeof(kbvh::BVHNode));
    std::memcpy(box, &aabb.bbMin, 16);
    std::memcpy(box + 4, &aabb.bbMax, 16);
    *root = r;
    if (sorted_keys) std::memcpy(sorted_keys, key.data(), 4 * (size_t)n);
    if (sorted_vals) std::memcpy(sorted_vals, val.data(), 4 * (size_t)n);
    return 0;
}

// oclBvhLines::compute over n segments. vertex: float2[2 n]; nodes: 32-byte BVHNode[2n - 1]
// out; root: in/out; sorted_keys / sorted_vals: uint32[n] out. Returns as clref_bvh_build.
int clref_bvh_lines_build(const float* vertex, uint32_t n, void* nodes, uint32_t* root, uint32_t* sorted_keys,
                          uint32_t* sorted_vals) {
    using namespace clc;
    if (n < 2) return -1;
    std::vector<float2> vtx(2 * (size_t)n);
    std::memcpy(vtx.data(), vertex, 16 * (size_t)n);
    // :67-74
    std::vector<uint> key(n), val(n);
    run_groups<false>(n, 1, [&] { kbvhl::clMorton(vtx.data(), key.data(), val.data()); });
    // :76-83
    const int rc = clref_radix_sort(key.data(), val.data(), n, 0, 32);
    if (rc) return rc;
    if (!keys_distinct(key)) return -5;
    // :84-112
    std::vector<kbvhl::BVHNode> bvh(2 * (size_t)n - 1);
    std::memset(bvh.data(), 0, bvh.size() * sizeof(kbvhl::BVHNode));
    uint r = *root;
    run_groups<false>(n - 1, 1, [&] { kbvhl::clCreateNodes(key.data(), val.data(), bvh.data()); });
    run_groups<false>(n - 1, 1, [&] { kbvhl::clLinkNodes(key.data(), bvh.data(), &r); });
    run_groups<false>(n, 1, [&] { kbvhl::clCreateLeaves(val.data(), bvh.data()); });
    run_groups<false>(n, 1, [&] { kbvhl::clComputeAABBs(vtx.data(), bvh.data(), reinterpret_cast<int*>(&r)); });
    std::memcpy(nodes, bvh.data(), bvh.size() * sizeof(kbvhl::BVHNode));
    *root = r;
    if (sorted_keys) std::memcpy(sorted_keys, key.data(), 4 * (size_t)n);
    if (sorted_vals) std::memcpy(sorted_vals, val.data(), 4 * (size_t)n);
    return 0;
}

}  // extern "C"
