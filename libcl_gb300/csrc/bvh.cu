// bvh.cu -- linear BVH over a triangle mesh: the oclBvhTrimesh replacement behind the C ABI
// (libCL/geom/oclBvhTrimesh.h:20-84, libCL/geom/oclBvhTrimesh.cpp:56-143,
// libCL/geom/oclBvhTrimesh.cl:33-298), the reference's second user of the radix sort; and its
// 2D sibling over line segments, the oclBvhLines replacement (libCL/geom/oclBvhLines.h:20-77,
// libCL/geom/oclBvhLines.cpp:48-115, libCL/geom/oclBvhLines.cl:27-245), which shares the node
// creation, linking, leaves and parent links (templated on the node type).
//
// One build, in the reference's order:
//   global bounding box (accumulated into the handle's box, which starts at zero and is never
//   reset, as the reference's is) -> 30-bit Morton key of every triangle centroid -> stable
//   sort of (key, triangle) on 32 bits -> internal node i (between sorted leaves i and i+1)
//   gets the highest bit (29..0) where keys i and i+1 differ -> each internal node links to
//   the nearer of its nearest left / right nodes with a higher bit (the one with the lower
//   bit; the root has neither) -> leaves take the free child slots -> boxes bottom-up.
// The reference finds the higher-bit neighbours by a linear scan per node and computes the
// boxes by one root-to-leaf descent per triangle with a visit flag per node. Here the scans
// skip 64- and 4096-node blocks by their maximum bit (same answer, bounded work) and the
// boxes are refitted bottom-up from parent links with a visit counter per node; min and max
// are evaluated with the reference's operand order, so every box is bit-identical.
#include <algorithm>
#include <cfloat>
#include <string>

#include "device.cuh"
#include "internal.h"

using namespace gbsph;

namespace {

constexpr int BVH_THREADS = 256;
constexpr uint32_t BLK = 64, SBLK = 4096;  // scan-skipping block sizes (SBLK = BLK * BLK)

// OpenCL's min / max of floats: min(x, y) = y < x ? y : x, max(x, y) = x < y ? y : x.
__device__ __forceinline__ float cl_min(float x, float y) { return y < x ? y : x; }
__device__ __forceinline__ float cl_max(float x, float y) { return x < y ? y : x; }
__device__ __forceinline__ float4 cl_min4(float4 a, float4 b) {
    return make_float4(cl_min(a.x, b.x), cl_min(a.y, b.y), cl_min(a.z, b.z), cl_min(a.w, b.w));
}
__device__ __forceinline__ float4 cl_max4(float4 a, float4 b) {
    return make_float4(cl_max(a.x, b.x), cl_max(a.y, b.y), cl_max(a.z, b.z), cl_max(a.w, b.w));
}

__device__ __forceinline__ uint32_t spread10(uint32_t x) {  // "code", libCL/geom/oclBvhTrimesh.cl:82-89
    x = (x | (x << 16)) & 0x030000FFu;
    x = (x | (x << 8)) & 0x0300F00Fu;
    x = (x | (x << 4)) & 0x030C30C3u;
    x = (x | (x << 2)) & 0x09249249u;
    return x;
}

// 16-bit interleave of clMorton, libCL/geom/oclBvhLines.cl:35-52.
__device__ __forceinline__ uint32_t spread16(uint32_t x) {
    x &= 0x0000FFFFu;
    x = (x | (x << 8)) & 0x00FF00FFu;
    x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u;
    x = (x | (x << 1)) & 0x55555555u;
    return x;
}

// Empty boxes of clCreateNodes: +-MAXFLOAT in the coordinate lanes (w = 0 for triangles).
__device__ __forceinline__ void box_init(gbsph_bvh_node& nd) {
    nd.bbMin[0] = nd.bbMin[1] = nd.bbMin[2] = FLT_MAX;
    nd.bbMin[3] = 0.f;
    nd.bbMax[0] = nd.bbMax[1] = nd.bbMax[2] = -FLT_MAX;
    nd.bbMax[3] = 0.f;
}
__device__ __forceinline__ void box_init(gbsph_bvh2d_node& nd) {
    nd.bbMin[0] = nd.bbMin[1] = FLT_MAX;
    nd.bbMax[0] = nd.bbMax[1] = -FLT_MAX;
}

// Per-block min / max of the vertices (all four lanes), combined with the handle's box by the
// last block to finish (clAABB, libCL/geom/oclBvhTrimesh.cl:33-76).
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_box(const float4* __restrict__ vertex, uint32_t nv,
                                                         float4* __restrict__ part, uint32_t* __restrict__ done,
                                                         float4* __restrict__ box) {
    __shared__ float4 smin[BVH_THREADS], smax[BVH_THREADS];
    __shared__ bool last;
    float4 mn = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), mx = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
    for (uint32_t i = blockIdx.x * BVH_THREADS + threadIdx.x; i < nv; i += gridDim.x * BVH_THREADS) {
        const float4 v = vertex[i];
        mn = cl_min4(mn, v);
        mx = cl_max4(mx, v);
    }
    smin[threadIdx.x] = mn;
    smax[threadIdx.x] = mx;
    __syncthreads();
    for (int s = BVH_THREADS / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) {
            smin[threadIdx.x] = cl_min4(smin[threadIdx.x], smin[threadIdx.x + s]);
            smax[threadIdx.x] = cl_max4(smax[threadIdx.x], smax[threadIdx.x + s]);
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        part[2 * blockIdx.x] = smin[0];
        part[2 * blockIdx.x + 1] = smax[0];
        __threadfence();
        last = atomicAdd(done, 1u) == gridDim.x - 1;
    }
    __syncthreads();
    if (last && threadIdx.x == 0) {
        __threadfence();
        const volatile float4* vp = part;  // written by other blocks: read past L1
        float4 a = box[0], b = box[1];
        for (uint32_t k = 0; k < gridDim.x; ++k) {
            const float4 lo = make_float4(vp[2 * k].x, vp[2 * k].y, vp[2 * k].z, vp[2 * k].w);
            const float4 hi = make_float4(vp[2 * k + 1].x, vp[2 * k + 1].y, vp[2 * k + 1].z, vp[2 * k + 1].w);
            a = cl_min4(a, lo);
            b = cl_max4(b, hi);
        }
        box[0] = a;
        box[1] = b;
        *done = 0;
    }
}

// clMorton (libCL/geom/oclBvhTrimesh.cl:91-103): key of the triangle's centroid in the box.
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_morton(const uint32_t* __restrict__ index,
                                                            const float4* __restrict__ vertex,
                                                            const float4* __restrict__ box, uint32_t n,
                                                            uint32_t nv, uint32_t* __restrict__ key,
                                                            uint32_t* __restrict__ val, uint32_t* err) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const uint32_t i0 = index[3 * g], i1 = index[3 * g + 1], i2 = index[3 * g + 2];
    if (i0 >= nv || i1 >= nv || i2 >= nv) atomicOr(err, DEV_ERR_KEY_RANGE);
    const float4 v0 = vertex[min(i0, nv - 1)], v1 = vertex[min(i1, nv - 1)], v2 = vertex[min(i2, nv - 1)];
    const float4 lo = box[0], hi = box[1];
    auto axis = [&](float a, float b, float c, float l, float h) {
        const float cen = __fdiv_rn(__fadd_rn(__fadd_rn(a, b), c), 3.0f);
        const float t = __fdiv_rn(__fsub_rn(cen, l), __fsub_rn(h, l));
        return spread10(__float2uint_rz(__fmul_rn(t, 1023.0f)));
    };
    key[g] = axis(v0.x, v1.x, v2.x, lo.x, hi.x) | (axis(v0.y, v1.y, v2.y, lo.y, hi.y) << 1) |
             (axis(v0.z, v1.z, v2.z, lo.z, hi.z) << 2);
    val[g] = g;
}

// clMorton of oclBvhLines (libCL/geom/oclBvhLines.cl:27-55): the segment's midpoint,
// 0.5 * (v0 + v1), truncated to integers, 16 bits per axis interleaved (x in the even bits).
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_morton_lines(const float2* __restrict__ vertex, uint32_t n,
                                                                  uint32_t* __restrict__ key,
                                                                  uint32_t* __restrict__ val) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const float2 v0 = vertex[2 * g], v1 = vertex[2 * g + 1];
    const uint32_t cx = __float2uint_rz(__fmul_rn(0.5f, __fadd_rn(v0.x, v1.x)));
    const uint32_t cy = __float2uint_rz(__fmul_rn(0.5f, __fadd_rn(v0.y, v1.y)));
    key[g] = spread16(cx) | (spread16(cy) << 1);
    val[g] = g;
}

// clCreateNodes (libCL/geom/oclBvhTrimesh.cl:119-143, libCL/geom/oclBvhLines.cl:71-95): the
// highest bit, of bits [0, TOP], where sorted keys i and i + 1 differ; and the block maxima of
// the bits.
template <class Node, int TOP>
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_nodes(const uint32_t* __restrict__ key, uint32_t m,
                                                           Node* __restrict__ node,
                                                           uint8_t* __restrict__ bits, uint8_t* __restrict__ bmax) {
    constexpr uint32_t MASK = TOP == 31 ? 0xFFFFFFFFu : (1u << (TOP + 1)) - 1u;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t bit = 0;
    if (i < m) {
        const uint32_t d = (key[i] ^ key[i + 1]) & MASK;
        bit = d ? 31u - (uint32_t)__clz(d) : 0u;
        Node nd;
        box_init(nd);
        nd.left = nd.right = -1;
        nd.bit = bit;
        nd.trav = 0;
        node[i] = nd;
        bits[i] = (uint8_t)bit;
    }
    // maximum bit of each 64-node block (blocks of 256 threads hold 4 of them)
    uint32_t v = i < m ? bit : 0u;
    for (int s = 16; s > 0; s >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, s));
    __shared__ uint32_t w[BVH_THREADS / 32];
    if ((threadIdx.x & 31) == 0) w[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < BVH_THREADS / BLK) {
        const uint32_t b = (blockIdx.x * BVH_THREADS) / BLK + threadIdx.x;
        if (b * BLK < m) bmax[b] = (uint8_t)max(w[2 * threadIdx.x], w[2 * threadIdx.x + 1]);
    }
}

// Maximum bit of each 4096-node super-block.
__global__ void k_bvh_smax(const uint8_t* __restrict__ bmax, uint32_t nb, uint8_t* __restrict__ smax) {
    const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s * (SBLK / BLK) >= nb) return;
    uint8_t v = 0;
    for (uint32_t b = s * (SBLK / BLK); b < min(nb, (s + 1) * (SBLK / BLK)); ++b) v = max(v, bmax[b]);
    smax[s] = v;
}

// Nearest node left of i (dir < 0) or right of i (dir > 0) whose bit exceeds `bit`, or -1:
// element steps inside a block, block steps inside a super-block, then super-block steps.
__device__ int nearest_higher(const uint8_t* __restrict__ bits, const uint8_t* __restrict__ bmax,
                              const uint8_t* __restrict__ smax, int m, int i, int dir, uint32_t bit) {
    int j = i + dir;
    while (j >= 0 && j < m) {
        if ((j % (int)BLK) == (dir > 0 ? 0 : (int)BLK - 1) && bmax[j / BLK] <= bit) {
            // skip this block; at a super-block boundary, skip super-blocks too
            if ((j % (int)SBLK) == (dir > 0 ? 0 : (int)SBLK - 1)) {
                int sb = j / (int)SBLK;
                while (sb >= 0 && sb * (int)SBLK < m && smax[sb] <= bit) sb += dir;
                if (sb < 0 || sb * (int)SBLK >= m) return -1;
                j = dir > 0 ? sb * (int)SBLK : min(m - 1, sb * (int)SBLK + (int)SBLK - 1);
                if ((j % (int)BLK) != (dir > 0 ? 0 : (int)BLK - 1) || bmax[j / BLK] > bit) continue;
            }
            j += dir * (int)BLK;
            continue;
        }
        if (bits[j] > bit) return j;
        j += dir;
    }
    return -1;
}

// clLinkNodes (libCL/geom/oclBvhTrimesh.cl:145-199, libCL/geom/oclBvhLines.cl:97-151).
// Several nodes can only claim the same slot (or the root) when sorted keys repeat (their
// bits are then 0); the largest claimant wins here, as in a sequential run of the
// reference's work-items.
template <class Node>
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_link(const uint8_t* __restrict__ bits,
                                                          const uint8_t* __restrict__ bmax,
                                                          const uint8_t* __restrict__ smax, int m,
                                                          Node* __restrict__ node,
                                                          uint32_t* __restrict__ root) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const uint32_t bit = bits[i];
    const int l = nearest_higher(bits, bmax, smax, m, i, -1, bit);
    const int r = nearest_higher(bits, bmax, smax, m, i, +1, bit);
    if (l < 0 && r < 0) {
        atomicMax(root, (uint32_t)i);  // one root unless keys repeat; then the last, as a sequential run
    } else if (r < 0 || (l >= 0 && bits[l] < bits[r])) {
        atomicMax(&node[l].right, i);
    } else {
        atomicMax(&node[r].left, i);
    }
}

// clCreateLeaves (libCL/geom/oclBvhTrimesh.cl:201-234, libCL/geom/oclBvhLines.cl:153-184):
// leaf n-1+g holds primitive val[g] in .bit and takes the free slot between internal nodes
// g-1 and g. (The leaf's box is written by the box pass.)
template <class Node>
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_leaves(const uint32_t* __restrict__ val, uint32_t n,
                                                            Node* __restrict__ node) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const uint32_t ls = n - 1, L = ls + g;
    Node nd;
    box_init(nd);
    nd.left = nd.right = 0;
    nd.bit = val[g];
    nd.trav = 0;
    node[L] = nd;
    if (g == 0) {
        node[0].left = (int32_t)L;
    } else if (g == ls) {
        node[ls - 1].right = (int32_t)L;
    } else if (node[g].left == -1) {
        node[g].left = (int32_t)L;
    } else if (node[g - 1].right == -1) {
        node[g - 1].right = (int32_t)L;
    }
}

// Parent links from the child slots, and the visit counters cleared.
template <class Node>
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_parents(const Node* __restrict__ node, uint32_t m,
                                                             int32_t* __restrict__ parent,
                                                             uint32_t* __restrict__ visits) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= m) return;
    const int32_t l = node[i].left, r = node[i].right;
    if (l >= 0) parent[l] = (int32_t)i;
    if (r >= 0) parent[r] = (int32_t)i;
    visits[i] = 0;
}

// Boxes (clComputeAABBs, libCL/geom/oclBvhTrimesh.cl:236-298): each leaf's box from its
// triangle; the second of a node's two children to arrive computes the node's box as
// min(left, right) / max(left, right) and goes on up; internal nodes end with trav = 2.
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_refit(const uint32_t* __restrict__ index,
                                                           const float4* __restrict__ vertex, uint32_t n, uint32_t nv,
                                                           gbsph_bvh_node* node, const int32_t* __restrict__ parent,
                                                           uint32_t* visits, const uint32_t* __restrict__ root) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const uint32_t L = n - 1 + g;
    const uint32_t tri = node[L].bit;
    float4 mn = make_float4(FLT_MAX, FLT_MAX, FLT_MAX, 0.f), mx = make_float4(-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.f);
    for (int k = 0; k < 3; ++k) {
        const float4 v = vertex[min(index[3 * tri + k], nv - 1)];
        mn = cl_min4(mn, v);
        mx = cl_max4(mx, v);
    }
    *reinterpret_cast<float4*>(node[L].bbMin) = mn;
    *reinterpret_cast<float4*>(node[L].bbMax) = mx;
    const uint32_t rt = *root;
    int32_t c = (int32_t)L;
    for (uint32_t depth = 0; depth < 2 * n && (uint32_t)c != rt; ++depth) {
        const int32_t p = parent[c];
        if (p < 0) return;  // not reachable from the root (repeated keys)
        __threadfence();
        if (atomicAdd(&visits[p], 1u) == 0) return;  // the other child is not done yet
        __threadfence();
        const volatile gbsph_bvh_node* vn = node;
        const int32_t l = vn[p].left, r = vn[p].right;
        float4 a, b;
        a.x = cl_min(vn[l].bbMin[0], vn[r].bbMin[0]);
        a.y = cl_min(vn[l].bbMin[1], vn[r].bbMin[1]);
        a.z = cl_min(vn[l].bbMin[2], vn[r].bbMin[2]);
        a.w = cl_min(vn[l].bbMin[3], vn[r].bbMin[3]);
        b.x = cl_max(vn[l].bbMax[0], vn[r].bbMax[0]);
        b.y = cl_max(vn[l].bbMax[1], vn[r].bbMax[1]);
        b.z = cl_max(vn[l].bbMax[2], vn[r].bbMax[2]);
        b.w = cl_max(vn[l].bbMax[3], vn[r].bbMax[3]);
        *reinterpret_cast<float4*>(node[p].bbMin) = a;
        *reinterpret_cast<float4*>(node[p].bbMax) = b;
        node[p].trav = 2;
        c = p;
    }
}

// Boxes of oclBvhLines (clComputeAABBs, libCL/geom/oclBvhLines.cl:186-245): each leaf's box
// from its segment's two vertices; the second of a node's two children to arrive computes
// min(left, right) / max(left, right) and goes on up. In the reference the first visitor
// leaves trav = 2 and the second swaps it for 3 before computing, so internal nodes end with
// trav = 3.
__global__ void __launch_bounds__(BVH_THREADS) k_bvh_refit_lines(const float2* __restrict__ vertex, uint32_t n,
                                                                 gbsph_bvh2d_node* node,
                                                                 const int32_t* __restrict__ parent,
                                                                 uint32_t* visits, const uint32_t* __restrict__ root) {
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    const uint32_t L = n - 1 + g;
    const uint32_t seg = node[L].bit;
    const float2 v0 = vertex[2 * seg], v1 = vertex[2 * seg + 1];
    const float2 mn = make_float2(cl_min(cl_min(FLT_MAX, v0.x), v1.x), cl_min(cl_min(FLT_MAX, v0.y), v1.y));
    const float2 mx = make_float2(cl_max(cl_max(-FLT_MAX, v0.x), v1.x), cl_max(cl_max(-FLT_MAX, v0.y), v1.y));
    *reinterpret_cast<float4*>(node[L].bbMin) = make_float4(mn.x, mn.y, mx.x, mx.y);
    const uint32_t rt = *root;
    int32_t c = (int32_t)L;
    for (uint32_t depth = 0; depth < 2 * n && (uint32_t)c != rt; ++depth) {
        const int32_t p = parent[c];
        if (p < 0) return;  // not reachable from the root (repeated keys)
        __threadfence();
        if (atomicAdd(&visits[p], 1u) == 0) return;  // the other child is not done yet
        __threadfence();
        const volatile gbsph_bvh2d_node* vn = node;
        const int32_t l = vn[p].left, r = vn[p].right;
        const float4 box = make_float4(cl_min(vn[l].bbMin[0], vn[r].bbMin[0]), cl_min(vn[l].bbMin[1], vn[r].bbMin[1]),
                                       cl_max(vn[l].bbMax[0], vn[r].bbMax[0]), cl_max(vn[l].bbMax[1], vn[r].bbMax[1]));
        *reinterpret_cast<float4*>(node[p].bbMin) = box;
        node[p].trav = 3;
        c = p;
    }
}

int grid(uint32_t n) { return (int)((n + BVH_THREADS - 1) / BVH_THREADS); }

}  // namespace

struct gbsph_bvh_s {
    int device = 0;
    gbsph_radix_sort_t sort = nullptr;
    uint32_t cap = 0;  // triangles the buffers hold
    uint32_t n = 0;    // triangles of the last build
    void* block = nullptr;
    gbsph_bvh_node* node = nullptr;
    uint32_t *key = nullptr, *val = nullptr, *visits = nullptr, *root = nullptr, *err = nullptr, *done = nullptr;
    int32_t* parent = nullptr;
    uint8_t *bits = nullptr, *bmax = nullptr, *smax = nullptr;
    float4* box = nullptr;   // [min, max], persists across builds
    float4* part = nullptr;  // per-block partial boxes
    std::string last_error;
};

namespace {

constexpr int BOX_BLOCKS = 1024;

int ensure(gbsph_bvh_s* h, uint32_t n) {
    if (n <= h->cap && h->block) return GBSPH_OK;
    if (h->block) cudaFree(h->block);
    h->block = nullptr;
    const size_t nn = 2 * (size_t)n, m = n;
    const size_t nb = (m + BLK - 1) / BLK, ns = (m + SBLK - 1) / SBLK;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t bytes = al(nn * sizeof(gbsph_bvh_node)) + 3 * al(m * 4) + al(nn * 4) + al(m) + al(nb) + al(ns) + 256;
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->block, bytes));
    char* p = (char*)h->block;
    h->node = (gbsph_bvh_node*)p;
    p += al(nn * sizeof(gbsph_bvh_node));
    h->key = (uint32_t*)p;
    p += al(m * 4);
    h->val = (uint32_t*)p;
    p += al(m * 4);
    h->visits = (uint32_t*)p;
    p += al(m * 4);
    h->parent = (int32_t*)p;
    p += al(nn * 4);
    h->bits = (uint8_t*)p;
    p += al(m);
    h->bmax = (uint8_t*)p;
    p += al(nb);
    h->smax = (uint8_t*)p;
    h->cap = n;
    return GBSPH_OK;
}

}  // namespace

extern "C" {

GBSPH_API int gbsph_bvh_create(gbsph_bvh_t* out) {
    if (!out) return GBSPH_ERR_ARGUMENT;
    *out = nullptr;
    gbsph_bvh_s* h = new gbsph_bvh_s();
    int rc = cudaGetDevice(&h->device) == cudaSuccess ? GBSPH_OK : GBSPH_ERR_CUDA;
    if (!rc) rc = gbsph_radix_sort_create(&h->sort);
    // small state: the persistent box (zero, as the reference's freshly allocated one), the
    // partial boxes, root, error word and the box kernel's block counter
    const size_t small = 2 * 16 + BOX_BLOCKS * 32 + 16;
    void* s = nullptr;
    if (!rc && cudaMalloc(&s, small) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMemset(s, 0, small) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (rc) {
        cudaGetLastError();
        if (s) cudaFree(s);
        if (h->sort) gbsph_radix_sort_destroy(h->sort);
        delete h;
        return rc;
    }
    h->box = (float4*)s;
    h->part = h->box + 2;
    h->root = (uint32_t*)(h->part + 2 * BOX_BLOCKS);
    h->err = h->root + 1;
    h->done = h->root + 2;
    *out = h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_bvh_destroy(gbsph_bvh_t h) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    cudaSetDevice(h->device);
    if (h->block) cudaFree(h->block);
    if (h->box) cudaFree(h->box);
    if (h->sort) gbsph_radix_sort_destroy(h->sort);
    delete h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_bvh_compute(gbsph_bvh_t h, const float* vertex, size_t n_vertices, const uint32_t* index,
                                size_t n_indices, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!vertex || !index) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null buffer");
    if (n_indices % 3 != 0) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "index count is not a multiple of 3");
    const size_t nt = n_indices / 3;
    if (nt < 2) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "a BVH needs at least 2 triangles");
    if (n_vertices == 0) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "no vertices");
    if (nt > SORT_MAX_KEYS - SORT_TILE || n_vertices > 0xFFFFFFFFull)
        return fail(&h->last_error, GBSPH_ERR_TOO_LARGE, "too many triangles or vertices");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    const uint32_t n = (uint32_t)nt, m = n - 1, nv = (uint32_t)n_vertices;
    int rc = ensure(h, n);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const float4* v4 = reinterpret_cast<const float4*>(vertex);
    const int bb = std::min(BOX_BLOCKS, std::max(1, (int)((nv + BVH_THREADS * 8 - 1) / (BVH_THREADS * 8))));
    k_bvh_box<<<bb, BVH_THREADS, 0, s>>>(v4, nv, h->part, h->done, h->box);
    k_bvh_morton<<<grid(n), BVH_THREADS, 0, s>>>(index, v4, h->box, n, nv, h->key, h->val, h->err);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    rc = gbsph_radix_sort_compute(h->sort, h->key, h->val, n, n, 0, 32, stream);
    if (rc) return fail(&h->last_error, rc, std::string("sort: ") + gbsph_radix_sort_last_error(h->sort));
    const uint32_t nb = (m + BLK - 1) / BLK;
    k_bvh_nodes<gbsph_bvh_node, 29><<<grid(m), BVH_THREADS, 0, s>>>(h->key, m, h->node, h->bits, h->bmax);
    k_bvh_smax<<<(unsigned)((nb + 255) / 256 / (SBLK / BLK) + 1), 256, 0, s>>>(h->bmax, nb, h->smax);
    GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(h->root, 0, 4, s));
    k_bvh_link<gbsph_bvh_node><<<grid(m), BVH_THREADS, 0, s>>>(h->bits, h->bmax, h->smax, (int)m, h->node, h->root);
    k_bvh_leaves<gbsph_bvh_node><<<grid(n), BVH_THREADS, 0, s>>>(h->val, n, h->node);
    GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(h->parent, 0xFF, (2 * (size_t)n - 1) * 4, s));
    k_bvh_parents<gbsph_bvh_node><<<grid(m), BVH_THREADS, 0, s>>>(h->node, m, h->parent, h->visits);
    k_bvh_refit<<<grid(n), BVH_THREADS, 0, s>>>(index, v4, n, nv, h->node, h->parent, h->visits, h->root);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    h->n = n;
    return GBSPH_OK;
}

GBSPH_API gbsph_bvh_node* gbsph_bvh_get_node_buffer(gbsph_bvh_t h, size_t* count) {
    if (!h) return nullptr;
    if (count) *count = h->n ? 2 * (size_t)h->n - 1 : 0;
    return h->node;
}

GBSPH_API size_t gbsph_bvh_get_node_count(gbsph_bvh_t h) { return h && h->n ? 2 * (size_t)h->n - 1 : 0; }

GBSPH_API int gbsph_bvh_get_root_node(gbsph_bvh_t h, uint32_t* root, void* stream) {
    if (!h || !root) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize((cudaStream_t)stream));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpy(root, h->root, 4, cudaMemcpyDeviceToHost));
    return GBSPH_OK;
}

GBSPH_API int gbsph_bvh_get_bounds(gbsph_bvh_t h, float* box8, void* stream) {
    if (!h || !box8) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize((cudaStream_t)stream));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpy(box8, h->box, 32, cudaMemcpyDeviceToHost));
    return GBSPH_OK;
}

GBSPH_API int gbsph_bvh_sync_status(gbsph_bvh_t h, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize((cudaStream_t)stream));
    const int src = gbsph_radix_sort_sync_status(h->sort, stream);
    if (src) return fail(&h->last_error, src, std::string("sort: ") + gbsph_radix_sort_last_error(h->sort));
    uint32_t bits = 0;
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpy(&bits, h->err, 4, cudaMemcpyDeviceToHost));
    if (bits) {
        GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->err, 0, 4));
        return fail(&h->last_error, dev_err_to_status(bits), "a triangle index is outside the vertex buffer");
    }
    return GBSPH_OK;
}

GBSPH_API const char* gbsph_bvh_last_error(gbsph_bvh_t h) { return h ? h->last_error.c_str() : "null handle"; }

}  // extern "C"

// ---- particle-vs-mesh collision -------------------------------------------------------------
// clCollideBVH (libCL/phys/oclFluid3D.cl:365-550), one work-item per particle, restated with
// round-to-nearest intrinsics (no contraction) so that it matches the CPU restatement bit for
// bit. OpenCL's implementation-defined helpers are fixed as: dot(a, b) = ((ax bx + ay by) +
// az bz) + aw bw; length / fast_length(a) = sqrt(dot(a, a)); normalize(a) = a / length(a)
// per lane; cross() of float4 has w = 0. The traversal keeps the reference's breadth-first
// order with its 256-entry circular queue, so the first colliding triangle is the same.

namespace {

struct F4 {
    float x, y, z, w;
};
__device__ __forceinline__ F4 f4(float4 a) { return {a.x, a.y, a.z, a.w}; }
__device__ __forceinline__ F4 add(F4 a, F4 b) {
    return {__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w)};
}
__device__ __forceinline__ F4 sub(F4 a, F4 b) {
    return {__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z), __fsub_rn(a.w, b.w)};
}
__device__ __forceinline__ F4 mul(F4 a, float s) {
    return {__fmul_rn(a.x, s), __fmul_rn(a.y, s), __fmul_rn(a.z, s), __fmul_rn(a.w, s)};
}
__device__ __forceinline__ F4 mulv(F4 a, F4 b) {
    return {__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y), __fmul_rn(a.z, b.z), __fmul_rn(a.w, b.w)};
}
__device__ __forceinline__ F4 divs(F4 a, float s) {
    return {__fdiv_rn(a.x, s), __fdiv_rn(a.y, s), __fdiv_rn(a.z, s), __fdiv_rn(a.w, s)};
}
__device__ __forceinline__ float dot(F4 a, F4 b) {
    return __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y)), __fmul_rn(a.z, b.z)),
                     __fmul_rn(a.w, b.w));
}
__device__ __forceinline__ float len(F4 a) { return __fsqrt_rn(dot(a, a)); }
__device__ __forceinline__ F4 normalize(F4 a) { return divs(a, len(a)); }
__device__ __forceinline__ F4 cross(F4 p, F4 q) {
    return {__fsub_rn(__fmul_rn(p.y, q.z), __fmul_rn(p.z, q.y)), __fsub_rn(__fmul_rn(p.z, q.x), __fmul_rn(p.x, q.z)),
            __fsub_rn(__fmul_rn(p.x, q.y), __fmul_rn(p.y, q.x)), 0.0f};
}

struct CollideParams {
    float dt, radius, pconst, density, h, mass;
};

// collideTriangle (libCL/phys/oclFluid3D.cl:380-459); `tri` is the first index slot.
__device__ bool collide_triangle(uint32_t tri, const uint32_t* __restrict__ index, const float4* __restrict__ vertex,
                                 uint32_t nv, F4& pos, F4& vel, F4& force, const CollideParams& P) {
    F4 V0 = f4(vertex[min(index[tri], nv - 1)]), V1 = f4(vertex[min(index[tri + 1], nv - 1)]),
       V2 = f4(vertex[min(index[tri + 2], nv - 1)]);
    V0.w = V1.w = V2.w = 0.0f;
    pos.w = 0.0f;
    const F4 u = sub(V1, V0), v = sub(V2, V0);
    F4 n = cross(u, v);
    if (dot(n, n) == 0.0f) return false;
    const F4 w0 = sub(pos, V0);
    const F4 disp = mul(vel, P.dt);
    const float a = dot(n, w0);
    if (a < 0.0f) return false;
    const float b = dot(n, disp);
    if (fabsf(b) < 0.000001f) return false;
    const float r = __fdiv_rn(-a, b);
    if (r < 0.0f) return false;
    const F4 I = add(pos, mul(disp, r));
    const float uu = dot(u, u), uv = dot(u, v), vv = dot(v, v);
    const F4 w = sub(I, V0);
    const float wu = dot(w, u), wv = dot(w, v);
    const float D = __fsub_rn(__fmul_rn(uv, uv), __fmul_rn(uu, vv));
    const float s = __fdiv_rn(__fsub_rn(__fmul_rn(uv, wv), __fmul_rn(vv, wu)), D);
    if (s < 0.0f || s > 1.0f) return false;
    const float t = __fdiv_rn(__fsub_rn(__fmul_rn(uv, wu), __fmul_rn(uu, wv)), D);
    if (t < 0.0f || __fadd_rn(s, t) > 1.0f) return false;
    n = normalize(n);
    const F4 Vc = sub(add(pos, disp), V0);
    const float dist = dot(Vc, n);
    const float depth = __fsub_rn(P.radius, dist);
    if (depth > 0.0f) {
        const F4 dPos = mul(mul(normalize(disp), dot(n, disp)), depth);
        const F4 dTan = sub(vel, mul(n, dot(n, vel)));
        force = add(force, divs(dTan, P.dt));
        const float hd = __fsub_rn(P.h, dist);
        force = add(force, mul(mul(mul(mul(n, hd), hd), __fdiv_rn(P.pconst, P.density)), P.mass));
        pos = add(pos, dPos);
        vel = {0.0f, 0.0f, 0.0f, 0.0f};
        return true;
    }
    return false;
}

// intersectBox + collideAABB (libCL/phys/oclFluid3D.cl:462-498).
__device__ bool collide_box(const gbsph_bvh_node& nd, F4 pos, F4 vel, float radius) {
    const F4 nr = normalize(vel);
    const F4 inv = {__fdiv_rn(1.0f, nr.x), __fdiv_rn(1.0f, nr.y), __fdiv_rn(1.0f, nr.z), __fdiv_rn(1.0f, nr.w)};
    const F4 bmin = {nd.bbMin[0], nd.bbMin[1], nd.bbMin[2], nd.bbMin[3]};
    const F4 bmax = {nd.bbMax[0], nd.bbMax[1], nd.bbMax[2], nd.bbMax[3]};
    const F4 tbot = mulv(inv, sub(bmin, pos)), ttop = mulv(inv, sub(bmax, pos));
    const float tminx = cl_min(ttop.x, tbot.x), tminy = cl_min(ttop.y, tbot.y), tminz = cl_min(ttop.z, tbot.z);
    const float tmaxx = cl_max(ttop.x, tbot.x), tmaxy = cl_max(ttop.y, tbot.y), tmaxz = cl_max(ttop.z, tbot.z);
    const float tnear = cl_max(cl_max(tminx, tminy), cl_max(tminx, tminz));
    const float tfar = cl_min(cl_min(tmaxx, tmaxy), cl_min(tmaxx, tmaxz));
    if (!(tfar > tnear)) return false;
    return tnear < cl_max(radius, len(vel));
}

constexpr uint32_t QUEUE_SIZE = 256;

__global__ void __launch_bounds__(BVH_THREADS) k_collide_bvh(float4* __restrict__ force, float4* __restrict__ position,
                                                             float4* __restrict__ velocity, uint32_t np,
                                                             CollideParams P, const gbsph_bvh_node* __restrict__ bvh,
                                                             uint32_t root, uint32_t n_nodes,
                                                             const uint32_t* __restrict__ index,
                                                             const float4* __restrict__ vertex, uint32_t nv,
                                                             uint32_t* err) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    F4 pos = f4(position[p]), vel = f4(velocity[p]), frc = f4(force[p]);
    uint32_t queue[QUEUE_SIZE];
    uint32_t head = 0, tail = 1;
    queue[0] = root;
    uint32_t steps = 0;
    while (head != tail) {
        const uint32_t it = queue[head];
        head = (head + 1) % QUEUE_SIZE;
        if (it >= n_nodes || ++steps > 4u * n_nodes + 4u) {  // not a tree: report and stop
            atomicOr(err, DEV_ERR_KEY_RANGE);
            return;
        }
        const uint32_t l = (uint32_t)bvh[it].left, r = (uint32_t)bvh[it].right;
        if (l == r) {
            if (collide_triangle(bvh[it].bit * 3u, index, vertex, nv, pos, vel, frc, P)) {
                position[p] = make_float4(pos.x, pos.y, pos.z, pos.w);
                velocity[p] = make_float4(vel.x, vel.y, vel.z, vel.w);
                force[p] = make_float4(frc.x, frc.y, frc.z, frc.w);
                break;
            }
        } else {
            if (l < n_nodes && collide_box(bvh[l], pos, vel, P.radius)) {
                queue[tail] = l;
                tail = (tail + 1) % QUEUE_SIZE;
            }
            if (r < n_nodes && collide_box(bvh[r], pos, vel, P.radius)) {
                queue[tail] = r;
                tail = (tail + 1) % QUEUE_SIZE;
            }
        }
    }
}

}  // namespace

extern "C" GBSPH_API int gbsph_bvh_collide(gbsph_bvh_t h, const gbsph_fluid3d_params* params, float* position,
                                           float* velocity, float* force, size_t n_particles, const float* vertex,
                                           size_t n_vertices, const uint32_t* index, void* stream) {
    if (!h || !params) return GBSPH_ERR_ARGUMENT;
    if (!position || !velocity || !force || !vertex || !index)
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null buffer");
    if (h->n == 0) return fail(&h->last_error, GBSPH_ERR_STATE, "collide before a BVH was built");
    if (n_particles == 0) return GBSPH_OK;
    if (n_particles > 0xFFFFFFFFull || n_vertices == 0 || n_vertices > 0xFFFFFFFFull)
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "bad particle or vertex count");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    uint32_t root = 0;
    cudaStream_t s = (cudaStream_t)stream;
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(&root, h->root, 4, cudaMemcpyDeviceToHost, s));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize(s));
    CollideParams P;
    P.dt = params->deltaTime;
    P.radius = params->particleRadius;
    P.pconst = params->pressureConstant;
    P.density = params->density;
    P.h = params->cellSize;
    P.mass = params->mass;
    const uint32_t np = (uint32_t)n_particles;
    k_collide_bvh<<<grid(np), BVH_THREADS, 0, s>>>(reinterpret_cast<float4*>(force), reinterpret_cast<float4*>(position),
                                                   reinterpret_cast<float4*>(velocity), np, P, h->node, root,
                                                   2 * h->n - 1, index, reinterpret_cast<const float4*>(vertex),
                                                   (uint32_t)n_vertices, h->err);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

// ------------------------------------------------------------------------------------------
// oclBvhLines replacement.
// ------------------------------------------------------------------------------------------
struct gbsph_bvh_lines_s {
    int device = 0;
    gbsph_radix_sort_t sort = nullptr;
    uint32_t cap = 0;  // segments the buffers hold
    uint32_t n = 0;    // segments of the last build
    void* block = nullptr;
    gbsph_bvh2d_node* node = nullptr;
    uint32_t *key = nullptr, *val = nullptr, *visits = nullptr, *root = nullptr;
    int32_t* parent = nullptr;
    uint8_t *bits = nullptr, *bmax = nullptr, *smax = nullptr;
    std::string last_error;
};

namespace {

int ensure_lines(gbsph_bvh_lines_s* h, uint32_t n) {
    if (n <= h->cap && h->block) return GBSPH_OK;
    if (h->block) cudaFree(h->block);
    h->block = nullptr;
    h->cap = 0;
    const size_t nn = 2 * (size_t)n, m = n;
    const size_t nb = (m + BLK - 1) / BLK, ns = (m + SBLK - 1) / SBLK;
    auto al = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t bytes = al(nn * sizeof(gbsph_bvh2d_node)) + 3 * al(m * 4) + al(nn * 4) + al(m) + al(nb) + al(ns) + 256;
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->block, bytes));
    char* p = (char*)h->block;
    h->node = (gbsph_bvh2d_node*)p;
    p += al(nn * sizeof(gbsph_bvh2d_node));
    h->key = (uint32_t*)p;
    p += al(m * 4);
    h->val = (uint32_t*)p;
    p += al(m * 4);
    h->visits = (uint32_t*)p;
    p += al(m * 4);
    h->parent = (int32_t*)p;
    p += al(nn * 4);
    h->bits = (uint8_t*)p;
    p += al(m);
    h->bmax = (uint8_t*)p;
    p += al(nb);
    h->smax = (uint8_t*)p;
    p += al(ns);
    h->root = (uint32_t*)p;
    h->cap = n;
    return GBSPH_OK;
}

}  // namespace

extern "C" {

GBSPH_API int gbsph_bvh_lines_create(gbsph_bvh_lines_t* out) {
    if (!out) return GBSPH_ERR_ARGUMENT;
    *out = nullptr;
    gbsph_bvh_lines_s* h = new gbsph_bvh_lines_s();
    int rc = cudaGetDevice(&h->device) == cudaSuccess ? GBSPH_OK : GBSPH_ERR_CUDA;
    if (!rc) rc = gbsph_radix_sort_create(&h->sort);
    if (rc) {
        cudaGetLastError();
        if (h->sort) gbsph_radix_sort_destroy(h->sort);
        delete h;
        return rc;
    }
    *out = h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_bvh_lines_destroy(gbsph_bvh_lines_t h) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    cudaSetDevice(h->device);
    if (h->block) cudaFree(h->block);
    if (h->sort) gbsph_radix_sort_destroy(h->sort);
    delete h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_bvh_lines_compute(gbsph_bvh_lines_t h, const float* vertex, size_t n_vertices, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!vertex) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null buffer");
    const size_t nl = n_vertices / 2;
    if (nl < 2) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "a BVH needs at least 2 segments");
    if (nl > SORT_MAX_KEYS - SORT_TILE) return fail(&h->last_error, GBSPH_ERR_TOO_LARGE, "too many segments");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    const uint32_t n = (uint32_t)nl, m = n - 1;
    int rc = ensure_lines(h, n);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const float2* v2 = reinterpret_cast<const float2*>(vertex);
    k_bvh_morton_lines<<<grid(n), BVH_THREADS, 0, s>>>(v2, n, h->key, h->val);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    rc = gbsph_radix_sort_compute(h->sort, h->key, h->val, n, n, 0, 32, stream);
    if (rc) return fail(&h->last_error, rc, std::string("sort: ") + gbsph_radix_sort_last_error(h->sort));
    const uint32_t nb = (m + BLK - 1) / BLK;
    k_bvh_nodes<gbsph_bvh2d_node, 31><<<grid(m), BVH_THREADS, 0, s>>>(h->key, m, h->node, h->bits, h->bmax);
    k_bvh_smax<<<(unsigned)((nb + 255) / 256 / (SBLK / BLK) + 1), 256, 0, s>>>(h->bmax, nb, h->smax);
    GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(h->root, 0, 4, s));
    k_bvh_link<gbsph_bvh2d_node><<<grid(m), BVH_THREADS, 0, s>>>(h->bits, h->bmax, h->smax, (int)m, h->node, h->root);
    k_bvh_leaves<gbsph_bvh2d_node><<<grid(n), BVH_THREADS, 0, s>>>(h->val, n, h->node);
    GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(h->parent, 0xFF, (2 * (size_t)n - 1) * 4, s));
    k_bvh_parents<gbsph_bvh2d_node><<<grid(m), BVH_THREADS, 0, s>>>(h->node, m, h->parent, h->visits);
    k_bvh_refit_lines<<<grid(n), BVH_THREADS, 0, s>>>(v2, n, h->node, h->parent, h->visits, h->root);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    h->n = n;
    return GBSPH_OK;
}

GBSPH_API gbsph_bvh2d_node* gbsph_bvh_lines_get_node_buffer(gbsph_bvh_lines_t h, size_t* count) {
    if (!h) return nullptr;
    if (count) *count = h->n ? 2 * (size_t)h->n - 1 : 0;
    return h->node;
}

GBSPH_API size_t gbsph_bvh_lines_get_node_count(gbsph_bvh_lines_t h) { return h && h->n ? 2 * (size_t)h->n - 1 : 0; }

GBSPH_API int gbsph_bvh_lines_get_root_node(gbsph_bvh_lines_t h, uint32_t* root, void* stream) {
    if (!h || !root) return GBSPH_ERR_ARGUMENT;
    if (!h->root) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "no build yet");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize((cudaStream_t)stream));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpy(root, h->root, 4, cudaMemcpyDeviceToHost));
    return GBSPH_OK;
}

GBSPH_API int gbsph_bvh_lines_sync_status(gbsph_bvh_lines_t h, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize((cudaStream_t)stream));
    const int src = gbsph_radix_sort_sync_status(h->sort, stream);
    if (src) return fail(&h->last_error, src, std::string("sort: ") + gbsph_radix_sort_last_error(h->sort));
    return GBSPH_OK;
}

GBSPH_API const char* gbsph_bvh_lines_last_error(gbsph_bvh_lines_t h) { return h ? h->last_error.c_str() : "null handle"; }

}  // extern "C"
