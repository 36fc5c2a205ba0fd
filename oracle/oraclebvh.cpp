// oraclebvh.cpp -- CPU restatement of the reference's BVH builds (triangle mesh and 2D line
// segments) and of its particle-vs-mesh collision.
//
// TEST INFRASTRUCTURE ONLY, like oracle3d.cpp: nothing in the product links or calls it.
// It follows oclBvhTrimesh::compute (libCL/geom/oclBvhTrimesh.cpp:56-143) and the kernels of
// libCL/geom/oclBvhTrimesh.cl step by step, one work-item at a time, with the reference's own
// algorithms (linear neighbour scans, per-triangle root-to-leaf descents with visit flags).
// OpenCL's float min(x, y) is y < x ? y : x and max(x, y) is x < y ? y : x; float-to-uint
// conversion truncates. Parity status: unpinned against executed reference output (no OpenCL
// device here); pinned by construction against the .cl source and by structural checks.

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/gbsph.h"

namespace {

inline float clmin(float x, float y) { return y < x ? y : x; }
inline float clmax(float x, float y) { return x < y ? y : x; }

// "code", libCL/geom/oclBvhTrimesh.cl:82-89
uint32_t code(uint32_t x) {
    x = (x | (x << 16)) & 0x030000FF;
    x = (x | (x << 8)) & 0x0300F00F;
    x = (x | (x << 4)) & 0x030C30C3;
    x = (x | (x << 2)) & 0x09249249;
    return x;
}

// float -> uint as the implicit OpenCL C conversion (truncation); NaN and negatives -> 0,
// which is what the GPU conversion gives.
uint32_t to_uint(float f) {
    if (!(f > 0.0f)) return 0;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

void init_node(gbsph_bvh_node& nd, int32_t l, int32_t r, uint32_t bit) {
    nd.bbMin[0] = nd.bbMin[1] = nd.bbMin[2] = FLT_MAX;
    nd.bbMin[3] = 0.0f;
    nd.bbMax[0] = nd.bbMax[1] = nd.bbMax[2] = -FLT_MAX;
    nd.bbMax[3] = 0.0f;
    nd.left = l;
    nd.right = r;
    nd.bit = bit;
    nd.trav = 0;
}

}  // namespace

extern "C" {

// One build. vertex: float4[nv]; index: uint32[3 n]; box: float[8] in/out (min xyzw, max
// xyzw; the reference's bfAABB, zero before the first build); nodes: [2n - 1]; root: in/out
// (the reference keeps mRootNode across builds). Returns 0, or -1 for n < 2.
int orc_bvh_build(const float* vertex, uint32_t nv, const uint32_t* index, uint32_t n, float* box,
                  gbsph_bvh_node* nodes, uint32_t* root, uint32_t* sorted_keys, uint32_t* sorted_vals) {
    if (n < 2) return -1;
    // clAABB (libCL/geom/oclBvhTrimesh.cl:33-76): min / max of every vertex, all four lanes,
    // into the persistent box
    for (uint32_t i = 0; i < nv; i++)
        for (int c = 0; c < 4; c++) {
            box[c] = clmin(box[c], vertex[4 * i + c]);
            box[4 + c] = clmax(box[4 + c], vertex[4 * i + c]);
        }
    // clMorton (:91-103)
    std::vector<uint32_t> key(n), val(n);
    for (uint32_t g = 0; g < n; g++) {
        const float* v0 = vertex + 4 * (size_t)index[3 * g];
        const float* v1 = vertex + 4 * (size_t)index[3 * g + 1];
        const float* v2 = vertex + 4 * (size_t)index[3 * g + 2];
        uint32_t k = 0;
        for (int c = 0; c < 3; c++) {
            const float cen = ((v0[c] + v1[c]) + v2[c]) / 3.0f;
            const float t = (cen - box[c]) / (box[4 + c] - box[c]);
            k |= code(to_uint(t * (float)0x3FF)) << c;
        }
        key[g] = k;
        val[g] = g;
    }
    // oclRadixSort on bits [0, 32): a stable sort
    std::vector<uint32_t> order(n);
    for (uint32_t i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
    std::vector<uint32_t> sk(n), sv(n);
    for (uint32_t i = 0; i < n; i++) {
        sk[i] = key[order[i]];
        sv[i] = val[order[i]];
    }
    const uint32_t m = n - 1;  // internal nodes
    // clCreateNodes (:119-143)
    for (uint32_t i = 0; i < m; i++) {
        uint32_t bit = 0;
        for (int b = 29; b >= 0; b--)
            if (((sk[i] >> b) & 1u) != ((sk[i + 1] >> b) & 1u)) {
                bit = (uint32_t)b;
                break;
            }
        init_node(nodes[i], -1, -1, bit);
    }
    // clLinkNodes (:145-199)
    for (uint32_t g = 0; g < m; g++) {
        const uint32_t bit = nodes[g].bit;
        int left = -1, right = -1;
        for (int i = (int)g - 1; i >= 0; i--)
            if (nodes[i].bit > bit) {
                left = i;
                break;
            }
        for (uint32_t i = g + 1; i < m; i++)
            if (nodes[i].bit > bit) {
                right = (int)i;
                break;
            }
        if (left != -1 || right != -1) {
            if (right == -1) nodes[left].right = (int32_t)g;
            else if (left == -1) nodes[right].left = (int32_t)g;
            else if (nodes[left].bit < nodes[right].bit) nodes[left].right = (int32_t)g;
            else nodes[right].left = (int32_t)g;
        } else {
            *root = g;
        }
    }
    // clCreateLeaves (:201-234)
    const uint32_t ls = n - 1;
    for (uint32_t g = 0; g < n; g++) {
        init_node(nodes[ls + g], 0, 0, sv[g]);
        if (g == 0) {
            nodes[0].left = (int32_t)(ls + g);
            continue;
        }
        if (g == ls) {
            nodes[ls - 1].right = (int32_t)(ls + g);
            continue;
        }
        if (nodes[g].left == -1) nodes[g].left = (int32_t)(g + ls);
        else if (nodes[g - 1].right == -1) nodes[g - 1].right = (int32_t)(g + ls);
    }
    // clComputeAABBs (:236-298): per triangle, descend by node index, box the leaf, then
    // climb: the first visitor of a node marks it and stops, the second computes its box
    for (uint32_t g = 0; g < n; g++) {
        std::vector<uint32_t> stack;
        stack.push_back(*root);
        for (;;) {
            gbsph_bvh_node& nd = nodes[stack.back()];
            if (nd.left == nd.right) {
                const uint32_t tri = nd.bit;
                float mn[4] = {FLT_MAX, FLT_MAX, FLT_MAX, 0.0f}, mx[4] = {-FLT_MAX, -FLT_MAX, -FLT_MAX, 0.0f};
                for (int k = 0; k < 3; k++)
                    for (int c = 0; c < 4; c++) {
                        const float v = vertex[4 * (size_t)index[3 * tri + k] + c];
                        mn[c] = clmin(mn[c], v);
                        mx[c] = clmax(mx[c], v);
                    }
                std::memcpy(nd.bbMin, mn, 16);
                std::memcpy(nd.bbMax, mx, 16);
                break;
            }
            stack.push_back(stack.back() >= g ? (uint32_t)nd.left : (uint32_t)nd.right);
            if (stack.size() > 2 * (size_t)n) return -2;  // not a tree
        }
        size_t top = stack.size() - 1;
        while (top--) {
            gbsph_bvh_node& nd = nodes[stack[top]];
            if (nd.trav == 0) {
                nd.trav = 2;
                break;
            }
            const gbsph_bvh_node& l = nodes[nd.left];
            const gbsph_bvh_node& r = nodes[nd.right];
            for (int c = 0; c < 4; c++) {
                nd.bbMin[c] = clmin(l.bbMin[c], r.bbMin[c]);
                nd.bbMax[c] = clmax(l.bbMax[c], r.bbMax[c]);
            }
        }
    }
    if (sorted_keys) std::memcpy(sorted_keys, sk.data(), 4 * (size_t)n);
    if (sorted_vals) std::memcpy(sorted_vals, sv.data(), 4 * (size_t)n);
    return 0;
}

}  // extern "C"

// ---- oclBvhLines (libCL/geom/oclBvhLines.cpp:48-115, libCL/geom/oclBvhLines.cl:27-245) ---------
namespace {

uint32_t code16(uint32_t x) {  // clMorton's interleave, libCL/geom/oclBvhLines.cl:35-52
    x &= 0x0000ffffu;
    x |= x << 8;
    x &= 0x00ff00ffu;
    x |= x << 4;
    x &= 0x0f0f0f0fu;
    x |= x << 2;
    x &= 0x33333333u;
    x |= x << 1;
    x &= 0x55555555u;
    return x;
}

void init_node2(gbsph_bvh2d_node& nd, int32_t l, int32_t r, uint32_t bit) {
    nd.bbMin[0] = nd.bbMin[1] = FLT_MAX;
    nd.bbMax[0] = nd.bbMax[1] = -FLT_MAX;
    nd.left = l;
    nd.right = r;
    nd.bit = bit;
    nd.trav = 0;
}

}  // namespace

extern "C" {

// One build over n segments. vertex: float2[2 n]; nodes: [2n - 1]; root: in/out (kept across
// builds, as mRootNode). Returns 0, -1 for n < 2, -2 if a descent does not reach a leaf.
int orc_bvh_lines_build(const float* vertex, uint32_t n, gbsph_bvh2d_node* nodes, uint32_t* root,
                        uint32_t* sorted_keys, uint32_t* sorted_vals) {
    if (n < 2) return -1;
    // clMorton (:27-55): midpoint 0.5 * (v0 + v1), truncated, 16 bits per axis interleaved
    std::vector<uint32_t> key(n), val(n);
    for (uint32_t g = 0; g < n; g++) {
        const float cx = 0.5f * (vertex[4 * (size_t)g] + vertex[4 * (size_t)g + 2]);
        const float cy = 0.5f * (vertex[4 * (size_t)g + 1] + vertex[4 * (size_t)g + 3]);
        key[g] = code16(to_uint(cx)) | (code16(to_uint(cy)) << 1);
        val[g] = g;
    }
    // oclRadixSort on bits [0, 32): a stable sort
    std::vector<uint32_t> order(n);
    for (uint32_t i = 0; i < n; i++) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
    std::vector<uint32_t> sk(n), sv(n);
    for (uint32_t i = 0; i < n; i++) {
        sk[i] = key[order[i]];
        sv[i] = val[order[i]];
    }
    const uint32_t m = n - 1;
    // clCreateNodes (:71-95): highest differing bit, 31 down to 0
    for (uint32_t i = 0; i < m; i++) {
        uint32_t bit = 0;
        for (int b = 31; b >= 0; b--)
            if (((sk[i] >> b) & 1u) != ((sk[i + 1] >> b) & 1u)) {
                bit = (uint32_t)b;
                break;
            }
        init_node2(nodes[i], -1, -1, bit);
    }
    // clLinkNodes (:97-151)
    for (uint32_t g = 0; g < m; g++) {
        const uint32_t bit = nodes[g].bit;
        int left = -1, right = -1;
        for (int i = (int)g - 1; i >= 0; i--)
            if (nodes[i].bit > bit) {
                left = i;
                break;
            }
        for (uint32_t i = g + 1; i < m; i++)
            if (nodes[i].bit > bit) {
                right = (int)i;
                break;
            }
        if (left != -1 || right != -1) {
            if (right == -1) nodes[left].right = (int32_t)g;
            else if (left == -1) nodes[right].left = (int32_t)g;
            else if (nodes[left].bit < nodes[right].bit) nodes[left].right = (int32_t)g;
            else nodes[right].left = (int32_t)g;
        } else {
            *root = g;
        }
    }
    // clCreateLeaves (:153-184): the leaf's box is left to clComputeAABBs
    const uint32_t ls = n - 1;
    for (uint32_t g = 0; g < n; g++) {
        gbsph_bvh2d_node& L = nodes[ls + g];
        L.bit = sv[g];
        L.left = L.right = 0;
        L.trav = 0;
        if (g == 0) {
            nodes[0].left = (int32_t)(ls + g);
            continue;
        }
        if (g == ls) {
            nodes[ls - 1].right = (int32_t)(ls + g);
            continue;
        }
        if (nodes[g].left == -1) nodes[g].left = (int32_t)(g + ls);
        else if (nodes[g - 1].right == -1) nodes[g - 1].right = (int32_t)(g + ls);
    }
    // clComputeAABBs (:186-245): per segment, step down by node index until a leaf, box it,
    // then climb: the first visitor leaves trav = 2 and stops; the second swaps 2 for 3 and
    // computes the node's box from its children
    for (uint32_t g = 0; g < n; g++) {
        std::vector<uint32_t> stack;
        stack.push_back(*root);
        for (;;) {
            const gbsph_bvh2d_node& nd = nodes[stack.back()];
            stack.push_back(stack.back() >= g ? (uint32_t)nd.left : (uint32_t)nd.right);
            if (stack.size() > 2 * (size_t)n) return -2;
            gbsph_bvh2d_node& c = nodes[stack.back()];
            if (c.left == c.right) {
                const uint32_t seg = c.bit;
                float mn[2] = {FLT_MAX, FLT_MAX}, mx[2] = {-FLT_MAX, -FLT_MAX};
                for (int k = 0; k < 2; k++)
                    for (int a = 0; a < 2; a++) {
                        const float v = vertex[4 * (size_t)seg + 2 * k + a];
                        mn[a] = clmin(mn[a], v);
                        mx[a] = clmax(mx[a], v);
                    }
                std::memcpy(c.bbMin, mn, 8);
                std::memcpy(c.bbMax, mx, 8);
                break;
            }
        }
        size_t top = stack.size() - 1;
        while (top--) {
            gbsph_bvh2d_node& nd = nodes[stack[top]];
            if (nd.trav == 0) {
                nd.trav = 2;
                break;
            }
            nd.trav = 3;
            const gbsph_bvh2d_node& l = nodes[nd.left];
            const gbsph_bvh2d_node& r = nodes[nd.right];
            for (int a = 0; a < 2; a++) {
                nd.bbMin[a] = clmin(l.bbMin[a], r.bbMin[a]);
                nd.bbMax[a] = clmax(l.bbMax[a], r.bbMax[a]);
            }
        }
    }
    if (sorted_keys) std::memcpy(sorted_keys, sk.data(), 4 * (size_t)n);
    if (sorted_vals) std::memcpy(sorted_vals, sv.data(), 4 * (size_t)n);
    return 0;
}

}  // extern "C"

// ---- clCollideBVH (libCL/phys/oclFluid3D.cl:365-550), one particle at a time ---------------
// Helpers fixed as in the library: dot = ((ax bx + ay by) + az bz) + aw bw, length =
// sqrt(dot(a, a)), normalize(a) = a / length(a) per lane, cross() with w = 0.
namespace {

struct F4 {
    float x, y, z, w;
};
F4 add(F4 a, F4 b) { return {a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w}; }
F4 sub(F4 a, F4 b) { return {a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w}; }
F4 mul(F4 a, float s) { return {a.x * s, a.y * s, a.z * s, a.w * s}; }
F4 mulv(F4 a, F4 b) { return {a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w}; }
F4 divs(F4 a, float s) { return {a.x / s, a.y / s, a.z / s, a.w / s}; }
float dot(F4 a, F4 b) { return ((a.x * b.x + a.y * b.y) + a.z * b.z) + a.w * b.w; }
float len(F4 a) { return std::sqrt(dot(a, a)); }
F4 normalize(F4 a) { return divs(a, len(a)); }
F4 cross(F4 p, F4 q) { return {p.y * q.z - p.z * q.y, p.z * q.x - p.x * q.z, p.x * q.y - p.y * q.x, 0.0f}; }
F4 load(const float* v, size_t i) { return {v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]}; }
void store(float* v, size_t i, F4 a) {
    v[4 * i] = a.x;
    v[4 * i + 1] = a.y;
    v[4 * i + 2] = a.z;
    v[4 * i + 3] = a.w;
}

bool collide_triangle(uint32_t tri, const uint32_t* index, const float* vertex, F4& pos, F4& vel, F4& force,
                      const gbsph_fluid3d_params& P) {
    F4 V0 = load(vertex, index[tri]), V1 = load(vertex, index[tri + 1]), V2 = load(vertex, index[tri + 2]);
    V0.w = V1.w = V2.w = 0.0f;
    pos.w = 0.0f;
    const F4 u = sub(V1, V0), v = sub(V2, V0);
    F4 n = cross(u, v);
    if (dot(n, n) == 0.0f) return false;
    const F4 w0 = sub(pos, V0);
    const F4 disp = mul(vel, P.deltaTime);
    const float a = dot(n, w0);
    if (a < 0.0f) return false;
    const float b = dot(n, disp);
    if (std::fabs(b) < 0.000001f) return false;
    const float r = -a / b;
    if (r < 0.0f) return false;
    const F4 I = add(pos, mul(disp, r));
    const float uu = dot(u, u), uv = dot(u, v), vv = dot(v, v);
    const F4 w = sub(I, V0);
    const float wu = dot(w, u), wv = dot(w, v);
    const float D = uv * uv - uu * vv;
    const float s = (uv * wv - vv * wu) / D;
    if (s < 0.0f || s > 1.0f) return false;
    const float t = (uv * wu - uu * wv) / D;
    if (t < 0.0f || (s + t) > 1.0f) return false;
    n = normalize(n);
    const F4 Vc = sub(add(pos, disp), V0);
    const float dist = dot(Vc, n);
    const float depth = P.particleRadius - dist;
    if (depth > 0.0f) {
        const F4 dPos = mul(mul(normalize(disp), dot(n, disp)), depth);
        const F4 dTan = sub(vel, mul(n, dot(n, vel)));
        force = add(force, divs(dTan, P.deltaTime));
        const float hd = P.cellSize - dist;
        force = add(force, mul(mul(mul(mul(n, hd), hd), P.pressureConstant / P.density), P.mass));
        pos = add(pos, dPos);
        vel = {0.0f, 0.0f, 0.0f, 0.0f};
        return true;
    }
    return false;
}

bool collide_box(const gbsph_bvh_node& nd, F4 pos, F4 vel, float radius) {
    const F4 nr = normalize(vel);
    const F4 inv = {1.0f / nr.x, 1.0f / nr.y, 1.0f / nr.z, 1.0f / nr.w};
    const F4 bmin = {nd.bbMin[0], nd.bbMin[1], nd.bbMin[2], nd.bbMin[3]};
    const F4 bmax = {nd.bbMax[0], nd.bbMax[1], nd.bbMax[2], nd.bbMax[3]};
    const F4 tbot = mulv(inv, sub(bmin, pos)), ttop = mulv(inv, sub(bmax, pos));
    const float tminx = clmin(ttop.x, tbot.x), tminy = clmin(ttop.y, tbot.y), tminz = clmin(ttop.z, tbot.z);
    const float tmaxx = clmax(ttop.x, tbot.x), tmaxy = clmax(ttop.y, tbot.y), tmaxz = clmax(ttop.z, tbot.z);
    const float tnear = clmax(clmax(tminx, tminy), clmax(tminx, tminz));
    const float tfar = clmin(clmin(tmaxx, tmaxy), clmin(tmaxx, tmaxz));
    if (!(tfar > tnear)) return false;
    return tnear < clmax(radius, len(vel));
}

}  // namespace

extern "C" {

// position / velocity / force: float4[np], updated in place for the particles that collide.
void orc_bvh_collide(const gbsph_fluid3d_params* P, float* position, float* velocity, float* force, uint32_t np,
                     const gbsph_bvh_node* bvh, uint32_t root, const uint32_t* index, const float* vertex) {
    for (uint32_t p = 0; p < np; p++) {
        F4 pos = load(position, p), vel = load(velocity, p), frc = load(force, p);
        uint32_t queue[256];
        uint32_t head = 0, tail = 1;
        queue[0] = root;
        while (head != tail) {
            const uint32_t it = queue[head];
            head = (head + 1) % 256;
            const uint32_t l = (uint32_t)bvh[it].left, r = (uint32_t)bvh[it].right;
            if (l == r) {
                if (collide_triangle(bvh[it].bit * 3, index, vertex, pos, vel, frc, *P)) {
                    store(position, p, pos);
                    store(velocity, p, vel);
                    store(force, p, frc);
                    break;
                }
            } else {
                if (collide_box(bvh[l], pos, vel, P->particleRadius)) {
                    queue[tail] = l;
                    tail = (tail + 1) % 256;
                }
                if (collide_box(bvh[r], pos, vel, P->particleRadius)) {
                    queue[tail] = r;
                    tail = (tail + 1) % 256;
                }
            }
        }
    }
}

}  // extern "C"
