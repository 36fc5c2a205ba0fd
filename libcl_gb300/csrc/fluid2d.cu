// fluid2d.cu -- the reference's 2D SPH model (double-density relaxation with an image-sampled
// wall field) on sm_103a: the oclFluid2D replacement behind the C ABI.
//
// Each reference kernel of libCL/phys/oclFluid2D.cl becomes one CUDA kernel with the same
// arithmetic in the same order (round-to-nearest intrinsics, no FMA contraction, IEEE sqrt
// and division), so results reproduce the FP32 restatement bit for bit. The sort is the
// library's one-sweep radix sort on the linear cell key. The scene sizes of this model (the
// reference default is 16,384 particles in a 40 x 36 cell container) are launch-bound, so the
// whole step is replayed as a CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_fp16.h>

#include "device.cuh"
#include "internal.h"

using namespace gbsph;

namespace {

// libCL/phys/oclFluid2D.cl:121-133, the OpenCL C macros evaluated in float.
constexpr float kRestDensity = 82.0f;
constexpr float kStiffness = 0.08f;
constexpr float kNearStiffness = 0.1f;
constexpr float kSurfaceTension = 21.00035f;
constexpr float kPi = 3.1415926535f;
constexpr float kParticleRadius = 0.05f / 5;
constexpr uint32_t EMPTY2 = 0xFFFFFFFFu;

struct P2 {
    float px, py, vx, vy, mass, unused;
};

struct K2 {
    float dT, h, cW, cH, cellSize, m, psize;
    float kNorm, kNearNorm;
    int ncx, ncy;
    uint32_t n, table;
    int W, H;  // wall image size
};

__device__ __forceinline__ float fm(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fa(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fs(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fd(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float len2(float x, float y) { return __fsqrt_rn(fa(fm(x, x), fm(y, y))); }
__device__ __forceinline__ float half_round(float x) { return __half2float(__float2half_rn(x)); }

// read_imagef with normalised coordinates, linear filtering and clamp-to-edge (OpenCL C spec).
__device__ __forceinline__ float4 sample(const float4* __restrict__ img, int W, int H, float s, float t) {
    const float u = fs(fm(s, (float)W), 0.5f), v = fs(fm(t, (float)H), 0.5f);
    const float fu = floorf(u), fv = floorf(v);
    const float a = fs(u, fu), b = fs(v, fv);
    int i0 = (int)fu, j0 = (int)fv;
    int i1 = i0 + 1, j1 = j0 + 1;
    i0 = min(max(i0, 0), W - 1);
    i1 = min(max(i1, 0), W - 1);
    j0 = min(max(j0, 0), H - 1);
    j1 = min(max(j1, 0), H - 1);
    const float w00 = fm(fs(1.f, a), fs(1.f, b)), w10 = fm(a, fs(1.f, b)), w01 = fm(fs(1.f, a), b), w11 = fm(a, b);
    const float4 t00 = img[(size_t)j0 * W + i0], t10 = img[(size_t)j0 * W + i1];
    const float4 t01 = img[(size_t)j1 * W + i0], t11 = img[(size_t)j1 * W + i1];
    float4 o;
    o.x = fa(fa(fa(fm(w00, t00.x), fm(w10, t10.x)), fm(w01, t01.x)), fm(w11, t11.x));
    o.y = fa(fa(fa(fm(w00, t00.y), fm(w10, t10.y)), fm(w01, t01.y)), fm(w11, t11.y));
    o.z = fa(fa(fa(fm(w00, t00.z), fm(w10, t10.z)), fm(w01, t01.z)), fm(w11, t11.z));
    o.w = fa(fa(fa(fm(w00, t00.w), fm(w10, t10.w)), fm(w01, t01.w)), fm(w11, t11.w));
    return o;
}

// clAdvanceState (libCL/phys/oclFluid2D.cl:173-182) fused with clHash (:61-69) and the
// digit histogram of the sort. Cell coordinates are clamped to the grid.
__global__ void k2_advance_hash(P2* __restrict__ st, float2* __restrict__ prev, uint32_t* __restrict__ keys,
                                uint32_t* __restrict__ hist, K2 k, int end_bit) {
    __shared__ uint32_t s_h[SORT_MAX_PASSES * SORT_RADIX];
    for (int i = threadIdx.x; i < SORT_MAX_PASSES * SORT_RADIX; i += blockDim.x) s_h[i] = 0;
    __syncthreads();
    const int passes = sort_passes(0, end_bit);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < k.n; i += gridDim.x * blockDim.x) {
        P2 p = st[i];
        prev[i] = make_float2(p.px, p.py);
        p.vx = fa(p.vx, fm(0.0f, k.dT));
        p.vy = fa(p.vy, fm(-9.81f, k.dT));
        p.px = fa(p.px, fm(p.vx, k.dT));
        p.py = fa(p.py, fm(p.vy, k.dT));
        st[i] = p;
        const int gx = min(max((int)floorf(fd(p.px, k.cellSize)), 0), k.ncx - 1);
        const int gy = min(max((int)floorf(fd(p.py, k.cellSize)), 0), k.ncy - 1);
        const uint32_t key = (uint32_t)(gy * k.ncx + gx);
        keys[i] = key;
        for (int q = 0; q < passes; ++q) {
            const int shift = q * SORT_RADIX_BITS;
            const int bits = min(SORT_RADIX_BITS, end_bit - shift);
            atomicAdd(&s_h[q * SORT_RADIX + ((key >> shift) & ((1u << bits) - 1u))], 1u);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * SORT_RADIX; i += blockDim.x)
        if (s_h[i]) atomicAdd(&hist[i], s_h[i]);
}

// clReorder (libCL/phys/oclFluid2D.cl:71-76): 24-byte particles.
__global__ void k2_reorder(const uint32_t* __restrict__ index, const P2* __restrict__ st, P2* __restrict__ srt, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) srt[i] = st[index[i]];
}

__device__ __forceinline__ void cells_of(const K2& k, float px, float py, int& x0, int& x1, int& y0, int& y1) {
    const int gx = (int)floorf(fd(px, k.cellSize)), gy = (int)floorf(fd(py, k.cellSize));
    x0 = max(gx - 1, 0);
    x1 = min(gx + 1, k.ncx - 1);
    y0 = max(gy - 1, 0);
    y1 = min(gy + 1, k.ncy - 1);
}

// The neighbour loops of clComputePressure / clComputePosition visit cells x = x0..x1 (outer),
// y = y0..y1 (inner) and the particles of each cell in sorted order, summing in that order.
// Here a warp takes one particle: the candidates (the cells' ranges, concatenated in the
// reference's order) are dealt to the lanes 32 at a time, each lane computes its candidate's
// terms, and the sums take the in-range terms one by one in candidate order (broadcast by
// shuffles), so every operation and its order are the reference's.
struct Cand2 {
    uint32_t pre;    // lane c < 9: candidates before cell c (of the concatenation)
    uint32_t start;  // lane c < 9: the cell's first sorted index
    uint32_t total;  // candidates of all cells (every lane)
};

__device__ __forceinline__ Cand2 cand2_setup(const K2& k, float px, float py, const uint32_t* __restrict__ cs,
                                             const uint32_t* __restrict__ ce) {
    const uint32_t lane = threadIdx.x & 31u;
    int x0, x1, y0, y1;
    cells_of(k, px, py, x0, x1, y0, y1);
    const int ny = y1 - y0 + 1, nc = (x1 - x0 + 1) * ny;
    uint32_t len = 0, st = 0;
    if ((int)lane < nc) {
        const int c = (y0 + (int)lane % ny) * k.ncx + x0 + (int)lane / ny;  // x outer, y inner
        st = cs[c];
        if (st != EMPTY2) len = ce[c] - st;
    }
    uint32_t incl = len;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if ((int)lane >= o) incl += v;
    }
    Cand2 c;
    c.pre = incl - len;
    c.start = st;
    c.total = __shfl_sync(0xffffffffu, incl, 8);
    return c;
}

// Sorted index of candidate k < total (from the per-cell values held by lanes 0..8).
__device__ __forceinline__ uint32_t cand2_index(const Cand2& c, uint32_t k) {
    uint32_t j = 0;
#pragma unroll
    for (int q = 0; q < 9; ++q) {
        const uint32_t pre = __shfl_sync(0xffffffffu, c.pre, q), st = __shfl_sync(0xffffffffu, c.start, q);
        if (k >= pre) j = st + (k - pre);
    }
    return j;
}

// clComputePressure (libCL/phys/oclFluid2D.cl:185-245), a warp per particle.
__global__ void k2_pressure(const P2* __restrict__ srt, float4* __restrict__ ps, const uint32_t* __restrict__ cs,
                            const uint32_t* __restrict__ ce, const float4* __restrict__ bstate, K2 k) {
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (i >= k.n) return;  // whole warps
    const P2 pi = srt[i];
    float density = 0.f, nearDensity = 0.f;
    const float4 wall = sample(bstate, k.W, k.H, fd(pi.px, k.cW), fd(pi.py, k.cH));
    if (wall.x != 0.f) {
        density = fa(density, wall.x);
        nearDensity = fa(nearDensity, wall.y);
    }
    const Cand2 c = cand2_setup(k, pi.px, pi.py, cs, ce);
    for (uint32_t base = 0; base < c.total; base += 32) {
        const uint32_t kk = base + lane;
        const uint32_t j = cand2_index(c, kk);
        bool in = false;
        float td = 0.f, tn = 0.f;
        if (kk < c.total && j != i) {
            const float dx = fs(srt[j].px, pi.px), dy = fs(srt[j].py, pi.py);
            const float r = len2(dx, dy);
            if (r > 0.0000001f && r < k.h) {
                const float a = fs(1.f, fd(r, k.h));
                td = fm(fm(fm(fm(k.m, a), a), a), k.kNorm);
                tn = fm(fm(fm(fm(fm(k.m, a), a), a), a), k.kNearNorm);
                in = true;
            }
        }
        for (uint32_t m = __ballot_sync(0xffffffffu, in); m; m &= m - 1) {
            const int b = __ffs(m) - 1;
            density = fa(density, __shfl_sync(0xffffffffu, td, b));
            nearDensity = fa(nearDensity, __shfl_sync(0xffffffffu, tn, b));
        }
    }
    if (lane == 0)
        ps[i] = make_float4(density, nearDensity, fm(kStiffness, fs(density, fm(k.m, kRestDensity))),
                            fm(kNearStiffness, nearDensity));
}

// clComputePosition (libCL/phys/oclFluid2D.cl:247-326), a warp per particle. The reference's
// viscosity term uses vel_j - vel_j (:299), which is zero, so it never contributes and is not
// evaluated here.
__global__ void k2_position(const P2* __restrict__ srt, const float4* __restrict__ ps, float2* __restrict__ relaxed,
                            const uint32_t* __restrict__ cs, const uint32_t* __restrict__ ce,
                            const float4* __restrict__ bstate, const float4* __restrict__ bvec, K2 k) {
    const uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31u;
    if (i >= k.n) return;  // whole warps
    const float4 si = ps[i];
    const P2 pi = srt[i];
    float rx = pi.px, ry = pi.py;
    const float dt2 = fm(k.dT, k.dT);
    const Cand2 c = cand2_setup(k, pi.px, pi.py, cs, ce);
    for (uint32_t base = 0; base < c.total; base += 32) {
        const uint32_t kk = base + lane;
        const uint32_t j = cand2_index(c, kk);
        bool in = false;
        float ux = 0.f, uy = 0.f, wx = 0.f, wy = 0.f;
        if (kk < c.total && j != i) {
            const float dx = fs(srt[j].px, pi.px), dy = fs(srt[j].py, pi.py);
            const float r = len2(dx, dy);
            if (r > 0.0000001f && r < k.h) {
                const float4 sj = ps[j];
                const float a = fs(1.f, fd(r, k.h));
                const float near = fm(fm(fm(fm(fa(si.w, sj.w), a), a), a), k.kNearNorm);
                const float far = fm(fm(fm(fa(si.z, sj.z), a), a), k.kNorm);
                const float d = fd(fm(dt2, fa(near, far)), 2.f);
                const float rm = fm(r, k.m);
                ux = fd(fm(dx, d), rm);
                uy = fd(fm(dy, d), rm);
                const float surf = fd(fm(fm(fm(dt2, fd(kSurfaceTension, k.m)), k.m),
                                         fa(fm(fm(fm(a, a), a), k.kNearNorm), fm(fm(a, a), k.kNorm))), 2.f);
                wx = fm(surf, dx);
                wy = fm(surf, dy);
                in = true;
            }
        }
        for (uint32_t m = __ballot_sync(0xffffffffu, in); m; m &= m - 1) {
            const int b = __ffs(m) - 1;
            rx = fs(rx, __shfl_sync(0xffffffffu, ux, b));
            ry = fs(ry, __shfl_sync(0xffffffffu, uy, b));
            rx = fa(rx, __shfl_sync(0xffffffffu, wx, b));
            ry = fa(ry, __shfl_sync(0xffffffffu, wy, b));
        }
    }
    if (lane != 0) return;
    const float4 wall = sample(bstate, k.W, k.H, fd(rx, k.cW), fd(ry, k.cH));
    if (wall.x != 0.f) {
        const float4 normal = sample(bvec, k.W, k.H, fd(rx, k.cW), fd(ry, k.cH));
        const float a = fs(1.f, fd(normal.z, k.h));
        const float near = fm(fm(fm(fm(fa(si.w, wall.w), a), a), a), k.kNearNorm);
        const float far = fm(fm(fm(fa(si.z, wall.z), a), a), k.kNorm);
        const float d = fd(fm(dt2, fa(near, far)), 2.f);
        rx = fa(rx, fd(fm(normal.x, d), k.m));
        ry = fa(ry, fd(fm(normal.y, d), k.m));
    }
    relaxed[i] = make_float2(rx, ry);
}

// clUpdateState (libCL/phys/oclFluid2D.cl:329-339).
__global__ void k2_update(P2* __restrict__ st, const float2* __restrict__ prev, const float2* __restrict__ relaxed,
                          const uint32_t* __restrict__ index, K2 k) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= k.n) return;
    const uint32_t o = index[i];
    const float2 pr = prev[o], rl = relaxed[i];
    float dx = fs(rl.x, pr.x), dy = fs(rl.y, pr.y);
    const float l = len2(dx, dy);
    const float cap = fm(4.0f, k.psize);
    const float lim = (cap < l) ? cap : l;  // min(l, 4 * particleSize) with the restatement's NaN rule
    dx = fd(fm(dx, lim), l);
    dy = fd(fm(dy, lim), l);
    P2 p = st[o];
    p.vx = fd(dx, k.dT);
    p.vy = fd(dy, k.dT);
    p.px = fa(pr.x, dx);
    p.py = fa(pr.y, dy);
    st[o] = p;
}

// clComputeBorder (libCL/phys/oclFluid2D.cl:358-443), one thread per pixel.
__global__ void k2_border(const float4* __restrict__ mask, int w, int h, float4* __restrict__ vout,
                          float4* __restrict__ sout, K2 k, float s) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= w || y >= h) return;
    const float pw = mask[(size_t)y * w + x].w;
    const int dW = (int)((double)fd(fm((float)w, k.h), k.cW) + 0.5);
    const int dH = (int)((double)fd(fm((float)h, k.h), k.cH) + 0.5);
    const float dX = fd(k.cW, (float)w), dY = fd(k.cH, (float)h);
    float dmin = 10000.f;
    float4 vec = make_float4(0.f, 0.f, 0.f, 0.f);
    float density = 0.f, nearDensity = 0.f;
    if (pw == 1.0f) {
        density = fm(fm(112.f, k.m), k.kNorm);
        nearDensity = fm(fm(112.f, k.m), k.kNearNorm);
        for (int i = max(x - dW, 0); i < min(x + dW, w); i++)
            for (int j = max(y - dH, 0); j < min(y + dH, h); j++) {
                if (mask[(size_t)j * w + i].w != 1.0f) {
                    const float dx = fs(fm((float)i, dX), fm((float)x, dX)), dy = fs(fm((float)j, dY), fm((float)y, dY));
                    const float r = len2(dx, dy);
                    if (r < dmin) {
                        vec.x = fd(dx, r);
                        vec.y = fd(dy, r);
                        vec.z = r;
                        dmin = r;
                    }
                }
            }
    } else {
        for (int i = max(x - dW, 0); i < min(x + dW, w); i++)
            for (int j = max(y - dH, 0); j < min(y + dH, h); j++) {
                if (mask[(size_t)j * w + i].w == 1.0f) {
                    const float dx = fs(fm((float)x, dX), fm((float)i, dX)), dy = fs(fm((float)y, dY), fm((float)j, dY));
                    const float r = len2(dx, dy);
                    if (r < k.h) {
                        const float a = fs(1.f, fd(r, k.h));
                        density = fa(density, fm(fm(fm(fm(fm(s, k.m), a), a), a), k.kNorm));
                        nearDensity = fa(nearDensity, fm(fm(fm(fm(fm(fm(s, k.m), a), a), a), a), k.kNearNorm));
                        if (r < dmin) {
                            vec.x = fd(dx, r);
                            vec.y = fd(dy, r);
                            vec.z = r;
                            dmin = r;
                        }
                    }
                }
            }
    }
    vout[(size_t)y * w + x] = make_float4(half_round(vec.x), half_round(vec.y), half_round(vec.z), half_round(vec.w));
    sout[(size_t)y * w + x] = make_float4(half_round(density), half_round(nearDensity),
                                          half_round(fm(kStiffness, fs(density, fm(k.m, kRestDensity)))),
                                          half_round(fm(kNearStiffness, nearDensity)));
}

int grid1(uint32_t n) { return (int)((n + 255) / 256); }

// clEmitter (libCL/phys/oclFluid2D.cl:342-352): particle emit+1 enters at x = 1 on one of
// four heights, with velocity (25, 1); the sixth field (`age` there) is set to 1.
__global__ void k2_emitter(P2* __restrict__ state, uint32_t n, uint32_t emit, float psize) {
    const uint32_t particle = blockIdx.x * blockDim.x + threadIdx.x;
    if (particle >= n) return;
    if (particle > emit && particle < emit + 2u) {
        P2 q = state[particle];
        q.px = 1.0f;
        q.py = __fadd_rn(14.0f, __fmul_rn((float)(particle % 4u * 12u), psize));
        q.vx = 25.0f;
        q.vy = 1.0f;
        q.unused = 1.0f;
        state[particle] = q;
    }
}

}  // namespace

struct gbsph_fluid2d_s {
    int device = 0;
    gbsph_fluid2d_params params{};
    bool compiled = false;
    size_t n = 128 * 128;
    void* state = nullptr;  // P2[n]
    bool state_owned = true;
    size_t state_count = 0;
    void* block = nullptr;  // internal per-particle arrays
    P2* sorted = nullptr;
    float4* pstate = nullptr;
    float2* relaxed = nullptr;
    float2* prev = nullptr;
    uint32_t *keys_a = nullptr, *keys_b = nullptr, *keys_c = nullptr, *vals_a = nullptr, *vals_b = nullptr, *index = nullptr;
    uint32_t* cs = nullptr;  // cell start / end, `table` entries each
    uint32_t* ce = nullptr;
    uint32_t table = 256;
    float4* bstate = nullptr;  // wall images W x H
    float4* bvec = nullptr;
    int W = 256, Hh = 256;
    void* scratch = nullptr;
    uint32_t* err = nullptr;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::vector<char> gkey;
    std::string last_error;
};

namespace {

using H2 = gbsph_fluid2d_s;

void default_params2d(gbsph_fluid2d_params* p) {
    // clInitFluid, libCL/phys/oclFluid2D.cl:136-151 (vmax and B are never set there)
    std::memset(p, 0, sizeof(*p));
    const float kH = (22 * 0.05f / 5);
    p->dT = (float)0.00433333333;
    p->h = kH;
    p->containerW = (float)17.68;
    p->containerH = (float)15.76;
    p->cellSize = 2 * p->h;
    p->cellCountX = (int)((double)(p->containerW / p->cellSize) + 0.5);
    p->cellCountY = (int)((double)(p->containerH / p->cellSize) + 0.5);
    p->particleSize = kParticleRadius;
    p->particleMass = 0.7f;
    p->p0 = kRestDensity;
}

K2 make_k2(const H2* h) {
    const gbsph_fluid2d_params& p = h->params;
    K2 k;
    std::memset(&k, 0, sizeof(k));
    k.dT = p.dT;
    k.h = p.h;
    k.cW = p.containerW;
    k.cH = p.containerH;
    k.cellSize = p.cellSize;
    k.m = p.particleMass;
    k.psize = p.particleSize;
    // kNorm / kNearNorm are macros of the compile-time kH (libCL/phys/oclFluid2D.cl:129-133)
    const float kH = (22 * 0.05f / 5);
    k.kNorm = (20 / (2 * kPi * kH * kH));
    k.kNearNorm = (30 / (2 * kPi * kH * kH));
    k.ncx = p.cellCountX;
    k.ncy = p.cellCountY;
    k.n = (uint32_t)h->n;
    k.table = h->table;
    k.W = h->W;
    k.H = h->Hh;
    return k;
}

void invalidate2(H2* h) {
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    h->gkey.clear();
}

int alloc_arrays2(H2* h, size_t n) {
    if (h->block) cudaFree(h->block);
    if (h->scratch) cudaFree(h->scratch);
    h->block = h->scratch = nullptr;
    const size_t n4 = (n + 63) & ~size_t(63);
    const size_t bytes = n4 * (24 + 16 + 8 + 8 + 6 * 4);
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->block, bytes));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->block, 0, bytes));
    char* p = (char*)h->block;
    h->pstate = (float4*)p;
    p += n4 * 16;
    h->sorted = (P2*)p;
    p += n4 * 24;
    h->relaxed = (float2*)p;
    p += n4 * 8;
    h->prev = (float2*)p;
    p += n4 * 8;
    uint32_t** arr[6] = {&h->keys_a, &h->keys_b, &h->keys_c, &h->vals_a, &h->vals_b, &h->index};
    for (auto a : arr) {
        *a = (uint32_t*)p;
        p += n4 * 4;
    }
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->scratch, onesweep_scratch_bytes((uint32_t)n, SORT_MAX_PASSES)));
    return GBSPH_OK;
}

int alloc_state2(H2* h, size_t n) {
    if (h->state_owned && h->state) cudaFree(h->state);
    h->state = nullptr;
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->state, std::max<size_t>(n, 1) * 24));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->state, 0, std::max<size_t>(n, 1) * 24));
    h->state_owned = true;
    h->state_count = n;
    return GBSPH_OK;
}

int alloc_border2(H2* h, int w, int hh) {
    if (h->bstate) cudaFree(h->bstate);
    if (h->bvec) cudaFree(h->bvec);
    h->bstate = h->bvec = nullptr;
    const size_t bytes = (size_t)w * hh * sizeof(float4);
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->bstate, bytes));
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->bvec, bytes));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->bstate, 0, bytes));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->bvec, 0, bytes));
    h->W = w;
    h->Hh = hh;
    invalidate2(h);
    return GBSPH_OK;
}

int alloc_table2(H2* h) {
    const gbsph_fluid2d_params& p = h->params;
    const uint32_t t = (uint32_t)(p.cellCountX * p.cellCountY) / 256 * 256 + 256;
    if (h->cs && t == h->table) return GBSPH_OK;
    if (h->cs) cudaFree(h->cs);
    h->cs = h->ce = nullptr;
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->cs, 2 * (size_t)t * 4));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->cs, 0xFF, 2 * (size_t)t * 4));
    h->ce = h->cs + t;
    h->table = t;
    invalidate2(h);
    return GBSPH_OK;
}

int bits_for2(uint64_t cells) {
    int b = 0;
    while (b < 32 && (1ull << b) < cells) b++;
    return std::max(b, 1);
}

#define RC2(x)                \
    do {                      \
        int _rc = (x);        \
        if (_rc) return _rc;  \
    } while (0)

int enqueue2(H2* h, const K2& k, cudaStream_t s) {
    const int end_bit = bits_for2((uint64_t)h->params.cellCountX * h->params.cellCountY);
    const int P = sort_passes(0, end_bit);
    GBSPH_CUDA_TRY(&h->last_error, onesweep_prepare(h->scratch, k.n, P, s));
    const int blocks = std::max(1, std::min(grid1(k.n), num_sms() * 8));
    k2_advance_hash<<<blocks, 256, 0, s>>>((P2*)h->state, h->prev, h->keys_a, (uint32_t*)h->scratch, k, end_bit);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    OnesweepArgs a;
    a.keys_in = h->keys_a;
    a.keys_out = h->keys_c;
    a.vals_out = h->index;
    a.tmp_keys[0] = h->keys_b;
    a.tmp_vals[0] = h->vals_b;
    a.tmp_keys[1] = h->keys_a;
    a.tmp_vals[1] = h->vals_a;
    a.n = k.n;
    a.start_bit = 0;
    a.end_bit = end_bit;
    a.scratch = h->scratch;
    a.err = h->err;
    GBSPH_CUDA_TRY(&h->last_error, onesweep_passes(a, s));
    k2_reorder<<<grid1(k.n), 256, 0, s>>>(h->index, (const P2*)h->state, h->sorted, k.n);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    GBSPH_CUDA_TRY(&h->last_error, cell_bounds_launch(h->keys_c, k.n, h->cs, h->ce, h->table, h->err, s));
    const unsigned wgrid = (unsigned)(((size_t)k.n * 32 + 255) / 256);  // a warp per particle
    k2_pressure<<<wgrid, 256, 0, s>>>(h->sorted, h->pstate, h->cs, h->ce, h->bstate, k);
    k2_position<<<wgrid, 256, 0, s>>>(h->sorted, h->pstate, h->relaxed, h->cs, h->ce, h->bstate, h->bvec, k);
    k2_update<<<grid1(k.n), 256, 0, s>>>((P2*)h->state, h->prev, h->relaxed, h->index, k);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

int validate2(H2* h) {
    const gbsph_fluid2d_params& p = h->params;
    const float v[9] = {p.dT, p.h, p.containerW, p.containerH, p.cellSize, p.particleSize, p.particleMass, p.p0, 0.f};
    for (float x : v)
        if (!std::isfinite(x)) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "parameters hold a NaN or infinity");
    if (!(p.cellSize > 0.f) || !(p.h > 0.f) || !(p.containerW > 0.f) || !(p.containerH > 0.f))
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "cellSize, h and the container must be > 0");
    if (p.cellCountX < 1 || p.cellCountY < 1 || (int64_t)p.cellCountX * p.cellCountY > (1 << 24))
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "cell counts must be in [1, 2^24] cells");
    return GBSPH_OK;
}

}  // namespace

extern "C" {

GBSPH_API int gbsph_fluid2d_default_params(gbsph_fluid2d_params* p) {
    if (!p) return GBSPH_ERR_ARGUMENT;
    default_params2d(p);
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid2d_create(gbsph_fluid2d_t* out) {
    if (!out) return GBSPH_ERR_ARGUMENT;
    *out = nullptr;
    H2* h = new H2();
    int rc = GBSPH_OK;
    if (cudaGetDevice(&h->device) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMalloc(&h->err, 256) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMemset(h->err, 0, 256) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    default_params2d(&h->params);
    if (!rc) rc = alloc_arrays2(h, h->n);
    if (!rc) rc = alloc_state2(h, h->n);
    if (!rc) rc = alloc_border2(h, 256, 256);
    if (!rc) rc = alloc_table2(h);
    if (rc) {
        cudaGetLastError();
        gbsph_fluid2d_destroy(h);
        return rc;
    }
    *out = h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid2d_destroy(gbsph_fluid2d_t h) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    cudaSetDevice(h->device);
    invalidate2(h);
    if (h->state_owned && h->state) cudaFree(h->state);
    void* ptrs[6] = {h->block, h->scratch, h->cs, h->bstate, h->bvec, h->err};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    delete h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid2d_compile(gbsph_fluid2d_t h) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    default_params2d(&h->params);
    RC2(alloc_table2(h));
    h->compiled = true;
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid2d_set_particle_count(gbsph_fluid2d_t h, size_t n) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (n == 0 || n > SORT_MAX_KEYS - SORT_TILE) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "bad particle count");
    if (!h->state_owned && h->state_count != n)
        return fail(&h->last_error, GBSPH_ERR_SIZE_MISMATCH, "borrowed state buffer does not hold n particles");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    invalidate2(h);
    h->n = n;
    RC2(alloc_arrays2(h, n));
    if (h->state_owned) RC2(alloc_state2(h, n));
    return GBSPH_OK;
}

GBSPH_API size_t gbsph_fluid2d_get_particle_count(gbsph_fluid2d_t h) { return h ? h->n : 0; }

GBSPH_API int gbsph_fluid2d_set_state_buffer(gbsph_fluid2d_t h, void* device_ptr, size_t count) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!device_ptr || (uintptr_t)device_ptr % 8) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null or misaligned state buffer");
    if (count != h->n)
        return fail(&h->last_error, GBSPH_ERR_SIZE_MISMATCH,
                    "state buffer holds " + std::to_string(count) + " particles, count is " + std::to_string(h->n));
    if (h->state_owned && h->state) {
        cudaSetDevice(h->device);
        cudaFree(h->state);
    }
    h->state = device_ptr;
    h->state_owned = false;
    h->state_count = count;
    invalidate2(h);
    return GBSPH_OK;
}

GBSPH_API void* gbsph_fluid2d_get_buffer(gbsph_fluid2d_t h, int which, size_t* count) {
    if (!h) return nullptr;
    size_t c = h->n;
    void* p = nullptr;
    switch (which) {
        case GBSPH2D_BUF_STATE: p = h->state; break;
        case GBSPH2D_BUF_SORTED_STATE: p = h->sorted; break;
        case GBSPH2D_BUF_INDEX: p = h->index; break;
        case GBSPH2D_BUF_CELL: p = h->keys_c; break;
        case GBSPH2D_BUF_PRESSURE: p = h->pstate; break;
        case GBSPH2D_BUF_RELAXED: p = h->relaxed; break;
        case GBSPH2D_BUF_PREVIOUS: p = h->prev; break;
        case GBSPH2D_BUF_BORDER_STATE: p = h->bstate; c = (size_t)h->W * h->Hh; break;
        case GBSPH2D_BUF_BORDER_VECTOR: p = h->bvec; c = (size_t)h->W * h->Hh; break;
        default: return nullptr;
    }
    if (count) *count = c;
    return p;
}

GBSPH_API gbsph_fluid2d_params* gbsph_fluid2d_get_params(gbsph_fluid2d_t h) { return h ? &h->params : nullptr; }

GBSPH_API int gbsph_fluid2d_compute_border(gbsph_fluid2d_t h, const float* mask, int width, int height, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!mask || width < 1 || height < 1 || (int64_t)width * height > (1 << 26))
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "bad wall mask");
    RC2(validate2(h));
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    if (width != h->W || height != h->Hh) RC2(alloc_border2(h, width, height));
    const K2 k = make_k2(h);
    const gbsph_fluid2d_params& p = h->params;
    const float dX = p.containerW / width, dY = p.containerH / height;
    const float s = (float)((double)(dX * dY) / (2 * M_PI * (double)p.particleSize * (double)p.particleSize));
    const dim3 blk(16, 16), grd((width + 15) / 16, (height + 15) / 16);
    k2_border<<<grd, blk, 0, (cudaStream_t)stream>>>((const float4*)mask, width, height, h->bvec, h->bstate, k, s);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid2d_emit(gbsph_fluid2d_t h, uint32_t emit, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!h->compiled) return fail(&h->last_error, GBSPH_ERR_NOT_COMPILED, "emit before compile()");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    k2_emitter<<<(unsigned)((h->n + 255) / 256), 256, 0, (cudaStream_t)stream>>>((P2*)h->state, (uint32_t)h->n, emit,
                                                                                h->params.particleSize);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid2d_compute(gbsph_fluid2d_t h, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!h->compiled) return fail(&h->last_error, GBSPH_ERR_NOT_COMPILED, "compute() before compile()");
    RC2(validate2(h));
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    RC2(alloc_table2(h));
    const K2 k = make_k2(h);
    std::vector<char> key(sizeof(K2) + 2 * sizeof(void*));
    std::memcpy(key.data(), &k, sizeof(K2));
    std::memcpy(key.data() + sizeof(K2), &h->state, sizeof(void*));
    std::memcpy(key.data() + sizeof(K2) + sizeof(void*), &h->bstate, sizeof(void*));
    if (!h->gexec || key != h->gkey) {
        invalidate2(h);
        GBSPH_CUDA_TRY(&h->last_error, cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue2(h, k, h->cap_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(h->cap_stream, &g);
        if (rc || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            return rc ? rc : fail(&h->last_error, GBSPH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        }
        const cudaError_t ie = cudaGraphInstantiate(&h->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            h->gexec = nullptr;
            return fail(&h->last_error, GBSPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        }
        h->gkey = key;
    }
    GBSPH_CUDA_TRY(&h->last_error, cudaGraphLaunch(h->gexec, (cudaStream_t)stream));
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid2d_get_cell_bounds(gbsph_fluid2d_t h, uint32_t* cell_start, uint32_t* cell_end,
                                            size_t n_cells, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!cell_start || !cell_end || n_cells != h->table)
        return fail(&h->last_error, GBSPH_ERR_SIZE_MISMATCH, "n_cells must equal the table size");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    cudaStream_t s = (cudaStream_t)stream;
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(cell_start, h->cs, n_cells * 4, cudaMemcpyDeviceToDevice, s));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(cell_end, h->ce, n_cells * 4, cudaMemcpyDeviceToDevice, s));
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid2d_sync_status(gbsph_fluid2d_t h, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t bits = 0;
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpy(&bits, h->err, 4, cudaMemcpyDeviceToHost));
    if (bits) {
        GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->err, 0, 4));
        return fail(&h->last_error, dev_err_to_status(bits), "device error word 0x" + std::to_string(bits));
    }
    return GBSPH_OK;
}

GBSPH_API const char* gbsph_fluid2d_last_error(gbsph_fluid2d_t h) { return h ? h->last_error.c_str() : "null handle"; }

}  // extern "C"
