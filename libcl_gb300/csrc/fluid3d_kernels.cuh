// fluid3d_kernels.cuh -- device code of the 3D (and 2D poly6/spiky) SPH step.
//
// Two families of neighbour kernels:
//   * "exact" kernels (thread per sorted particle) restate clCalculateDensity /
//     clCalculateForces (libCL/phys/oclFluid3D.cl:150-255) operation for operation with
//     round-to-nearest intrinsics (no FMA contraction, IEEE sqrt and division), visiting the
//     27 (or 9) neighbour cells in the reference's z, y, x order. In REFERENCE_HASH mode that
//     includes visiting a bucket twice when two neighbour cells hash to it. They reproduce the
//     FP32 restatement bit for bit and serve the parity modes.
//   * "brick" kernels (LINEAR_GRID only) are the fast path. A persistent CTA takes a brick of
//     W cells along x, loads the cell table of the 9 (or 3) neighbour rows, copies those rows'
//     contiguous particle ranges into shared memory with cp.async.bulk on one mbarrier, and
//     each warp evaluates one target cell: lanes = (target, candidate stride) so candidate
//     loads are shared-memory broadcasts; partial sums are combined with shuffles. FMA and
//     rsqrt are used, so results agree with the restatement within FP32 tolerance.
#pragma once

#include "device.cuh"
#include "internal.h"

namespace gbsph {

constexpr uint32_t EMPTY = 0xFFFFFFFFu;
constexpr uint32_t REF_BUCKETS = 262144u;  // BUCKETS, libCL/phys/oclFluid3D.cl:32
constexpr int BRICK_THREADS = 256;
constexpr int BRICK_WARPS = BRICK_THREADS / 32;
constexpr int BRICK_W_MAX = 16;
constexpr int BRICK_SLOTS = BRICK_W_MAX + 2;

// One scene of a batch (LINEAR_GRID): its particles, cells and bricks are consecutive ranges
// of the batch's arrays, and its gas constant, viscosity, box and grid are its own.
struct SceneDev {
    uint32_t part_off, cell_off, brick_off, n;
    int nx, ny, nz, bxn;
    float4 origin, box_min, box_max;
    float stiff, cvisc, pad0, pad1;
};

// Kernel-side parameters, passed by value.
struct KParams {
    float dt, radius, h, mass, p0, rho0, stiff, cvisc, cpress, kconst, vlimit;
    float h2;         // h*h
    float r2_thresh;  // smallest float x with sqrtf(x) >= h, so (sqrtf(r2) < h) == (r2 < r2_thresh)
    float4 gravity, box_min, box_max, origin;
    int nx, ny, nz;
    int key_mode, dims;
    int end_bit;     // sort bits [0, end_bit)
    int digit_bits;  // sort digit width (bits per pass)
    int bw, bxn;  // brick width (cells) and bricks per x row
    uint32_t n;
    uint32_t table_cells;
    const SceneDev* scenes;  // batches only: n_scenes entries, sorted by part/cell/brick offsets
    int n_scenes;
    float4* rec_force;  // when set: receives each particle's force after the clip box, before the clamp
    // When set (brick kernels): slot *rec_slot of rec_nbr (rec_n4 * NBR_CAP words per slot)
    // receives each particle's in-range neighbours (itself included) as sorted indices,
    // NBR_CAP per particle, and slot *rec_slot of rec_cnt (rec_n4 words) their number, or
    // REC_SCAN where the list overflowed or the brick was not staged.
    uint32_t* rec_nbr;
    uint32_t* rec_cnt;
    const uint32_t* rec_slot;
    uint32_t rec_n4;
};

// Index of the scene whose range [off, next off) holds v (binary search over `n` scenes).
template <int FIELD>
__device__ __forceinline__ int scene_of(const SceneDev* __restrict__ sc, int n, uint32_t v) {
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const uint32_t o = FIELD == 0 ? sc[mid].part_off : (FIELD == 1 ? sc[mid].cell_off : sc[mid].brick_off);
        if (o <= v) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// ---- keys ---------------------------------------------------------------------------------

// gridPosition (libCL/phys/oclFluid3D.cl:34-42); LINEAR_GRID subtracts the grid origin.
__device__ __forceinline__ void grid_position(const KParams& kp, float4 p, int& gx, int& gy, int& gz) {
    if (kp.key_mode == GBSPH_KEY_LINEAR_GRID) {
        p.x = __fsub_rn(p.x, kp.origin.x);
        p.y = __fsub_rn(p.y, kp.origin.y);
        p.z = __fsub_rn(p.z, kp.origin.z);
    }
    gx = (int)floorf(__fdiv_rn(p.x, kp.h));
    gy = (int)floorf(__fdiv_rn(p.y, kp.h));
    gz = kp.dims == 2 ? 0 : (int)floorf(__fdiv_rn(p.z, kp.h));
}

// hashKey (libCL/phys/oclFluid3D.cl:44-52).
__device__ __forceinline__ uint32_t hash_key(int x, int y, int z) {
    uint32_t n = (73856093u * (uint32_t)x) ^ (19349663u * (uint32_t)y) ^ (83492791u * (uint32_t)z);
    return n % REF_BUCKETS;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return min(max(v, lo), hi); }

__device__ __forceinline__ uint32_t linear_key(const KParams& kp, int x, int y, int z) {
    x = clampi(x, 0, kp.nx - 1);
    y = clampi(y, 0, kp.ny - 1);
    z = clampi(z, 0, kp.nz - 1);
    return (uint32_t)x + (uint32_t)kp.nx * ((uint32_t)y + (uint32_t)kp.ny * (uint32_t)z);
}

__device__ __forceinline__ uint32_t particle_key(const KParams& kp, float4 p) {
    int gx, gy, gz;
    grid_position(kp, p, gx, gy, gz);
    return kp.key_mode == GBSPH_KEY_LINEAR_GRID ? linear_key(kp, gx, gy, gz) : hash_key(gx, gy, gz);
}

// clHash (libCL/phys/oclFluid3D.cl:57-64) fused with the digit histogram of every sort pass
// (the index is implicit: the first sort pass generates values 0..n-1). With CLEAR, the
// linear cell table entries of the previous step's occupied cells are reset (the previous
// sorted keys are still in `prev_keys`), replacing a full fill of the table.
template <bool CLEAR>
__global__ void __launch_bounds__(256) k_hash(const float4* __restrict__ pos, KParams kp,
                                              uint32_t* __restrict__ keys,
                                              uint32_t* __restrict__ hist,
                                              const uint32_t* __restrict__ prev_keys,
                                              uint2* __restrict__ table) {
    __shared__ uint32_t s_h[SORT_MAX_PASSES * SORT_RADIX];
    for (int i = threadIdx.x; i < SORT_MAX_PASSES * SORT_RADIX; i += blockDim.x) s_h[i] = 0;
    __syncthreads();
    const int passes = sort_passes(0, kp.end_bit, kp.digit_bits);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < kp.n; i += gridDim.x * blockDim.x) {
        const uint32_t k = particle_key(kp, pos[i]);
        keys[i] = k;
        for (int p = 0; p < passes; ++p) {
            const int shift = p * kp.digit_bits;
            const int bits = min(kp.digit_bits, kp.end_bit - shift);
            atomicAdd(&s_h[p * SORT_RADIX + ((k >> shift) & ((1u << bits) - 1u))], 1u);
        }
        if (CLEAR) {
            const uint32_t pk = prev_keys[i];
            if ((i == 0 || prev_keys[i - 1] != pk) && pk < kp.table_cells) table[pk] = make_uint2(EMPTY, EMPTY);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * SORT_RADIX; i += blockDim.x)
        if (s_h[i]) atomicAdd(&hist[i], s_h[i]);
}

// clReorder (libCL/phys/oclFluid3D.cl:66-72), used when the gather is not fused into the
// last sort pass.
static __global__ void k_reorder(const uint32_t* __restrict__ index, const float4* __restrict__ pos,
                          const float4* __restrict__ vel, float4* __restrict__ spos,
                          float4* __restrict__ svel, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t s = index[i];
    spos[i] = pos[s];
    svel[i] = vel[s];
}

// Cell bounds into the interleaved LINEAR_GRID table, plus the list of occupied bricks,
// for BOUNDS_TILE consecutive sorted keys per CTA (BOUNDS_ITEMS per thread, strided by the
// block). A key that starts a cell writes the cell's first index, one that ends it the end;
// a key whose brick differs from its predecessor's appends the brick id: the CTA's appends
// take ranks from a shared counter and reserve their slots with one global atomic (one
// counter address, so per-key atomics would queue behind each other).
constexpr uint32_t BOUNDS_ITEMS = 4;
constexpr uint32_t BOUNDS_TILE = 256 * BOUNDS_ITEMS;

// Tile `tile` of the keys; COH: the keys were written earlier in the same launch.
template <bool COH = false, class BrickOf>
__device__ __forceinline__ void bounds_tile(const uint32_t* __restrict__ keys, const KParams& kp,
                                            uint2* __restrict__ table, uint32_t* __restrict__ bricks,
                                            uint32_t* __restrict__ n_bricks, uint32_t* err, BrickOf brick_of,
                                            uint32_t tile) {
    __shared__ uint32_t s_cnt, s_base;
    if (threadIdx.x == 0) s_cnt = 0;
    __syncthreads();
    uint32_t bid[BOUNDS_ITEMS], rank[BOUNDS_ITEMS];
    const uint32_t i0 = tile * BOUNDS_TILE + threadIdx.x;
#pragma unroll
    for (uint32_t it = 0; it < BOUNDS_ITEMS; ++it) {
        const uint32_t i = i0 + it * blockDim.x;
        rank[it] = EMPTY;
        bid[it] = 0;
        if (i >= kp.n) continue;
        const uint32_t k = ld_phase<COH>(keys + i);
        if (k >= kp.table_cells) {
            atomicOr(err, DEV_ERR_KEY_RANGE);
            continue;
        }
        const uint32_t prev = i > 0 ? ld_phase<COH>(keys + i - 1) : EMPTY;
        const uint32_t next = i + 1 < kp.n ? ld_phase<COH>(keys + i + 1) : EMPTY;
        if (k != prev) table[k].x = i;
        if (k != next) table[k].y = i + 1;
        bid[it] = brick_of(k);
        if (prev == EMPTY || bid[it] != brick_of(prev)) rank[it] = atomicAdd(&s_cnt, 1u);
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_cnt) s_base = atomicAdd(n_bricks, s_cnt);
    __syncthreads();
#pragma unroll
    for (uint32_t it = 0; it < BOUNDS_ITEMS; ++it)
        if (rank[it] != EMPTY) bricks[s_base + rank[it]] = bid[it];
}

// Single scene: brick id = x/W + bxn*(y + ny*z).
static __global__ void __launch_bounds__(256) k_bounds_linear(const uint32_t* __restrict__ keys, KParams kp,
                                                              uint2* __restrict__ table, uint32_t* __restrict__ bricks,
                                                              uint32_t* __restrict__ n_bricks, uint32_t* err) {
    const uint32_t nx = (uint32_t)kp.nx, bw = (uint32_t)kp.bw, bxn = (uint32_t)kp.bxn;
    bounds_tile(keys, kp, table, bricks, n_bricks, err,
                [=](uint32_t k) { return (k % nx) / bw + bxn * (k / nx); }, blockIdx.x);
}

// Batch version of k_hash: each particle keys into its own scene's grid; the key is the
// scene's cell offset plus the local linear key. The body takes the block's histogram
// buffer (SORT_MAX_PASSES * SORT_RADIX words of shared memory) from the caller.
template <bool CLEAR>
__device__ __forceinline__ void hash_batch_run(uint32_t* s_h, const float4* __restrict__ pos, const KParams& kp,
                                               uint32_t* __restrict__ keys, uint32_t* __restrict__ hist,
                                               const uint32_t* __restrict__ prev_keys, uint2* __restrict__ table) {
    for (int i = threadIdx.x; i < SORT_MAX_PASSES * SORT_RADIX; i += blockDim.x) s_h[i] = 0;
    __syncthreads();
    const int passes = sort_passes(0, kp.end_bit, kp.digit_bits);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < kp.n; i += gridDim.x * blockDim.x) {
        const SceneDev& d = kp.scenes[scene_of<0>(kp.scenes, kp.n_scenes, i)];
        const float4 p = pos[i];
        const int gx = (int)floorf(__fdiv_rn(__fsub_rn(p.x, d.origin.x), kp.h));
        const int gy = (int)floorf(__fdiv_rn(__fsub_rn(p.y, d.origin.y), kp.h));
        const int gz = (int)floorf(__fdiv_rn(__fsub_rn(p.z, d.origin.z), kp.h));
        const uint32_t k = d.cell_off + (uint32_t)clampi(gx, 0, d.nx - 1) +
                           (uint32_t)d.nx * ((uint32_t)clampi(gy, 0, d.ny - 1) + (uint32_t)d.ny * (uint32_t)clampi(gz, 0, d.nz - 1));
        keys[i] = k;
        for (int q = 0; q < passes; ++q) {
            const int shift = q * kp.digit_bits;
            const int bits = min(kp.digit_bits, kp.end_bit - shift);
            atomicAdd(&s_h[q * SORT_RADIX + ((k >> shift) & ((1u << bits) - 1u))], 1u);
        }
        if (CLEAR) {
            const uint32_t pk = prev_keys[i];
            if ((i == 0 || prev_keys[i - 1] != pk) && pk < kp.table_cells) table[pk] = make_uint2(EMPTY, EMPTY);
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < passes * SORT_RADIX; i += blockDim.x)
        if (s_h[i]) atomicAdd(&hist[i], s_h[i]);
    __syncthreads();  // s_h is free for the caller
}

template <bool CLEAR>
__global__ void __launch_bounds__(256) k_hash_batch(const float4* __restrict__ pos, KParams kp,
                                                    uint32_t* __restrict__ keys, uint32_t* __restrict__ hist,
                                                    const uint32_t* __restrict__ prev_keys, uint2* __restrict__ table) {
    __shared__ uint32_t s_h[SORT_MAX_PASSES * SORT_RADIX];
    hash_batch_run<CLEAR>(s_h, pos, kp, keys, hist, prev_keys, table);
}

__device__ __forceinline__ uint32_t batch_brick_of(const KParams& kp, uint32_t k) {
    const SceneDev& d = kp.scenes[scene_of<1>(kp.scenes, kp.n_scenes, k)];
    const uint32_t local = k - d.cell_off, nx = (uint32_t)d.nx;
    return d.brick_off + (local % nx) / (uint32_t)kp.bw + (uint32_t)d.bxn * (local / nx);
}

// Batch version of k_bounds_linear: brick ids are global (scene brick offset + local id).
static __global__ void __launch_bounds__(256) k_bounds_batch(const uint32_t* __restrict__ keys, KParams kp,
                                                             uint2* __restrict__ table, uint32_t* __restrict__ bricks,
                                                             uint32_t* __restrict__ n_bricks, uint32_t* err) {
    bounds_tile(keys, kp, table, bricks, n_bricks, err, [&](uint32_t k) { return batch_brick_of(kp, k); }, blockIdx.x);
}

// Splits the interleaved table into two arrays (for inspection through the ABI).
static __global__ void k_table_split(const uint2* __restrict__ table, uint32_t cells,
                              uint32_t* __restrict__ cs, uint32_t* __restrict__ ce) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cells) return;
    const uint2 e = table[i];
    cs[i] = e.x;
    ce[i] = e.x == EMPTY ? EMPTY : e.y;
}

// ---- exact (reference-order) neighbour kernels ---------------------------------------------

struct SplitTable {  // REFERENCE_HASH: bfCellStart / bfCellEnd
    const uint32_t* cs;
    const uint32_t* ce;
    __device__ __forceinline__ uint2 get(uint32_t k) const { return make_uint2(cs[k], ce[k]); }
};
struct PairTable {  // LINEAR_GRID: interleaved
    const uint2* t;
    __device__ __forceinline__ uint2 get(uint32_t k) const { return t[k]; }
};

// Calls f(start, end) for each non-empty neighbour cell in the reference's visiting order.
template <int MODE, class Table, class F>
__device__ __forceinline__ void for_each_neighbour_cell(const KParams& kp, const Table& tab, float4 p, F&& f) {
    int gx, gy, gz;
    grid_position(kp, p, gx, gy, gz);
    const int zr = kp.dims == 2 ? 0 : 1;
    if (MODE == GBSPH_KEY_LINEAR_GRID) {
        gx = clampi(gx, 0, kp.nx - 1);
        gy = clampi(gy, 0, kp.ny - 1);
        gz = kp.dims == 2 ? 0 : clampi(gz, 0, kp.nz - 1);
    }
    for (int z = -zr; z <= zr; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                uint32_t cell;
                if (MODE == GBSPH_KEY_LINEAR_GRID) {
                    const int cx = gx + x, cy = gy + y, cz = gz + z;
                    if (cx < 0 || cy < 0 || cz < 0 || cx >= kp.nx || cy >= kp.ny || cz >= kp.nz) continue;
                    cell = (uint32_t)cx + (uint32_t)kp.nx * ((uint32_t)cy + (uint32_t)kp.ny * (uint32_t)cz);
                } else {
                    cell = hash_key(gx + x, gy + y, gz + z);
                }
                const uint2 e = tab.get(cell);
                if (e.x == EMPTY) continue;
                f(e.x, e.y);
            }
}

// fast_length of (a - b) with w = 0 is the correctly rounded sqrt of exact_r2 =
// ((x*x + y*y) + z*z). The correctly rounded sqrt is monotone, so sqrt(r2) < h exactly when
// r2 < kp.r2_thresh (the least float whose sqrt is >= h): the kernels test r2 and take the
// root of in-range candidates only.
__device__ __forceinline__ float exact_r2(float vx, float vy, float vz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)), __fmul_rn(vz, vz));
}

// In-range neighbours the exact density kernel records per particle for the exact force
// kernel (sorted indices in visiting order); a particle with more is scanned again.
constexpr uint32_t XL_CAP = 64;

// clCalculateDensity, libCL/phys/oclFluid3D.cl:150-200. With RECORD, the in-range neighbours
// j (visiting order, repeats of a bucket visited twice included) go to xl[k * n + particle]
// (entry-major, so that the force kernel's threads, stepping through their lists together,
// read consecutive words) and their number to xc[particle].
template <int MODE, class Table, bool RECORD>
__global__ void __launch_bounds__(256) k_density_exact(float4* __restrict__ spos, float4* __restrict__ svel,
                                                       Table tab, KParams kp, uint32_t* __restrict__ xl,
                                                       uint32_t* __restrict__ xc) {
    const uint32_t particle = blockIdx.x * blockDim.x + threadIdx.x;
    if (particle >= kp.n) return;
    const float4 posI = spos[particle];
    float density = 0.0f;
    int count = 0;
    uint32_t* mine = RECORD ? xl + particle : nullptr;
    for_each_neighbour_cell<MODE>(kp, tab, posI, [&](uint32_t start, uint32_t end) {
        for (uint32_t j = start; j < end; j++) {
            if (j == particle) continue;
            const float4 pj = spos[j];
            const float r2 = exact_r2(__fsub_rn(posI.x, pj.x), __fsub_rn(posI.y, pj.y), __fsub_rn(posI.z, pj.z));
            if (r2 < kp.r2_thresh) {  // fast_length < h
                const float vlen = __fsqrt_rn(r2);
                const float t = __fsub_rn(__fmul_rn(kp.h, kp.h), __fmul_rn(vlen, vlen));
                density = __fadd_rn(density, __fmul_rn(__fmul_rn(t, t), t));
                if (RECORD && (uint32_t)count < XL_CAP) mine[(size_t)count * kp.n] = j;
                count++;
            }
        }
    });
    if (RECORD) xc[particle] = (uint32_t)count;
    // The reference writes .w in place while other work-items read .xyz only. Here the
    // candidates' positions are loaded as whole float4s, so a load may race with another
    // thread's write of that particle's .w; the loaded .w is never used (the sums take .xyz
    // only), so the race cannot change a result.
    if (count > 2) {
        density = fmaxf(1.0f, __fmul_rn(__fmul_rn(kp.mass, kp.kconst), density));
        reinterpret_cast<float*>(spos)[4 * (size_t)particle + 3] = density;
        reinterpret_cast<float*>(svel)[4 * (size_t)particle + 3] =
            __fadd_rn(kp.p0, __fmul_rn(kp.stiff, __fsub_rn(density, kp.rho0)));
    } else {
        reinterpret_cast<float*>(spos)[4 * (size_t)particle + 3] = kp.rho0;
        reinterpret_cast<float*>(svel)[4 * (size_t)particle + 3] = kp.p0;
    }
}

// clCalculateForces, libCL/phys/oclFluid3D.cl:202-255: force[index[i]] += SPH force, w = 0.
// With LISTED, a particle whose in-range neighbours the density kernel recorded (xc <= XL_CAP)
// takes them from its list, in the same visiting order, instead of scanning the buckets again:
// the same pairs in the same order, so the same sums, but the warp's threads step through
// their pairs together rather than each meeting its in-range candidates at different steps.
template <int MODE, class Table, bool LISTED>
__global__ void __launch_bounds__(256) k_forces_exact(const float4* __restrict__ spos,
                                                      const float4* __restrict__ svel,
                                                      float4* __restrict__ force,
                                                      const uint32_t* __restrict__ index,
                                                      Table tab, KParams kp, const uint32_t* __restrict__ xl,
                                                      const uint32_t* __restrict__ xc) {
    const uint32_t particle = blockIdx.x * blockDim.x + threadIdx.x;
    if (particle >= kp.n) return;
    const float4 posI = spos[particle], velI = svel[particle];
    float px = 0.f, py = 0.f, pz = 0.f, qx = 0.f, qy = 0.f, qz = 0.f;
    // one pair with the neighbour's position and velocity at hand
    auto pair_at = [&](const float4& posJ, const float4& velJ) {
        const float vx = __fsub_rn(posI.x, posJ.x), vy = __fsub_rn(posI.y, posJ.y), vz = __fsub_rn(posI.z, posJ.z);
        const float r2 = exact_r2(vx, vy, vz);
        if (r2 < kp.r2_thresh) {  // fast_length < h
            const float vlen = __fsqrt_rn(r2);
            const float density2 = __fmul_rn(posI.w, posJ.w);
            const float s = __fdiv_rn(__fadd_rn(velI.w, velJ.w), density2);
            const float hr = __fsub_rn(kp.h, vlen);
            px = __fadd_rn(px, __fmul_rn(s, __fmul_rn(__fmul_rn(__fdiv_rn(vx, vlen), hr), hr)));
            py = __fadd_rn(py, __fmul_rn(s, __fmul_rn(__fmul_rn(__fdiv_rn(vy, vlen), hr), hr)));
            pz = __fadd_rn(pz, __fmul_rn(s, __fmul_rn(__fmul_rn(__fdiv_rn(vz, vlen), hr), hr)));
            qx = __fadd_rn(qx, __fmul_rn(__fdiv_rn(__fsub_rn(velJ.x, velI.x), density2), hr));
            qy = __fadd_rn(qy, __fmul_rn(__fdiv_rn(__fsub_rn(velJ.y, velI.y), density2), hr));
            qz = __fadd_rn(qz, __fmul_rn(__fdiv_rn(__fsub_rn(velJ.z, velI.z), density2), hr));
        }
    };
    auto pair = [&](uint32_t j) {
        const float4 posJ = spos[j];
        const float vx = __fsub_rn(posI.x, posJ.x), vy = __fsub_rn(posI.y, posJ.y), vz = __fsub_rn(posI.z, posJ.z);
        if (exact_r2(vx, vy, vz) < kp.r2_thresh) pair_at(posJ, svel[j]);
    };
    const uint32_t nl = LISTED ? xc[particle] : EMPTY;
    if (LISTED && nl <= XL_CAP) {
        // the recorded neighbours in their order; the next one's index, position and velocity
        // are loaded while the current pair is computed
        const uint32_t* mine = xl + particle;
        float4 pn = posI, vn = velI;
        if (nl) {
            const uint32_t j0 = mine[0];
            pn = spos[j0];
            vn = svel[j0];
        }
        for (uint32_t k = 0; k < nl; ++k) {
            const float4 posJ = pn, velJ = vn;
            if (k + 1 < nl) {
                const uint32_t jn = mine[(size_t)(k + 1) * kp.n];
                pn = spos[jn];
                vn = svel[jn];
            }
            pair_at(posJ, velJ);
        }
    } else {
        for_each_neighbour_cell<MODE>(kp, tab, posI, [&](uint32_t start, uint32_t end) {
            for (uint32_t j = start; j < end; j++)
                if (j != particle) pair(j);
        });
    }
    const uint32_t o = index[particle];
    float4 f = force[o];
    f.x = __fadd_rn(f.x, __fmul_rn(__fadd_rn(__fmul_rn(kp.cpress, px), __fmul_rn(kp.cvisc, qx)), kp.mass));
    f.y = __fadd_rn(f.y, __fmul_rn(__fadd_rn(__fmul_rn(kp.cpress, py), __fmul_rn(kp.cvisc, qy)), kp.mass));
    f.z = __fadd_rn(f.z, __fmul_rn(__fadd_rn(__fmul_rn(kp.cpress, pz), __fmul_rn(kp.cvisc, qz)), kp.mass));
    f.w = 0.0f;
    force[o] = f;
}

// ---- post stages ---------------------------------------------------------------------------

// repulsionForce walls of clClipBox (libCL/phys/oclFluid3D.cl:304-361): EPSILON 1e-5,
// stiffness 2000, damping 256, in the order y-min, y-max, z-min, z-max, x-min, x-max.
__device__ __forceinline__ void add_wall(float& fa, float& fw, float sign, float diff, float vn) {
    if (diff > 0.00001f) {
        const float mag = __fsub_rn(__fmul_rn(2000.0f, diff), __fmul_rn(256.0f, __fmul_rn(sign, vn)));
        fa = __fadd_rn(fa, __fmul_rn(sign, mag));
        fw = __fadd_rn(fw, __fmul_rn(0.0f, mag));
    }
}

__device__ __forceinline__ float4 clip_box_force(const KParams& kp, const float4& box_min, const float4& box_max,
                                                  float4 pos, float4 vel, float4 f) {
    const float r = kp.radius;
    add_wall(f.y, f.w, 1.0f, __fsub_rn(r, __fsub_rn(pos.y, box_min.y)), vel.y);
    add_wall(f.y, f.w, -1.0f, __fsub_rn(r, __fsub_rn(box_max.y, pos.y)), vel.y);
    if (kp.dims != 2) {
        add_wall(f.z, f.w, 1.0f, __fsub_rn(r, __fsub_rn(pos.z, box_min.z)), vel.z);
        add_wall(f.z, f.w, -1.0f, __fsub_rn(r, __fsub_rn(box_max.z, pos.z)), vel.z);
    }
    add_wall(f.x, f.w, 1.0f, __fsub_rn(r, __fsub_rn(pos.x, box_min.x)), vel.x);
    add_wall(f.x, f.w, -1.0f, __fsub_rn(r, __fsub_rn(box_max.x, pos.x)), vel.x);
    return f;
}

__device__ __forceinline__ float4 clip_box_force(const KParams& kp, float4 pos, float4 vel, float4 f) {
    return clip_box_force(kp, kp.box_min, kp.box_max, pos, vel, f);
}

// clIntegrateForce (libCL/phys/oclFluid3D.cl:258-271): clamp |F|, v += F*dt on 4 lanes.
__device__ __forceinline__ float4 integrate_force(const KParams& kp, float4 v, float4 f) {
    const float speed = __fsqrt_rn(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(f.x, f.x), __fmul_rn(f.y, f.y)),
                                                       __fmul_rn(f.z, f.z)), __fmul_rn(f.w, f.w)));
    if (speed > kp.vlimit) {
        const float s = __fdiv_rn(kp.vlimit, speed);
        f.x = __fmul_rn(f.x, s);
        f.y = __fmul_rn(f.y, s);
        f.z = __fmul_rn(f.z, s);
        f.w = __fmul_rn(f.w, s);
    }
    v.x = __fadd_rn(v.x, __fmul_rn(f.x, kp.dt));
    v.y = __fadd_rn(v.y, __fmul_rn(f.y, kp.dt));
    v.z = __fadd_rn(v.z, __fmul_rn(f.z, kp.dt));
    v.w = __fadd_rn(v.w, __fmul_rn(f.w, kp.dt));
    return v;
}

// clIntegrateVelocity (libCL/phys/oclFluid3D.cl:284-291): all four lanes.
__device__ __forceinline__ float4 integrate_velocity(const KParams& kp, float4 p, float4 v) {
    return make_float4(__fadd_rn(p.x, __fmul_rn(v.x, kp.dt)), __fadd_rn(p.y, __fmul_rn(v.y, kp.dt)),
                       __fadd_rn(p.z, __fmul_rn(v.z, kp.dt)), __fadd_rn(p.w, __fmul_rn(v.w, kp.dt)));
}

static __global__ void k_clip_box(const float4* __restrict__ spos, const float4* __restrict__ svel,
                           float4* __restrict__ force, const uint32_t* __restrict__ index, KParams kp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    const uint32_t o = index[i];
    const float4 f = clip_box_force(kp, spos[i], svel[i], force[o]);
    force[o] = f;
    if (kp.rec_force) kp.rec_force[o] = f;
}

static __global__ void k_integrate_force(float4* __restrict__ vel, const float4* __restrict__ force, KParams kp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    vel[i] = integrate_force(kp, vel[i], force[i]);
}

static __global__ void k_gravity(float4* __restrict__ force, KParams kp) {  // clGravity, :294-298
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    force[i] = kp.gravity;
}

static __global__ void k_integrate_velocity(float4* __restrict__ pos, const float4* __restrict__ vel, KParams kp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    pos[i] = integrate_velocity(kp, pos[i], vel[i]);
}

// clEmitter (libCL/phys/oclFluid3D.cl:273-282): particles emit+1 .. emit+99 are placed on a
// 10-wide sheet at y = 0.6 (index = emit - particle, negative, with C's truncating / and %)
// and given velocity (0, emit_speed, 0). The z lane `0.6 + index%10*2*radius` adds the float
// product to the double literal 0.6 in double and rounds the sum to float once (OpenCL C on a
// device with doubles, as the reference's kernels compile on the host and GPU OpenCL stacks).
static __global__ void k_emitter(float4* __restrict__ pos, float4* __restrict__ vel, uint32_t n, uint32_t emit,
                                 float emit_speed, float radius) {
    const uint32_t particle = blockIdx.x * blockDim.x + threadIdx.x;
    if (particle >= n) return;
    if (particle > emit && particle < emit + 100u) {
        const int index = (int)(emit - particle);
        const float dz = __fmul_rn((float)(index % 10 * 2), radius);
        pos[particle] = make_float4(__fmul_rn((float)(index / 10 * 2), radius), 0.6f,
                                    __double2float_rn(__dadd_rn(0.6, (double)dz)), 1.0f);
        vel[particle] = make_float4(0.0f, emit_speed, 0.0f, 1.0f);
    }
}

// clip + integrate-force + gravity + integrate-velocity in one pass over sorted slots.
// Equivalent to the four reference kernels because index is a permutation.
static __global__ void k_post_fused(const float4* __restrict__ spos, const float4* __restrict__ svel,
                             const uint32_t* __restrict__ index, float4* __restrict__ pos,
                             float4* __restrict__ vel, float4* __restrict__ force, KParams kp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    const uint32_t o = index[i];
    const float4 f = clip_box_force(kp, spos[i], svel[i], force[o]);
    if (kp.rec_force) kp.rec_force[o] = f;
    const float4 v = integrate_force(kp, vel[o], f);
    vel[o] = v;
    force[o] = kp.gravity;
    pos[o] = integrate_velocity(kp, pos[o], v);
}

// ---- brick (fast, LINEAR_GRID) neighbour kernels ---------------------------------------------

struct BrickShared {
    uint32_t off[9][BRICK_SLOTS + 1];  // lower bounds of each cell inside the row's range
    uint32_t lo[9];                    // first sorted index of the row's range
    uint32_t rcnt[9];                  // candidates of the row
    uint32_t base[9];                  // offset of the row in the staging buffer
    uint32_t brick;                    // index into the occupied-brick list
    // the brick's scene: grid, cell-table offset and the parameters that vary per scene
    int nx, ny, nz, bxn;
    uint32_t cell_off, lbrick;  // lbrick: the brick's id within its scene
    float stiff, cvisc;
    float4 box_min, box_max;
    unsigned long long bar;
};

// Loads the brick's scene, geometry and neighbour-row ranges into S. A single scene takes its
// grid and parameters from kp; in a batch (BATCH) the brick id is global and its scene is
// found in kp.scenes. Returns the brick's first cell x and cell count through x0/ncell.
template <int DIMS, bool BATCH>
__device__ __forceinline__ void brick_setup(BrickShared& S, const KParams& kp, uint32_t bid,
                                            const uint2* __restrict__ table, uint32_t* err, int& x0,
                                            int& ncell) {
    constexpr int R = DIMS == 3 ? 9 : 3;
    const int W = kp.bw;
    const int t = threadIdx.x;
    // a single scene's grid comes from kp (no barrier needed); a batch's from its scene
    // table, through shared memory. The barrier after the table loads publishes S's scene
    // fields before any warp reads them.
    if (t == 0) {
        if (BATCH) {
            const int sc = scene_of<2>(kp.scenes, kp.n_scenes, bid);
            const SceneDev& d = kp.scenes[sc];
            S.nx = d.nx;
            S.ny = d.ny;
            S.nz = d.nz;
            S.bxn = d.bxn;
            S.cell_off = d.cell_off;
            S.stiff = d.stiff;
            S.cvisc = d.cvisc;
            S.box_min = d.box_min;
            S.box_max = d.box_max;
            S.lbrick = bid - d.brick_off;
        } else {
            S.nx = kp.nx;
            S.ny = kp.ny;
            S.nz = kp.nz;
            S.bxn = kp.bxn;
            S.cell_off = 0;
            S.stiff = kp.stiff;
            S.cvisc = kp.cvisc;
            S.box_min = kp.box_min;
            S.box_max = kp.box_max;
            S.lbrick = bid;
        }
    }
    if (BATCH) __syncthreads();
    const uint32_t lb = BATCH ? S.lbrick : bid;
    const int nx = BATCH ? S.nx : kp.nx, ny = BATCH ? S.ny : kp.ny, nz = BATCH ? S.nz : kp.nz;
    const uint32_t bxn = BATCH ? (uint32_t)S.bxn : (uint32_t)kp.bxn;
    const int bx = (int)(lb % bxn);
    const uint32_t yz = lb / bxn;
    const int y = (int)(yz % (uint32_t)ny);
    const int z = (int)(yz / (uint32_t)ny);
    x0 = bx * W;
    ncell = min(W, nx - x0);
    const uint2* tab = BATCH ? table + S.cell_off : table;
    // a warp per row (warp w takes rows w, w + BRICK_WARPS, ...): lane c reads the range of the
    // row's column c (cell x0 - 1 + c), a warp scan of the counts gives the columns' offsets
    // inside the row's range, and the first non-empty column its start
    const int lane = t & 31;
    for (int r = t >> 5; r < R; r += BRICK_WARPS) {
        const int cy = y + (r % 3) - 1;
        const int cz = DIMS == 3 ? z + (r / 3) - 1 : 0;
        const int cx = x0 - 1 + lane;
        uint32_t cnt = 0, st = 0;
        if (lane < W + 2 && cx >= 0 && cx < nx && cy >= 0 && cy < ny && cz >= 0 && cz < nz) {
            const uint2 e = tab[(uint32_t)cx + (uint32_t)nx * ((uint32_t)cy + (uint32_t)ny * (uint32_t)cz)];
            if (e.x != EMPTY) {
                cnt = e.y - e.x;
                st = e.x;
            }
        }
        uint32_t inc = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        const uint32_t total = __shfl_sync(0xffffffffu, inc, 31);
        const uint32_t nonempty = __ballot_sync(0xffffffffu, cnt != 0u);
        const uint32_t lo = nonempty ? __shfl_sync(0xffffffffu, st, __ffs(nonempty) - 1) : 0u;
        const bool bad = (uint64_t)lo + total > kp.n;  // inconsistent table: report, use an empty row
        // column W + 2 (and beyond) has no count, so its exclusive offset is the row's total
        if (lane <= W + 2) S.off[r][lane] = bad ? 0u : inc - cnt;
        if (lane == 0) {
            S.lo[r] = bad ? 0u : lo;
            S.rcnt[r] = bad ? 0u : total;
            if (bad) atomicOr(err, DEV_ERR_KEY_RANGE);
        }
    }
    __syncthreads();
}

// Warp 0: the rows' bases in the staging buffer (a scan of their counts), then, if the brick
// fits, lane 0 arms the mbarrier `bar` with the byte count and lane r copies row r. No barrier:
// the other warps learn whether the brick is staged from brick_total and wait on `bar`
// (brick_wait's barrier then publishes the bases).
template <int DIMS, int NARR>
__device__ __forceinline__ void brick_stage(BrickShared& S, float4* s_buf, uint32_t cap,
                                            const float4* __restrict__ a0, const float4* __restrict__ a1,
                                            uint64_t* bar) {
    constexpr int R = DIMS == 3 ? 9 : 3;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const uint32_t rc = lane < R ? S.rcnt[lane] : 0u;
        uint32_t inc = rc;
#pragma unroll
        for (int o = 1; o < 16; o <<= 1) {
            const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += v;
        }
        const uint32_t base = inc - rc, total = __shfl_sync(0xffffffffu, inc, R - 1);
        if (lane < R) S.base[lane] = base;
        if (total <= cap && total > 0) {
            if (lane == 0) mbar_arrive_expect_tx(bar, total * 16u * NARR);
            __syncwarp();
            if (lane < R && rc) {
                // this lane's generic-proxy accesses (shared memory, and global memory that an
                // earlier phase of a persistent kernel wrote) before its bulk copies
                fence_proxy_async_smem();
                fence_proxy_async_global();
                bulk_g2s(s_buf + base, a0 + S.lo[lane], rc * 16u, bar);
                if (NARR > 1) bulk_g2s(s_buf + cap + base, a1 + S.lo[lane], rc * 16u, bar);
            }
        }
    }
}

// Candidates the brick stages: the sum of its rows' counts (known to every thread after the
// set-up's barrier).
template <int DIMS>
__device__ __forceinline__ uint32_t brick_total(const BrickShared& S) {
    constexpr int R = DIMS == 3 ? 9 : 3;
    uint32_t a = 0;
#pragma unroll
    for (int r = 0; r < R; ++r) a += S.rcnt[r];
    return a;
}

// Waits for the staged copies (every thread), then a barrier. Returns false to every thread
// if any thread's wait hit its limit, after draining the copies still in flight (bounded).
__device__ __forceinline__ bool brick_wait(uint64_t* bar, uint32_t& phase, uint32_t* err) {
    bool ok = mbar_wait_bounded(bar, phase);
    if (!ok) atomicOr(err, DEV_ERR_MBAR_TIMEOUT);
    ok = __syncthreads_and(ok);
    phase ^= 1u;
    if (!ok && threadIdx.x == 0) {
        // drain the copies still in flight (bounded) before this CTA's shared memory goes away
        mbar_wait_bounded(bar, phase ^ 1u);
    }
    return ok;
}

// Tree reduction over the Q lanes {q*tg + ti} that share a target.
__device__ __forceinline__ float reduce_q(float v, uint32_t q, uint32_t Q, uint32_t tg) {
    for (uint32_t s = 1; s < Q; s <<= 1) {
        const float o = __shfl_down_sync(0xffffffffu, v, s * tg);
        if ((q & (2 * s - 1)) == 0 && q + s < Q) v += o;
    }
    return v;
}

// Staged candidates per brick. The density and force kernels use the same value so that they
// stage (or fall back for) exactly the same bricks: the neighbour lists the density kernel
// records are indices into that staging.
constexpr uint32_t BRICK_CAP = 1536;
constexpr uint32_t NBR_CAP = 64;         // neighbour slots per particle (uint16), split over the Q lanes
constexpr uint32_t WLIST_STRIDE = NBR_CAP + 8;  // shared-memory stride per target (halves; 16-byte rows)
constexpr uint32_t LIST_STAGE_MAX = 160;        // targets per brick whose lists the force kernel stages
constexpr uint32_t GROUP_MAX = 16;              // targets a warp takes at once (both passes)
constexpr uint32_t NBR_SUBLISTS = 8;            // at most 8 lanes (sub-lists) per target
constexpr uint64_t NBR_SCAN = 1ull << 63;       // nbr_meta: the force pass scans for this target
constexpr uint32_t REC_SCAN = 0xFFFFFFFFu;      // rec_cnt: no recorded list for this particle


// Dynamic shared memory of the brick kernels.
constexpr size_t DENSITY_SMEM = (size_t)BRICK_CAP * 16 + (size_t)BRICK_WARPS * GROUP_MAX * WLIST_STRIDE * 2;
// force: staged positions and velocities, then the lists, list lengths and permutation
// entries of up to LIST_STAGE_MAX targets (the last two rounded out to 16-byte copies)
constexpr size_t FORCE_LIST_BYTES = (size_t)LIST_STAGE_MAX * NBR_CAP * 2;
constexpr size_t FORCE_META_BYTES = (size_t)(LIST_STAGE_MAX + 2) * 8;
constexpr size_t FORCE_INDEX_BYTES = (size_t)(LIST_STAGE_MAX + 4) * 4;
constexpr size_t FORCE_SMEM = (size_t)BRICK_CAP * 32 + FORCE_LIST_BYTES + FORCE_META_BYTES + FORCE_INDEX_BYTES;

// Slots of each lane's sub-list when Q lanes share a target: sub-list q holds slots
// [q * sub, (q + 1) * sub) of the target's NBR_CAP slots.
__device__ __forceinline__ uint32_t nbr_sub(uint32_t Q) { return NBR_CAP / Q; }

// Lane layout of a group of tg targets (1 <= tg <= GROUP_MAX) on a warp: lane = q * tg + ti
// serves target ti with stride q of Q = min(32 / tg, NBR_SUBLISTS) (lanes with q >= Q idle).
// tq packs ti | q << 8;
// info packs Q | nbr_sub(Q) << 8; group << ti is the mask of the lanes serving target ti.
// Both neighbour passes use it, so the density pass's sub-lists are the force pass's.
struct LaneMap {
    uint16_t tq[GROUP_MAX + 1][32];
    uint32_t info[GROUP_MAX + 1];
    uint32_t group[GROUP_MAX + 1];
};

__device__ __forceinline__ void lane_map_init(LaneMap& L) {
    for (uint32_t i = threadIdx.x; i < (GROUP_MAX + 1) * 32; i += blockDim.x) {
        const uint32_t tg = i / 32, lane = i % 32;
        if (tg == 0) {
            L.tq[0][lane] = 0;
            if (lane == 0) L.info[0] = L.group[0] = 0;
            continue;
        }
        const uint32_t Q = min(32 / tg, NBR_SUBLISTS);
        L.tq[tg][lane] = (uint16_t)((lane % tg) | ((lane / tg) << 8));
        if (lane == 0) {
            uint32_t m = 0;
            for (uint32_t k = 0; k < Q; ++k) m |= 1u << (k * tg);
            L.info[tg] = Q | (nbr_sub(Q) << 8);
            L.group[tg] = m;
        }
    }
}

// Density + pressure for every particle of the occupied bricks (persistent CTAs).
// Writes sorted position .w = density and sorted velocity .w = pressure, as
// clCalculateDensity does (libCL/phys/oclFluid3D.cl:189-199). A warp takes a target cell and
// up to GROUP_MAX of its particles at a time; lanes (target ti, stride q) walk the 9 (or 3)
// neighbour rows of the cell (3 consecutive cells each, contiguous in the staging buffer),
// lane q taking candidates q, q + Q, ... of every row, so candidate loads are shared-memory
// broadcasts. Every target also meets itself (r^2 = 0, term h^6, count 1); that term is
// removed after the sum instead of testing the index of every candidate. Each lane records
// its in-range candidates (the target itself included) as staged indices in its own
// sub-list of nbr[gi][NBR_CAP] (in candidate order); the lists' lengths are the counts the
// reference's count > 2 test uses and go to nbr_meta[gi] (one byte per sub-list), or
// nbr_meta[gi] = NBR_SCAN when a sub-list overflowed or the brick could not be staged.
typedef uint8_t SubListCounts[BRICK_WARPS][GROUP_MAX][NBR_SUBLISTS];  // sub-list lengths per warp group

// The body of k_density_brick, on shared memory the caller provides: s_buf (DENSITY_SMEM
// bytes), S2 (two brick records, used in turn, so that a warp may start the next brick's
// set-up while others still compute this one), L and wcnt. The batched step's persistent
// kernel runs it as one of its phases. Returns false if a bulk-copy wait gave up (the CTA left
// the loop).
template <int DIMS, bool BATCH>
__device__ __forceinline__ bool density_brick_run(float4* s_buf, BrickShared* S2, LaneMap& L, SubListCounts& wcnt,
                                                  float4* __restrict__ spos, float4* __restrict__ svel,
                                                  const uint2* __restrict__ table, const uint32_t* __restrict__ bricks,
                                                  uint32_t* counters, const KParams& kp, uint16_t* __restrict__ nbr,
                                                  uint64_t* __restrict__ nbr_meta, uint32_t* err) {
    constexpr int R = DIMS == 3 ? 9 : 3;
    constexpr int RC = DIMS == 3 ? 4 : 1;  // the brick's own row
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint16_t* wlist = reinterpret_cast<uint16_t*>(s_buf + BRICK_CAP) + warp * GROUP_MAX * WLIST_STRIDE;
    lane_map_init(L);
    uint64_t* bar = reinterpret_cast<uint64_t*>(&S2[0].bar);
    if (t == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    uint32_t phase = 0;
    const uint32_t n_bricks = __ldcg(counters);  // written by the bounds pass (an earlier kernel or phase)
    const float h2 = kp.h2, thr = kp.r2_thresh;
    const uint32_t buf_a = smem_addr(s_buf);
    // Brick k uses record S2[k & 1]. Its id was fetched at the start of brick k - 1 and is read
    // after that brick's barriers; the set-up's barrier of brick k (all warps are done with
    // brick k - 1) comes before the copies into the staging buffer.
    if (t == 0) S2[0].brick = atomicAdd(&counters[1], 1u);
    __syncthreads();
    for (uint32_t it = 0;; it ^= 1u) {
        BrickShared& S = S2[it];
        const uint32_t b = S.brick;
        if (b >= n_bricks) break;
        if (t == 0) S2[it ^ 1u].brick = atomicAdd(&counters[1], 1u);
        int x0, ncell;
        brick_setup<DIMS, BATCH>(S, kp, bricks[b], table, err, x0, ncell);
        brick_stage<DIMS, 1>(S, s_buf, BRICK_CAP, spos, nullptr, bar);
        const uint32_t total = brick_total<DIMS>(S);
        const bool staged = total <= BRICK_CAP && total > 0;
        if (staged && !brick_wait(bar, phase, err)) return false;
        for (int c = warp; c < ncell; c += BRICK_WARPS) {
            const uint32_t t0 = S.off[RC][c + 1], nt = S.off[RC][c + 2] - t0;
            for (uint32_t g0 = 0; g0 < nt; g0 += GROUP_MAX) {
                const uint32_t tg = min(GROUP_MAX, nt - g0);
                const uint32_t e = L.tq[tg][lane], f = L.info[tg];
                const uint32_t ti = e & 0xFFu, q = e >> 8, Q = f & 0xFFu, sub = f >> 8;
                const bool active = q < Q;
                const uint32_t tl = t0 + g0 + ti;
                const uint32_t gi = S.lo[RC] + tl;
                const float4 pi = staged ? s_buf[S.base[RC] + tl] : spos[gi];
                uint16_t* my = wlist + ti * WLIST_STRIDE + q * sub;
                float acc = 0.0f;
                uint32_t nk = 0;  // in-range candidates of this lane (the target itself included)
                if (active && staged) {
                    // 32-bit shared-memory addresses stepped per candidate: the candidate's
                    // position (16 bytes) and this lane's next list slot, wa, which stops one
                    // slot past the sub-list (the next lane's first slot, or the row's padding).
                    // A lane that gets there has overflowed (nk = sub): its target is then
                    // scanned by the force pass and none of its sub-lists is read.
                    const uint32_t my_a = smem_addr(my), w_end = my_a + 2u * sub, step = Q * 16u;
                    uint32_t wa = my_a;
#pragma unroll 1
                    for (int r = 0; r < R; ++r) {
                        const uint32_t lo = S.off[r][c], len = S.off[r][c + 3] - lo;
                        uint32_t v = S.base[r] + lo + q;  // staged index of the candidate
                        uint32_t a = buf_a + v * 16u;
                        const uint32_t a_end = buf_a + (S.base[r] + lo + len) * 16u;
#pragma unroll 4
                        for (; a < a_end; a += step, v += Q) {
                            const float4 pj = lds_f4(a);
                            const float dx = pi.x - pj.x, dy = pi.y - pj.y;
                            float r2 = fmaf(dy, dy, dx * dx);
                            if (DIMS == 3) {
                                const float dz = pi.z - pj.z;
                                r2 = fmaf(dz, dz, r2);
                            }
                            const bool in = r2 < thr;
                            const float tt = in ? h2 - r2 : 0.0f;
                            acc = fmaf(tt * tt, tt, acc);
                            // branch-free append: the slot after the last real entry is
                            // overwritten by the next candidate. The target and coincident
                            // particles (r^2 = 0) are listed; the force pass skips them.
                            sts_u16(wa, v);
                            wa = min(wa + (in ? 2u : 0u), w_end);
                        }
                    }
                    nk = (wa - my_a) >> 1;  // at most sub: an overflowed lane counts sub
                } else if (active) {  // unstaged brick: candidates from global memory, no lists
#pragma unroll 1
                    for (int r = 0; r < R; ++r) {
                        const uint32_t lo = S.off[r][c], len = S.off[r][c + 3] - lo;
                        const float4* rp = spos + S.lo[r] + lo;
                        for (uint32_t k = q; k < len; k += Q) {
                            const float4 pj = rp[k];
                            const float dx = pi.x - pj.x, dy = pi.y - pj.y;
                            float r2 = fmaf(dy, dy, dx * dx);
                            if (DIMS == 3) {
                                const float dz = pi.z - pj.z;
                                r2 = fmaf(dz, dz, r2);
                            }
                            const bool in = r2 < thr;
                            const float tt = in ? h2 - r2 : 0.0f;
                            acc = fmaf(tt * tt, tt, acc);
                            nk += in ? 1u : 0u;
                        }
                    }
                }
                const bool ovf = !staged || nk >= sub;
                if (kp.rec_nbr) {
                    // recording (an adjoint's recomputation): the target's sub-lists, concatenated
                    // in q order, as sorted indices; lane q writes its own entries after those
                    // of the lanes q' < q of its target
                    uint32_t before = active ? nk : 0u;
#pragma unroll
                    for (uint32_t st = 1; st < NBR_SUBLISTS; st <<= 1) {
                        const uint32_t v = __shfl_up_sync(0xffffffffu, before, (st * tg) & 31u);
                        if (q >= st && st < Q) before += v;
                    }
                    before -= active ? nk : 0u;  // exclusive
                    const uint32_t anyovf = __ballot_sync(0xffffffffu, active && ovf) & (L.group[tg] << ti);
                    if (active && !anyovf) {
                        const size_t slot = *kp.rec_slot;
                        uint32_t* out = kp.rec_nbr + (slot * kp.rec_n4 + gi) * NBR_CAP + before;
                        for (uint32_t e = 0; e < nk; ++e) {
                            const uint32_t sidx = my[e];
                            uint32_t g = sidx;
#pragma unroll
                            for (int r = 0; r < R; ++r)
                                if (sidx >= S.base[r]) g = sidx - S.base[r] + S.lo[r];
                            out[e] = g;
                        }
                    }
                }
                acc = reduce_q(acc, q, Q, tg);
                const float cnt = reduce_q((float)nk, q, Q, tg);
                const uint32_t om = __ballot_sync(0xffffffffu, active && ovf) & (L.group[tg] << ti);
                // the target's sub-list lengths, one byte each, gathered through shared memory
                if (active) wcnt[warp][ti][q] = (uint8_t)min(nk, 127u);
                __syncwarp();
                if (active && q == 0) {
                    acc -= h2 * h2 * h2;  // the target's own term
                    const float count = cnt - 1.0f;
                    float rho = kp.rho0, p = kp.p0;
                    if (count > 2.5f) {
                        rho = fmaxf(1.0f, kp.mass * kp.kconst * acc);
                        p = kp.p0 + S.stiff * (rho - kp.rho0);
                    }
                    spos[gi] = make_float4(pi.x, pi.y, pi.z, rho);
                    reinterpret_cast<float*>(svel)[4 * (size_t)gi + 3] = p;
                    const uint64_t lens = *reinterpret_cast<const uint64_t*>(wcnt[warp][ti]);
                    nbr_meta[gi] = om ? NBR_SCAN : (Q < 8 ? lens & ((1ull << (8 * Q)) - 1ull) : lens);
                    if (kp.rec_cnt) kp.rec_cnt[(size_t)*kp.rec_slot * kp.rec_n4 + gi] = om ? REC_SCAN : (uint32_t)(cnt + 0.5f);
                }
                // copy the group's lists out. A brick's lists fill the brick's targets' rows of
                // nbr, stored chunk-major: the 16-byte chunk ch (entries 8ch..8ch+7) of the
                // brick's u-th target is uint4 number ch * ntarg + u (so that the force pass,
                // one lane per target, reads consecutive chunks); half-warps copy one chunk of
                // up to 16 consecutive targets each.
                __syncwarp();
                if (staged) {
                    const uint32_t u0 = t0 + g0 - S.off[RC][1], ntarg = S.off[RC][ncell + 1] - S.off[RC][1];
                    uint4* dst = reinterpret_cast<uint4*>(nbr + (size_t)(S.lo[RC] + S.off[RC][1]) * NBR_CAP);
                    const uint32_t row = (uint32_t)lane & 15u;
                    if (row < tg)
                        for (uint32_t ch = (uint32_t)lane >> 4; ch < NBR_CAP / 8; ch += 2)
                            dst[(size_t)ch * ntarg + u0 + row] =
                                *reinterpret_cast<const uint4*>(wlist + row * WLIST_STRIDE + ch * 8u);
                }
                __syncwarp();
            }
        }
    }
    return true;
}

template <int DIMS, bool BATCH>
__global__ void __launch_bounds__(BRICK_THREADS, 4) k_density_brick(float4* __restrict__ spos,
                                                                 float4* __restrict__ svel,
                                                                 const uint2* __restrict__ table,
                                                                 const uint32_t* __restrict__ bricks,
                                                                 uint32_t* counters, KParams kp,
                                                                 uint16_t* __restrict__ nbr,
                                                                 uint64_t* __restrict__ nbr_meta, uint32_t* err) {
    extern __shared__ float4 s_buf[];  // [BRICK_CAP] positions, then per-warp neighbour lists
    __shared__ BrickShared S[2];
    __shared__ LaneMap L;
    __shared__ __align__(8) SubListCounts wcnt;
    density_brick_run<DIMS, BATCH>(s_buf, S, L, wcnt, spos, svel, table, bricks, counters, kp, nbr, nbr_meta, err);
}

// Pressure + viscosity contribution of one in-range neighbour (acc: pressure xyz, viscosity xyz).
template <int DIMS>
__device__ __forceinline__ void force_pair(const float4& pi, const float4& vi, float inv_rho_i, const float4& pj,
                                           const float4& vj, float h, float* acc) {
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = DIMS == 3 ? pi.z - pj.z : 0.0f;
    float r2 = fmaf(dy, dy, dx * dx);
    if (DIMS == 3) r2 = fmaf(dz, dz, r2);
    const float inv = rsqrtf(r2);
    const float vlen = r2 * inv;
    const float hr = h - vlen;
    const float dd = inv_rho_i * __frcp_rn(pj.w);  // 1 / (rho_i rho_j)
    const float sp = (vi.w + vj.w) * dd * hr * hr * inv;
    acc[0] = fmaf(sp, dx, acc[0]);
    acc[1] = fmaf(sp, dy, acc[1]);
    acc[2] = fmaf(sp, dz, acc[2]);
    const float cv = hr * dd;
    acc[3] = fmaf(vj.x - vi.x, cv, acc[3]);
    acc[4] = fmaf(vj.y - vi.y, cv, acc[4]);
    acc[5] = fmaf(vj.z - vi.z, cv, acc[5]);
}

// Reciprocal with the approximate (about 1 ulp) hardware instruction.
__device__ __forceinline__ float rcp_approx(float x) {
    float r;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

// force_pair on the force pass's staged copies. The target's w lanes hold a_i = 1/rho_i
// (position) and b_i = p_i/rho_i (velocity); the neighbour's hold rho_j and p_j as the density
// pass wrote them, from which a_j = rcp(rho_j) and b_j = p_j a_j are formed here:
// (p_i + p_j) / (rho_i rho_j) = b_i a_j + a_i b_j. Skips r = 0 (the target itself, which its
// list holds, and coincident particles).
template <int DIMS>
__device__ __forceinline__ void force_pair_pre(const float4& pi, const float4& vi, const float4& pj,
                                               const float4& vj, float h, float* acc) {
    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = DIMS == 3 ? pi.z - pj.z : 0.0f;
    float r2 = fmaf(dy, dy, dx * dx);
    if (DIMS == 3) r2 = fmaf(dz, dz, r2);
    if (!(r2 > 0.0f)) return;
    const float inv = rsqrtf(r2);
    const float hr = h - r2 * inv;
    const float aj = rcp_approx(pj.w), bj = vj.w * aj;
    const float dd = pi.w * aj;  // 1 / (rho_i rho_j)
    const float sp = fmaf(vi.w, aj, pi.w * bj) * (hr * hr * inv);
    acc[0] = fmaf(sp, dx, acc[0]);
    acc[1] = fmaf(sp, dy, acc[1]);
    acc[2] = fmaf(sp, dz, acc[2]);
    const float cv = hr * dd;
    acc[3] = fmaf(vj.x - vi.x, cv, acc[3]);
    acc[4] = fmaf(vj.y - vi.y, cv, acc[4]);
    acc[5] = fmaf(vj.z - vi.z, cv, acc[5]);
}

// Forces (pressure + viscosity) for every particle of the occupied bricks
// (clCalculateForces, libCL/phys/oclFluid3D.cl:202-255). The brick's rows are staged exactly
// as in k_density_brick; two lanes take a target and evaluate the in-range pairs that the
// density kernel recorded in the target's sub-lists. A target whose sub-lists overflowed is
// scanned over its rows by its whole warp after the list walk; in an unstaged brick both lanes
// scan the rows in global memory. With FUSED the clip-box, integrate-force, gravity and
// integrate-velocity stages follow in registers; otherwise the SPH force is added to
// force[index[i]] (with w = 0) as clCalculateForces does.
// The body of k_force_brick, on shared memory the caller provides: s_buf (FORCE_SMEM bytes:
// [BRICK_CAP] positions, [BRICK_CAP] velocities, then the neighbour lists of up to
// LIST_STAGE_MAX targets), S and L. COH: the sorted state and the lists were written earlier
// in the same launch, so the direct loads of them go through L2 only. Returns false if a
// bulk-copy wait gave up (the CTA left the loop).
template <int DIMS, bool FUSED, bool BATCH, bool COH = false>
__device__ __forceinline__ bool force_brick_run(float4* s_buf, BrickShared* S2, LaneMap& L,
                                                const float4* __restrict__ spos, const float4* __restrict__ svel,
                                                const uint32_t* __restrict__ index, float4* __restrict__ pos,
                                                float4* __restrict__ vel, float4* __restrict__ force,
                                                const uint2* __restrict__ table, const uint32_t* __restrict__ bricks,
                                                uint32_t* counters, const KParams& kp,
                                                const uint16_t* __restrict__ nbr,
                                                const uint64_t* __restrict__ nbr_meta, uint32_t* err) {
    constexpr int R = DIMS == 3 ? 9 : 3;
    constexpr int RC = DIMS == 3 ? 4 : 1;
    const int t = threadIdx.x, lane = t & 31;
    lane_map_init(L);
    uint64_t* bar = reinterpret_cast<uint64_t*>(&S2[0].bar);
    if (t == 0) {
        mbar_init(bar, 1);
        fence_mbar_init();
    }
    uint32_t phase = 0;
    const uint32_t n_bricks = __ldcg(counters);  // written by the bounds pass (an earlier kernel or phase)
    const float4* s_pos = s_buf;
    const float4* s_vel = s_buf + BRICK_CAP;
    uint16_t* s_lists = reinterpret_cast<uint16_t*>(s_buf + 2 * BRICK_CAP);
    uint64_t* s_meta = reinterpret_cast<uint64_t*>(reinterpret_cast<char*>(s_lists) + FORCE_LIST_BYTES);
    uint32_t* s_index = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(s_meta) + FORCE_META_BYTES);
    // records used in turn, as in density_brick_run
    if (t == 0) S2[0].brick = atomicAdd(&counters[2], 1u);
    __syncthreads();
    for (uint32_t it = 0;; it ^= 1u) {
        BrickShared& S = S2[it];
        const uint32_t b = S.brick;
        if (b >= n_bricks) break;
        if (t == 0) S2[it ^ 1u].brick = atomicAdd(&counters[2], 1u);
        int x0, ncell;
        brick_setup<DIMS, BATCH>(S, kp, bricks[b], table, err, x0, ncell);
        // the brick's targets are consecutive particles: stage their lists with the rows
        const uint32_t tfirst = S.lo[RC] + S.off[RC][1];
        const uint32_t ntarg = S.off[RC][ncell + 1] - S.off[RC][1];
        const bool lists_staged = ntarg <= LIST_STAGE_MAX && S.rcnt[RC] > 0;
        // warp 0: row bases (a scan of the rows' counts); if the brick fits, lane 0 arms the
        // mbarrier with the byte count, lane r copies row r's positions and velocities, and lanes
        // R .. R + 2 the targets' lists, list lengths and permutation entries
        if (t < 32) {
            const uint32_t rc = lane < R ? S.rcnt[lane] : 0u;
            uint32_t inc = rc;
#pragma unroll
            for (int o = 1; o < 16; o <<= 1) {
                const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += v;
            }
            const uint32_t base = inc - rc, total = __shfl_sync(0xffffffffu, inc, R - 1);
            if (lane < R) S.base[lane] = base;
            if (total <= BRICK_CAP && total > 0) {
                const uint32_t lbytes = lists_staged ? ntarg * NBR_CAP * 2 : 0u;
                // list lengths and permutation entries of the targets, from 16-byte boundaries
                const uint32_t mbytes = lists_staged ? (((tfirst + ntarg + 1u) & ~1u) - (tfirst & ~1u)) * 8u : 0u;
                const uint32_t ibytes = lists_staged ? (((tfirst + ntarg + 3u) & ~3u) - (tfirst & ~3u)) * 4u : 0u;
                if (lane == 0) mbar_arrive_expect_tx(bar, total * 32u + lbytes + mbytes + ibytes);
                __syncwarp();
                if (lane < R && rc) {
                    fence_proxy_async_smem();  // as in brick_stage
                    fence_proxy_async_global();
                    bulk_g2s(s_buf + base, spos + S.lo[lane], rc * 16u, bar);
                    bulk_g2s(s_buf + BRICK_CAP + base, svel + S.lo[lane], rc * 16u, bar);
                }
                if (lbytes && lane >= R && lane < R + 3) {
                    fence_proxy_async_smem();
                    fence_proxy_async_global();
                    if (lane == R) bulk_g2s(s_lists, nbr + (size_t)tfirst * NBR_CAP, lbytes, bar);
                    else if (lane == R + 1) bulk_g2s(s_meta, nbr_meta + (tfirst & ~1u), mbytes, bar);
                    else bulk_g2s(s_index, index + (tfirst & ~3u), ibytes, bar);
                }
            }
        }
        const uint32_t total = brick_total<DIMS>(S);
        const bool staged = total <= BRICK_CAP && total > 0;
        if (staged && !brick_wait(bar, phase, err)) return false;
        // P = 2 lanes per target: the brick's targets are consecutive in the centre row, so the
        // CTA takes 128 of them at a time whatever cell they are in; the two lanes of a target
        // split its list (or, in an unstaged brick, take alternate candidates of each row) and
        // their partial sums are added with a shuffle. The summation order depends on neither
        // the brick width nor the brick's target count, as long as the brick is staged.
        const uint32_t tbeg = S.off[RC][1];
        constexpr uint32_t lp = 1u, P = 1u << lp;
        for (uint32_t u0 = 0; u0 < ntarg; u0 += BRICK_THREADS >> lp) {
            const uint32_t u = u0 + ((uint32_t)t >> lp), p = (uint32_t)t & (P - 1u);
            const bool active = u < ntarg;
            const uint32_t tl = tbeg + u;
            const uint32_t gi = S.lo[RC] + tl;
            float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
            float4 pi = make_float4(0.f, 0.f, 0.f, 0.f), vi = pi, f_o = pi, v_o = pi, p_o = pi;
            uint32_t o = 0, Q = 0, sub = 0, c = 0;
            uint64_t meta = NBR_SCAN;
            if (active) {
                // the target's cell and its place in the density pass's groups (its sub-lists)
                while (c + 1 < (uint32_t)ncell && S.off[RC][c + 2] <= tl) ++c;
                const uint32_t c0 = S.off[RC][c + 1], nt = S.off[RC][c + 2] - c0;
                const uint32_t g0 = (tl - c0) & ~(GROUP_MAX - 1u);
                const uint32_t f = L.info[min(GROUP_MAX, nt - g0)];
                Q = f & 0xFFu;
                sub = f >> 8;
                pi = staged ? s_pos[S.base[RC] + tl] : ld_phase<COH>(spos + gi);
                vi = staged ? s_vel[S.base[RC] + tl] : ld_phase<COH>(svel + gi);
                if (staged) {  // the target's w lanes: 1/rho and p/rho (force_pair_pre)
                    pi.w = rcp_approx(pi.w);
                    vi.w *= pi.w;
                }
                if (p == 0) {  // prefetch what the integration needs
                    o = (staged && lists_staged) ? s_index[gi - (tfirst & ~3u)] : ld_phase<COH>(index + gi);
                    f_o = force[o];
                    if (FUSED) {
                        v_o = vel[o];
                        p_o = pos[o];
                    }
                }
                meta = !staged ? NBR_SCAN : (lists_staged ? s_meta[gi - (tfirst & ~1u)] : ld_phase<COH>(nbr_meta + gi));
            }
            const bool scan = (meta & NBR_SCAN) != 0;
            // Sub-lists that start on 16-byte chunks and pair up (Q = 2, 4, 8) can be walked a
            // chunk at a time; a warp whose listed targets are all of that kind does so. Any
            // other warp walks every listed target in one flat loop (the same loop for every
            // layout, so that its lanes stay together). Both visit a target's entries in the
            // same order, which depends on the target's own sub-lists only: with Q even lane p
            // takes sub-lists p, p + 2, ... whole, otherwise entries p, p + 2, ... of the
            // concatenated sub-lists.
            const bool whole = (Q % P) == 0 && (sub & 7u) == 0;
            const bool chunked = __all_sync(0xffffffffu, scan || whole);
            if (active) {
                const float inv_rho_i = staged ? pi.w : 1.0f / pi.w;
                if (!scan) {
                    // slot s of the target's list sits at chunk-major position
                    // ((s >> 3) * ntarg + u) * 8 + (s & 7)
                    const uint16_t* lst = (lists_staged ? s_lists : nbr + (size_t)tfirst * NBR_CAP) + (gi - tfirst) * 8u;
                    const uint32_t n8 = ntarg * 8u;
                    if (!chunked) {
                        // (q, k): the next entry's sub-list and place in it; m: the lane's count
                        const bool pairs = (Q % P) == 0;
                        const uint32_t dq = pairs ? P : 1u, dk = pairs ? 1u : P;
                        uint32_t q = pairs ? p : 0u, k = pairs ? 0u : p, m;
                        if (pairs) {  // bytes p, p + 2, ... of meta
                            m = (uint32_t)(((meta & (0x00FF00FF00FF00FFull << (8 * p))) * 0x0101010101010101ull) >> 56);
                        } else {
                            const uint32_t n = (uint32_t)((meta * 0x0101010101010101ull) >> 56);
                            m = n > p ? (n - p + P - 1u) / P : 0u;
                        }
                        uint32_t nq = (uint32_t)(meta >> (8 * q)) & 127u;
                        auto settle = [&]() {
                            while (k >= nq && q + dq < Q) {
                                k -= nq;
                                q += dq;
                                nq = (uint32_t)(meta >> (8 * q)) & 127u;
                            }
                        };
                        settle();
#pragma unroll 1
                        for (uint32_t i = 0; i < m; ++i) {
                            const uint32_t s = q * sub + k;
                            const uint32_t li = (s >> 3) * n8 + (s & 7u);
                            // staged lists are in shared memory, the others in global memory
                            const uint32_t i0 = lists_staged ? lst[li] : ld_phase<COH>(lst + li);
                            force_pair_pre<DIMS>(pi, vi, s_pos[i0], s_vel[i0], kp.h, acc);
                            k += dk;
                            settle();
                        }
                    } else {
#pragma unroll 1
                        for (uint32_t q = p; q < Q; q += P) {
                            const uint32_t n = (uint32_t)(meta >> (8 * q)) & 127u;
                            const uint4* l4 = reinterpret_cast<const uint4*>(lst);
                            for (uint32_t k0 = 0; k0 < n; k0 += 8) {
                                const size_t li = (size_t)((q * sub + k0) >> 3) * ntarg;
                                const uint4 v = lists_staged ? l4[li] : ld_phase<COH>(l4 + li);
                                const uint32_t w[4] = {v.x, v.y, v.z, v.w};
                                const uint32_t m = min(8u, n - k0);
#pragma unroll
                                for (uint32_t e = 0; e < 8; ++e) {
                                    if (e >= m) break;
                                    const uint32_t idx = (w[e >> 1] >> (16 * (e & 1))) & 0xFFFFu;
                                    force_pair_pre<DIMS>(pi, vi, s_pos[idx], s_vel[idx], kp.h, acc);
                                }
                            }
                        }
                    }
                } else if (!staged) {  // unstaged brick: both lanes scan the rows in global memory
#pragma unroll 1
                    for (int r = 0; r < R; ++r) {
                        const float4* rp = spos + S.lo[r];
                        const float4* rv = svel + S.lo[r];
                        const uint32_t hi = S.off[r][c + 3];
                        for (uint32_t j = S.off[r][c] + p; j < hi; j += P) {
                            const float4 pj = ld_phase<COH>(rp + j);
                            const float dx = pi.x - pj.x, dy = pi.y - pj.y;
                            float r2 = fmaf(dy, dy, dx * dx);
                            if (DIMS == 3) {
                                const float dz = pi.z - pj.z;
                                r2 = fmaf(dz, dz, r2);
                            }
                            if (r2 < kp.r2_thresh && r2 > 0.0f)
                                force_pair<DIMS>(pi, vi, inv_rho_i, pj, ld_phase<COH>(rv + j), kp.h, acc);
                        }
                    }
                }
            }
            if (staged) {
                // Targets of a staged brick whose sub-lists overflowed: the whole warp scans
                // each one's rows in turn (lane l takes candidates l, l + 32, ... of every
                // row) and the sum goes to the target's first lane.
                uint32_t pend = __ballot_sync(0xffffffffu, active && scan && p == 0);
                while (pend) {
                    const int src = __ffs(pend) - 1;
                    pend &= pend - 1u;
                    const float4 ps = make_float4(__shfl_sync(0xffffffffu, pi.x, src), __shfl_sync(0xffffffffu, pi.y, src),
                                                  __shfl_sync(0xffffffffu, pi.z, src), __shfl_sync(0xffffffffu, pi.w, src));
                    const float4 vs = make_float4(__shfl_sync(0xffffffffu, vi.x, src), __shfl_sync(0xffffffffu, vi.y, src),
                                                  __shfl_sync(0xffffffffu, vi.z, src), __shfl_sync(0xffffffffu, vi.w, src));
                    const uint32_t cs = __shfl_sync(0xffffffffu, c, src);
                    float a[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
                    for (int r = 0; r < R; ++r) {
                        const float4* rp = s_pos + S.base[r];
                        const float4* rv = s_vel + S.base[r];
                        const uint32_t hi = S.off[r][cs + 3];
                        for (uint32_t j = S.off[r][cs] + (uint32_t)lane; j < hi; j += 32) {
                            const float4 pj = rp[j];
                            const float dx = ps.x - pj.x, dy = ps.y - pj.y;
                            float r2 = fmaf(dy, dy, dx * dx);
                            if (DIMS == 3) {
                                const float dz = ps.z - pj.z;
                                r2 = fmaf(dz, dz, r2);
                            }
                            if (r2 < kp.r2_thresh) force_pair_pre<DIMS>(ps, vs, pj, rv[j], kp.h, a);
                        }
                    }
                    for (int m = 16; m > 0; m >>= 1) {
#pragma unroll
                        for (int k = 0; k < 6; ++k) a[k] += __shfl_xor_sync(0xffffffffu, a[k], m);
                    }
                    if (lane == src) {
#pragma unroll
                        for (int k = 0; k < 6; ++k) acc[k] = a[k];
                    }
                }
            }
            for (uint32_t m = P >> 1; m > 0; m >>= 1) {
#pragma unroll
                for (int k = 0; k < 6; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], m);
            }
            if (active && p == 0) {
                float4 fs = f_o;
                const float cvisc = S.cvisc;
                fs.x = __fadd_rn(fs.x, __fmul_rn(__fadd_rn(__fmul_rn(kp.cpress, acc[0]), __fmul_rn(cvisc, acc[3])), kp.mass));
                fs.y = __fadd_rn(fs.y, __fmul_rn(__fadd_rn(__fmul_rn(kp.cpress, acc[1]), __fmul_rn(cvisc, acc[4])), kp.mass));
                fs.z = __fadd_rn(fs.z, __fmul_rn(__fadd_rn(__fmul_rn(kp.cpress, acc[2]), __fmul_rn(cvisc, acc[5])), kp.mass));
                fs.w = 0.0f;
                if (FUSED) {
                    fs = clip_box_force(kp, S.box_min, S.box_max, pi, vi, fs);
                    if (kp.rec_force) kp.rec_force[o] = fs;
                    const float4 v = integrate_force(kp, v_o, fs);
                    vel[o] = v;
                    force[o] = kp.gravity;
                    pos[o] = integrate_velocity(kp, p_o, v);
                } else {
                    force[o] = fs;
                }
            }
        }
        __syncthreads();  // every warp is done with the brick before the next one's set-up
    }
    return true;
}

template <int DIMS, bool FUSED, bool BATCH>
__global__ void __launch_bounds__(BRICK_THREADS, 3) k_force_brick(const float4* __restrict__ spos,
                                                               const float4* __restrict__ svel,
                                                               const uint32_t* __restrict__ index,
                                                               float4* __restrict__ pos,
                                                               float4* __restrict__ vel,
                                                               float4* __restrict__ force,
                                                               const uint2* __restrict__ table,
                                                               const uint32_t* __restrict__ bricks,
                                                               uint32_t* counters, KParams kp,
                                                               const uint16_t* __restrict__ nbr,
                                                               const uint64_t* __restrict__ nbr_meta,
                                                               uint32_t* err) {
    extern __shared__ float4 s_buf[];
    __shared__ BrickShared S[2];
    __shared__ LaneMap L;
    force_brick_run<DIMS, FUSED, BATCH>(s_buf, S, L, spos, svel, index, pos, vel, force, table, bricks, counters, kp,
                                        nbr, nbr_meta, err);
}

}  // namespace gbsph
