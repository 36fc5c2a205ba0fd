// cell_kernels.cuh -- the fast (LINEAR_GRID) neighbour passes: density/pressure and
// forces + integration over bricks of cells, with in-range bitmasks between the two passes.
//
// A persistent CTA takes a brick of W cells along x and stages the particle ranges of its 9
// (or 3) neighbour rows in shared memory with cp.async.bulk (brick_setup / brick_stage in
// fluid3d_kernels.cuh). Each warp then takes one cell of the brick at a time. The cell's
// candidates are the particles of the 3 x 3 (x 3) block of cells around it: for every
// neighbour row r, the cells x-1 .. x+1, which are consecutive in sorted order. Concatenated
// row after row they form the cell's candidate sequence k = 0 .. nk-1, which is the same for
// every target of the cell and does not depend on how cells are grouped into bricks.
//
// Density (k_density_cells): the warp holds up to GT targets of the cell in registers and its
// 32 lanes take 32 candidates per round (lane l: k = 32 j + l), so one shared-memory load of
// a candidate is tested against all GT targets. Per round and target, a warp ballot of the
// in-range test is the target's 32-bit in-range mask for candidates 32 j .. 32 j + 31; the
// masks (at most MASK_WORDS per target) are the only thing the force pass needs from this
// pass besides the densities. Partial sums are combined by a transposing butterfly that
// leaves target i's sum on lane 4 i.
//
// Forces (k_force_cells): the same cells and candidate sequences; Q = 32 / GT' lanes take a
// target (GT' = the group's target count rounded up to a power of two) and lane q of a target
// evaluates its in-range candidates whose position in their mask word is q modulo Q, in
// candidate order; the Q partial sums are added by a shuffle tree. Clip box, clamp, gravity
// and both integrations follow in registers.
//
// Summation orders depend only on a cell's own particles and candidate sequence, so results
// are deterministic and independent of the brick width and of how work is scheduled.
#pragma once

#include "fluid3d_kernels.cuh"

namespace gbsph {

constexpr uint32_t GT = 8;                 // targets a warp holds at once
constexpr uint32_t MASK_WORDS = 16;        // in-range mask words per particle (candidates <= 512)
constexpr uint32_t MASK_STAGE_WORDS = 4096;  // mask words of a brick the force pass stages
constexpr uint32_t CELL_INDEX_STAGE = 512;   // permutation entries of a brick the force pass stages
constexpr float FAR_AWAY = 1.0e30f;          // coordinate of a padding candidate (r^2 overflows)

constexpr size_t DENSITY_CELLS_SMEM = (size_t)BRICK_CAP * 16;
constexpr size_t FORCE_CELLS_SMEM = (size_t)BRICK_CAP * 32 + (size_t)MASK_STAGE_WORDS * 4 + (size_t)(CELL_INDEX_STAGE + 4) * 4;

// Per-warp map of a cell's candidate sequence: cum[r] = candidates before row r (cum[R] = nk,
// cum[R + 1] = EMPTY as a sentinel); adj[r] = staged (or sorted) index of the row's first
// candidate minus cum[r], so candidate k of row r is at index k + adj[r].
template <int R>
struct CellMap {
    uint32_t cum[BRICK_WARPS][R + 2];
    uint32_t adj_s[BRICK_WARPS][R];
    uint32_t adj_g[BRICK_WARPS][R];
};

// Builds the warp's map for cell c of the brick; returns nk (all lanes).
template <int R>
__device__ __forceinline__ uint32_t cell_map(CellMap<R>& M, const BrickShared& S, int warp, int lane, int c) {
    uint32_t len = 0, st_s = 0, st_g = 0;
    if (lane < R) {
        const uint32_t lo = S.off[lane][c];
        len = S.off[lane][c + 3] - lo;
        st_s = S.base[lane] + lo;
        st_g = S.lo[lane] + lo;
    }
    uint32_t inc = len;
#pragma unroll
    for (int o = 1; o < 16; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
    }
    const uint32_t nk = __shfl_sync(0xffffffffu, inc, R - 1);
    if (lane < R) {
        const uint32_t cum = inc - len;
        M.cum[warp][lane] = cum;
        M.adj_s[warp][lane] = st_s - cum;
        M.adj_g[warp][lane] = st_g - cum;
    }
    if (lane == R) M.cum[warp][R] = nk;
    if (lane == R + 1) M.cum[warp][R + 1] = EMPTY;
    __syncwarp();
    return nk;
}

// A lane's position in the candidate sequence: row r, where row r + 1 starts, and the row's
// index adjustment. Advanced monotonically.
struct CellCursor {
    uint32_t r, next, adj;
};

template <int R, bool STAGED>
__device__ __forceinline__ void cursor_start(const CellMap<R>& M, int warp, CellCursor& cu) {
    cu.r = 0;
    cu.next = M.cum[warp][1];
    cu.adj = STAGED ? M.adj_s[warp][0] : M.adj_g[warp][0];
}

template <int R, bool STAGED>
__device__ __forceinline__ uint32_t cursor_index(const CellMap<R>& M, int warp, CellCursor& cu, uint32_t k) {
    while (k >= cu.next) {
        ++cu.r;
        cu.next = M.cum[warp][cu.r + 1];
        cu.adj = STAGED ? M.adj_s[warp][cu.r < R ? cu.r : R - 1] : M.adj_g[warp][cu.r < R ? cu.r : R - 1];
    }
    return k + cu.adj;
}

// Sorted index of candidate k (for the recorded lists); k < nk.
template <int R>
__device__ __forceinline__ uint32_t cursor_sorted(const CellMap<R>& M, int warp, const CellCursor& cu, uint32_t k) {
    return k + M.adj_g[warp][cu.r];
}

// Transposing butterfly: v[i] (i < GT) summed over the warp; lane 4 i ends with target i's sum.
__device__ __forceinline__ float warp_sum8(const float (&v)[GT], int lane) {
    const bool b4 = lane & 16, b3 = lane & 8, b2 = lane & 4;
    float v4[4], v2[2];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float keep = b4 ? v[i + 4] : v[i], send = b4 ? v[i] : v[i + 4];
        v4[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float keep = b3 ? v4[i + 2] : v4[i], send = b3 ? v4[i] : v4[i + 2];
        v2[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    float v1;
    {
        const float keep = b2 ? v2[1] : v2[0], send = b2 ? v2[0] : v2[1];
        v1 = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
    v1 += __shfl_xor_sync(0xffffffffu, v1, 2);
    v1 += __shfl_xor_sync(0xffffffffu, v1, 1);
    return v1;
}

// Density + pressure of every particle of the occupied bricks (clCalculateDensity,
// libCL/phys/oclFluid3D.cl:150-200): sorted position .w = density, sorted velocity .w =
// pressure. Writes the in-range masks: word j of the brick's u-th target (the brick's targets
// are the consecutive sorted particles of its centre row) at masks[tfirst * MASK_WORDS + j *
// ntarg + u]; a cell with more than 32 * MASK_WORDS candidates writes none (the force pass
// tests those candidates itself). Every target meets itself (r^2 = 0, term h^6, counted);
// that term is removed after the sum and the count excludes it, as the reference's j !=
// particle test does. While an adjoint records (kp.rec_nbr), the in-range candidates'
// sorted indices (the target included) go to its tape slot in candidate order.
template <int DIMS, bool BATCH>
__global__ void __launch_bounds__(BRICK_THREADS, 3) k_density_cells(float4* __restrict__ spos, float4* __restrict__ svel,
                                                                 const uint2* __restrict__ table,
                                                                 const uint32_t* __restrict__ bricks, uint32_t* counters,
                                                                 KParams kp, uint32_t* __restrict__ masks, uint32_t* err) {
    constexpr int R = DIMS == 3 ? 9 : 3;
    constexpr int RC = DIMS == 3 ? 4 : 1;
    extern __shared__ float4 s_buf[];  // [BRICK_CAP] staged positions
    __shared__ BrickShared S;
    __shared__ CellMap<R> M;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) {
        mbar_init(reinterpret_cast<uint64_t*>(&S.bar), 1);
        fence_mbar_init();
    }
    uint32_t phase = 0;
    const uint32_t n_bricks = counters[0];
    const float h2 = kp.h2, thr = kp.r2_thresh, h6 = kp.h2 * kp.h2 * kp.h2;
    const uint32_t buf_a = smem_addr(s_buf);
    if (t == 0) S.brick = atomicAdd(&counters[1], 1u);
    for (;;) {
        __syncthreads();
        const uint32_t b = S.brick;
        if (b >= n_bricks) break;
        uint32_t next_brick = 0;
        if (t == 0) next_brick = atomicAdd(&counters[1], 1u);
        int x0, ncell;
        brick_setup<DIMS, BATCH>(S, kp, bricks[b], table, err, x0, ncell);
        const bool staged = brick_stage<DIMS, 1>(S, s_buf, BRICK_CAP, spos, nullptr);
        if (staged && !brick_wait(S, phase, err)) return;
        const uint32_t tbeg = S.off[RC][1];
        const uint32_t tfirst = S.lo[RC] + tbeg, ntarg = S.off[RC][ncell + 1] - tbeg;
        uint32_t* mb = masks + (size_t)tfirst * MASK_WORDS;
        for (int c = warp; c < ncell; c += BRICK_WARPS) {
            const uint32_t nk = cell_map<R>(M, S, warp, lane, c);
            const uint32_t rounds = (nk + 31u) >> 5;
            const bool keep = rounds <= MASK_WORDS;
            const uint32_t t0 = S.off[RC][c + 1], nt = S.off[RC][c + 2] - t0;
            for (uint32_t g0 = 0; g0 < nt; g0 += GT) {
                const uint32_t g = min(GT, nt - g0);
                const uint32_t tl0 = t0 + g0;  // the group's first target in the centre row
                float px[GT], py[GT], pz[GT], acc[GT];
#pragma unroll
                for (uint32_t i = 0; i < GT; ++i) {
                    float4 p = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (i < g) p = staged ? s_buf[S.base[RC] + tl0 + i] : spos[S.lo[RC] + tl0 + i];
                    px[i] = p.x;
                    py[i] = p.y;
                    pz[i] = p.z;
                    acc[i] = 0.0f;
                }
                uint32_t cnt = 0;       // lane i < g: in-range candidates of target i
                uint32_t rbase[GT];     // recording: entries written so far per target
#pragma unroll
                for (uint32_t i = 0; i < GT; ++i) rbase[i] = 0;
                size_t rec0 = 0;
                if (kp.rec_nbr) rec0 = (size_t)*kp.rec_slot * kp.rec_n4;
                CellCursor cu;
                if (staged) cursor_start<R, true>(M, warp, cu);
                else cursor_start<R, false>(M, warp, cu);
#pragma unroll 1
                for (uint32_t j = 0; j < rounds; ++j) {
                    const uint32_t k = (j << 5) + (uint32_t)lane;
                    const bool valid = k < nk;
                    float4 pj = make_float4(FAR_AWAY, FAR_AWAY, FAR_AWAY, 0.f);
                    if (valid) {
                        if (staged) pj = lds_f4(buf_a + cursor_index<R, true>(M, warp, cu, k) * 16u);
                        else pj = spos[cursor_index<R, false>(M, warp, cu, k)];
                    }
                    uint32_t mine = 0;
#pragma unroll
                    for (uint32_t i = 0; i < GT; ++i) {
                        if (i < g) {
                            const float dx = px[i] - pj.x, dy = py[i] - pj.y;
                            float r2 = fmaf(dy, dy, dx * dx);
                            if (DIMS == 3) {
                                const float dz = pz[i] - pj.z;
                                r2 = fmaf(dz, dz, r2);
                            }
                            const bool in = r2 < thr;
                            const float tt = in ? h2 - r2 : 0.0f;
                            acc[i] = fmaf(tt * tt, tt, acc[i]);
                            const uint32_t w = __ballot_sync(0xffffffffu, in);
                            mine = lane == (int)i ? w : mine;
                            if (kp.rec_nbr) {
                                const uint32_t pos = rbase[i] + __popc(w & lanemask_lt());
                                if (in && pos < NBR_CAP)
                                    kp.rec_nbr[(rec0 + S.lo[RC] + tl0 + i) * NBR_CAP + pos] =
                                        cursor_sorted<R>(M, warp, cu, k);
                                rbase[i] += __popc(w);
                            }
                        }
                    }
                    if ((uint32_t)lane < g) {
                        cnt += __popc(mine);
                        if (keep) mb[(size_t)j * ntarg + (tl0 - tbeg) + lane] = mine;
                    }
                }
                const float sum = warp_sum8(acc, lane);
                const float tot = __shfl_sync(0xffffffffu, sum, (lane & 7) * 4);
                if ((uint32_t)lane < g) {
                    const uint32_t gi = S.lo[RC] + tl0 + lane;
                    const float a = tot - h6;  // the target's own term
                    const uint32_t count = cnt - 1u;
                    float rho = kp.rho0, p = kp.p0;
                    if (count > 2u) {
                        rho = fmaxf(1.0f, kp.mass * kp.kconst * a);
                        p = kp.p0 + S.stiff * (rho - kp.rho0);
                    }
                    reinterpret_cast<float*>(spos)[4 * (size_t)gi + 3] = rho;
                    reinterpret_cast<float*>(svel)[4 * (size_t)gi + 3] = p;
                    if (kp.rec_cnt) kp.rec_cnt[rec0 + gi] = cnt > NBR_CAP ? REC_SCAN : cnt;
                }
            }
        }
        if (t == 0) S.brick = next_brick;  // read by every thread after the barrier at the top
    }
}

// A candidate's position and velocity as the force pass uses them: w lanes a = 1/rho and
// b = p/rho (force_pair_pre). From the staging buffer (already converted) or from global
// memory (converted here with the same instruction, so both paths give the same bits).
template <bool STAGED>
__device__ __forceinline__ void force_candidate(const float4* s_pos, const float4* s_vel, const float4* __restrict__ spos,
                                                const float4* __restrict__ svel, uint32_t idx, float4& pj, float4& vj) {
    if (STAGED) {
        pj = s_pos[idx];
        vj = s_vel[idx];
    } else {
        pj = spos[idx];
        vj = svel[idx];
        const float a = rcp_approx(pj.w);
        pj.w = a;
        vj.w *= a;
    }
}

// Forces (pressure + viscosity; clCalculateForces, libCL/phys/oclFluid3D.cl:202-255) for every
// particle of the occupied bricks, from the in-range masks of k_density_cells. With FUSED the
// clip-box, integrate-force, gravity and integrate-velocity stages follow in registers;
// otherwise the SPH force is added to force[index[i]] (w = 0) as clCalculateForces does.
template <int DIMS, bool FUSED, bool BATCH>
__global__ void __launch_bounds__(BRICK_THREADS, 3) k_force_cells(const float4* __restrict__ spos,
                                                               const float4* __restrict__ svel,
                                                               const uint32_t* __restrict__ index,
                                                               float4* __restrict__ pos, float4* __restrict__ vel,
                                                               float4* __restrict__ force, const uint2* __restrict__ table,
                                                               const uint32_t* __restrict__ bricks, uint32_t* counters,
                                                               KParams kp, const uint32_t* __restrict__ masks,
                                                               uint32_t* err) {
    constexpr int R = DIMS == 3 ? 9 : 3;
    constexpr int RC = DIMS == 3 ? 4 : 1;
    // [BRICK_CAP] positions, [BRICK_CAP] velocities, the brick's mask words, its permutation entries
    extern __shared__ float4 s_buf[];
    __shared__ BrickShared S;
    __shared__ CellMap<R> M;
    __shared__ uint32_t s_rounds, s_mstaged, s_istaged;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0) {
        mbar_init(reinterpret_cast<uint64_t*>(&S.bar), 1);
        fence_mbar_init();
    }
    uint32_t phase = 0;
    const uint32_t n_bricks = counters[0];
    float4* s_pos = s_buf;
    float4* s_vel = s_buf + BRICK_CAP;
    uint32_t* s_mask = reinterpret_cast<uint32_t*>(s_buf + 2 * BRICK_CAP);
    uint32_t* s_index = s_mask + MASK_STAGE_WORDS;
    if (t == 0) S.brick = atomicAdd(&counters[2], 1u);
    for (;;) {
        __syncthreads();
        const uint32_t b = S.brick;
        if (b >= n_bricks) break;
        uint32_t next_brick = 0;
        if (t == 0) next_brick = atomicAdd(&counters[2], 1u);
        int x0, ncell;
        brick_setup<DIMS, BATCH>(S, kp, bricks[b], table, err, x0, ncell);
        const uint32_t tbeg = S.off[RC][1];
        const uint32_t tfirst = S.lo[RC] + tbeg, ntarg = S.off[RC][ncell + 1] - tbeg;
        if (warp == 0) {
            // mask words per target the brick needs: the most rounds of any of its cells
            uint32_t nk = 0;
            if (lane < ncell)
                for (int r = 0; r < R; ++r) nk += S.off[r][lane + 3] - S.off[r][lane];
            const uint32_t rd = __reduce_max_sync(0xffffffffu, (nk + 31u) >> 5);
            if (lane == 0) {
                uint32_t acc = 0;
                for (int r = 0; r < R; ++r) {
                    S.base[r] = acc;
                    acc += S.rcnt[r];
                }
                S.total = acc;
                const uint32_t rw = min(rd, MASK_WORDS);
                // 16-byte copies: whole words from a 16-byte aligned start
                const uint32_t mwords = (rw * ntarg + 3u) & ~3u;
                const uint32_t i0 = tfirst & ~3u, iwords = ((tfirst + ntarg + 3u) & ~3u) - i0;
                const bool rows = acc <= BRICK_CAP && acc > 0;
                const bool mst = rows && mwords > 0 && mwords <= MASK_STAGE_WORDS;
                const bool ist = rows && iwords <= CELL_INDEX_STAGE + 4;
                s_rounds = rw;
                s_mstaged = mst;
                s_istaged = ist;
                if (rows) {
                    fence_proxy_async_smem();
                    mbar_arrive_expect_tx(reinterpret_cast<uint64_t*>(&S.bar),
                                          acc * 32u + (mst ? mwords * 4u : 0u) + (ist ? iwords * 4u : 0u));
                    for (int r = 0; r < R; ++r) {
                        if (!S.rcnt[r]) continue;
                        bulk_g2s(s_pos + S.base[r], spos + S.lo[r], S.rcnt[r] * 16u, reinterpret_cast<uint64_t*>(&S.bar));
                        bulk_g2s(s_vel + S.base[r], svel + S.lo[r], S.rcnt[r] * 16u, reinterpret_cast<uint64_t*>(&S.bar));
                    }
                    if (mst)
                        bulk_g2s(s_mask, masks + (size_t)tfirst * MASK_WORDS, mwords * 4u,
                                 reinterpret_cast<uint64_t*>(&S.bar));
                    if (ist) bulk_g2s(s_index, index + i0, iwords * 4u, reinterpret_cast<uint64_t*>(&S.bar));
                }
            }
        }
        __syncthreads();
        const bool staged = S.total <= BRICK_CAP && S.total > 0;
        const bool mstaged = s_mstaged, istaged = s_istaged;
        if (staged) {
            if (!brick_wait(S, phase, err)) return;
            for (uint32_t k = t; k < S.total; k += BRICK_THREADS) {  // w lanes: 1/rho and p/rho
                const float a = rcp_approx(s_pos[k].w);
                s_pos[k].w = a;
                s_vel[k].w *= a;
            }
            __syncthreads();
        }
        const uint32_t* mglob = masks + (size_t)tfirst * MASK_WORDS;
        const uint32_t i0 = tfirst & ~3u;
        for (int c = warp; c < ncell; c += BRICK_WARPS) {
            const uint32_t nk = cell_map<R>(M, S, warp, lane, c);
            const uint32_t rounds = (nk + 31u) >> 5;
            const bool scan = rounds > MASK_WORDS;  // no masks: test every candidate
            const uint32_t t0 = S.off[RC][c + 1], nt = S.off[RC][c + 2] - t0;
            for (uint32_t g0 = 0; g0 < nt; g0 += GT) {
                const uint32_t g = min(GT, nt - g0);
                const uint32_t lq = g > 4 ? 2u : (g > 2 ? 3u : (g > 1 ? 4u : 5u));  // log2 Q
                const uint32_t Q = 1u << lq;
                const uint32_t ti = (uint32_t)lane >> lq, q = (uint32_t)lane & (Q - 1u);
                const bool active = ti < g;
                const uint32_t tl = t0 + g0 + (active ? ti : 0u);
                const uint32_t u = tl - tbeg;
                const uint32_t gi = S.lo[RC] + tl;
                float4 pi, vi;
                if (staged) {
                    pi = s_pos[S.base[RC] + tl];
                    vi = s_vel[S.base[RC] + tl];
                } else {
                    force_candidate<false>(s_pos, s_vel, spos, svel, gi, pi, vi);
                }
                uint32_t o = 0;
                float4 f_o = make_float4(0.f, 0.f, 0.f, 0.f), v_o = f_o, p_o = f_o;
                if (active && q == 0) {  // what the integration needs, fetched early
                    o = istaged ? s_index[gi - i0] : index[gi];
                    f_o = force[o];
                    if (FUSED) {
                        v_o = vel[o];
                        p_o = pos[o];
                    }
                }
                float acc[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                if (active) {
                    CellCursor cu;
                    if (staged) cursor_start<R, true>(M, warp, cu);
                    else cursor_start<R, false>(M, warp, cu);
                    if (!scan) {
                        const uint32_t pat = (Q == 32u ? 1u : 0xFFFFFFFFu / ((1u << Q) - 1u)) << q;
#pragma unroll 1
                        for (uint32_t j = 0; j < rounds; ++j) {
                            const uint32_t wi = j * ntarg + u;
                            uint32_t w = (mstaged ? s_mask[wi] : mglob[wi]) & pat;
                            while (w) {
                                const uint32_t bit = (uint32_t)(__ffs(w) - 1);
                                w &= w - 1u;
                                const uint32_t k = (j << 5) + bit;
                                float4 pj, vj;
                                if (staged) force_candidate<true>(s_pos, s_vel, spos, svel, cursor_index<R, true>(M, warp, cu, k), pj, vj);
                                else force_candidate<false>(s_pos, s_vel, spos, svel, cursor_index<R, false>(M, warp, cu, k), pj, vj);
                                force_pair_pre<DIMS>(pi, vi, pj, vj, kp.h, acc);
                            }
                        }
                    } else {
#pragma unroll 1
                        for (uint32_t k = q; k < nk; k += Q) {
                            float4 pj, vj;
                            if (staged) force_candidate<true>(s_pos, s_vel, spos, svel, cursor_index<R, true>(M, warp, cu, k), pj, vj);
                            else force_candidate<false>(s_pos, s_vel, spos, svel, cursor_index<R, false>(M, warp, cu, k), pj, vj);
                            const float dx = pi.x - pj.x, dy = pi.y - pj.y;
                            float r2 = fmaf(dy, dy, dx * dx);
                            if (DIMS == 3) {
                                const float dz = pi.z - pj.z;
                                r2 = fmaf(dz, dz, r2);
                            }
                            if (r2 < kp.r2_thresh) force_pair_pre<DIMS>(pi, vi, pj, vj, kp.h, acc);
                        }
                    }
                }
                for (uint32_t m = 1; m < Q; m <<= 1) {
#pragma unroll
                    for (int e = 0; e < 6; ++e) acc[e] += __shfl_xor_sync(0xffffffffu, acc[e], m);
                }
                if (active && q == 0) {
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
        }
        if (t == 0) S.brick = next_brick;  // read by every thread after the barrier at the top
    }
}

}  // namespace gbsph
