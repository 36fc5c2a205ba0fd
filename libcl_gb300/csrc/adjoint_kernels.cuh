// adjoint_kernels.cuh -- reverse-mode derivative of the LINEAR_GRID 3D step (density, forces,
// clip box, clamp, symplectic Euler; libCL/phys/oclFluid3D.cl:150-298,304-361) with the
// forward permutation and neighbour sets held fixed. For one step, in sorted order i with
// particle o = index[i]:
//   rho_i = max(1, m K S_i) if count_i > 2 else rho0,   S_i = sum_j (h^2 - r_ij^2)^3
//   p_i   = p0 + k (rho_i - rho0)
//   F_i   = F0_o + m [Cp sum_j (p_i+p_j)/(rho_i rho_j) d_ij (h-r)^2 / r
//                   + Cv sum_j (v_j-v_i)/(rho_i rho_j) (h-r)] + walls(x_i, v_i)
//   v'_o  = v_o + clamp(F_i) dt,   x'_o = x_o + v'_o dt
// with d_ij = x_i - x_j, r = |d_ij|, Cv = mu * 45 / (pi h^6). The neighbour relation is
// symmetric, so the loss terms of a pair {i, j} depend only on w_i - w_j (w = m dL/dF) and
// dL/dS_i + dL/dS_j: each kernel gathers over its own particle's neighbours (the list the
// forward's density pass recorded, or the cells) and nothing is scattered (deterministic, no
// atomics). The count > 2, max(1, .), clamp and wall branches are
// differentiated on the side the forward step took.
#pragma once

#include "fluid3d_access.h"

namespace gbsph {

// ---- the recorded step ----------------------------------------------------------------------

// What the backward pass of one step reads: the forward's sorted keys and permutation, the
// sorted state with w = density (positions) and pressure (velocities), and the force after
// the clip box in particle order.
struct StepTape {
    uint32_t* index;
    uint32_t* keys;
    float4* spos;
    float4* svel;
    float4* fwall;
    const uint32_t* nbr;  // the density pass's neighbour lists (NBR_CAP per particle, sorted indices)
    const uint32_t* cnt;  // their lengths, or REC_SCAN: walk the cells instead
};

static __global__ void k_tape_record(StepTape dst, const uint32_t* __restrict__ index,
                                     const uint32_t* __restrict__ keys, const float4* __restrict__ spos,
                                     const float4* __restrict__ svel, const float4* __restrict__ fwall, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dst.index[i] = index[i];
    dst.keys[i] = keys[i];
    dst.spos[i] = spos[i];
    dst.svel[i] = svel[i];
    dst.fwall[i] = fwall[i];
}

// Lanes that share a particle in the gather kernels below: lane q takes entries q, q + 4, ...
// of the particle's list (or candidates q, q + 4, ... of each neighbour cell), and the lanes'
// partial sums are added with shuffles in a fixed order (deterministic).
constexpr uint32_t ADJ_LANES = 4;

__device__ __forceinline__ float adj_lane_sum(float v) {
#pragma unroll
    for (uint32_t m = ADJ_LANES >> 1; m > 0; m >>= 1) v += __shfl_xor_sync(0xffffffffu, v, m);
    return v;
}

// Calls f(j, dx, dy, dz, r2) for every neighbour j != i with sqrtf(r2) < h among candidates
// q, q + ADJ_LANES, ... of each of the 27 neighbour cells of the LINEAR_GRID table (z, y, x
// order).
template <class F>
__device__ __forceinline__ void for_each_neighbour(const KParams& kp, const uint2* __restrict__ table,
                                                   const float4* __restrict__ spos, uint32_t i, const float4& pi,
                                                   uint32_t q, F&& f) {
    int gx, gy, gz;
    grid_position(kp, pi, gx, gy, gz);
    gx = clampi(gx, 0, kp.nx - 1);
    gy = clampi(gy, 0, kp.ny - 1);
    gz = clampi(gz, 0, kp.nz - 1);
    for (int z = -1; z <= 1; z++) {
        const int cz = gz + z;
        if (cz < 0 || cz >= kp.nz) continue;
        for (int y = -1; y <= 1; y++) {
            const int cy = gy + y;
            if (cy < 0 || cy >= kp.ny) continue;
            const uint32_t row = (uint32_t)kp.nx * ((uint32_t)cy + (uint32_t)kp.ny * (uint32_t)cz);
            for (int x = -1; x <= 1; x++) {
                const int cx = gx + x;
                if (cx < 0 || cx >= kp.nx) continue;
                const uint2 e = table[row + (uint32_t)cx];
                if (e.x == EMPTY) continue;
                for (uint32_t j = e.x + q; j < e.y; j += ADJ_LANES) {
                    if (j == i) continue;
                    const float4 pj = spos[j];
                    const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
                    const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
                    if (r2 < kp.r2_thresh) f(j, dx, dy, dz, r2);
                }
            }
        }
    }
}

// Calls f(j, dx, dy, dz, r2) for lane q's share of the neighbours j != i of the recorded step:
// entries q, q + ADJ_LANES, ... of the list the density pass recorded for i, or (list
// overflowed, brick not staged) lane q's candidates of the cell walk.
template <class F>
__device__ __forceinline__ void for_each_recorded(const KParams& kp, const StepTape& t, const uint2* __restrict__ table,
                                                  uint32_t i, const float4& pi, uint32_t q, F&& f) {
    const uint32_t n = t.cnt[i];
    if (n == REC_SCAN) {
        for_each_neighbour(kp, table, t.spos, i, pi, q, f);
        return;
    }
    const uint32_t* l = t.nbr + (size_t)i * NBR_CAP;
    for (uint32_t e = q; e < n; e += ADJ_LANES) {
        const uint32_t j = l[e];
        if (j == i) continue;
        const float4 pj = t.spos[j];
        const float dx = pi.x - pj.x, dy = pi.y - pj.y, dz = pi.z - pj.z;
        const float r2 = fmaf(dz, dz, fmaf(dy, dy, dx * dx));
        if (r2 < kp.r2_thresh) f(j, dx, dy, dz, r2);
    }
}

// Integration, clamp and walls, backwards, plus the step's cell table. In: dL/dx', dL/dv'
// (particle order). Out (sorted order): w = m dL/dF, and dL/dx, dL/dv without the SPH terms.
// The table `own` (clean on entry) receives this step's cell ranges; if `keys_next` is set,
// the ranges of that step are erased from `other`, which this step does not read.
static __global__ void __launch_bounds__(256) k_adj_post(StepTape t, const float4* __restrict__ gx,
                                                         const float4* __restrict__ gv, float4* __restrict__ w,
                                                         float4* __restrict__ gxs, float4* __restrict__ gvs,
                                                         uint2* __restrict__ own, uint2* __restrict__ other,
                                                         const uint32_t* __restrict__ keys_next, KParams kp) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kp.n) return;
    const uint32_t k = t.keys[i];
    if (k < kp.table_cells) {
        if (i == 0 || t.keys[i - 1] != k) own[k].x = i;
        if (i + 1 == kp.n || t.keys[i + 1] != k) own[k].y = i + 1;
    }
    if (keys_next) {
        const uint32_t kn = keys_next[i];
        if ((i == 0 || keys_next[i - 1] != kn) && kn < kp.table_cells) other[kn] = make_uint2(EMPTY, EMPTY);
    }
    const uint32_t o = t.index[i];
    const float4 x = t.spos[i], f = t.fwall[o], g_x = gx[o], g_v = gv[o];
    // x' = x + v' dt, v' = v + clamp(F) dt
    const float3 gvt = make_float3(fmaf(g_x.x, kp.dt, g_v.x), fmaf(g_x.y, kp.dt, g_v.y), fmaf(g_x.z, kp.dt, g_v.z));
    float3 gf = make_float3(gvt.x * kp.dt, gvt.y * kp.dt, gvt.z * kp.dt);
    const float f2 = f.x * f.x + f.y * f.y + f.z * f.z + f.w * f.w;
    const float speed = sqrtf(f2);
    if (speed > kp.vlimit) {  // clamp(F) = L F / |F|: dL/dF = (L / |F|) (g - F (F.g) / |F|^2)
        const float s = kp.vlimit / speed, fg = (f.x * gf.x + f.y * gf.y + f.z * gf.z) / f2;
        gf = make_float3(s * (gf.x - f.x * fg), s * (gf.y - f.y * fg), s * (gf.z - f.z * fg));
    }
    // an active wall adds 2000 * (r - distance) - 256 * (normal . v) along its normal:
    // -2000 to dF_a/dx_a and -256 to dF_a/dv_a for either wall of axis a
    float3 ax = make_float3(0.f, 0.f, 0.f), av = make_float3(0.f, 0.f, 0.f);
    const float r = kp.radius;
    auto wall = [&](float diff, float ga, float& cx, float& cv) {
        if (diff > 0.00001f) {
            cx -= 2000.0f * ga;
            cv -= 256.0f * ga;
        }
    };
    wall(r - (x.y - kp.box_min.y), gf.y, ax.y, av.y);
    wall(r - (kp.box_max.y - x.y), gf.y, ax.y, av.y);
    wall(r - (x.z - kp.box_min.z), gf.z, ax.z, av.z);
    wall(r - (kp.box_max.z - x.z), gf.z, ax.z, av.z);
    wall(r - (x.x - kp.box_min.x), gf.x, ax.x, av.x);
    wall(r - (kp.box_max.x - x.x), gf.x, ax.x, av.x);
    w[i] = make_float4(kp.mass * gf.x, kp.mass * gf.y, kp.mass * gf.z, 0.f);
    gxs[i] = make_float4(g_x.x + ax.x, g_x.y + ax.y, g_x.z + ax.z, 0.f);
    gvs[i] = make_float4(gvt.x + av.x, gvt.y + av.y, gvt.z + av.z, 0.f);
}

// SPH force and pressure law, backwards (gather over neighbours): adds the pair terms to
// dL/dx and dL/dv, writes dL/dS (zero where the forward clamped the density to 1 or set it to
// rho0 because count <= 2), and accumulates per particle (particle order, FP64) the stiffness
// term (rho - rho0) dL/dp and the viscosity term dL/dmu = (45 / (pi h^6)) w . B.
// ADJ_LANES threads per particle.
static __global__ void __launch_bounds__(256) k_adj_force(StepTape t, const uint2* __restrict__ table,
                                                          const float4* __restrict__ w, float4* __restrict__ gxs,
                                                          float4* __restrict__ gvs, float* __restrict__ gS,
                                                          double2* __restrict__ acc, KParams kp, float c45) {
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gt / ADJ_LANES, q = gt % ADJ_LANES;
    const bool live = i < kp.n;
    const float4* __restrict__ spos = t.spos;
    const float4* __restrict__ svel = t.svel;
    const float4 xi = live ? spos[i] : make_float4(0.f, 0.f, 0.f, 1.f), vi = live ? svel[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 wi = live ? w[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float rho_i = xi.w, p_i = vi.w, h = kp.h, cp = kp.cpress, cv = kp.cvisc;
    float3 ax = make_float3(0.f, 0.f, 0.f), av = make_float3(0.f, 0.f, 0.f), bsum = make_float3(0.f, 0.f, 0.f);
    float ap = 0.f, arho = 0.f;
    int count = 0;
    if (live) for_each_recorded(kp, t, table, i, xi, q, [&](uint32_t j, float dx, float dy, float dz, float r2) {
        count++;
        if (!(r2 > 0.0f)) return;  // coincident particles exert no force
        const float4 xj = spos[j], vj = svel[j], wj = w[j];
        const float rinv = rsqrtf(r2), r = r2 * rinv, hr = h - r;
        const float D = 1.0f / (rho_i * xj.w), P = p_i + vj.w;
        const float phi = hr * hr * rinv;                         // (h - r)^2 / r
        const float dphi_r = -hr * (h + r) * rinv * rinv * rinv;  // phi'(r) / r
        const float dwx = wi.x - wj.x, dwy = wi.y - wj.y, dwz = wi.z - wj.z;
        const float dvx = vj.x - vi.x, dvy = vj.y - vi.y, dvz = vj.z - vi.z;
        const float ddw = dx * dwx + dy * dwy + dz * dwz;
        const float dwu = phi * ddw;  // (w_i - w_j) . d phi
        const float dwdv = dwx * dvx + dwy * dvy + dwz * dvz;
        const float cJ = cp * P * D, cD = cv * D * dwdv * rinv, cvh = cv * D * hr;
        ax.x += cJ * fmaf(dphi_r * dx, ddw, phi * dwx) - cD * dx;
        ax.y += cJ * fmaf(dphi_r * dy, ddw, phi * dwy) - cD * dy;
        ax.z += cJ * fmaf(dphi_r * dz, ddw, phi * dwz) - cD * dz;
        av.x -= cvh * dwx;
        av.y -= cvh * dwy;
        av.z -= cvh * dwz;
        ap += cp * D * dwu;
        arho -= (D / rho_i) * fmaf(cp * P, dwu, cv * hr * dwdv);
        const float dh = D * hr;
        bsum.x += dvx * dh;
        bsum.y += dvy * dh;
        bsum.z += dvz * dh;
    });
    ax = make_float3(adj_lane_sum(ax.x), adj_lane_sum(ax.y), adj_lane_sum(ax.z));
    av = make_float3(adj_lane_sum(av.x), adj_lane_sum(av.y), adj_lane_sum(av.z));
    bsum = make_float3(adj_lane_sum(bsum.x), adj_lane_sum(bsum.y), adj_lane_sum(bsum.z));
    ap = adj_lane_sum(ap);
    arho = adj_lane_sum(arho);
    count = (int)adj_lane_sum((float)count);
    if (!live || q != 0) return;
    float4 g = gxs[i];
    gxs[i] = make_float4(g.x + ax.x, g.y + ax.y, g.z + ax.z, 0.f);
    g = gvs[i];
    gvs[i] = make_float4(g.x + av.x, g.y + av.y, g.z + av.z, 0.f);
    const bool active = count > 2 && rho_i > 1.0f;  // rho = max(1, m K S) took the m K S side
    gS[i] = active ? kp.mass * kp.kconst * fmaf(kp.stiff, ap, arho) : 0.f;
    const uint32_t o = t.index[i];
    double2 a = acc[o];
    a.x += (double)((rho_i - kp.rho0) * ap);
    a.y += (double)(c45 * (wi.x * bsum.x + wi.y * bsum.y + wi.z * bsum.z));
    acc[o] = a;
}

// Density sum, backwards: dL/dx_i += -6 sum_j (h^2 - r^2)^2 d_ij (dL/dS_i + dL/dS_j); the
// step's input gradients go back to particle order.
// ADJ_LANES threads per particle.
static __global__ void __launch_bounds__(256) k_adj_density(StepTape t, const uint2* __restrict__ table,
                                                            const float* __restrict__ gS,
                                                            const float4* __restrict__ gxs,
                                                            const float4* __restrict__ gvs, float4* __restrict__ gx,
                                                            float4* __restrict__ gv, KParams kp) {
    const uint32_t gt = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t i = gt / ADJ_LANES, q = gt % ADJ_LANES;
    const bool live = i < kp.n;
    const float4 xi = live ? t.spos[i] : make_float4(0.f, 0.f, 0.f, 0.f);
    const float gSi = live ? gS[i] : 0.f;
    float3 a = make_float3(0.f, 0.f, 0.f);
    if (live) for_each_recorded(kp, t, table, i, xi, q, [&](uint32_t j, float dx, float dy, float dz, float r2) {
        const float tt = kp.h2 - r2;
        const float c = -6.0f * tt * tt * (gSi + gS[j]);
        a.x = fmaf(c, dx, a.x);
        a.y = fmaf(c, dy, a.y);
        a.z = fmaf(c, dz, a.z);
    });
    a = make_float3(adj_lane_sum(a.x), adj_lane_sum(a.y), adj_lane_sum(a.z));
    if (!live || q != 0) return;
    const uint32_t o = t.index[i];
    const float4 g = gxs[i];
    gx[o] = make_float4(g.x + a.x, g.y + a.y, g.z + a.z, 0.f);
    gv[o] = gvs[i];
}

// Sums the per-particle (stiffness, viscosity) terms in a fixed order into out[0], out[1].
static __global__ void __launch_bounds__(1024) k_adj_reduce(const double2* __restrict__ acc, uint32_t n,
                                                            double* __restrict__ out) {
    __shared__ double s[2][1024];
    double a = 0.0, b = 0.0;
    for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) {
        const double2 v = acc[i];
        a += v.x;
        b += v.y;
    }
    s[0][threadIdx.x] = a;
    s[1][threadIdx.x] = b;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if ((int)threadIdx.x < st) {
            s[0][threadIdx.x] += s[0][threadIdx.x + st];
            s[1][threadIdx.x] += s[1][threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = s[0][0];
        out[1] = s[1][0];
    }
}

}  // namespace gbsph
