// oracle2d.cpp -- CPU restatement of the reference's 2D SPH step (double-density relaxation).
//
// TEST INFRASTRUCTURE ONLY (see oracle3d.cpp for the rules and the parity status). Follows
// libCL/phys/oclFluid2D.cl and the driver libCL/phys/oclFluid2D.cpp:256-362 operation for
// operation in FP32 (compiled with -ffp-contract=off):
//   * `length(v)` -> sqrtf(x*x + y*y);
//   * read_imagef with CLK_NORMALIZED_COORDS_TRUE | CLK_FILTER_LINEAR | CLK_ADDRESS_CLAMP_TO_EDGE
//     -> the OpenCL bilinear formula in FP32 (u = s*W - 0.5, weights from frac(u), texel
//     indices clamped to the image), with (1-a)(1-b), a(1-b), (1-a)b, ab summed in that order;
//   * the RGBA half-float wall images -> float arrays whose values are rounded to half
//     precision (round to nearest even) when written;
//   * cell coordinates are clamped to the grid before the key is formed (the reference writes
//     outside its table when a particle leaves the container; results are the same whenever
//     particles stay inside it).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/gbsph.h"

namespace {

// libCL/phys/oclFluid2D.cl:121-133, evaluated in float like the OpenCL C macros.
const float kRestDensity = 82.0f;
const float kStiffness = 0.08f;
const float kNearStiffness = 0.1f;
const float kSurfaceTension = 21.00035f;
const float kPi = 3.1415926535f;
const float kParticleRadius = 0.05f / 5;
const float kH = (22 * 0.05f / 5);
const float kNorm = (20 / (2 * kPi * kH * kH));
const float kNearNorm = (30 / (2 * kPi * kH * kH));
const float kEps = 0.0000001f;
const uint32_t kEmpty = 0xFFFFFFFFu;

inline float half_round(float x) { return (float)(_Float16)x; }

struct P2 {
    float px, py, vx, vy, mass, unused;
};

inline float len2(float x, float y) { return std::sqrt(x * x + y * y); }

// Bilinear, normalised, clamp-to-edge sample of a float4 image (OpenCL C spec, filtering).
void sample(const float* img, int W, int H, float s, float t, float out[4]) {
    const float u = s * (float)W - 0.5f, v = t * (float)H - 0.5f;
    const float fu = std::floor(u), fv = std::floor(v);
    const float a = u - fu, b = v - fv;
    int i0 = (int)fu, j0 = (int)fv;
    int i1 = i0 + 1, j1 = j0 + 1;
    i0 = std::min(std::max(i0, 0), W - 1);
    i1 = std::min(std::max(i1, 0), W - 1);
    j0 = std::min(std::max(j0, 0), H - 1);
    j1 = std::min(std::max(j1, 0), H - 1);
    const float w00 = (1 - a) * (1 - b), w10 = a * (1 - b), w01 = (1 - a) * b, w11 = a * b;
    for (int c = 0; c < 4; c++) {
        const float t00 = img[4 * ((size_t)j0 * W + i0) + c], t10 = img[4 * ((size_t)j0 * W + i1) + c];
        const float t01 = img[4 * ((size_t)j1 * W + i0) + c], t11 = img[4 * ((size_t)j1 * W + i1) + c];
        out[c] = ((w00 * t00 + w10 * t10) + w01 * t01) + w11 * t11;
    }
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

}  // namespace

extern "C" {

// clInitFluid (libCL/phys/oclFluid2D.cl:136-151); vmax and B are never set by the reference.
void orc2d_default_params(gbsph_fluid2d_params* p) {
    std::memset(p, 0, sizeof(*p));
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

// compile(): (cellCountX*cellCountY/256 + 1)*256 table entries (libCL/phys/oclFluid2D.cpp:240-243).
uint32_t orc2d_table_size(const gbsph_fluid2d_params* p) {
    const uint32_t c = (uint32_t)(p->cellCountX * p->cellCountY);
    return (c / 256 + 1) * 256;
}

// clComputeBorder (libCL/phys/oclFluid2D.cl:358-443) over a W x H float4 mask.
void orc2d_compute_border(const float* mask, int w, int h, const gbsph_fluid2d_params* P, float* vec_out,
                          float* state_out) {
    const int dW = (int)((double)(w * P->h / P->containerW) + 0.5);
    const int dH = (int)((double)(h * P->h / P->containerH) + 0.5);
    const float dX = P->containerW / w, dY = P->containerH / h;
    const float s = (float)((double)(dX * dY) / (2 * M_PI * (double)P->particleSize * (double)P->particleSize));
    for (int y = 0; y < h; y++)
        for (int x = 0; x < w; x++) {
            const float pixel_w = mask[4 * ((size_t)y * w + x) + 3];
            float dmin = 10000;
            float vec[4] = {0, 0, 0, 0};
            float density = 0, nearDensity = 0;
            if (pixel_w == 1.0f) {
                density = 112 * P->particleMass * kNorm;
                nearDensity = 112 * P->particleMass * kNearNorm;
                for (int i = std::max(x - dW, 0); i < std::min(x + dW, w); i++)
                    for (int j = std::max(y - dH, 0); j < std::min(y + dH, h); j++) {
                        if (mask[4 * ((size_t)j * w + i) + 3] != 1.0f) {
                            const float dx = i * dX - x * dX, dy = j * dY - y * dY;
                            const float r = len2(dx, dy);
                            if (r < dmin) {
                                vec[0] = dx / r;
                                vec[1] = dy / r;
                                vec[2] = r;
                                dmin = r;
                            }
                        }
                    }
            } else {
                for (int i = std::max(x - dW, 0); i < std::min(x + dW, w); i++)
                    for (int j = std::max(y - dH, 0); j < std::min(y + dH, h); j++) {
                        if (mask[4 * ((size_t)j * w + i) + 3] == 1.0f) {
                            const float dx = x * dX - i * dX, dy = y * dY - j * dY;
                            const float r = len2(dx, dy);
                            if (r < P->h) {
                                const float a = 1 - r / P->h;
                                density += s * P->particleMass * a * a * a * kNorm;
                                nearDensity += s * P->particleMass * a * a * a * a * kNearNorm;
                                if (r < dmin) {
                                    vec[0] = dx / r;
                                    vec[1] = dy / r;
                                    vec[2] = r;
                                    dmin = r;
                                }
                            }
                        }
                    }
            }
            float* v = vec_out + 4 * ((size_t)y * w + x);
            float* st = state_out + 4 * ((size_t)y * w + x);
            for (int c = 0; c < 4; c++) v[c] = half_round(vec[c]);
            st[0] = half_round(density);
            st[1] = half_round(nearDensity);
            st[2] = half_round(kStiffness * (density - P->particleMass * kRestDensity));
            st[3] = half_round(kNearStiffness * nearDensity);
        }
}

int orc_stable_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int startBit, int endBit);

// One oclFluid2D::compute (libCL/phys/oclFluid2D.cpp:256-362) on host arrays. `state` is
// gbsph_particle2d[n] (updated in place); the wall images are W x H float4. Outputs the
// sorted keys, index, sorted state, per-particle State (float4), relaxed positions
// (float2, cell order), previous positions (float2, particle order) and the cell table.
void orc2d_step(float* state, uint32_t n, const gbsph_fluid2d_params* P, const float* border_state,
                const float* border_vec, int W, int H, uint32_t* cell, uint32_t* index, float* sorted,
                float* pstate, float* relaxed, float* prev, uint32_t* cellStart, uint32_t* cellEnd) {
    P2* st = reinterpret_cast<P2*>(state);
    P2* srt = reinterpret_cast<P2*>(sorted);
    const float dT = P->dT, m = P->particleMass, h = P->h;
    // clAdvanceState (:173-182)
    for (uint32_t i = 0; i < n; i++) {
        prev[2 * i] = st[i].px;
        prev[2 * i + 1] = st[i].py;
        st[i].vx += 0.0f * dT;
        st[i].vy += -9.81f * dT;
        st[i].px += st[i].vx * dT;
        st[i].py += st[i].vy * dT;
    }
    // clHash (:61-69), coordinates clamped to the grid
    for (uint32_t i = 0; i < n; i++) {
        const int gx = clampi((int)std::floor(st[i].px / P->cellSize), 0, P->cellCountX - 1);
        const int gy = clampi((int)std::floor(st[i].py / P->cellSize), 0, P->cellCountY - 1);
        cell[i] = (uint32_t)(gy * P->cellCountX + gx);
        index[i] = i;
    }
    orc_stable_sort(cell, index, n, 0, 24);
    for (uint32_t i = 0; i < n; i++) srt[i] = st[index[i]];  // clReorder (:71-76)
    // clInitBounds + clFindBounds (:78-113)
    const uint32_t table = (uint32_t)(P->cellCountX * P->cellCountY) / 256 * 256 + 256;
    for (uint32_t c = 0; c < table; c++) cellStart[c] = cellEnd[c] = kEmpty;
    for (uint32_t p = 0; p < n; p++) {
        if (p == 0) {
            cellStart[cell[0]] = 0;
            continue;
        }
        if (cell[p] != cell[p - 1]) {
            cellEnd[cell[p - 1]] = p;
            cellStart[cell[p]] = p;
        }
        if (p == n - 1) cellEnd[cell[p]] = n;
    }
    auto cells_of = [&](const P2& pi, int& x0, int& x1, int& y0, int& y1) {
        const int gx = (int)std::floor(pi.px / P->cellSize), gy = (int)std::floor(pi.py / P->cellSize);
        x0 = std::max(gx - 1, 0);
        x1 = std::min(gx + 1, P->cellCountX - 1);
        y0 = std::max(gy - 1, 0);
        y1 = std::min(gy + 1, P->cellCountY - 1);
    };
    // clComputePressure (:185-245)
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        const uint32_t i = (uint32_t)ii;
        const P2 pi = srt[i];
        int x0, x1, y0, y1;
        cells_of(pi, x0, x1, y0, y1);
        float density = 0, nearDensity = 0;
        float wall[4];
        sample(border_state, W, H, pi.px / P->containerW, pi.py / P->containerH, wall);
        if (wall[0] != 0) {
            density += wall[0];
            nearDensity += wall[1];
        }
        for (int x = x0; x <= x1; x++)
            for (int y = y0; y <= y1; y++) {
                const int c = y * P->cellCountX + x;
                const uint32_t start = cellStart[c];
                if (start == kEmpty) continue;
                const uint32_t end = cellEnd[c];
                for (uint32_t j = start; j < end; j++) {
                    if (j == i) continue;
                    const float dx = srt[j].px - pi.px, dy = srt[j].py - pi.py;
                    const float r = len2(dx, dy);
                    if (r > kEps && r < h) {
                        const float a = 1 - r / h;
                        density += m * a * a * a * kNorm;
                        nearDensity += m * a * a * a * a * kNearNorm;
                    }
                }
            }
        float* s4 = pstate + 4 * (size_t)i;
        s4[0] = density;
        s4[1] = nearDensity;
        s4[2] = kStiffness * (density - m * kRestDensity);
        s4[3] = kNearStiffness * nearDensity;
    }
    // clComputePosition (:247-326); the viscosity term uses vel_j - vel_j == 0 (:299), so it
    // never contributes, exactly as in the reference.
#pragma omp parallel for schedule(dynamic, 64)
    for (int64_t ii = 0; ii < (int64_t)n; ii++) {
        const uint32_t i = (uint32_t)ii;
        const float* si = pstate + 4 * (size_t)i;
        const P2 pi = srt[i];
        int x0, x1, y0, y1;
        cells_of(pi, x0, x1, y0, y1);
        float rx = pi.px, ry = pi.py;
        for (int x = x0; x <= x1; x++)
            for (int y = y0; y <= y1; y++) {
                const int c = y * P->cellCountX + x;
                const uint32_t start = cellStart[c];
                if (start == kEmpty) continue;
                const uint32_t end = cellEnd[c];
                for (uint32_t j = start; j < end; j++) {
                    if (j == i) continue;
                    const float dx = srt[j].px - pi.px, dy = srt[j].py - pi.py;
                    const float r = len2(dx, dy);
                    if (r > kEps && r < h) {
                        const float* sj = pstate + 4 * (size_t)j;
                        const float a = 1 - r / h;
                        const float d = (dT * dT) * ((si[3] + sj[3]) * a * a * a * kNearNorm + (si[2] + sj[2]) * a * a * kNorm) / 2;
                        rx -= dx * d / (r * m);
                        ry -= dy * d / (r * m);
                        const float s = (dT * dT) * (kSurfaceTension / m) * m * (a * a * a * kNearNorm + a * a * kNorm) / 2;
                        rx += s * dx;
                        ry += s * dy;
                    }
                }
            }
        float wall[4];
        sample(border_state, W, H, rx / P->containerW, ry / P->containerH, wall);
        if (wall[0] != 0) {
            float normal[4];
            sample(border_vec, W, H, rx / P->containerW, ry / P->containerH, normal);
            const float a = 1 - normal[2] / h;
            const float d = (dT * dT) * ((si[3] + wall[3]) * a * a * a * kNearNorm + (si[2] + wall[2]) * a * a * kNorm) / 2;
            rx += normal[0] * d / m;
            ry += normal[1] * d / m;
        }
        relaxed[2 * (size_t)i] = rx;
        relaxed[2 * (size_t)i + 1] = ry;
    }
    // clUpdateState (:329-339)
    for (uint32_t i = 0; i < n; i++) {
        const uint32_t o = index[i];
        float dx = relaxed[2 * (size_t)i] - prev[2 * (size_t)o], dy = relaxed[2 * (size_t)i + 1] - prev[2 * (size_t)o + 1];
        const float l = len2(dx, dy);
        const float lim = std::min(l, 4.0f * P->particleSize);
        dx = dx * lim / l;
        dy = dy * lim / l;
        st[o].vx = dx / dT;
        st[o].vy = dy / dT;
        st[o].px = prev[2 * (size_t)o] + dx;
        st[o].py = prev[2 * (size_t)o + 1] + dy;
    }
}

}  // extern "C"
