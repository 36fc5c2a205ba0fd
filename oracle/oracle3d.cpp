// oracle3d.cpp -- CPU restatement of the reference's 3D SPH step and radix sort.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product library links, loads or calls this
// code; only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg do, and only
// as the checker (or the timed CPU baseline), never as the thing measured or shipped.
//
// Parity status: the reference (jochenstier/libcl) is OpenCL C whose host code needs GL
// headers and whose kernels need an OpenCL device; neither exists here, and the reference's
// own tests (libCL/TEST/main.cpp) hold no golden vectors or known answers for this path
// (the sort test only checks that keys do not decrease, TEST/main.cpp:168-175). This file
// is therefore pinned by construction against the `.cl` sources it restates line by line
// (each function cites the file:line it follows), by the properties the reference's test
// does check (sortedness), and by std::stable_sort as the definition of a stable LSD sort.
// In that sense parity is "unpinned" against executed reference output.
//
// Floating-point conventions (all stated where used):
//   * `fast_length(v)` (implementation-defined precision in OpenCL) -> sqrtf(x*x+y*y+z*z+w*w)
//   * `pow(x, 3.0f)` -> x*x*x
//   * every `/` is an IEEE division; the file is compiled with -ffp-contract=off so that no
//     FMA contraction happens on either host architecture.
// Physics is templated on the scalar type: T=float is the FP32 restatement, T=double the
// FP64 oracle of the same step. Cell keys are always computed in FP32 from the FP32
// positions so both share the forward permutation.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "../include/gbsph.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

const uint32_t kEmpty = 0xFFFFFFFFu;
const uint32_t kBuckets = 262144u;  // BUCKETS, libCL/phys/oclFluid3D.cl:32

template <class T>
struct V4 {
    T x, y, z, w;
};

template <class T>
inline V4<T> load4(const T* p, size_t i) {
    return V4<T>{p[4 * i + 0], p[4 * i + 1], p[4 * i + 2], p[4 * i + 3]};
}
template <class T>
inline void store4(T* p, size_t i, const V4<T>& v) {
    p[4 * i + 0] = v.x;
    p[4 * i + 1] = v.y;
    p[4 * i + 2] = v.z;
    p[4 * i + 3] = v.w;
}

// gridPosition, libCL/phys/oclFluid3D.cl:34-42: (int)floor(position/cellSize) per axis.
// In LINEAR_GRID mode the position is first shifted by the grid origin.
inline void grid_position(const gbsph_fluid3d_params& P, float px, float py, float pz, int g[3]) {
    if (P.keyMode == GBSPH_KEY_LINEAR_GRID) {
        px = px - P.gridOrigin[0];
        py = py - P.gridOrigin[1];
        pz = pz - P.gridOrigin[2];
    }
    g[0] = (int)std::floor(px / P.cellSize);
    g[1] = (int)std::floor(py / P.cellSize);
    g[2] = (int)std::floor(pz / P.cellSize);
    if (P.dims == 2) g[2] = 0;
}

// hashKey, libCL/phys/oclFluid3D.cl:44-52: uint32 wrap-around products, XOR, mod 262144.
inline uint32_t hash_key(int gx, int gy, int gz) {
    const uint32_t p1 = 73856093u, p2 = 19349663u, p3 = 83492791u;
    uint32_t n = (p1 * (uint32_t)gx) ^ (p2 * (uint32_t)gy) ^ (p3 * (uint32_t)gz);
    return n % kBuckets;
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// LINEAR_GRID key (an extension): clamp the cell to the grid, then x + nx*(y + ny*z).
inline uint32_t linear_key(const gbsph_fluid3d_params& P, int gx, int gy, int gz) {
    gx = clampi(gx, 0, P.gridDim[0] - 1);
    gy = clampi(gy, 0, P.gridDim[1] - 1);
    gz = clampi(gz, 0, P.gridDim[2] - 1);
    return (uint32_t)gx + (uint32_t)P.gridDim[0] * ((uint32_t)gy + (uint32_t)P.gridDim[1] * (uint32_t)gz);
}

inline uint32_t cell_key(const gbsph_fluid3d_params& P, const int g[3]) {
    return P.keyMode == GBSPH_KEY_LINEAR_GRID ? linear_key(P, g[0], g[1], g[2])
                                              : hash_key(g[0], g[1], g[2]);
}

inline size_t table_size(const gbsph_fluid3d_params& P) {
    if (P.keyMode == GBSPH_KEY_LINEAR_GRID)
        return (size_t)P.gridDim[0] * (size_t)P.gridDim[1] * (size_t)(P.dims == 2 ? 1 : P.gridDim[2]);
    return kBuckets;
}

// The list of neighbour-cell keys visited for a particle in grid cell g, in the order of
// the reference's loops (z outer, then y, then x; libCL/phys/oclFluid3D.cl:160-166).
// REFERENCE_HASH keeps duplicates (a bucket hit twice is visited twice). LINEAR_GRID visits
// the clamped cells that exist (each once).
inline int neighbour_cells(const gbsph_fluid3d_params& P, const int g[3], uint32_t out[27]) {
    int n = 0;
    const int zr = (P.dims == 2) ? 0 : 1;
    for (int z = -zr; z <= zr; z++)
        for (int y = -1; y <= 1; y++)
            for (int x = -1; x <= 1; x++) {
                if (P.keyMode == GBSPH_KEY_LINEAR_GRID) {
                    int cx = clampi(g[0], 0, P.gridDim[0] - 1) + x;
                    int cy = clampi(g[1], 0, P.gridDim[1] - 1) + y;
                    int cz = (P.dims == 2) ? 0 : clampi(g[2], 0, P.gridDim[2] - 1) + z;
                    if (cx < 0 || cy < 0 || cz < 0 || cx >= P.gridDim[0] || cy >= P.gridDim[1] ||
                        (P.dims != 2 && cz >= P.gridDim[2]))
                        continue;
                    out[n++] = linear_key(P, cx, cy, cz);
                } else {
                    out[n++] = hash_key(g[0] + x, g[1] + y, g[2] + z);
                }
            }
    return n;
}

// ---------------------------------------------------------------------------------------
// Radix sort: restatement of libCL/sort/oclRadixSort.cl:20-222 driven as in
// libCL/sort/oclRadixSort.cpp:62-144 (256-item work-groups, 4-bit digits, per pass:
// clBlockSort -> clBlockScan -> clBlockPrefix -> clReorder). Work-groups are executed one
// after another; barriers become loop boundaries.
// ---------------------------------------------------------------------------------------
const int kBits = 4, kRadix = 16, kBlock = 256;

void block_sort(const uint32_t* keyIn, uint32_t* keyOut, const uint32_t* valIn, uint32_t* valOut,
                uint32_t startbit, uint32_t* blockScan, uint32_t* blockOffset, uint32_t size,
                int totalBlocks, int blockid) {
    // libCL/sort/oclRadixSort.cl:20-112
    uint32_t key[kBlock], val[kBlock], prefixSum[kBlock], nk[kBlock], nv[kBlock];
    for (int t = 0; t < kBlock; t++) {
        uint32_t g = (uint32_t)blockid * kBlock + t;
        key[t] = 0xFFFFFFFFu;
        val[t] = 0xFFFFFFFFu;
        if (g < size) {
            key[t] = keyIn[g];
            val[t] = valIn[g];
        }
    }
    for (uint32_t bit = startbit; bit < startbit + kBits; bit++) {  // :45-64, 1-bit split
        for (int t = 0; t < kBlock; t++) prefixSum[t] = !((key[t] >> bit) & 1u);
        for (int i = 1; i < kBlock; i++) prefixSum[i] += prefixSum[i - 1];
        for (int t = 0; t < kBlock; t++) {
            uint32_t lsb = !((key[t] >> bit) & 1u);
            uint32_t address = lsb ? prefixSum[t] - 1 : prefixSum[kBlock - 1] - prefixSum[t] + t;
            nk[address] = key[t];
            nv[address] = val[t];
        }
        std::memcpy(key, nk, sizeof(key));
        std::memcpy(val, nv, sizeof(val));
    }
    for (int t = 0; t < kBlock; t++) {  // :66-70
        uint32_t g = (uint32_t)blockid * kBlock + t;
        if (g < size) {
            keyOut[g] = key[t];
            valOut[g] = val[t];
        }
    }
    uint32_t offset[kRadix] = {0};  // :75-110, digit start and count within the block
    uint32_t dig[kBlock];
    for (int t = 0; t < kBlock; t++) dig[t] = (key[t] >> startbit) & 0xFu;
    for (int t = 1; t < kBlock; t++)
        if (dig[t] != dig[t - 1]) offset[dig[t]] = t;
    for (int d = 0; d < kRadix; d++) blockOffset[blockid * kRadix + d] = offset[d];
    for (int t = 1; t < kBlock; t++)
        if (dig[t] != dig[t - 1]) offset[dig[t - 1]] = t - offset[dig[t - 1]];
    offset[dig[kBlock - 1]] = kBlock - offset[dig[kBlock - 1]];
    for (int d = 0; d < kRadix; d++) blockScan[d * totalBlocks + blockid] = offset[d];
}

}  // namespace

extern "C" {

// oclRadixSort::compute (libCL/sort/oclRadixSort.cpp:62-144) on host arrays. Returns 0, or
// the reference's failures: -2 (sizes differ), -3 (n >= 4,194,304), -4 (bit range % 4).
int orc_radix_sort_reference(uint32_t* keys, uint32_t* vals, uint32_t n_keys, uint32_t n_vals,
                             int startBit, int endBit) {
    if (n_keys != n_vals) return -2;
    const uint32_t cMaxArraySize = 256u * 256u * 256u * 4u / 16u;  // :24
    if (n_keys >= cMaxArraySize) return -3;
    if ((endBit - startBit) % kBits != 0) return -4;
    if (n_keys == 0) return 0;
    const uint32_t n = n_keys;
    const int blocks = (int)std::ceil((float)n / kBlock);
    std::vector<uint32_t> tk(n), tv(n), scan((size_t)blocks * kRadix), boff((size_t)blocks * kRadix);
    for (int j = startBit; j < endBit; j += kBits) {
#pragma omp parallel for schedule(static)
        for (int b = 0; b < blocks; b++)
            block_sort(keys, tk.data(), vals, tv.data(), (uint32_t)j, scan.data(), boff.data(), n, blocks, b);
        // clBlockScan + clBlockPrefix (:114-187): together an exclusive scan of the
        // digit-major count array, in chunks of 1024 whose totals are then prefixed.
        uint32_t run = 0;
        for (size_t i = 0; i < scan.size(); i++) {
            uint32_t c = scan[i];
            scan[i] = run;
            run += c;
        }
        // clReorder (:189-222): index = totalOffset[radix] + threadid - blockOffset[radix]
#pragma omp parallel for schedule(static)
        for (int b = 0; b < blocks; b++)
            for (int t = 0; t < kBlock; t++) {
                uint32_t g = (uint32_t)b * kBlock + t;
                if (g >= n) break;
                uint32_t key = tk[g], val = tv[g];
                uint32_t radix = (key >> j) & 0xFu;
                uint32_t index = scan[radix * blocks + b] + t - boff[b * kRadix + radix];
                keys[index] = key;
                vals[index] = val;
            }
    }
    return 0;
}

// The definition a stable LSD sort on bits [startBit, endBit) must meet: std::stable_sort
// by the extracted bit field. Any size.
int orc_stable_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int startBit, int endBit) {
    if (startBit < 0 || endBit > 32 || endBit < startBit) return -4;
    const int width = endBit - startBit;
    const uint64_t mask = width >= 32 ? 0xFFFFFFFFull : ((1ull << width) - 1ull);
    std::vector<uint64_t> packed(n);  // (field << 32) | original position
    for (uint32_t i = 0; i < n; i++)
        packed[i] = ((((uint64_t)keys[i] >> startBit) & mask) << 32) | i;
    std::vector<uint32_t> k0(keys, keys + n), v0(vals, vals + n);
    std::sort(packed.begin(), packed.end());  // position tie-break == stability
    for (uint32_t i = 0; i < n; i++) {
        uint32_t src = (uint32_t)(packed[i] & 0xFFFFFFFFu);
        keys[i] = k0[src];
        vals[i] = v0[src];
    }
    return 0;
}

// clEnqueueFillBuffer(0xFFFFFFFF) x2 + clFindBounds (libCL/phys/oclFluid3D.cpp:309-315,
// libCL/phys/oclFluid3D.cl:85-113). As in the reference, particle 0 only sets cellStart,
// so for n == 1 cellEnd stays empty. Keys >= n_cells are skipped (out of the reference's
// bounds); the count of skipped keys is returned.
int orc_find_bounds(const uint32_t* cell, uint32_t n, uint32_t* cellStart, uint32_t* cellEnd,
                    uint32_t n_cells) {
    for (uint32_t c = 0; c < n_cells; c++) cellStart[c] = cellEnd[c] = kEmpty;
    int skipped = 0;
    for (uint32_t p = 0; p < n; p++) {
        uint32_t hash = cell[p];
        if (hash >= n_cells) {
            skipped++;
            continue;
        }
        if (p == 0) {
            cellStart[hash] = 0;
            continue;
        }
        uint32_t prev = cell[p - 1];
        if (hash != prev) {
            if (prev < n_cells) cellEnd[prev] = p;
            cellStart[hash] = p;
        }
        if (p == n - 1) cellEnd[hash] = n;
    }
    return skipped;
}

// The kernel constants clInitFluid forms (libCL/phys/oclFluid3D.cl:145-147 with the macros
// DensityConstant, ViscosityConstant, PressureConstant of :123-128) for a cell size h and a
// viscosity mu: out = (kernelConstant, viscosityConstant, pressureConstant). M_PI_F is a
// float: 64.0*M_PI_F is a double product, but M_PI_F * pow(h, 6.0f) is a float product,
// divided into -45.0 in double.
void orc_kernel_constants(float h, float mu, float* out) {
    const float pi_f = 3.14159274101257f;  // M_PI_F
    out[0] = (float)(315.0 / (64.0 * (double)pi_f * (double)std::pow(h, 9.0f)));
    out[1] = (float)(-(double)mu * (-45.0 / (double)(pi_f * std::pow(h, 6.0f))));
    out[2] = (float)(-(-45.0 / (double)(pi_f * std::pow(h, 6.0f))));
}

// clInitFluid, libCL/phys/oclFluid3D.cl:130-148 (double literals evaluated in double,
// pow() of float arguments in float), plus the hard-coded kernel arguments of
// libCL/phys/oclFluid3D.cpp:256-268.
void orc_init_fluid_params(gbsph_fluid3d_params* p) {
    std::memset(p, 0, sizeof(*p));
    p->deltaTime = (float)0.005;
    p->mass = (float)0.006;
    p->density = 1000;
    p->viscosity = (float)6.0;
    p->pressure = 0;
    p->velocitylimit = 500;
    p->stiffness = 1;
    p->spacing = (float)(0.87 * (double)std::pow(p->mass / p->density, 1 / 3.0f));
    p->particleRadius = (float)(0.5 * (double)p->spacing);
    p->cellSize = (float)(2.0 * (double)p->spacing);
    float k[3];
    orc_kernel_constants(p->cellSize, p->viscosity, k);
    p->kernelConstant = k[0];
    p->viscosityConstant = k[1];
    p->pressureConstant = k[2];
    p->gravity[0] = -9.8f * 0.0f;
    p->gravity[1] = -9.8f * 0.0f;
    p->gravity[2] = -9.8f * 1.0f;
    p->gravity[3] = -9.8f * 0.0f;
    for (int i = 0; i < 3; i++) {
        p->boxMin[i] = -1;
        p->boxMax[i] = 1;
    }
    p->keyMode = GBSPH_KEY_REFERENCE_HASH;
    p->dims = 3;
}

// clHash, libCL/phys/oclFluid3D.cl:57-64.
void orc_hash(const float* pos, uint32_t n, const gbsph_fluid3d_params* P, uint32_t* cell,
              uint32_t* index) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        int g[3];
        grid_position(*P, pos[4 * i], pos[4 * i + 1], pos[4 * i + 2], g);
        cell[i] = cell_key(*P, g);
        index[i] = (uint32_t)i;
    }
}

// clReorder, libCL/phys/oclFluid3D.cl:66-72.
void orc_reorder(const uint32_t* index, const float* pos, const float* vel, float* spos,
                 float* svel, uint32_t n) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        std::memcpy(spos + 4 * i, pos + 4 * (size_t)index[i], 16);
        std::memcpy(svel + 4 * i, vel + 4 * (size_t)index[i], 16);
    }
}

}  // extern "C"

namespace {

// clCalculateDensity, libCL/phys/oclFluid3D.cl:150-200.
template <class T>
void density_t(T* position, T* velocity, const float* fpos, const uint32_t* cellStart,
               const uint32_t* cellEnd, uint32_t n, const gbsph_fluid3d_params& P) {
    const T h = (T)P.cellSize;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t particle = 0; particle < (int64_t)n; particle++) {
        V4<T> posI = load4(position, particle);
        T density = 0;
        int g[3];
        grid_position(P, fpos[4 * particle], fpos[4 * particle + 1], fpos[4 * particle + 2], g);
        uint32_t cells[27];
        int nc = neighbour_cells(P, g, cells);
        int count = 0;
        for (int c = 0; c < nc; c++) {
            uint32_t start = cellStart[cells[c]];
            if (start == kEmpty) continue;
            uint32_t end = cellEnd[cells[c]];
            for (uint32_t j = start; j < end; j++) {
                if (j == (uint32_t)particle) continue;
                V4<T> pj = load4(position, j);
                T vx = posI.x - pj.x, vy = posI.y - pj.y, vz = posI.z - pj.z, vw = 0;
                T vlen = std::sqrt(vx * vx + vy * vy + vz * vz + vw * vw);  // fast_length
                if (vlen < h) {
                    T t = h * h - vlen * vlen;  // DensityVariable: pow(h*h - r*r, 3)
                    density += t * t * t;
                    count++;
                }
            }
        }
        // written after the whole neighbour loop; reads of .w above see the old values only
        // through posI (the reference reads position[j].w nowhere in this kernel)
        if (count > 2) {
            density = std::max((T)1.0, (T)P.mass * (T)P.kernelConstant * density);
            position[4 * particle + 3] = density;
            velocity[4 * particle + 3] = (T)P.pressure + (T)P.stiffness * (density - (T)P.density);
        } else {
            position[4 * particle + 3] = (T)P.density;
            velocity[4 * particle + 3] = (T)P.pressure;
        }
    }
}

// clCalculateForces, libCL/phys/oclFluid3D.cl:202-255.
template <class T>
void forces_t(const T* position, const T* velocity, T* force, const uint32_t* index,
              const float* fpos, const uint32_t* cellStart, const uint32_t* cellEnd, uint32_t n,
              const gbsph_fluid3d_params& P) {
    const T h = (T)P.cellSize;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t particle = 0; particle < (int64_t)n; particle++) {
        V4<T> posI = load4(position, particle), velI = load4(velocity, particle);
        T px = 0, py = 0, pz = 0;              // pressure (w stays 0)
        T qx = 0, qy = 0, qz = 0;              // viscosity (w is discarded)
        int g[3];
        grid_position(P, fpos[4 * particle], fpos[4 * particle + 1], fpos[4 * particle + 2], g);
        uint32_t cells[27];
        int nc = neighbour_cells(P, g, cells);
        for (int c = 0; c < nc; c++) {
            uint32_t start = cellStart[cells[c]];
            if (start == kEmpty) continue;
            uint32_t end = cellEnd[cells[c]];
            for (uint32_t j = start; j < end; j++) {
                if (j == (uint32_t)particle) continue;
                V4<T> posJ = load4(position, j);
                T vx = posI.x - posJ.x, vy = posI.y - posJ.y, vz = posI.z - posJ.z, vw = 0;
                T vlen = std::sqrt(vx * vx + vy * vy + vz * vz + vw * vw);
                if (vlen < h) {
                    V4<T> velJ = load4(velocity, j);
                    T density2 = posI.w * posJ.w;
                    T pressure2 = velI.w + velJ.w;
                    // pressure2/density2*PressureVariable(h, vector/vlen, vlen)
                    T s = pressure2 / density2;
                    T hr = h - vlen;
                    px += s * ((vx / vlen) * hr * hr);
                    py += s * ((vy / vlen) * hr * hr);
                    pz += s * ((vz / vlen) * hr * hr);
                    // (velJ-velI)/density2*ViscosityVariable(h, vlen)
                    qx += ((velJ.x - velI.x) / density2) * hr;
                    qy += ((velJ.y - velI.y) / density2) * hr;
                    qz += ((velJ.z - velI.z) / density2) * hr;
                }
            }
        }
        size_t o = index[particle];
        T m = (T)P.mass, cp = (T)P.pressureConstant, cv = (T)P.viscosityConstant;
        force[4 * o + 0] += (cp * px + cv * qx) * m;
        force[4 * o + 1] += (cp * py + cv * qy) * m;
        force[4 * o + 2] += (cp * pz + cv * qz) * m;
        force[4 * o + 3] = 0;
    }
}

// repulsionForce + clClipBox, libCL/phys/oclFluid3D.cl:304-361 (EPSILON 1e-5,
// BOUNDARY_STIFFNESS 2000, BOUNDARY_DAMPENING 256). Walls in the reference's order:
// y-min, y-max, z-min, z-max, x-min, x-max (z walls skipped when dims == 2).
template <class T>
void clip_box_t(const T* position, const T* velocity, T* force, const uint32_t* index,
                uint32_t n, const gbsph_fluid3d_params& P) {
    const T eps = (T)0.00001f, K = 2000, D = 256, r = (T)P.particleRadius;
#pragma omp parallel for schedule(static)
    for (int64_t particle = 0; particle < (int64_t)n; particle++) {
        V4<T> pos = load4(position, particle), vel = load4(velocity, particle);
        size_t o = index[particle];
        V4<T> f = load4(force, o);
        auto wall = [&](int axis, T sign, T diff) {
            if (diff > eps) {
                T vn = axis == 0 ? vel.x : (axis == 1 ? vel.y : vel.z);
                // normal*(K*dist - D*dot(normal, velocity)); dot over 4 lanes, normal.w = 0
                T mag = K * diff - D * (sign * vn);
                if (axis == 0) f.x += sign * mag;
                if (axis == 1) f.y += sign * mag;
                if (axis == 2) f.z += sign * mag;
                f.w += (T)0 * mag;
            }
        };
        wall(1, 1, r - (pos.y - (T)P.boxMin[1]));
        wall(1, -1, r - ((T)P.boxMax[1] - pos.y));
        if (P.dims != 2) {
            wall(2, 1, r - (pos.z - (T)P.boxMin[2]));
            wall(2, -1, r - ((T)P.boxMax[2] - pos.z));
        }
        wall(0, 1, r - (pos.x - (T)P.boxMin[0]));
        wall(0, -1, r - ((T)P.boxMax[0] - pos.x));
        store4(force, o, f);
    }
}

// clIntegrateForce, libCL/phys/oclFluid3D.cl:258-271.
template <class T>
void integrate_force_t(T* vel, const T* force, uint32_t n, const gbsph_fluid3d_params& P) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        V4<T> v = load4(vel, i), f = load4(force, i);
        T speed = std::sqrt(f.x * f.x + f.y * f.y + f.z * f.z + f.w * f.w);
        if (speed > (T)P.velocitylimit) {
            T s = (T)P.velocitylimit / speed;
            f.x *= s;
            f.y *= s;
            f.z *= s;
            f.w *= s;
        }
        T dt = (T)P.deltaTime;
        v.x += f.x * dt;
        v.y += f.y * dt;
        v.z += f.z * dt;
        v.w += f.w * dt;
        store4(vel, i, v);
    }
}

// clGravity, libCL/phys/oclFluid3D.cl:294-298 (the -9.8f factor is folded into
// params.gravity, which holds the value written).
template <class T>
void gravity_t(T* force, uint32_t n, const gbsph_fluid3d_params& P) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++)
        store4(force, i, V4<T>{(T)P.gravity[0], (T)P.gravity[1], (T)P.gravity[2], (T)P.gravity[3]});
}

// clIntegrateVelocity, libCL/phys/oclFluid3D.cl:284-291 (all four lanes).
template <class T>
void integrate_velocity_t(T* pos, const T* vel, uint32_t n, const gbsph_fluid3d_params& P) {
    T dt = (T)P.deltaTime;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++)
        for (int c = 0; c < 4; c++) pos[4 * i + c] += vel[4 * i + c] * dt;
}

template <class T>
void to_t(const float* src, T* dst, size_t count) {
    for (size_t i = 0; i < count; i++) dst[i] = (T)src[i];
}

// One whole step in the order of oclFluid3D::compute (libCL/phys/oclFluid3D.cpp:293-342).
// pos/vel/force are in/out float4[n]; the FP32 positions `fpos_key` (same as pos for T=float)
// give the keys. Outputs the sorted keys, index, sorted pos/vel (w = density / pressure) and
// the cell tables. `ref_sort` selects the restated reference sort (else std::stable_sort).
// If `fwall` is set it receives the force after the clip box (particle order).
template <class T>
int step_t(T* pos, T* vel, T* force, const float* fpos_key, uint32_t n,
           const gbsph_fluid3d_params& P, uint32_t* cell, uint32_t* index, T* spos, T* svel,
           uint32_t* cellStart, uint32_t* cellEnd, int ref_sort, T* fwall = nullptr) {
    orc_hash(fpos_key, n, &P, cell, index);
    int rc = ref_sort ? orc_radix_sort_reference(cell, index, n, n, 0, 24)
                      : orc_stable_sort(cell, index, n, 0, 24);
    if (rc) return rc;
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++)
        for (int c = 0; c < 4; c++) {
            spos[4 * i + c] = pos[4 * (size_t)index[i] + c];
            svel[4 * i + c] = vel[4 * (size_t)index[i] + c];
        }
    const uint32_t ncell = (uint32_t)table_size(P);
    orc_find_bounds(cell, n, cellStart, cellEnd, ncell);
    // the neighbour loops key off the FP32 sorted positions
    std::vector<float> fs(4 * (size_t)n);
    for (size_t i = 0; i < n; i++)
        std::memcpy(&fs[4 * i], fpos_key + 4 * (size_t)index[i], 16);
    density_t<T>(spos, svel, fs.data(), cellStart, cellEnd, n, P);
    forces_t<T>(spos, svel, force, index, fs.data(), cellStart, cellEnd, n, P);
    clip_box_t<T>(spos, svel, force, index, n, P);
    if (fwall) std::memcpy(fwall, force, 4 * sizeof(T) * (size_t)n);
    integrate_force_t<T>(vel, force, n, P);
    gravity_t<T>(force, n, P);
    integrate_velocity_t<T>(pos, vel, n, P);
    return 0;
}

}  // namespace

extern "C" {

// Single stages on FP32 arrays, fed whatever prior state the caller holds (used to compare
// one GPU stage against the restatement on identical inputs).
void orc_density(float* spos, float* svel, const uint32_t* cellStart, const uint32_t* cellEnd,
                 uint32_t n, const gbsph_fluid3d_params* P) {
    std::vector<float> fs(spos, spos + 4 * (size_t)n);
    density_t<float>(spos, svel, fs.data(), cellStart, cellEnd, n, *P);
}
void orc_forces(const float* spos, const float* svel, float* force, const uint32_t* index,
                const uint32_t* cellStart, const uint32_t* cellEnd, uint32_t n,
                const gbsph_fluid3d_params* P) {
    forces_t<float>(spos, svel, force, index, spos, cellStart, cellEnd, n, *P);
}
void orc_clip_box(const float* spos, const float* svel, float* force, const uint32_t* index,
                  uint32_t n, const gbsph_fluid3d_params* P) {
    clip_box_t<float>(spos, svel, force, index, n, *P);
}
void orc_integrate_force(float* vel, const float* force, uint32_t n, const gbsph_fluid3d_params* P) {
    integrate_force_t<float>(vel, force, n, *P);
}
void orc_gravity(float* force, uint32_t n, const gbsph_fluid3d_params* P) { gravity_t<float>(force, n, *P); }
void orc_integrate_velocity(float* pos, const float* vel, uint32_t n, const gbsph_fluid3d_params* P) {
    integrate_velocity_t<float>(pos, vel, n, *P);
}

// FP64 single stages: positions/velocities/forces in double, keys from `fpos` (float4).
void orc_density_f64(double* spos, double* svel, const float* fspos, const uint32_t* cellStart,
                     const uint32_t* cellEnd, uint32_t n, const gbsph_fluid3d_params* P) {
    density_t<double>(spos, svel, fspos, cellStart, cellEnd, n, *P);
}
void orc_forces_f64(const double* spos, const double* svel, double* force, const uint32_t* index,
                    const float* fspos, const uint32_t* cellStart, const uint32_t* cellEnd,
                    uint32_t n, const gbsph_fluid3d_params* P) {
    forces_t<double>(spos, svel, force, index, fspos, cellStart, cellEnd, n, *P);
}

// Whole step, FP32. Returns 0 or the sort's failure code.
int orc_step(float* pos, float* vel, float* force, uint32_t n, const gbsph_fluid3d_params* P,
             uint32_t* cell, uint32_t* index, float* spos, float* svel, uint32_t* cellStart,
             uint32_t* cellEnd, int ref_sort) {
    return step_t<float>(pos, vel, force, pos, n, *P, cell, index, spos, svel, cellStart, cellEnd, ref_sort);
}

// Whole step, FP64 state; keys from the FP32 copy `fpos_key` of the positions (the caller
// keeps it in sync, e.g. by rounding the FP64 positions after each step).
int orc_step_f64(double* pos, double* vel, double* force, const float* fpos_key, uint32_t n,
                 const gbsph_fluid3d_params* P, uint32_t* cell, uint32_t* index, double* spos,
                 double* svel, uint32_t* cellStart, uint32_t* cellEnd) {
    return step_t<double>(pos, vel, force, fpos_key, n, *P, cell, index, spos, svel, cellStart,
                          cellEnd, 0);
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// FP64 adjoint of the LINEAR_GRID step (hand-derived reverse of clCalculateDensity,
// clCalculateForces, clClipBox, clIntegrateForce and clIntegrateVelocity,
// libCL/phys/oclFluid3D.cl:150-298,304-361), with each step's permutation and neighbour
// sets held fixed. Per step, in sorted order i with particle o = index[i], d = x_i - x_j,
// r = |d|, D = 1/(rho_i rho_j), w = m dL/dF:
//   integration:  dL/dv += dt dL/dx';  dL/dF = dt dL/dv (through the clamp's Jacobian when
//                 |F| exceeded the limit); active walls add -2000 dL/dF_a to dL/dx_a and
//                 -256 dL/dF_a to dL/dv_a
//   forces:       per pair, with dw = w_i - w_j, phi = (h-r)^2/r, dv = v_j - v_i:
//                 dL/dx_i += Cp (p_i+p_j) D (phi dw + phi'(r)/r (d.dw) d) - Cv D (dw.dv)/r d
//                 dL/dv_i -= Cv D (h-r) dw
//                 dL/dp_i += Cp D phi (d.dw)
//                 dL/drho_i -= D/rho_i (Cp (p_i+p_j) phi (d.dw) + Cv (h-r) (dw.dv))
//   pressure law: dL/dS_i = m K (dL/drho_i + k dL/dp_i) where rho = m K S (else 0),
//                 dL/dk += (rho_i - rho0) dL/dp_i, dL/dmu += 45/(pi h^6) w_i . sum_j D (h-r) dv
//   density:      dL/dx_i += -6 sum_j (h^2 - r^2)^2 (dL/dS_i + dL/dS_j) d
// Each pair's terms depend on i and j symmetrically, so every sum gathers over i's own
// neighbours (the same loops as the forward kernels).
// ---------------------------------------------------------------------------------------
namespace {

struct TapeF64 {
    std::vector<uint32_t> cell, index, cs, ce;
    std::vector<double> spos, svel, fwall;
    std::vector<float> fs;  // FP32 sorted positions: the cell lookups
};

void record_step_f64(double* pos, double* vel, double* force, uint32_t n, const gbsph_fluid3d_params& P,
                     TapeF64& t) {
    const size_t cells = table_size(P);
    t.cell.resize(n);
    t.index.resize(n);
    t.cs.resize(cells);
    t.ce.resize(cells);
    t.spos.resize(4 * (size_t)n);
    t.svel.resize(4 * (size_t)n);
    t.fwall.resize(4 * (size_t)n);
    std::vector<float> fpos(4 * (size_t)n);
    for (size_t i = 0; i < 4 * (size_t)n; i++) fpos[i] = (float)pos[i];
    step_t<double>(pos, vel, force, fpos.data(), n, P, t.cell.data(), t.index.data(), t.spos.data(),
                   t.svel.data(), t.cs.data(), t.ce.data(), 0, t.fwall.data());
    t.fs.resize(4 * (size_t)n);
    for (size_t i = 0; i < n; i++) std::memcpy(&t.fs[4 * i], &fpos[4 * (size_t)t.index[i]], 16);
}

// Calls f(j, dx, dy, dz, r) for every neighbour j != i with r < h (FP64 distances, cells
// from the FP32 positions), as the forward loops of density_t / forces_t visit them.
template <class F>
void for_neighbours_f64(const TapeF64& t, const gbsph_fluid3d_params& P, int64_t i, F&& f) {
    const double h = P.cellSize;
    int g[3];
    grid_position(P, t.fs[4 * i], t.fs[4 * i + 1], t.fs[4 * i + 2], g);
    uint32_t cells[27];
    const int nc = neighbour_cells(P, g, cells);
    const double* xi = &t.spos[4 * i];
    for (int c = 0; c < nc; c++) {
        const uint32_t start = t.cs[cells[c]];
        if (start == kEmpty) continue;
        const uint32_t end = t.ce[cells[c]];
        for (uint32_t j = start; j < end; j++) {
            if (j == (uint32_t)i) continue;
            const double* xj = &t.spos[4 * (size_t)j];
            const double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
            const double r = std::sqrt(dx * dx + dy * dy + dz * dz);
            if (r < h) f(j, dx, dy, dz, r);
        }
    }
}

// One step backwards: gx/gv (particle order) hold dL/d(state after the step) on entry and
// dL/d(state before the step) on return; acc_k / acc_mu (particle order) accumulate.
void adjoint_step_f64(const TapeF64& t, uint32_t n, const gbsph_fluid3d_params& P, double* gx, double* gv,
                      double* acc_k, double* acc_mu) {
    const double dt = P.deltaTime, h = P.cellSize, m = P.mass, cp = P.pressureConstant, cv = P.viscosityConstant;
    const double mK = (double)P.mass * (double)P.kernelConstant, k = P.stiffness, rho0 = P.density;
    const double pi = (double)(float)M_PI;
    const double c45 = 45.0 / (pi * std::pow((double)P.cellSize, 6.0));
    std::vector<double> w(3 * (size_t)n), gxs(3 * (size_t)n), gvs(3 * (size_t)n), gS(n);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        const size_t o = t.index[i];
        const double* x = &t.spos[4 * i];
        const double* f = &t.fwall[4 * o];
        double gvt[3], gf[3];
        for (int a = 0; a < 3; a++) {
            gvt[a] = gv[4 * o + a] + dt * gx[4 * o + a];
            gf[a] = dt * gvt[a];
        }
        const double f2 = f[0] * f[0] + f[1] * f[1] + f[2] * f[2] + f[3] * f[3];
        const double speed = std::sqrt(f2);
        if (speed > (double)P.velocitylimit) {
            const double s = (double)P.velocitylimit / speed, fg = (f[0] * gf[0] + f[1] * gf[1] + f[2] * gf[2]) / f2;
            for (int a = 0; a < 3; a++) gf[a] = s * (gf[a] - f[a] * fg);
        }
        double ax[3] = {0, 0, 0}, av[3] = {0, 0, 0};
        const double r = P.particleRadius, eps = (double)0.00001f;
        auto wall = [&](int a, double diff) {
            if (diff > eps) {
                ax[a] -= 2000.0 * gf[a];
                av[a] -= 256.0 * gf[a];
            }
        };
        wall(1, r - (x[1] - (double)P.boxMin[1]));
        wall(1, r - ((double)P.boxMax[1] - x[1]));
        wall(2, r - (x[2] - (double)P.boxMin[2]));
        wall(2, r - ((double)P.boxMax[2] - x[2]));
        wall(0, r - (x[0] - (double)P.boxMin[0]));
        wall(0, r - ((double)P.boxMax[0] - x[0]));
        for (int a = 0; a < 3; a++) {
            w[3 * i + a] = m * gf[a];
            gxs[3 * i + a] = gx[4 * o + a] + ax[a];
            gvs[3 * i + a] = gvt[a] + av[a];
        }
    }
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        const double* xi = &t.spos[4 * i];
        const double* vi = &t.svel[4 * i];
        const double* wi = &w[3 * i];
        const double rho_i = xi[3], p_i = vi[3];
        double ax[3] = {0, 0, 0}, av[3] = {0, 0, 0}, b[3] = {0, 0, 0}, ap = 0, arho = 0;
        int count = 0;
        for_neighbours_f64(t, P, i, [&](uint32_t j, double dx, double dy, double dz, double r) {
            count++;
            if (!(r > 0)) return;
            const double* xj = &t.spos[4 * (size_t)j];
            const double* vj = &t.svel[4 * (size_t)j];
            const double* wj = &w[3 * (size_t)j];
            const double hr = h - r, D = 1.0 / (rho_i * xj[3]), Pp = p_i + vj[3];
            const double phi = hr * hr / r, dphi_r = -hr * (h + r) / (r * r * r);
            const double d[3] = {dx, dy, dz};
            const double dw[3] = {wi[0] - wj[0], wi[1] - wj[1], wi[2] - wj[2]};
            const double dv[3] = {vj[0] - vi[0], vj[1] - vi[1], vj[2] - vi[2]};
            const double ddw = d[0] * dw[0] + d[1] * dw[1] + d[2] * dw[2];
            const double dwdv = dw[0] * dv[0] + dw[1] * dv[1] + dw[2] * dv[2];
            for (int a = 0; a < 3; a++) {
                ax[a] += cp * Pp * D * (phi * dw[a] + dphi_r * ddw * d[a]) - cv * D * dwdv / r * d[a];
                av[a] -= cv * D * hr * dw[a];
                b[a] += D * hr * dv[a];
            }
            ap += cp * D * phi * ddw;
            arho -= D / rho_i * (cp * Pp * phi * ddw + cv * hr * dwdv);
        });
        for (int a = 0; a < 3; a++) {
            gxs[3 * i + a] += ax[a];
            gvs[3 * i + a] += av[a];
        }
        gS[i] = (count > 2 && rho_i > 1.0) ? mK * (arho + k * ap) : 0.0;
        const size_t o = t.index[i];
        acc_k[o] += (rho_i - rho0) * ap;
        acc_mu[o] += c45 * (wi[0] * b[0] + wi[1] * b[1] + wi[2] * b[2]);
    }
    const double h2 = h * h;
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; i++) {
        double a[3] = {0, 0, 0};
        for_neighbours_f64(t, P, i, [&](uint32_t j, double dx, double dy, double dz, double r) {
            const double tt = h2 - r * r;
            const double c = -6.0 * tt * tt * (gS[i] + gS[j]);
            a[0] += c * dx;
            a[1] += c * dy;
            a[2] += c * dz;
        });
        const size_t o = t.index[i];
        for (int q = 0; q < 3; q++) {
            gx[4 * o + q] = gxs[3 * i + q] + a[q];
            gv[4 * o + q] = gvs[3 * i + q];
        }
        gx[4 * o + 3] = 0;
        gv[4 * o + 3] = 0;
    }
}

}  // namespace

extern "C" {

// `steps` FP64 steps in place (keys from the positions rounded to FP32 before each step).
int orc_run_f64(double* pos, double* vel, double* force, uint32_t n, const gbsph_fluid3d_params* P,
                uint32_t steps) {
    TapeF64 t;
    for (uint32_t s = 0; s < steps; s++) record_step_f64(pos, vel, force, n, *P, t);
    return 0;
}

// Reverse-mode gradients of a loss on the state after `steps` FP64 steps from (pos0, vel0,
// force0): given dL/dpos, dL/dvel of the final state (float4-strided doubles; gvel may be
// NULL), writes dL/dpos0, dL/dvel0 and gparams[0] = dL/dstiffness, gparams[1] =
// dL/dviscosity. Checkpoints every `every` steps and recomputes each segment.
int orc_adjoint_f64(const double* pos0, const double* vel0, const double* force0, uint32_t n,
                    const gbsph_fluid3d_params* P, uint32_t steps, uint32_t every, const double* gpos,
                    const double* gvel, double* gpos0, double* gvel0, double* gparams) {
    if (P->keyMode != GBSPH_KEY_LINEAR_GRID || P->dims != 3 || every == 0) return -1;
    const size_t N4 = 4 * (size_t)n;
    const uint32_t nseg = (steps + every - 1) / every;
    std::vector<std::vector<double>> ck(nseg, std::vector<double>(3 * N4));
    std::vector<double> pos(pos0, pos0 + N4), vel(vel0, vel0 + N4), force(force0, force0 + N4);
    TapeF64 scratch;
    for (uint32_t s = 0; s < steps; s++) {
        if (s % every == 0) {
            std::vector<double>& c = ck[s / every];
            std::memcpy(c.data(), pos.data(), N4 * 8);
            std::memcpy(c.data() + N4, vel.data(), N4 * 8);
            std::memcpy(c.data() + 2 * N4, force.data(), N4 * 8);
        }
        record_step_f64(pos.data(), vel.data(), force.data(), n, *P, scratch);
    }
    std::vector<double> gx(gpos, gpos + N4), gv(N4, 0.0), acc_k(n, 0.0), acc_mu(n, 0.0);
    if (gvel) std::memcpy(gv.data(), gvel, N4 * 8);
    std::vector<TapeF64> tape(every);
    for (uint32_t seg = nseg; seg-- > 0;) {
        const uint32_t s0 = seg * every, s1 = std::min(steps, s0 + every);
        const std::vector<double>& c = ck[seg];
        std::memcpy(pos.data(), c.data(), N4 * 8);
        std::memcpy(vel.data(), c.data() + N4, N4 * 8);
        std::memcpy(force.data(), c.data() + 2 * N4, N4 * 8);
        for (uint32_t s = s0; s < s1; s++) record_step_f64(pos.data(), vel.data(), force.data(), n, *P, tape[s - s0]);
        for (uint32_t s = s1; s-- > s0;) adjoint_step_f64(tape[s - s0], n, *P, gx.data(), gv.data(), acc_k.data(), acc_mu.data());
    }
    if (gpos0) std::memcpy(gpos0, gx.data(), N4 * 8);
    if (gvel0) std::memcpy(gvel0, gv.data(), N4 * 8);
    if (gparams) {
        double a = 0, b = 0;
        for (uint32_t i = 0; i < n; i++) {
            a += acc_k[i];
            b += acc_mu[i];
        }
        gparams[0] = a;
        gparams[1] = b;
    }
    return 0;
}

// The FP64 adjoint along a given trajectory: states_pos / states_vel hold the float4 state
// before each of the `steps` steps (step-major, float32, e.g. read back from the GPU after
// every step); force0 is the force buffer before the first step (later steps start from the
// gravity vector, as the step leaves it). Each step is re-linearised in FP64 around the given
// state, so branch decisions and neighbour sets follow that trajectory.
int orc_adjoint_states_f64(const float* states_pos, const float* states_vel, const double* force0, uint32_t n,
                           const gbsph_fluid3d_params* P, uint32_t steps, const double* gpos, const double* gvel,
                           double* gpos0, double* gvel0, double* gparams) {
    if (P->keyMode != GBSPH_KEY_LINEAR_GRID || P->dims != 3) return -1;
    const size_t N4 = 4 * (size_t)n;
    std::vector<double> gx(gpos, gpos + N4), gv(N4, 0.0), acc_k(n, 0.0), acc_mu(n, 0.0);
    if (gvel) std::memcpy(gv.data(), gvel, N4 * 8);
    std::vector<double> pos(N4), vel(N4), force(N4);
    TapeF64 t;
    for (uint32_t s = steps; s-- > 0;) {
        for (size_t i = 0; i < N4; i++) {
            pos[i] = states_pos[s * N4 + i];
            vel[i] = states_vel[s * N4 + i];
        }
        if (s == 0) {
            std::memcpy(force.data(), force0, N4 * 8);
        } else {
            for (size_t i = 0; i < n; i++)
                for (int c = 0; c < 4; c++) force[4 * i + c] = P->gravity[c];
        }
        record_step_f64(pos.data(), vel.data(), force.data(), n, *P, t);
        adjoint_step_f64(t, n, *P, gx.data(), gv.data(), acc_k.data(), acc_mu.data());
    }
    if (gpos0) std::memcpy(gpos0, gx.data(), N4 * 8);
    if (gvel0) std::memcpy(gvel0, gv.data(), N4 * 8);
    if (gparams) {
        double a = 0, b = 0;
        for (uint32_t i = 0; i < n; i++) {
            a += acc_k[i];
            b += acc_mu[i];
        }
        gparams[0] = a;
        gparams[1] = b;
    }
    return 0;
}

}  // extern "C"
