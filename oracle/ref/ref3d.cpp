// ref3d.cpp -- the reference's 3D SPH kernels (libCL/phys/oclFluid3D.cl, compiled
// unchanged apart from oracle/ref/rewrite.py's edits) driven as oclFluid3D::compute
// enqueues them (libCL/phys/oclFluid3D.cpp:293-342).
//
// TEST INFRASTRUCTURE ONLY: the checker that pins the oracle restatement (oracle3d.cpp) to
// the reference's own kernels, and the reference arm's CPU step. Nothing in the product
// library links it.
#include <cstdint>
#include <cstring>
#include <vector>

#include "clshim.h"

namespace clc {
namespace k3d {
#include "oclFluid3D.cl.inc"

// clInitFluid's constant lines (:145-147), through the reference's own macros (:123-128).
inline void kernel_constants(System* param) {
    param->kernelConstant = DensityConstant(param->cellSize);
    param->viscosityConstant = -param->viscosity * ViscosityConstant(param->cellSize);
    param->pressureConstant = -PressureConstant(param->cellSize);
}
}  // namespace k3d
}  // namespace clc

extern "C" int clref_radix_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int startBit, int endBit);

namespace {
using namespace clc;
const size_t kLocal = 256;         // oclFluid3D::cLocalSize, libCL/phys/oclFluid3D.cpp:16
const size_t kBuckets = 262144;    // oclFluid3D::cBucketCount, :17
static_assert(sizeof(k3d::System) == 13 * sizeof(float), "System is 13 floats");
static_assert(sizeof(k3d::BVHNode) == 48, "BVHNode is 48 bytes");

std::vector<float4> load4(const float* p, size_t n) {
    std::vector<float4> v(n);
    std::memcpy((void*)v.data(), p, n * sizeof(float4));
    return v;
}
void store4(float* p, const std::vector<float4>& v) { std::memcpy(p, (const void*)v.data(), v.size() * sizeof(float4)); }
float4 f4(const float* p) { return float4(p[0], p[1], p[2], p[3]); }
size_t local_for(size_t n) { return n % kLocal == 0 ? kLocal : 1; }
}  // namespace

extern "C" {

// clInitFluid (libCL/phys/oclFluid3D.cl:130-148), one work-item as clEnqueueTask runs it.
void clref3d_init_fluid(float* system13) {
    k3d::System s;
    std::memset(&s, 0, sizeof(s));
    run_groups(1, 1, [&] { k3d::clInitFluid(&s); });
    std::memcpy(system13, &s, sizeof(s));
}

// The three kernel constants (density, viscosity, pressure) as clInitFluid forms them for
// a given cell size and viscosity.
void clref3d_kernel_constants(float cell_size, float viscosity, float* out3) {
    k3d::System p;
    std::memset(&p, 0, sizeof(p));
    p.cellSize = cell_size;
    p.viscosity = viscosity;
    k3d::kernel_constants(&p);
    out3[0] = p.kernelConstant;
    out3[1] = p.viscosityConstant;
    out3[2] = p.pressureConstant;
}

// One oclFluid3D::compute on host arrays (pos, vel, force: float[4 n], updated in place).
// system13: the System block (:15-30); gravity_arg, box_min, box_max: the float4 kernel
// arguments of clGravity and clClipBox (bindBuffers, libCL/phys/oclFluid3D.cpp:256-268).
// Outputs: sorted keys and permutation, sorted position/velocity (.w = density/pressure),
// the 262,144-bucket cell table, and (when force_pre is not null) the force array as
// clCalculateForces leaves it. Returns 0; -1 when n is not a multiple of the local size
// 256 (the OpenCL 1.x NDRange rule the reference's launches rely on); the sort's codes.
int clref3d_step(float* pos, float* vel, float* force, uint32_t n, const float* system13, const float* gravity_arg,
                 const float* box_min, const float* box_max, uint32_t* cell, uint32_t* index, float* spos,
                 float* svel, uint32_t* cell_start, uint32_t* cell_end, float* force_pre) {
    if (n == 0 || n % kLocal != 0) return -1;
    k3d::System S;
    std::memcpy(&S, system13, sizeof(S));
    std::vector<float4> P = load4(pos, n), V = load4(vel, n), F = load4(force, n);
    std::vector<float4> SP(n), SV(n);
    const float4 g = f4(gravity_arg), bmin = f4(box_min), bmax = f4(box_max);
    uint* c = cell;
    uint* ix = index;
    uint* cs = cell_start;
    uint* ce = cell_end;

    run_groups(n, kLocal, [&] { k3d::clHash(c, ix, P.data(), &S); });                         // :295
    int rc = clref_radix_sort(c, ix, n, 0, 24);                                                // :299
    if (rc != 0) return rc;
    run_groups(n, kLocal, [&] { k3d::clReorder(ix, P.data(), V.data(), SP.data(), SV.data()); });  // :304
    for (size_t i = 0; i < kBuckets; i++) cs[i] = ce[i] = 0xFFFFFFFFu;                         // :309-313
    run_groups_coro(n, kLocal, [&] {                                                           // :315
        thread_local std::vector<uint> localHash(kLocal + 1);
        return k3d::clFindBounds(cs, ce, c, localHash.data());
    });
    run_groups(n, kLocal, [&] { k3d::clCalculateDensity(SP.data(), SV.data(), cs, ce, &S); });     // :318
    run_groups(n, kLocal, [&] { k3d::clCalculateForces(SP.data(), SV.data(), F.data(), ix, cs, ce, &S); });  // :321
    if (force_pre) store4(force_pre, F);
    run_groups(n, kLocal, [&] { k3d::clClipBox(SP.data(), SV.data(), F.data(), ix, &S, bmin, bmax); });  // :332
    run_groups(n, kLocal, [&] { k3d::clIntegrateForce(V.data(), F.data(), &S); });             // :334
    run_groups(n, kLocal, [&] { k3d::clGravity(F.data(), g); });                                // :336
    run_groups(n, kLocal, [&] { k3d::clIntegrateVelocity(P.data(), V.data(), &S); });          // :338
    store4(pos, P);
    store4(vel, V);
    store4(force, F);
    store4(spos, SP);
    store4(svel, SV);
    return 0;
}

// clEmitter (libCL/phys/oclFluid3D.cl:273-282) over n work-items.
void clref3d_emit(float* pos, float* vel, uint32_t n, uint32_t emit, float emit_speed, const float* system13) {
    k3d::System S;
    std::memcpy(&S, system13, sizeof(S));
    std::vector<float4> P = load4(pos, n), V = load4(vel, n);
    run_groups(n, local_for(n), [&] { k3d::clEmitter(P.data(), V.data(), emit, emit_speed, &S); });
    store4(pos, P);
    store4(vel, V);
}

// clCollideBVH (libCL/phys/oclFluid3D.cl:498-550) over n work-items: force, position and
// velocity float[4 n] updated in place; nodes: 48-byte BVHNode records; triangle: 3
// vertex indices per triangle; vertex: float[4 V].
void clref3d_collide_bvh(float* force, float* pos, float* vel, uint32_t n, const float* system13, const void* nodes,
                         uint32_t n_nodes, uint32_t root, const uint32_t* triangle, const float* vertex,
                         uint32_t n_vertex) {
    k3d::System S;
    std::memcpy(&S, system13, sizeof(S));
    std::vector<float4> P = load4(pos, n), V = load4(vel, n), F = load4(force, n), X = load4(vertex, n_vertex);
    std::vector<k3d::BVHNode> bvh(n_nodes);
    std::memcpy((void*)bvh.data(), nodes, n_nodes * sizeof(k3d::BVHNode));
    run_groups(n, local_for(n), [&] {
        k3d::clCollideBVH(F.data(), P.data(), V.data(), &S, bvh.data(), root, (const uint*)triangle, X.data());
    });
    store4(pos, P);
    store4(vel, V);
    store4(force, F);
}

}  // extern "C"
