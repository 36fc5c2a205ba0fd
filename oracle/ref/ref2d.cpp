// ref2d.cpp -- the reference's 2D SPH kernels (libCL/phys/oclFluid2D.cl, compiled
// unchanged apart from oracle/ref/rewrite.py's edits) driven as oclFluid2D::compute and
// oclFluid2D::computeBorder enqueue them (libCL/phys/oclFluid2D.cpp:131-146,256-362).
//
// TEST INFRASTRUCTURE ONLY: the checker that pins the oracle restatement (oracle2d.cpp) to
// the reference's own kernels. Nothing in the product library links it.
#include <cstdint>
#include <cstring>
#include <vector>

#include "clshim.h"

namespace clc {
namespace k2d {
#include "oclFluid2D.cl.inc"
}  // namespace k2d
}  // namespace clc

extern "C" int clref_radix_sort(uint32_t* keys, uint32_t* vals, uint32_t n, int startBit, int endBit);

namespace {
using namespace clc;
const size_t kLocal = 256;  // oclFluid2D::cLocalSize, libCL/phys/oclFluid2D.h:79
static_assert(sizeof(k2d::System) == 48, "System is 12 four-byte fields");
static_assert(sizeof(k2d::Particle) == 24, "Particle is 24 bytes");
static_assert(sizeof(k2d::State) == 16, "State is one float4");

// The wall images as the reference creates them: RGBA half-float texels
// (libCL/phys/oclFluid2D.cpp:72-75). `values` are float RGBA texels.
struct half_image {
    std::vector<_Float16> texels;
    image im;
    half_image(const float* values, int w, int h) : texels((size_t)4 * w * h) {
        for (size_t i = 0; i < texels.size(); i++) texels[i] = values ? (_Float16)values[i] : (_Float16)0.0f;
        im = image{w, h, IMG_HALF_RGBA, texels.data()};
    }
    void to_float(float* out) const {
        for (size_t i = 0; i < texels.size(); i++) out[i] = (float)texels[i];
    }
};

uint32_t table_size(const k2d::System& S) {  // compile(), libCL/phys/oclFluid2D.cpp:240-243
    const size_t c = (size_t)(S.cellCountX * S.cellCountY);
    return (uint32_t)((c / kLocal + 1) * kLocal);
}
}  // namespace

extern "C" {

// clInitFluid (libCL/phys/oclFluid2D.cl:136-151), one work-item; fields it does not set
// stay zero.
void clref2d_init_fluid(void* params) {
    k2d::System s;
    std::memset(&s, 0, sizeof(s));
    run_groups(1, 1, [&] { k2d::clInitFluid(&s); });
    std::memcpy(params, &s, sizeof(s));
}

uint32_t clref2d_table_size(const void* params) {
    k2d::System S;
    std::memcpy(&S, params, sizeof(S));
    return table_size(S);
}

// computeBorder (libCL/phys/oclFluid2D.cpp:131-146): clComputeBorder over a w x h range.
// mask: float RGBA [h][w][4] (the caller's image); vec_out, state_out: the two half-float
// images it writes, returned as floats [h][w][4].
void clref2d_compute_border(const float* mask, int w, int h, const void* params, float* vec_out, float* state_out) {
    k2d::System S;
    std::memcpy(&S, params, sizeof(S));
    std::vector<float> m(mask, mask + (size_t)4 * w * h);
    image in{w, h, IMG_FLOAT_RGBA, m.data()};
    half_image vec(nullptr, w, h), st(nullptr, w, h);
    image2d_t pin = &in, pvec = &vec.im, pst = &st.im;
    run_items_2d((size_t)w, (size_t)h, [&] { k2d::clComputeBorder(pin, pvec, pst, &S); });
    vec.to_float(vec_out);
    st.to_float(state_out);
}

// One oclFluid2D::compute on a host Particle array (state: float[6 n], updated in place).
// border_state / border_vec: the wall images as float RGBA [h][w][4] (stored as half
// floats, as the reference's images are). Outputs: sorted keys and permutation, sorted
// particles, the (density, near density, pressure, near pressure) array, the relaxed and
// previous positions, and the cell table. Returns 0; -1 when n is not a multiple of 256;
// -5 when a particle's key falls outside the cell table (the reference would write
// outside it: it does not clamp, libCL/phys/oclFluid2D.cl:61-69,105-111); the sort's codes.
int clref2d_step(float* state, uint32_t n, const void* params, const float* border_state, const float* border_vec,
                 int w, int h, uint32_t* cell, uint32_t* index, float* sorted, float* pstate, float* relaxed,
                 float* prev, uint32_t* cell_start, uint32_t* cell_end) {
    if (n == 0 || n % kLocal != 0) return -1;
    k2d::System S;
    std::memcpy(&S, params, sizeof(S));
    const uint32_t cells = table_size(S);
    std::vector<k2d::Particle> st(n), srt(n);
    std::memcpy((void*)st.data(), state, (size_t)n * sizeof(k2d::Particle));
    std::vector<float2> prevPos(n), relaxedPos(n);
    std::vector<k2d::State> pressure(n);
    half_image bstate(border_state, w, h), bvec(border_vec, w, h);
    image2d_t pbs = &bstate.im, pbv = &bvec.im;
    uint* c = cell;
    uint* ix = index;
    uint* cs = cell_start;
    uint* ce = cell_end;

    run_groups(n, kLocal, [&] { k2d::clAdvanceState(st.data(), prevPos.data(), &S); });   // :260
    run_groups(n, kLocal, [&] { k2d::clHash(c, ix, st.data(), &S); });                     // :263
    for (uint32_t i = 0; i < n; i++)
        if (c[i] >= cells) return -5;
    int rc = clref_radix_sort(c, ix, n, 0, 24);                                            // :267
    if (rc != 0) return rc;
    run_groups(n, kLocal, [&] { k2d::clReorder(ix, st.data(), srt.data()); });             // :285
    run_groups(cells, kLocal, [&] { k2d::clInitBounds(cs, ce); });                          // :288
    run_groups_coro(n, kLocal, [&] {                                                       // :290
        thread_local std::vector<uint> localHash(kLocal + 1);
        return k2d::clFindBounds(cs, ce, c, localHash.data());
    });
    run_groups(n, kLocal, [&] { k2d::clComputePressure(srt.data(), pressure.data(), cs, ce, pbs, &S); });  // :293
    run_groups(n, kLocal, [&] {                                                            // :311
        k2d::clComputePosition(srt.data(), pressure.data(), relaxedPos.data(), cs, ce, pbs, pbv, &S);
    });
    run_groups(n, kLocal, [&] {                                                            // :327
        k2d::clUpdateState(st.data(), prevPos.data(), relaxedPos.data(), ix, &S);
    });
    std::memcpy(state, (const void*)st.data(), (size_t)n * sizeof(k2d::Particle));
    std::memcpy(sorted, (const void*)srt.data(), (size_t)n * sizeof(k2d::Particle));
    std::memcpy(pstate, (const void*)pressure.data(), (size_t)n * sizeof(k2d::State));
    std::memcpy(relaxed, (const void*)relaxedPos.data(), (size_t)n * sizeof(float2));
    std::memcpy(prev, (const void*)prevPos.data(), (size_t)n * sizeof(float2));
    return 0;
}

// clEmitter (libCL/phys/oclFluid2D.cl:342-352) over n work-items.
void clref2d_emit(float* state, uint32_t n, uint32_t emit, const void* params) {
    k2d::System S;
    std::memcpy(&S, params, sizeof(S));
    std::vector<k2d::Particle> st(n);
    std::memcpy((void*)st.data(), state, (size_t)n * sizeof(k2d::Particle));
    run_groups(n, n % kLocal == 0 ? kLocal : 1, [&] { k2d::clEmitter(st.data(), emit, &S); });
    std::memcpy(state, (const void*)st.data(), (size_t)n * sizeof(k2d::Particle));
}

}  // extern "C"
