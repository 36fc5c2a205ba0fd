// adjoint3d.cu -- host side of the 3D step's adjoint (gbsph_adjoint3d_*).
//
// forward(): `steps` ordinary compute() calls on the fluid, with a copy of (position, velocity,
// force) taken before every K-th step. backward(): for each segment of K steps, last first,
// the fluid is reset to the segment's checkpoint and stepped again with force recording on;
// after each step the permutation, sorted keys, sorted state and the force after the clip box
// are copied into the segment's tape (one kernel), and the density pass writes each
// particle's neighbour list (sorted indices) into the step's tape slot. The step's adjoint
// then runs in reverse over the tape: post (integration, clamp, walls; builds the step's cell
// table) -> force (gather over the lists) -> density (gather over the lists); particles
// without a list (overflow, unstaged brick) walk the cell table. The recomputed steps are the
// same kernels on the same inputs, so the tape holds exactly the forward's states.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "adjoint_kernels.cuh"

using namespace gbsph;

struct gbsph_adjoint3d_s {
    gbsph_fluid3d_t fluid = nullptr;
    int device = 0;
    uint32_t steps = 0, every = 0, nseg = 0;
    size_t n = 0, n4 = 0;
    void* block = nullptr;  // checkpoints, final state, tape, work arrays
    float4* ckpt = nullptr;  // nseg x {pos, vel, force} x n4
    float4* fin = nullptr;   // {pos, vel, force} x n4
    char* tape = nullptr;    // `every` slots
    uint32_t* lists = nullptr;  // `every` slots of n4 x NBR_CAP recorded neighbours
    uint32_t* lcnt = nullptr;   // `every` slots of n4 list lengths
    uint32_t* slot_dev = nullptr;  // the slot the recording step writes
    uint32_t* slot_ids = nullptr;  // 0, 1, ..., every - 1 (copied into slot_dev)
    float4 *w = nullptr, *gxs = nullptr, *gvs = nullptr, *gx = nullptr, *gv = nullptr, *rec = nullptr;
    float* gS = nullptr;
    double2* acc = nullptr;
    uint2* tables = nullptr;  // two cell tables, used by alternate steps
    size_t table_cells = 0;
    bool forward_done = false;
    gbsph_fluid3d_params params{};
    std::string last_error;
};

namespace {

using A = gbsph_adjoint3d_s;

#define RC(x)                \
    do {                     \
        int _rc = (x);       \
        if (_rc) return _rc; \
    } while (0)

size_t slot_bytes(size_t n4) { return n4 * (4 + 4 + 16 + 16 + 16); }

StepTape slot(const A* a, uint32_t k) {
    char* p = a->tape + slot_bytes(a->n4) * k;
    StepTape t;
    t.nbr = a->lists + (size_t)k * a->n4 * NBR_CAP;
    t.cnt = a->lcnt + (size_t)k * a->n4;
    t.spos = (float4*)p;
    p += a->n4 * 16;
    t.svel = (float4*)p;
    p += a->n4 * 16;
    t.fwall = (float4*)p;
    p += a->n4 * 16;
    t.index = (uint32_t*)p;
    p += a->n4 * 4;
    t.keys = (uint32_t*)p;
    return t;
}

int grid1(size_t n) { return (int)((n + 255) / 256); }

// Copies the fluid's (position, velocity, force) to `dst` (3 x n4) or back.
int copy_state(A* a, const FluidAccess& fa, float4* st, bool to_fluid, cudaStream_t s) {
    float4* f[3] = {fa.pos, fa.vel, fa.force};
    for (int k = 0; k < 3; k++) {
        float4* d = to_fluid ? f[k] : st + k * a->n4;
        const float4* src = to_fluid ? st + k * a->n4 : f[k];
        GBSPH_CUDA_TRY(&a->last_error, cudaMemcpyAsync(d, src, a->n * 16, cudaMemcpyDeviceToDevice, s));
    }
    return GBSPH_OK;
}

int check_fluid(A* a, FluidAccess* fa, KParams* kp) {
    const int rc = fluid3d_access(a->fluid, fa, kp);
    if (rc) return fail(&a->last_error, rc, std::string("fluid: ") + gbsph_fluid3d_last_error(a->fluid));
    if (!fa->compiled) return fail(&a->last_error, GBSPH_ERR_NOT_COMPILED, "the fluid is not compiled");
    if (fa->n != a->n) return fail(&a->last_error, GBSPH_ERR_SIZE_MISMATCH, "the fluid's particle count changed");
    if (fa->has_hook) return fail(&a->last_error, GBSPH_ERR_STATE, "the adjoint needs a fluid without an integrate hook");
    if (kp->key_mode != GBSPH_KEY_LINEAR_GRID || kp->dims != 3)
        return fail(&a->last_error, GBSPH_ERR_ARGUMENT, "the adjoint needs keyMode LINEAR_GRID and dims 3");
    if (kp->table_cells != a->table_cells || !a->tables) {
        if (a->tables) cudaFree(a->tables);
        a->tables = nullptr;
        a->table_cells = 0;
        GBSPH_CUDA_TRY(&a->last_error, cudaMalloc(&a->tables, 2ull * kp->table_cells * sizeof(uint2)));
        a->table_cells = kp->table_cells;
    }
    return GBSPH_OK;
}

// Clears the fluid's record pointer on every exit path of backward().
struct RecordGuard {
    gbsph_fluid3d_t f;
    ~RecordGuard() { fluid3d_set_record(f, nullptr); }
};

int backward_segment(A* a, const FluidAccess& fa, const KParams& kp, uint32_t seg, float c45, cudaStream_t s) {
    const uint32_t s0 = seg * a->every, s1 = std::min(a->steps, s0 + a->every);
    RC(copy_state(a, fa, a->ckpt + (size_t)seg * 3 * a->n4, true, s));
    for (uint32_t st = s0; st < s1; st++) {
        const uint32_t k = st - s0;  // the tape slot this step's lists go to
        GBSPH_CUDA_TRY(&a->last_error, cudaMemcpyAsync(a->slot_dev, a->slot_ids + k, 4, cudaMemcpyDeviceToDevice, s));
        // no list unless the step's density pass records one (the per-stage kernels do not)
        GBSPH_CUDA_TRY(&a->last_error, cudaMemsetAsync(a->lcnt + (size_t)k * a->n4, 0xFF, a->n4 * 4, s));
        const int rc = gbsph_fluid3d_compute(a->fluid, (void*)s);
        if (rc) return fail(&a->last_error, rc, std::string("recompute: ") + gbsph_fluid3d_last_error(a->fluid));
        k_tape_record<<<grid1(a->n), 256, 0, s>>>(slot(a, st - s0), fa.index, fa.keys, fa.spos, fa.svel, a->rec,
                                                   (uint32_t)a->n);
        GBSPH_CUDA_TRY(&a->last_error, cudaGetLastError());
    }
    GBSPH_CUDA_TRY(&a->last_error, cudaMemsetAsync(a->tables, 0xFF, 2ull * a->table_cells * sizeof(uint2), s));
    for (uint32_t st = s1; st-- > s0;) {
        const StepTape t = slot(a, st - s0);
        uint2* own = a->tables + (size_t)(st & 1) * a->table_cells;
        uint2* other = a->tables + (size_t)((st + 1) & 1) * a->table_cells;
        const uint32_t* keys_next = st + 1 < s1 ? slot(a, st + 1 - s0).keys : nullptr;
        k_adj_post<<<grid1(a->n), 256, 0, s>>>(t, a->gx, a->gv, a->w, a->gxs, a->gvs, own, other, keys_next, kp);
        k_adj_force<<<grid1(a->n * ADJ_LANES), 256, 0, s>>>(t, own, a->w, a->gxs, a->gvs, a->gS, a->acc, kp, c45);
        k_adj_density<<<grid1(a->n * ADJ_LANES), 256, 0, s>>>(t, own, a->gS, a->gxs, a->gvs, a->gx, a->gv, kp);
        GBSPH_CUDA_TRY(&a->last_error, cudaGetLastError());
    }
    return GBSPH_OK;
}

}  // namespace

extern "C" {

GBSPH_API int gbsph_adjoint3d_create(gbsph_adjoint3d_t* out, gbsph_fluid3d_t fluid, uint32_t steps,
                                     uint32_t checkpoint_every) {
    if (!out) return GBSPH_ERR_ARGUMENT;
    *out = nullptr;
    if (!fluid || steps == 0 || checkpoint_every == 0) return GBSPH_ERR_ARGUMENT;
    A* a = new A();
    a->fluid = fluid;
    a->steps = steps;
    a->every = std::min(checkpoint_every, steps);
    a->nseg = (steps + a->every - 1) / a->every;
    a->n = gbsph_fluid3d_get_particle_count(fluid);
    a->n4 = (a->n + 63) & ~size_t(63);
    const size_t n4 = a->n4;
    const size_t list_words = (size_t)a->every * n4 * (NBR_CAP + 1);
    const size_t bytes = (size_t)a->nseg * 3 * n4 * 16 + 3 * n4 * 16 + a->every * slot_bytes(n4) +
                         6 * n4 * 16 + n4 * 4 + n4 * 16 + list_words * 4 + ((size_t)a->every + 64) * 4;
    if (cudaGetDevice(&a->device) != cudaSuccess || cudaMalloc(&a->block, bytes) != cudaSuccess) {
        cudaGetLastError();
        delete a;
        return GBSPH_ERR_CUDA;
    }
    char* p = (char*)a->block;
    a->ckpt = (float4*)p;
    p += (size_t)a->nseg * 3 * n4 * 16;
    a->fin = (float4*)p;
    p += 3 * n4 * 16;
    a->tape = p;
    p += a->every * slot_bytes(n4);
    float4** f4[6] = {&a->w, &a->gxs, &a->gvs, &a->gx, &a->gv, &a->rec};
    for (auto q : f4) {
        *q = (float4*)p;
        p += n4 * 16;
    }
    a->acc = (double2*)p;
    p += n4 * 16;
    a->gS = (float*)p;
    p += n4 * 4;
    a->lists = (uint32_t*)p;
    p += (size_t)a->every * n4 * NBR_CAP * 4;
    a->lcnt = (uint32_t*)p;
    p += (size_t)a->every * n4 * 4;
    a->slot_dev = (uint32_t*)p;
    a->slot_ids = a->slot_dev + 64;
    std::vector<uint32_t> ids(a->every);
    for (uint32_t k = 0; k < a->every; k++) ids[k] = k;
    if (cudaMemcpy(a->slot_ids, ids.data(), (size_t)a->every * 4, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(a->block);
        delete a;
        return GBSPH_ERR_CUDA;
    }
    *out = a;
    return GBSPH_OK;
}

GBSPH_API int gbsph_adjoint3d_destroy(gbsph_adjoint3d_t a) {
    if (!a) return GBSPH_ERR_ARGUMENT;
    cudaSetDevice(a->device);
    if (a->block) cudaFree(a->block);
    if (a->tables) cudaFree(a->tables);
    delete a;
    return GBSPH_OK;
}

GBSPH_API int gbsph_adjoint3d_forward(gbsph_adjoint3d_t a, void* stream) {
    if (!a) return GBSPH_ERR_ARGUMENT;
    a->forward_done = false;
    FluidAccess fa;
    KParams kp;
    RC(check_fluid(a, &fa, &kp));
    cudaStream_t s = (cudaStream_t)stream;
    for (uint32_t st = 0; st < a->steps; st++) {
        if (st % a->every == 0) RC(copy_state(a, fa, a->ckpt + (size_t)(st / a->every) * 3 * a->n4, false, s));
        const int rc = gbsph_fluid3d_compute(a->fluid, stream);
        if (rc) return fail(&a->last_error, rc, std::string("forward: ") + gbsph_fluid3d_last_error(a->fluid));
    }
    RC(copy_state(a, fa, a->fin, false, s));
    std::memcpy(&a->params, gbsph_fluid3d_get_params(a->fluid), sizeof(a->params));
    a->forward_done = true;
    return GBSPH_OK;
}

GBSPH_API int gbsph_adjoint3d_backward(gbsph_adjoint3d_t a, const float* grad_position, const float* grad_velocity,
                                       float* grad_position0, float* grad_velocity0, double* grad_params,
                                       void* stream) {
    if (!a) return GBSPH_ERR_ARGUMENT;
    if (!grad_position) return fail(&a->last_error, GBSPH_ERR_ARGUMENT, "grad_position is required");
    if (!a->forward_done) return fail(&a->last_error, GBSPH_ERR_STATE, "backward() before forward()");
    if (std::memcmp(&a->params, gbsph_fluid3d_get_params(a->fluid), sizeof(a->params)) != 0)
        return fail(&a->last_error, GBSPH_ERR_STATE, "the fluid's parameters changed since forward()");
    FluidAccess fa;
    KParams kp;
    RC(check_fluid(a, &fa, &kp));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t bytes = a->n * 16;
    GBSPH_CUDA_TRY(&a->last_error, cudaMemcpyAsync(a->gx, grad_position, bytes, cudaMemcpyDeviceToDevice, s));
    if (grad_velocity)
        GBSPH_CUDA_TRY(&a->last_error, cudaMemcpyAsync(a->gv, grad_velocity, bytes, cudaMemcpyDeviceToDevice, s));
    else
        GBSPH_CUDA_TRY(&a->last_error, cudaMemsetAsync(a->gv, 0, bytes, s));
    GBSPH_CUDA_TRY(&a->last_error, cudaMemsetAsync(a->acc, 0, a->n * sizeof(double2), s));
    // dCv/dmu for the viscosity constant mu * 45 / (pi h^6) (pi rounded to float as in the
    // parameter derivation)
    const double pi = (double)(float)M_PI;
    const float c45 = (float)(45.0 / (pi * std::pow((double)a->params.cellSize, 6.0)));
    {
        RecordGuard guard{a->fluid};
        fluid3d_set_record(a->fluid, a->rec, a->lists, a->lcnt, a->slot_dev, (uint32_t)a->n4);
        for (uint32_t seg = a->nseg; seg-- > 0;) RC(backward_segment(a, fa, kp, seg, c45, s));
    }
    RC(copy_state(a, fa, a->fin, true, s));
    if (grad_params) {
        k_adj_reduce<<<1, 1024, 0, s>>>(a->acc, (uint32_t)a->n, grad_params);
        GBSPH_CUDA_TRY(&a->last_error, cudaGetLastError());
    }
    if (grad_position0)
        GBSPH_CUDA_TRY(&a->last_error, cudaMemcpyAsync(grad_position0, a->gx, bytes, cudaMemcpyDeviceToDevice, s));
    if (grad_velocity0)
        GBSPH_CUDA_TRY(&a->last_error, cudaMemcpyAsync(grad_velocity0, a->gv, bytes, cudaMemcpyDeviceToDevice, s));
    return GBSPH_OK;
}

GBSPH_API const char* gbsph_adjoint3d_last_error(gbsph_adjoint3d_t a) { return a ? a->last_error.c_str() : "null handle"; }

}  // extern "C"
