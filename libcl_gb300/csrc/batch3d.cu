// batch3d.cu -- many independent 3D scenes advanced together (gbsph_batch3d_*).
//
// The scenes' particles are concatenated; each scene owns a slice of one global cell table
// (key = scene cell offset + the scene's own linear key) and a range of brick ids, so one
// hash, one sort, one bounds pass, one density and one force launch advance every scene. The
// brick kernels find a brick's scene by binary search over the scene table and take its gas
// constant, viscosity, box and grid from there; particles of different scenes are never in
// the same brick, so scenes cannot interact. The step is replayed as one CUDA graph; an
// autotuner picks the brick width.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fluid3d_kernels.cuh"

using namespace gbsph;

struct gbsph_batch3d_s {
    int device = 0;
    gbsph_fluid3d_params shared{};
    std::vector<gbsph_scene3d_desc> scenes;
    std::vector<SceneDev> sdev_host;
    SceneDev* sdev = nullptr;
    size_t n = 0, cells = 0;
    void* block = nullptr;  // every per-particle array
    float4 *pos = nullptr, *vel = nullptr, *force = nullptr, *spos = nullptr, *svel = nullptr;
    uint32_t *keys_a = nullptr, *keys_b = nullptr, *keys_c = nullptr, *vals_a = nullptr, *vals_b = nullptr;
    uint32_t *index = nullptr, *bricks = nullptr;
    uint16_t* nbr = nullptr;
    uint64_t* nbr_meta = nullptr;
    uint2* table = nullptr;
    bool table_clean = false;
    void* scratch = nullptr;
    uint32_t* err = nullptr;
    int bw = 8, use_graph = 1, sdev_bw = -1;
    int dens_blocks = 0, force_blocks = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::vector<char> gkey;
    std::string last_error;
};

namespace {

using B = gbsph_batch3d_s;

void binvalidate(B* h) {
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    h->gkey.clear();
}

void bfree(B* h) {
    void* ptrs[5] = {h->block, h->table, h->scratch, h->sdev, nullptr};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    h->block = nullptr;
    h->table = nullptr;
    h->scratch = nullptr;
    h->sdev = nullptr;
    h->n = h->cells = 0;
}

int bits_for_b(uint64_t cells) {
    int b = 0;
    while (b < 32 && (1ull << b) < cells) b++;
    return std::max(b, 1);
}

uint32_t* bcounters(B* h) { return (uint32_t*)((char*)h->scratch + SORT_USER_COUNTER_OFFSET); }

// Scene table for the current brick width (brick offsets depend on it).
int upload_scenes(B* h) {
    if (h->sdev_bw == h->bw) return GBSPH_OK;
    uint32_t brick_off = 0;
    for (auto& d : h->sdev_host) {
        d.bxn = (d.nx + h->bw - 1) / h->bw;
        d.brick_off = brick_off;
        brick_off += (uint32_t)d.bxn * (uint32_t)d.ny * (uint32_t)d.nz;
    }
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpy(h->sdev, h->sdev_host.data(), h->sdev_host.size() * sizeof(SceneDev),
                                              cudaMemcpyHostToDevice));
    h->sdev_bw = h->bw;
    binvalidate(h);
    return GBSPH_OK;
}

KParams make_kp(const B* h) {
    const gbsph_fluid3d_params& p = h->shared;
    KParams k;
    std::memset(&k, 0, sizeof(k));
    k.dt = p.deltaTime;
    k.radius = p.particleRadius;
    k.h = p.cellSize;
    k.mass = p.mass;
    k.p0 = p.pressure;
    k.rho0 = p.density;
    k.cpress = p.pressureConstant;
    k.kconst = p.kernelConstant;
    k.vlimit = p.velocitylimit;
    k.h2 = p.cellSize * p.cellSize;
    // smallest float x with sqrtf(x) >= h
    uint32_t lo = 0, hi = 0x7f800000u;
    while (hi - lo > 1) {
        const uint32_t mid = lo + (hi - lo) / 2;
        float f;
        std::memcpy(&f, &mid, 4);
        if (std::sqrt(f) >= p.cellSize) hi = mid;
        else lo = mid;
    }
    std::memcpy(&k.r2_thresh, &hi, 4);
    k.gravity = make_float4(p.gravity[0], p.gravity[1], p.gravity[2], p.gravity[3]);
    k.key_mode = GBSPH_KEY_LINEAR_GRID;
    k.dims = 3;
    k.end_bit = bits_for_b(h->cells);
    k.bw = h->bw;
    k.n = (uint32_t)h->n;
    k.table_cells = (uint32_t)h->cells;
    k.scenes = h->sdev;
    k.n_scenes = (int)h->scenes.size();
    return k;
}

#define BRC(x)                \
    do {                      \
        int _rc = (x);        \
        if (_rc) return _rc;  \
    } while (0)

int enqueue_batch(B* h, const KParams& kp, cudaStream_t s) {
    const bool clear = h->table_clean;
    if (!clear) GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(h->table, 0xFF, h->cells * sizeof(uint2), s));
    h->table_clean = false;
    GBSPH_CUDA_TRY(&h->last_error, onesweep_prepare(h->scratch, kp.n, sort_passes(0, kp.end_bit), s));
    const int blocks = std::max(1, std::min((int)((kp.n + 255) / 256), num_sms() * 8));
    if (clear)
        k_hash_batch<true><<<blocks, 256, 0, s>>>(h->pos, kp, h->keys_a, (uint32_t*)h->scratch, h->keys_c, h->table);
    else
        k_hash_batch<false><<<blocks, 256, 0, s>>>(h->pos, kp, h->keys_a, (uint32_t*)h->scratch, nullptr, nullptr);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    OnesweepArgs a;
    a.keys_in = h->keys_a;
    a.keys_out = h->keys_c;
    a.vals_out = h->index;
    a.tmp_keys[0] = h->keys_b;
    a.tmp_vals[0] = h->vals_b;
    a.tmp_keys[1] = h->keys_a;
    a.tmp_vals[1] = h->vals_a;
    a.n = kp.n;
    a.end_bit = kp.end_bit;
    a.scratch = h->scratch;
    a.err = h->err;
    a.gather.n_gather = 2;
    a.gather.src[0] = h->pos;
    a.gather.src[1] = h->vel;
    a.gather.dst[0] = h->spos;
    a.gather.dst[1] = h->svel;
    GBSPH_CUDA_TRY(&h->last_error, onesweep_passes(a, s));
    k_bounds_batch<<<(kp.n + BOUNDS_TILE - 1) / BOUNDS_TILE, 256, 0, s>>>(h->keys_c, kp, h->table, h->bricks, bcounters(h), h->err);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    h->table_clean = true;
    k_density_brick<3, true><<<h->dens_blocks, BRICK_THREADS, DENSITY_SMEM, s>>>(h->spos, h->svel, h->table, h->bricks,
                                                                                bcounters(h), kp, h->nbr, h->nbr_meta, h->err);
    k_force_brick<3, true, true><<<h->force_blocks, BRICK_THREADS, FORCE_SMEM, s>>>(
        h->spos, h->svel, h->index, h->pos, h->vel, h->force, h->table, h->bricks, bcounters(h), kp, h->nbr, h->nbr_meta,
        h->err);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

int bcompute(B* h, cudaStream_t s, bool allow_graph) {
    BRC(upload_scenes(h));
    const KParams kp = make_kp(h);
    if (!h->use_graph || !allow_graph || !h->table_clean) {
        const int rc = enqueue_batch(h, kp, s);
        if (rc) h->table_clean = false;
        return rc;
    }
    std::vector<char> key(sizeof(KParams));
    std::memcpy(key.data(), &kp, sizeof(KParams));
    if (!h->gexec || key != h->gkey) {
        binvalidate(h);
        GBSPH_CUDA_TRY(&h->last_error, cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_batch(h, kp, h->cap_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(h->cap_stream, &g);
        if (rc || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            h->table_clean = false;
            return rc ? rc : fail(&h->last_error, GBSPH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        }
        const cudaError_t ie = cudaGraphInstantiate(&h->gexec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            h->gexec = nullptr;
            h->table_clean = false;
            return fail(&h->last_error, GBSPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        }
        h->gkey = key;
    }
    const cudaError_t le = cudaGraphLaunch(h->gexec, s);
    if (le != cudaSuccess) {
        h->table_clean = false;
        return fail(&h->last_error, GBSPH_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(le));
    }
    h->table_clean = true;
    return GBSPH_OK;
}

}  // namespace

extern "C" {

GBSPH_API int gbsph_batch3d_create(gbsph_batch3d_t* out) {
    if (!out) return GBSPH_ERR_ARGUMENT;
    *out = nullptr;
    B* h = new B();
    int rc = GBSPH_OK;
    if (cudaGetDevice(&h->device) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMalloc(&h->err, 256) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMemset(h->err, 0, 256) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc) {
        int nb = 0;
        const int sms = num_sms();
        if (cudaFuncSetAttribute(k_density_brick<3, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)DENSITY_SMEM) ||
            cudaFuncSetAttribute(k_force_brick<3, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)FORCE_SMEM) ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_density_brick<3, true>, BRICK_THREADS, DENSITY_SMEM))
            rc = GBSPH_ERR_CUDA;
        h->dens_blocks = std::max(1, nb) * sms;
        if (!rc && cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force_brick<3, true, true>, BRICK_THREADS, FORCE_SMEM))
            rc = GBSPH_ERR_CUDA;
        h->force_blocks = std::max(1, nb) * sms;
    }
    if (rc) {
        cudaGetLastError();
        gbsph_batch3d_destroy(h);
        return rc;
    }
    *out = h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_batch3d_destroy(gbsph_batch3d_t h) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    cudaSetDevice(h->device);
    binvalidate(h);
    bfree(h);
    if (h->err) cudaFree(h->err);
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    delete h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_batch3d_set_scenes(gbsph_batch3d_t h, const gbsph_fluid3d_params* shared,
                                       const gbsph_scene3d_desc* scenes, int n_scenes) {
    if (!h || !shared || !scenes || n_scenes < 1) return GBSPH_ERR_ARGUMENT;
    if (!(shared->cellSize > 0.0f) || !std::isfinite(shared->deltaTime) || !std::isfinite(shared->mass))
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "shared parameters: cellSize must be > 0 and values finite");
    uint64_t n = 0, cells = 0;
    for (int i = 0; i < n_scenes; i++) {
        const gbsph_scene3d_desc& d = scenes[i];
        if (d.n_particles == 0 || d.gridDim[0] < 1 || d.gridDim[1] < 1 || d.gridDim[2] < 1 ||
            !std::isfinite(d.stiffness) || !std::isfinite(d.viscosity))
            return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "scene " + std::to_string(i) + ": bad description");
        n += d.n_particles;
        cells += (uint64_t)d.gridDim[0] * d.gridDim[1] * d.gridDim[2];
    }
    if (n > SORT_MAX_KEYS - SORT_TILE || cells > (1ull << 30))
        return fail(&h->last_error, GBSPH_ERR_TOO_LARGE, "batch has too many particles or cells");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    binvalidate(h);
    bfree(h);
    h->shared = *shared;
    h->shared.dims = 3;
    h->scenes.assign(scenes, scenes + n_scenes);
    h->sdev_host.assign(n_scenes, SceneDev{});
    uint32_t part_off = 0, cell_off = 0;
    for (int i = 0; i < n_scenes; i++) {
        const gbsph_scene3d_desc& d = scenes[i];
        SceneDev& e = h->sdev_host[i];
        std::memset(&e, 0, sizeof(e));
        e.part_off = part_off;
        e.cell_off = cell_off;
        e.n = d.n_particles;
        e.nx = d.gridDim[0];
        e.ny = d.gridDim[1];
        e.nz = d.gridDim[2];
        e.origin = make_float4(d.gridOrigin[0], d.gridOrigin[1], d.gridOrigin[2], 0.f);
        e.box_min = make_float4(d.boxMin[0], d.boxMin[1], d.boxMin[2], 0.f);
        e.box_max = make_float4(d.boxMax[0], d.boxMax[1], d.boxMax[2], 0.f);
        e.stiff = d.stiffness;
        gbsph_fluid3d_params tmp = *shared;
        tmp.dims = 3;
        tmp.viscosity = d.viscosity;
        gbsph_fluid3d_params_derive(&tmp);
        e.cvisc = tmp.viscosityConstant;
        part_off += d.n_particles;
        cell_off += (uint32_t)(d.gridDim[0] * d.gridDim[1] * d.gridDim[2]);
    }
    h->n = n;
    h->cells = cells;
    const size_t n4 = (n + 63) & ~size_t(63);
    const size_t bytes = n4 * (5 * 16 + 7 * 4 + NBR_CAP * 2 + 8);
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->block, bytes));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->block, 0, bytes));
    char* p = (char*)h->block;
    float4** f4[5] = {&h->pos, &h->vel, &h->force, &h->spos, &h->svel};
    for (auto a : f4) {
        *a = (float4*)p;
        p += n4 * 16;
    }
    uint32_t** u4[7] = {&h->keys_a, &h->keys_b, &h->keys_c, &h->vals_a, &h->vals_b, &h->index, &h->bricks};
    for (auto a : u4) {
        *a = (uint32_t*)p;
        p += n4 * 4;
    }
    h->nbr = (uint16_t*)p;
    p += n4 * NBR_CAP * 2;
    h->nbr_meta = (uint64_t*)p;
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->table, cells * sizeof(uint2)));
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->scratch, onesweep_scratch_bytes((uint32_t)n, SORT_MAX_PASSES)));
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->sdev, n_scenes * sizeof(SceneDev)));
    h->sdev_bw = -1;
    h->table_clean = false;
    return upload_scenes(h);
}

GBSPH_API void* gbsph_batch3d_get_buffer(gbsph_batch3d_t h, int which, size_t* count) {
    if (!h) return nullptr;
    if (count) *count = h->n;
    switch (which) {
        case GBSPH_BUF_POSITION: return h->pos;
        case GBSPH_BUF_VELOCITY: return h->vel;
        case GBSPH_BUF_FORCE: return h->force;
        case GBSPH_BUF_SORTED_POSITION: return h->spos;
        case GBSPH_BUF_SORTED_VELOCITY: return h->svel;
        case GBSPH_BUF_INDEX: return h->index;
        case GBSPH_BUF_CELL: return h->keys_c;
        default: return nullptr;
    }
}

GBSPH_API int gbsph_batch3d_scene_range(gbsph_batch3d_t h, int s, size_t* first, size_t* count) {
    if (!h || s < 0 || s >= (int)h->scenes.size()) return GBSPH_ERR_ARGUMENT;
    if (first) *first = h->sdev_host[s].part_off;
    if (count) *count = h->sdev_host[s].n;
    return GBSPH_OK;
}

GBSPH_API int gbsph_batch3d_set_option(gbsph_batch3d_t h, int option, int value) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (option == GBSPH_OPT_CUDA_GRAPH) {
        h->use_graph = value ? 1 : 0;
    } else if (option == GBSPH_OPT_BRICK_WIDTH) {
        if (value < 1 || value > BRICK_W_MAX) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "brick width must be in [1, 16]");
        h->bw = value;
    } else {
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "unknown option");
    }
    binvalidate(h);
    return GBSPH_OK;
}

GBSPH_API int gbsph_batch3d_compute(gbsph_batch3d_t h, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (h->n == 0) return fail(&h->last_error, GBSPH_ERR_STATE, "no scenes");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    return bcompute(h, (cudaStream_t)stream, true);
}

GBSPH_API int gbsph_batch3d_autotune(gbsph_batch3d_t h, void* stream, int* best_width) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (h->n == 0) return fail(&h->last_error, GBSPH_ERR_STATE, "no scenes");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    cudaStream_t s = (cudaStream_t)stream;
    const size_t st = ((h->n + 63) & ~size_t(63)) * sizeof(float4);  // pos, vel, force are adjacent
    void* saved = nullptr;
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&saved, 3 * st));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(saved, h->pos, 3 * st, cudaMemcpyDeviceToDevice, s));  // pos, vel, force
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int widths[3] = {4, 8, 16};
    float best = 1e30f;
    int best_w = h->bw, rc = GBSPH_OK;
    for (int w : widths) {
        h->bw = w;
        binvalidate(h);
        for (int i = 0; i < 2 && !rc; i++) rc = bcompute(h, s, true);  // eager + capture
        if (!rc) cudaEventRecord(e0, s);
        for (int i = 0; i < 3 && !rc; i++) rc = bcompute(h, s, true);
        if (rc) break;
        cudaEventRecord(e1, s);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
            best = ms;
            best_w = w;
        }
        cudaMemcpyAsync(h->pos, saved, 3 * st, cudaMemcpyDeviceToDevice, s);
    }
    cudaStreamSynchronize(s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(saved);
    h->bw = best_w;
    h->table_clean = false;
    binvalidate(h);
    if (best_width) *best_width = best_w;
    return rc;
}

GBSPH_API int gbsph_batch3d_sync_status(gbsph_batch3d_t h, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t bits = 0;
    GBSPH_CUDA_TRY(&h->last_error, cudaMemcpy(&bits, h->err, 4, cudaMemcpyDeviceToHost));
    if (bits) {
        GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->err, 0, 4));
        h->table_clean = false;
        return fail(&h->last_error, dev_err_to_status(bits), "device error word 0x" + std::to_string(bits));
    }
    return GBSPH_OK;
}

GBSPH_API const char* gbsph_batch3d_last_error(gbsph_batch3d_t h) { return h ? h->last_error.c_str() : "null handle"; }

}  // extern "C"
