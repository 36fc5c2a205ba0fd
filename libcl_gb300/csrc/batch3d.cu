// batch3d.cu -- many independent 3D scenes advanced together (gbsph_batch3d_*).
//
// The scenes' particles are concatenated; each scene owns a slice of one global cell table
// (key = scene cell offset + the scene's own linear key) and a range of brick ids, so one
// hash, one sort, one bounds pass, one density and one force launch advance every scene. The
// brick kernels find a brick's scene by binary search over the scene table and take its gas
// constant, viscosity, box and grid from there; particles of different scenes are never in
// the same brick, so scenes cannot interact. The step is replayed as one CUDA graph of one
// kernel per stage, or runs as one persistent cooperative kernel (k_batch_step); an
// autotuner picks the form, the brick width, the sort's digit width and its tile size.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fluid3d_kernels.cuh"
#include "grid_sync.cuh"
#include "onesweep.cuh"

using namespace gbsph;

namespace {

// ---- the persistent step ------------------------------------------------------------------

// Where k_batch_step keeps its grid barrier's words: offset in the sort scratch's caller
// counters (zeroed with the scratch before each step), on a cache line of their own.
constexpr uint32_t GRID_SYNC_WORD = 32;

struct BatchStepArgs {
    float4 *pos, *vel, *force, *spos, *svel;
    uint32_t *keys_a, *keys_b, *keys_c, *vals_a, *vals_b, *index, *bricks;
    uint16_t* nbr;
    uint64_t* nbr_meta;
    uint2* table;
    uint32_t* scratch;
    uint32_t* err;
    int clear;  // reset the previous step's table entries (keys_c) in the hash phase
};

// Dynamic shared memory of k_batch_step: each phase carves its own layout out of one buffer
// (the force phase's is the largest).
constexpr size_t STEP_SMEM = FORCE_SMEM;
static_assert(DENSITY_SMEM + sizeof(SubListCounts) <= STEP_SMEM, "density phase layout");
static_assert(onesweep_smem_words(SORT_ITEMS) * 4 <= STEP_SMEM, "sort phase layout");
static_assert(SORT_MAX_PASSES * SORT_RADIX * 4 <= STEP_SMEM, "hash phase layout");

// One step of every scene in one launch: hash + digit histograms, the radix-sort passes (the
// last gathers the sorted state), cell bounds + occupied bricks, density, forces +
// integration, with a grid-wide barrier between phases. Every phase takes its work from an
// atomic queue (sort tiles, brick ids) or strides over the grid, so the grid is whatever is
// resident: occupancy x SMs. Data written by one phase and read by a later one is read
// through L2 (ld_phase<true>) or by bulk copies after the barrier's proxy fence.
template <int ITEMS>
__global__ void __launch_bounds__(BRICK_THREADS, 3) k_batch_step(BatchStepArgs a, KParams kp) {
    extern __shared__ float4 s_dyn[];
    __shared__ BrickShared S[2];  // the brick phases use the two records in turn
    __shared__ LaneMap L;
    __shared__ uint32_t s_flag;
    uint32_t* words = reinterpret_cast<uint32_t*>(s_dyn);
    uint32_t* counters = a.scratch + SORT_USER_COUNTER_OFFSET / 4;
    GridSync gs{counters + GRID_SYNC_WORD, a.err, 0u, gridDim.x};

    if (a.clear) hash_batch_run<true>(words, a.pos, kp, a.keys_a, a.scratch, a.keys_c, a.table);
    else hash_batch_run<false>(words, a.pos, kp, a.keys_a, a.scratch, nullptr, nullptr);
    if (!gs.sync(&s_flag)) return;

    const int P = sort_passes(0, kp.end_bit, kp.digit_bits);
    const uint32_t tiles = sort_tiles(kp.n, SORT_THREADS * ITEMS);
    const OnesweepSmem sm = onesweep_smem<ITEMS>(words);
    SortGather g;
    g.n_gather = 2;
    g.src[0] = a.pos;
    g.src[1] = a.vel;
    g.dst[0] = a.spos;
    g.dst[1] = a.svel;
    const uint32_t* kin = a.keys_a;
    const uint32_t* vin = nullptr;
    for (int p = 0; p < P; ++p) {
        const bool last = p == P - 1;
        uint32_t* kout = last ? a.keys_c : ((p & 1) ? a.keys_a : a.keys_b);
        uint32_t* vout = last ? a.index : ((p & 1) ? a.vals_a : a.vals_b);
        const int shift = p * kp.digit_bits, bits = min(kp.digit_bits, kp.end_bit - shift);
        if (p == 0 && last) {
            while (onesweep_tile<true, 2, ITEMS, true>(sm, kin, vin, kout, vout, kp.n, shift, bits, p, tiles, a.scratch,
                                                       a.err, g)) {
            }
        } else if (p == 0) {
            while (onesweep_tile<true, 0, ITEMS, true>(sm, kin, vin, kout, vout, kp.n, shift, bits, p, tiles, a.scratch,
                                                       a.err, g)) {
            }
        } else if (last) {
            while (onesweep_tile<false, 2, ITEMS, true>(sm, kin, vin, kout, vout, kp.n, shift, bits, p, tiles,
                                                        a.scratch, a.err, g)) {
            }
        } else {
            while (onesweep_tile<false, 0, ITEMS, true>(sm, kin, vin, kout, vout, kp.n, shift, bits, p, tiles,
                                                        a.scratch, a.err, g)) {
            }
        }
        if (!gs.sync(&s_flag)) return;
        kin = kout;
        vin = vout;
    }

    const uint32_t btiles = (kp.n + BOUNDS_TILE - 1) / BOUNDS_TILE;
    for (uint32_t tile = blockIdx.x; tile < btiles; tile += gridDim.x)
        bounds_tile<true>(a.keys_c, kp, a.table, a.bricks, counters, a.err,
                          [&](uint32_t k) { return batch_brick_of(kp, k); }, tile);
    if (!gs.sync(&s_flag)) return;

    SubListCounts& wcnt = *reinterpret_cast<SubListCounts*>(reinterpret_cast<char*>(s_dyn) + DENSITY_SMEM);
    const bool ok = density_brick_run<3, true>(s_dyn, S, L, wcnt, a.spos, a.svel, a.table, a.bricks, counters, kp,
                                               a.nbr, a.nbr_meta, a.err);
    __syncthreads();
    if (threadIdx.x == 0) {
        if (ok) mbar_inval(reinterpret_cast<uint64_t*>(&S[0].bar));  // the force phase initialises it again
        else gs.abort();
    }
    if (!gs.sync(&s_flag)) return;

    force_brick_run<3, true, true, true>(s_dyn, S, L, a.spos, a.svel, a.index, a.pos, a.vel, a.force, a.table, a.bricks,
                                         counters, kp, a.nbr, a.nbr_meta, a.err);
}

}  // namespace

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
    int digit_bits = SORT_RADIX_BITS;  // bits per sort pass (5 to 8)
    int sort_items = 0;                // keys per thread of a sort tile (8 or 16; 0: by key count)
    int persistent = 0;                // 1: the step is one cooperative k_batch_step launch
    bool persistent_graph_ok = true;   // false once capturing the cooperative launch failed
    int step_blocks[2] = {0, 0};       // resident k_batch_step CTAs (8 and 16 keys per thread)
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
    k.digit_bits = h->digit_bits;
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
    GBSPH_CUDA_TRY(&h->last_error, onesweep_prepare(h->scratch, kp.n, sort_passes(0, kp.end_bit, kp.digit_bits), s));
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
    a.digit_bits = kp.digit_bits;
    a.items = h->sort_items;
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

int sort_items_of(const B* h) { return h->sort_items ? h->sort_items : sort_items_for((uint32_t)h->n); }

// The persistent form: table reset (when needed) and scratch clear, then one cooperative
// launch; replayed as a graph like the staged form (eagerly if the driver cannot capture a
// cooperative launch).
int enqueue_persistent(B* h, const KParams& kp, cudaStream_t s) {
    const bool clear = h->table_clean;
    if (!clear) GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(h->table, 0xFF, h->cells * sizeof(uint2), s));
    h->table_clean = false;
    GBSPH_CUDA_TRY(&h->last_error, onesweep_prepare(h->scratch, kp.n, sort_passes(0, kp.end_bit, kp.digit_bits), s));
    BatchStepArgs a;
    a.pos = h->pos;
    a.vel = h->vel;
    a.force = h->force;
    a.spos = h->spos;
    a.svel = h->svel;
    a.keys_a = h->keys_a;
    a.keys_b = h->keys_b;
    a.keys_c = h->keys_c;
    a.vals_a = h->vals_a;
    a.vals_b = h->vals_b;
    a.index = h->index;
    a.bricks = h->bricks;
    a.nbr = h->nbr;
    a.nbr_meta = h->nbr_meta;
    a.table = h->table;
    a.scratch = (uint32_t*)h->scratch;
    a.err = h->err;
    a.clear = clear ? 1 : 0;
    KParams k = kp;
    void* args[2] = {&a, &k};
    const bool big = sort_items_of(h) == 16;
    const void* fn = big ? (const void*)k_batch_step<16> : (const void*)k_batch_step<8>;
    GBSPH_CUDA_TRY(&h->last_error, cudaLaunchCooperativeKernel(fn, dim3(h->step_blocks[big ? 1 : 0]), dim3(BRICK_THREADS),
                                                               args, STEP_SMEM, s));
    h->table_clean = true;
    return GBSPH_OK;
}

int bcompute(B* h, cudaStream_t s, bool allow_graph) {
    BRC(upload_scenes(h));
    const KParams kp = make_kp(h);
    if (sort_passes(0, kp.end_bit, kp.digit_bits) > SORT_MAX_PASSES)
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT,
                    std::to_string(kp.digit_bits) + "-bit digits need more than four passes over " +
                        std::to_string(kp.end_bit) + "-bit keys");
    auto enqueue = [&](cudaStream_t st) { return h->persistent ? enqueue_persistent(h, kp, st) : enqueue_batch(h, kp, st); };
    if (!h->use_graph || !allow_graph || !h->table_clean || (h->persistent && !h->persistent_graph_ok)) {
        const int rc = enqueue(s);
        if (rc) h->table_clean = false;
        return rc;
    }
    std::vector<char> key(sizeof(KParams));
    std::memcpy(key.data(), &kp, sizeof(KParams));
    if (!h->gexec || key != h->gkey) {
        binvalidate(h);
        GBSPH_CUDA_TRY(&h->last_error, cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue(h->cap_stream);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(h->cap_stream, &g);
        cudaError_t ie = cudaSuccess;
        if (!rc && ce == cudaSuccess) ie = cudaGraphInstantiate(&h->gexec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (rc || ce != cudaSuccess || ie != cudaSuccess) {
            h->gexec = nullptr;
            h->table_clean = false;
            if (h->persistent) {  // a cooperative launch that this driver cannot capture: run it eagerly
                cudaGetLastError();
                h->persistent_graph_ok = false;
                h->last_error = std::string("the persistent step could not be captured (") +
                                cudaGetErrorString(ce != cudaSuccess ? ce : ie) + "); it runs eagerly";
                const int rc2 = enqueue(s);
                if (rc2) h->table_clean = false;
                return rc2;
            }
            if (rc) return rc;
            return fail(&h->last_error, GBSPH_ERR_CUDA,
                        std::string(ce != cudaSuccess ? "graph capture: " : "graph instantiate: ") +
                            cudaGetErrorString(ce != cudaSuccess ? ce : ie));
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
        const void* steps[2] = {(const void*)k_batch_step<8>, (const void*)k_batch_step<16>};
        for (int i = 0; i < 2 && !rc; i++) {
            if (cudaFuncSetAttribute(steps[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)STEP_SMEM) ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, steps[i], BRICK_THREADS, STEP_SMEM))
                rc = GBSPH_ERR_CUDA;
            h->step_blocks[i] = nb * sms;  // 0: the persistent form cannot run here
        }
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
    } else if (option == GBSPH_OPT_RADIX_BITS) {
        if (value < 5 || value > SORT_RADIX_BITS) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "radix bits must be in [5, 8]");
        h->digit_bits = value;
    } else if (option == GBSPH_OPT_SORT_TILE) {
        if (value != 0 && value != 8 && value != 16)
            return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "sort tile must be 0, 8 or 16 keys per thread");
        h->sort_items = value;
    } else if (option == GBSPH_OPT_PERSISTENT) {
        if (value && (h->step_blocks[0] == 0 || h->step_blocks[1] == 0))
            return fail(&h->last_error, GBSPH_ERR_STATE, "the persistent step does not fit on this device");
        h->persistent = value ? 1 : 0;
    } else {
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "unknown option");
    }
    binvalidate(h);
    return GBSPH_OK;
}

GBSPH_API int gbsph_batch3d_get_option(gbsph_batch3d_t h, int option, int* value) {
    if (!h || !value) return GBSPH_ERR_ARGUMENT;
    switch (option) {
        case GBSPH_OPT_CUDA_GRAPH: *value = h->use_graph; break;
        case GBSPH_OPT_BRICK_WIDTH: *value = h->bw; break;
        case GBSPH_OPT_RADIX_BITS: *value = h->digit_bits; break;
        case GBSPH_OPT_SORT_TILE: *value = h->sort_items; break;
        case GBSPH_OPT_PERSISTENT: *value = h->persistent; break;
        default: return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "unknown option");
    }
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
    // every combination of brick width x digit width x sort tile x step form
    const int widths[3] = {4, 8, 16}, digits[3] = {6, 7, 8}, items[2] = {8, 16};
    const int forms = (h->step_blocks[0] && h->step_blocks[1]) ? 2 : 1;
    const int end_bit = bits_for_b(h->cells);
    float best = 1e30f;
    int best_w = h->bw, best_d = h->digit_bits, best_i = h->sort_items, best_p = h->persistent, rc = GBSPH_OK;
    for (int c = 0; c < 3 * 3 * 2 * forms && !rc; c++) {
        const int w = widths[c / (3 * 2 * forms)], d = digits[(c / (2 * forms)) % 3], it = items[(c / forms) % 2],
                  pf = c % forms;
        if (sort_passes(0, end_bit, d) > SORT_MAX_PASSES) continue;
        h->bw = w;
        h->digit_bits = d;
        h->sort_items = it;
        h->persistent = pf;
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
            best_d = d;
            best_i = it;
            best_p = pf;
        }
        cudaMemcpyAsync(h->pos, saved, 3 * st, cudaMemcpyDeviceToDevice, s);
    }
    cudaStreamSynchronize(s);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(saved);
    h->bw = best_w;
    h->digit_bits = best_d;
    h->sort_items = best_i;
    h->persistent = best_p;
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
