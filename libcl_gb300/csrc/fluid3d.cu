// fluid3d.cu -- host side of the 3D SPH fluid: the oclFluid3D replacement behind the C ABI.
//
// One step (libCL/phys/oclFluid3D.cpp:293-342) is enqueued on the caller's stream as:
//   memset(sort scratch) -> k_hash (+digit histogram, +sparse clear of last step's cells)
//   -> one-sweep passes (last pass gathers sorted position/velocity = clReorder)
//   -> cell bounds (+ occupied-brick list) -> density -> forces (+clip/integrate/gravity)
// and, once the cell table is in steady state, replayed as a captured CUDA graph.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "fluid3d_access.h"

using namespace gbsph;

namespace {


struct DevBuf {
    void* ptr = nullptr;
    size_t count = 0;
    bool owned = false;
};

float bits_to_float(uint32_t b) {
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}

// Smallest float x >= 0 with sqrtf(x) >= h. sqrtf is correctly rounded and monotone, so for
// every float r2 >= 0: (sqrtf(r2) < h) == (r2 < threshold).
float r2_threshold(float h) {
    if (!(h > 0.0f)) return 0.0f;  // nothing is nearer than h
    if (std::isinf(h)) return h;   // every finite distance is
    uint32_t lo = 0, hi = 0x7f800000u;  // sqrtf(+0) = 0 < h, sqrtf(inf) = inf >= h
    while (hi - lo > 1) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (std::sqrt(bits_to_float(mid)) >= h) hi = mid;
        else lo = mid;
    }
    return bits_to_float(hi);
}

int bits_for(uint64_t cells) {  // number of key bits to sort so that every key < cells is covered
    int b = 0;
    while (b < 32 && (1ull << b) < cells) b++;
    return std::max(b, 1);
}

}  // namespace

struct gbsph_fluid3d_s {
    int device = 0;
    gbsph_fluid3d_params params{};
    bool compiled = false;
    size_t n = 256;
    DevBuf buf[3];  // position, velocity, force
    size_t n_alloc = 0;
    void* pblock = nullptr;  // per-particle internal arrays
    float4* spos = nullptr;
    float4* svel = nullptr;
    uint32_t *keys_a = nullptr, *keys_b = nullptr, *keys_c = nullptr;
    uint32_t *vals_a = nullptr, *vals_b = nullptr, *index = nullptr, *bricks = nullptr;
    uint16_t* nbr = nullptr;      // per particle NBR_CAP neighbour slots (density -> forces)
    uint64_t* nbr_meta = nullptr;  // per particle: sub-list lengths, scan flag (bit 63)
    uint32_t* hash_tables = nullptr;  // cell start / end, REF_BUCKETS each
    uint32_t* xlist = nullptr;        // REFERENCE_HASH fused step: XL_CAP neighbours + count per particle
    size_t xlist_n = 0;
    uint2* table = nullptr;           // LINEAR_GRID interleaved table
    size_t table_cells = 0;
    bool table_clean = false;  // table empty except the runs of keys_c
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    uint32_t* err = nullptr;
    float4* rec_force = nullptr;  // set by an adjoint while it records a step
    uint32_t* rec_nbr = nullptr;
    uint32_t* rec_cnt = nullptr;
    const uint32_t* rec_slot = nullptr;
    uint32_t rec_n4 = 0;
    gbsph_fluid3d_hook_fn hook = nullptr;
    void* hook_user = nullptr;
    int opt_fused = 1, opt_graph = 1, opt_bw = 16, opt_profile = 0;
    cudaEvent_t ev[6] = {};
    bool ev_valid = false;
    int dens_blocks = 0, force_blocks = 0;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::vector<char> gkey;
    // compute_host: the step with its host copies, captured separately
    cudaStream_t io_stream = nullptr;
    cudaEvent_t io_ev[5] = {};  // fork, position, velocity and force uploaded, side copies done
    float4* io_grav = nullptr;  // n copies of the gravity vector: the fused step's force output
    size_t io_grav_n = 0;
    cudaGraphExec_t gexec_io = nullptr;
    std::vector<char> gkey_io;
    // getParamBuffer: a device copy of `params`, refreshed on the stream before a step whenever
    // the host struct differs from the copy last written (`dparams_shadow`)
    gbsph_fluid3d_params* dparams = nullptr;
    gbsph_fluid3d_params dparams_shadow{};
    bool dparams_valid = false;
    std::string last_error;
};

namespace {

using H = gbsph_fluid3d_s;

__global__ void k_store_params(gbsph_fluid3d_params* __restrict__ out, gbsph_fluid3d_params p) {
    if (threadIdx.x == 0) *out = p;
}

// Brings the device copy of the parameters up to date on `s` (no-op when unchanged). The
// struct travels as a kernel argument, so later host edits cannot race with the write.
int refresh_param_buffer(H* h, cudaStream_t s) {
    if (h->dparams_valid && std::memcmp(&h->dparams_shadow, &h->params, sizeof(h->params)) == 0) return GBSPH_OK;
    k_store_params<<<1, 32, 0, s>>>(h->dparams, h->params);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    h->dparams_shadow = h->params;
    h->dparams_valid = true;
    return GBSPH_OK;
}

void default_params(gbsph_fluid3d_params* p) {
    // clInitFluid, libCL/phys/oclFluid3D.cl:130-148 (double literals evaluated in double)
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
    p->dims = 3;
    gbsph_fluid3d_params_derive(p);
    // hard-coded kernel arguments, libCL/phys/oclFluid3D.cpp:256-268
    p->gravity[0] = -9.8f * 0.0f;
    p->gravity[1] = -9.8f * 0.0f;
    p->gravity[2] = -9.8f * 1.0f;
    p->gravity[3] = -9.8f * 0.0f;
    for (int i = 0; i < 3; i++) {
        p->boxMin[i] = -1.0f;
        p->boxMax[i] = 1.0f;
    }
    p->keyMode = GBSPH_KEY_REFERENCE_HASH;
}

bool finite_all(const float* v, int n) {
    for (int i = 0; i < n; i++)
        if (!std::isfinite(v[i])) return false;
    return true;
}

int validate_params(H* h) {
    const gbsph_fluid3d_params& p = h->params;
    if (!finite_all(&p.deltaTime, 13) || !finite_all(p.gravity, 4) || !std::isfinite(p.boxMin[0]) ||
        !std::isfinite(p.boxMin[1]) || !std::isfinite(p.boxMax[0]) || !std::isfinite(p.boxMax[1]) ||
        !finite_all(p.gridOrigin, 3))
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "parameters hold a NaN or infinity");
    if (!(p.cellSize > 0.0f)) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "cellSize must be > 0");
    if (p.dims != 2 && p.dims != 3) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "dims must be 2 or 3");
    if (p.keyMode == GBSPH_KEY_LINEAR_GRID) {
        const int64_t nz = p.dims == 2 ? 1 : p.gridDim[2];
        if (p.gridDim[0] < 1 || p.gridDim[1] < 1 || nz < 1)
            return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "gridDim must be positive");
        if ((int64_t)p.gridDim[0] * p.gridDim[1] * nz > (1ll << 30))
            return fail(&h->last_error, GBSPH_ERR_TOO_LARGE, "grid has more than 2^30 cells");
    } else if (p.keyMode != GBSPH_KEY_REFERENCE_HASH) {
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "unknown keyMode");
    }
    return GBSPH_OK;
}

KParams make_kparams(const H* h) {
    const gbsph_fluid3d_params& p = h->params;
    KParams k;
    std::memset(&k, 0, sizeof(k));  // padding too: the struct is compared bytewise as a graph key
    k.dt = p.deltaTime;
    k.radius = p.particleRadius;
    k.h = p.cellSize;
    k.mass = p.mass;
    k.p0 = p.pressure;
    k.rho0 = p.density;
    k.stiff = p.stiffness;
    k.cvisc = p.viscosityConstant;
    k.cpress = p.pressureConstant;
    k.kconst = p.kernelConstant;
    k.vlimit = p.velocitylimit;
    k.h2 = p.cellSize * p.cellSize;
    k.r2_thresh = r2_threshold(p.cellSize);
    k.gravity = make_float4(p.gravity[0], p.gravity[1], p.gravity[2], p.gravity[3]);
    k.box_min = make_float4(p.boxMin[0], p.boxMin[1], p.boxMin[2], p.boxMin[3]);
    k.box_max = make_float4(p.boxMax[0], p.boxMax[1], p.boxMax[2], p.boxMax[3]);
    k.origin = make_float4(p.gridOrigin[0], p.gridOrigin[1], p.gridOrigin[2], 0.0f);
    k.key_mode = p.keyMode;
    k.dims = p.dims;
    if (p.keyMode == GBSPH_KEY_LINEAR_GRID) {
        k.nx = p.gridDim[0];
        k.ny = p.gridDim[1];
        k.nz = p.dims == 2 ? 1 : p.gridDim[2];
        k.table_cells = (uint32_t)((uint64_t)k.nx * k.ny * k.nz);
        k.end_bit = bits_for(k.table_cells);
    } else {
        k.nx = k.ny = k.nz = 0;
        k.table_cells = REF_BUCKETS;
        k.end_bit = 18;  // keys < 2^18; the reference sorts bits [0, 24) of the same keys
    }
    k.digit_bits = SORT_RADIX_BITS;
    k.bw = h->opt_bw;
    k.bxn = k.nx > 0 ? (k.nx + k.bw - 1) / k.bw : 0;
    k.n = (uint32_t)h->n;
    k.rec_force = h->rec_force;
    k.rec_nbr = h->rec_nbr;
    k.rec_cnt = h->rec_cnt;
    k.rec_slot = h->rec_slot;
    k.rec_n4 = h->rec_n4;
    return k;
}

void invalidate_graph(H* h) {
    if (h->gexec) cudaGraphExecDestroy(h->gexec);
    h->gexec = nullptr;
    h->gkey.clear();
    if (h->gexec_io) cudaGraphExecDestroy(h->gexec_io);
    h->gexec_io = nullptr;
    h->gkey_io.clear();
}

// Host state of gbsph_fluid3d_compute_host: three float4[n] inputs and outputs.
struct HostIO {
    const float* in[3];
    float* out[3];
};

void free_particle_arrays(H* h) {
    if (h->pblock) cudaFree(h->pblock);
    h->pblock = nullptr;
    if (h->scratch) cudaFree(h->scratch);
    h->scratch = nullptr;
    h->n_alloc = 0;
}

int alloc_particle_arrays(H* h, size_t n) {
    free_particle_arrays(h);
    const size_t n4 = (n + 63) & ~size_t(63);
    const size_t bytes = n4 * (2 * 16 + 7 * 4 + NBR_CAP * 2 + 8);
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->pblock, bytes));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->pblock, 0, bytes));
    char* p = (char*)h->pblock;
    h->spos = (float4*)p;
    p += n4 * 16;
    h->svel = (float4*)p;
    p += n4 * 16;
    uint32_t** arr[7] = {&h->keys_a, &h->keys_b, &h->keys_c, &h->vals_a, &h->vals_b, &h->index, &h->bricks};
    for (auto a : arr) {
        *a = (uint32_t*)p;
        p += n4 * 4;
    }
    h->nbr = (uint16_t*)p;
    p += n4 * NBR_CAP * 2;
    h->nbr_meta = (uint64_t*)p;
    h->scratch_bytes = onesweep_scratch_bytes((uint32_t)n, SORT_MAX_PASSES);
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->scratch, h->scratch_bytes));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->scratch, 0, h->scratch_bytes));
    h->n_alloc = n;
    h->table_clean = false;
    return GBSPH_OK;
}

int alloc_owned(H* h, int which, size_t n) {
    DevBuf& b = h->buf[which];
    if (b.owned && b.ptr) cudaFree(b.ptr);
    b = DevBuf();
    GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&b.ptr, std::max<size_t>(n, 1) * 16));
    GBSPH_CUDA_TRY(&h->last_error, cudaMemset(b.ptr, 0, std::max<size_t>(n, 1) * 16));
    b.count = n;
    b.owned = true;
    return GBSPH_OK;
}

// Makes the cell tables match the current parameters.
int ensure_tables(H* h) {
    if (h->params.keyMode == GBSPH_KEY_LINEAR_GRID) {
        const size_t cells = (size_t)h->params.gridDim[0] * h->params.gridDim[1] *
                             (size_t)(h->params.dims == 2 ? 1 : h->params.gridDim[2]);
        if (cells != h->table_cells || !h->table) {
            if (h->table) cudaFree(h->table);
            h->table = nullptr;
            h->table_cells = 0;
            GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->table, cells * sizeof(uint2)));
            h->table_cells = cells;
            h->table_clean = false;
            invalidate_graph(h);
        }
    } else {
        if (!h->hash_tables) {
            GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->hash_tables, 2 * (size_t)REF_BUCKETS * 4));
            GBSPH_CUDA_TRY(&h->last_error, cudaMemset(h->hash_tables, 0xFF, 2 * (size_t)REF_BUCKETS * 4));
        }
        if (h->xlist_n != h->n_alloc) {  // the fused step's neighbour lists
            if (h->xlist) cudaFree(h->xlist);
            h->xlist = nullptr;
            h->xlist_n = 0;
            GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->xlist, std::max<size_t>(h->n_alloc, 1) * (XL_CAP + 1) * 4));
            h->xlist_n = h->n_alloc;
            invalidate_graph(h);
        }
    }
    return GBSPH_OK;
}

uint32_t* counters(H* h) { return (uint32_t*)((char*)h->scratch + SORT_USER_COUNTER_OFFSET); }
float4* P4(H* h, int w) { return (float4*)h->buf[w].ptr; }

int grid1(uint32_t n) { return (int)((n + 255) / 256); }

// ---- stage launchers ----------------------------------------------------------------------

int st_hash(H* h, const KParams& kp, cudaStream_t s, bool clear) {
    GBSPH_CUDA_TRY(&h->last_error, onesweep_prepare(h->scratch, kp.n, sort_passes(0, kp.end_bit), s));
    const int blocks = std::max(1, std::min(grid1(kp.n), num_sms() * 8));
    if (clear)
        k_hash<true><<<blocks, 256, 0, s>>>(P4(h, 0), kp, h->keys_a, (uint32_t*)h->scratch, h->keys_c, h->table);
    else
        k_hash<false><<<blocks, 256, 0, s>>>(P4(h, 0), kp, h->keys_a, (uint32_t*)h->scratch, nullptr, nullptr);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

// Sorts the keys; with `gather` the last pass also gathers the sorted positions and, with
// gather_vel, the sorted velocities.
int st_sort(H* h, const KParams& kp, cudaStream_t s, bool gather, cudaEvent_t before_last = nullptr,
            bool gather_vel = true) {
    OnesweepArgs a;
    a.keys_in = h->keys_a;
    a.vals_in = nullptr;
    a.keys_out = h->keys_c;
    a.vals_out = h->index;
    a.tmp_keys[0] = h->keys_b;
    a.tmp_vals[0] = h->vals_b;
    a.tmp_keys[1] = h->keys_a;
    a.tmp_vals[1] = h->vals_a;
    a.n = kp.n;
    a.start_bit = 0;
    a.end_bit = kp.end_bit;
    a.scratch = h->scratch;
    a.err = h->err;
    if (gather) {
        a.gather.n_gather = gather_vel ? 2 : 1;
        a.gather.src[0] = P4(h, 0);
        a.gather.src[1] = P4(h, 1);
        a.gather.dst[0] = h->spos;
        a.gather.dst[1] = h->svel;
    }
    a.before_last = before_last;
    GBSPH_CUDA_TRY(&h->last_error, onesweep_passes(a, s));
    return GBSPH_OK;
}

// Sorted velocities gathered on their own (when the velocity upload is still in flight while
// the sort runs).
__global__ void k_gather_velocity(const uint32_t* __restrict__ index, const float4* __restrict__ vel,
                                  float4* __restrict__ svel, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) svel[i] = vel[index[i]];
}

int st_reorder(H* h, const KParams& kp, cudaStream_t s) {
    k_reorder<<<grid1(kp.n), 256, 0, s>>>(h->index, P4(h, 0), P4(h, 1), h->spos, h->svel, kp.n);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

int st_bounds(H* h, const KParams& kp, cudaStream_t s, bool full_clear) {
    if (kp.key_mode == GBSPH_KEY_LINEAR_GRID) {
        if (full_clear) GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(h->table, 0xFF, h->table_cells * sizeof(uint2), s));
        GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(counters(h), 0, 16, s));
        k_bounds_linear<<<(kp.n + BOUNDS_TILE - 1) / BOUNDS_TILE, 256, 0, s>>>(h->keys_c, kp, h->table, h->bricks, counters(h), h->err);
        GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    } else {
        GBSPH_CUDA_TRY(&h->last_error, cell_bounds_launch(h->keys_c, kp.n, h->hash_tables,
                                                          h->hash_tables + REF_BUCKETS, REF_BUCKETS, h->err, s));
    }
    return GBSPH_OK;
}

// Exact (reference-order) density and forces. With lists (the fused REFERENCE_HASH step, where
// the two run back to back on the same sorted state) the density kernel records each
// particle's in-range neighbours and the force kernel walks them instead of the buckets.
int st_density_exact(H* h, const KParams& kp, cudaStream_t s, bool lists = false) {
    uint32_t* xl = h->xlist;
    uint32_t* xc = h->xlist ? h->xlist + (size_t)h->xlist_n * XL_CAP : nullptr;
    if (kp.key_mode == GBSPH_KEY_LINEAR_GRID)
        k_density_exact<GBSPH_KEY_LINEAR_GRID, PairTable, false><<<grid1(kp.n), 256, 0, s>>>(
            h->spos, h->svel, PairTable{h->table}, kp, nullptr, nullptr);
    else if (lists && xl)
        k_density_exact<GBSPH_KEY_REFERENCE_HASH, SplitTable, true><<<grid1(kp.n), 256, 0, s>>>(
            h->spos, h->svel, SplitTable{h->hash_tables, h->hash_tables + REF_BUCKETS}, kp, xl, xc);
    else
        k_density_exact<GBSPH_KEY_REFERENCE_HASH, SplitTable, false><<<grid1(kp.n), 256, 0, s>>>(
            h->spos, h->svel, SplitTable{h->hash_tables, h->hash_tables + REF_BUCKETS}, kp, nullptr, nullptr);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

int st_forces_exact(H* h, const KParams& kp, cudaStream_t s, bool lists = false) {
    const uint32_t* xl = h->xlist;
    const uint32_t* xc = h->xlist ? h->xlist + (size_t)h->xlist_n * XL_CAP : nullptr;
    if (kp.key_mode == GBSPH_KEY_LINEAR_GRID)
        k_forces_exact<GBSPH_KEY_LINEAR_GRID, PairTable, false><<<grid1(kp.n), 256, 0, s>>>(
            h->spos, h->svel, P4(h, 2), h->index, PairTable{h->table}, kp, nullptr, nullptr);
    else if (lists && xl)
        k_forces_exact<GBSPH_KEY_REFERENCE_HASH, SplitTable, true><<<grid1(kp.n), 256, 0, s>>>(
            h->spos, h->svel, P4(h, 2), h->index, SplitTable{h->hash_tables, h->hash_tables + REF_BUCKETS}, kp, xl, xc);
    else
        k_forces_exact<GBSPH_KEY_REFERENCE_HASH, SplitTable, false><<<grid1(kp.n), 256, 0, s>>>(
            h->spos, h->svel, P4(h, 2), h->index, SplitTable{h->hash_tables, h->hash_tables + REF_BUCKETS}, kp,
            nullptr, nullptr);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

int st_density_brick(H* h, const KParams& kp, cudaStream_t s) {
    auto launch = [&](auto kern) {
        kern<<<h->dens_blocks, BRICK_THREADS, DENSITY_SMEM, s>>>(h->spos, h->svel, h->table, h->bricks, counters(h), kp,
                                                                 h->nbr, h->nbr_meta, h->err);
    };
    if (kp.dims == 2) launch(k_density_brick<2, false>);
    else launch(k_density_brick<3, false>);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

int st_force_brick(H* h, const KParams& kp, cudaStream_t s, bool fused) {
    auto launch = [&](auto kern) {
        kern<<<h->force_blocks, BRICK_THREADS, FORCE_SMEM, s>>>(h->spos, h->svel, h->index, P4(h, 0), P4(h, 1), P4(h, 2),
                                                                h->table, h->bricks, counters(h), kp, h->nbr,
                                                                h->nbr_meta, h->err);
    };
    if (kp.dims == 2) {
        if (fused) launch(k_force_brick<2, true, false>);
        else launch(k_force_brick<2, false, false>);
    } else {
        if (fused) launch(k_force_brick<3, true, false>);
        else launch(k_force_brick<3, false, false>);
    }
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

int st_post(H* h, const KParams& kp, int stage, cudaStream_t s) {
    const int g = grid1(kp.n);
    switch (stage) {
        case GBSPH_STAGE_CLIP_BOX: k_clip_box<<<g, 256, 0, s>>>(h->spos, h->svel, P4(h, 2), h->index, kp); break;
        case GBSPH_STAGE_INTEGRATE_FORCE: k_integrate_force<<<g, 256, 0, s>>>(P4(h, 1), P4(h, 2), kp); break;
        case GBSPH_STAGE_GRAVITY: k_gravity<<<g, 256, 0, s>>>(P4(h, 2), kp); break;
        case GBSPH_STAGE_INTEGRATE_VELOCITY: k_integrate_velocity<<<g, 256, 0, s>>>(P4(h, 0), P4(h, 1), kp); break;
        default: return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "not a post stage");
    }
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

int run_hook(H* h, cudaStream_t s) {
    const int rc = h->hook(h, (void*)s, h->hook_user);
    if (rc != 0) return fail(&h->last_error, GBSPH_ERR_STATE, "integrate hook returned " + std::to_string(rc));
    return GBSPH_OK;
}

#define RC(x)                   \
    do {                        \
        int _rc = (x);          \
        if (_rc) return _rc;    \
    } while (0)

// The reference's kernel sequence, one kernel per stage (GBSPH_OPT_FUSED = 0).
int enqueue_staged(H* h, const KParams& kp, cudaStream_t s) {
    h->table_clean = false;
    RC(st_hash(h, kp, s, false));
    RC(st_sort(h, kp, s, false));
    RC(st_reorder(h, kp, s));
    RC(st_bounds(h, kp, s, true));
    RC(st_density_exact(h, kp, s));
    RC(st_forces_exact(h, kp, s));
    if (h->hook) return run_hook(h, s);
    for (int st = GBSPH_STAGE_CLIP_BOX; st <= GBSPH_STAGE_INTEGRATE_VELOCITY; ++st) RC(st_post(h, kp, st, s));
    return GBSPH_OK;
}

// With GBSPH_OPT_PROFILE: an event between stages (gbsph_fluid3d_stage_times) and an NVTX
// range per stage (named as the stage times; seen by nsys / ncu --nvtx, free otherwise).
int mark(H* h, int i, cudaStream_t s) {
    if (!h->opt_profile) return GBSPH_OK;
    static const char* const kStage[5] = {"gbsph front_end", "gbsph sort", "gbsph bounds", "gbsph density",
                                          "gbsph forces"};
    if (i > 0) nvtxRangePop();
    if (i < 5) nvtxRangePushA(kStage[i]);
    if (!h->ev[i]) GBSPH_CUDA_TRY(&h->last_error, cudaEventCreate(&h->ev[i]));
    GBSPH_CUDA_TRY(&h->last_error, cudaEventRecord(h->ev[i], s));
    return GBSPH_OK;
}

// The fused step (default). With `io` the step also uploads its state from host memory and
// downloads it after: position first on `s`; velocity and force on a side stream, waited for
// just before the sort's last pass (which gathers velocities) and before the force pass, so
// their transfers overlap the hash, the sort and the density pass; the three downloads follow
// the force pass.
int enqueue_fused(H* h, const KParams& kp, cudaStream_t s, const HostIO* io = nullptr) {
    const bool linear = kp.key_mode == GBSPH_KEY_LINEAR_GRID;
    const bool clear = linear && h->table_clean;
    const size_t bytes = (size_t)kp.n * 16;
    h->ev_valid = false;
    // Without a hook the fused step leaves the gravity vector in every force entry, so the force
    // output is known before the step runs: it is downloaded from io_grav on the side stream
    // while the step computes (after the force input has been read from the same host array).
    const bool grav_out = io && !h->hook && h->io_grav && h->io_grav_n >= kp.n;
    if (io) {
        // the uploads one after another on the side stream (position first: the hash needs it;
        // velocity next: the last sort pass gathers it; force last: the force pass reads it)
        GBSPH_CUDA_TRY(&h->last_error, cudaEventRecord(h->io_ev[0], s));
        GBSPH_CUDA_TRY(&h->last_error, cudaStreamWaitEvent(h->io_stream, h->io_ev[0], 0));
        for (int w = 0; w < 3; w++) {
            GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(P4(h, w), io->in[w], bytes, cudaMemcpyHostToDevice, h->io_stream));
            GBSPH_CUDA_TRY(&h->last_error, cudaEventRecord(h->io_ev[1 + w], h->io_stream));
        }
        if (grav_out) {
            k_gravity<<<grid1(kp.n), 256, 0, h->io_stream>>>(h->io_grav, kp);
            GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
            GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(io->out[2], h->io_grav, bytes, cudaMemcpyDeviceToHost, h->io_stream));
        }
        GBSPH_CUDA_TRY(&h->last_error, cudaEventRecord(h->io_ev[4], h->io_stream));
    }
    RC(mark(h, 0, s));
    if (linear && !h->table_clean)
        GBSPH_CUDA_TRY(&h->last_error, cudaMemsetAsync(h->table, 0xFF, h->table_cells * sizeof(uint2), s));
    h->table_clean = false;
    if (io) GBSPH_CUDA_TRY(&h->last_error, cudaStreamWaitEvent(s, h->io_ev[1], 0));
    RC(st_hash(h, kp, s, clear));
    RC(mark(h, 1, s));
    // with host input the sort does not wait for the velocity upload: the sorted velocities
    // are gathered after the cell bounds (before the density pass, which writes their w)
    RC(st_sort(h, kp, s, true, nullptr, io == nullptr));
    auto gather_velocity = [&]() -> int {
        if (!io) return GBSPH_OK;
        GBSPH_CUDA_TRY(&h->last_error, cudaStreamWaitEvent(s, h->io_ev[2], 0));
        k_gather_velocity<<<grid1(kp.n), 256, 0, s>>>(h->index, P4(h, 1), h->svel, kp.n);
        GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
        return GBSPH_OK;
    };
    RC(mark(h, 2, s));
    if (linear) {
        // counters were zeroed with the sort scratch in st_hash
        k_bounds_linear<<<(kp.n + BOUNDS_TILE - 1) / BOUNDS_TILE, 256, 0, s>>>(h->keys_c, kp, h->table, h->bricks, counters(h), h->err);
        GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
        h->table_clean = true;
        RC(gather_velocity());
        RC(mark(h, 3, s));
        RC(st_density_brick(h, kp, s));
        RC(mark(h, 4, s));
        if (io) GBSPH_CUDA_TRY(&h->last_error, cudaStreamWaitEvent(s, h->io_ev[3], 0));
        RC(st_force_brick(h, kp, s, h->hook == nullptr));
    } else {
        RC(st_bounds(h, kp, s, true));
        RC(gather_velocity());
        RC(mark(h, 3, s));
        RC(st_density_exact(h, kp, s, true));
        RC(mark(h, 4, s));
        if (io) GBSPH_CUDA_TRY(&h->last_error, cudaStreamWaitEvent(s, h->io_ev[3], 0));
        RC(st_forces_exact(h, kp, s, true));
        if (!h->hook) {
            k_post_fused<<<grid1(kp.n), 256, 0, s>>>(h->spos, h->svel, h->index, P4(h, 0), P4(h, 1), P4(h, 2), kp);
            GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
        }
    }
    RC(mark(h, 5, s));
    h->ev_valid = h->opt_profile != 0;
    if (h->hook) RC(run_hook(h, s));
    if (io) {
        for (int w = 0; w < (grav_out ? 2 : 3); w++)
            GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(io->out[w], P4(h, w), bytes, cudaMemcpyDeviceToHost, s));
        GBSPH_CUDA_TRY(&h->last_error, cudaStreamWaitEvent(s, h->io_ev[4], 0));
    }
    return GBSPH_OK;
}

std::vector<char> graph_key(const H* h, const KParams& kp) {
    std::vector<char> k(sizeof(KParams) + 3 * sizeof(void*) + 4 * sizeof(int));
    char* p = k.data();
    std::memcpy(p, &kp, sizeof(KParams));
    p += sizeof(KParams);
    for (int i = 0; i < 3; i++) {
        std::memcpy(p, &h->buf[i].ptr, sizeof(void*));
        p += sizeof(void*);
    }
    int o[4] = {h->opt_fused, h->opt_bw, (int)h->table_cells, 0};
    std::memcpy(p, o, sizeof(o));
    return k;
}

int setup_kernels(H* h) {
    const int sms = num_sms();
    int nb = 0;
    const int dsm = (int)DENSITY_SMEM, fsm = (int)FORCE_SMEM;
    GBSPH_CUDA_TRY(&h->last_error, cudaFuncSetAttribute(k_density_brick<3, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dsm));
    GBSPH_CUDA_TRY(&h->last_error, cudaFuncSetAttribute(k_density_brick<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, dsm));
    GBSPH_CUDA_TRY(&h->last_error, cudaFuncSetAttribute(k_force_brick<3, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm));
    GBSPH_CUDA_TRY(&h->last_error, cudaFuncSetAttribute(k_force_brick<3, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm));
    GBSPH_CUDA_TRY(&h->last_error, cudaFuncSetAttribute(k_force_brick<2, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm));
    GBSPH_CUDA_TRY(&h->last_error, cudaFuncSetAttribute(k_force_brick<2, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm));
    GBSPH_CUDA_TRY(&h->last_error, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_density_brick<3, false>, BRICK_THREADS, DENSITY_SMEM));
    h->dens_blocks = std::max(1, nb) * sms;
    GBSPH_CUDA_TRY(&h->last_error, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force_brick<3, true, false>, BRICK_THREADS, FORCE_SMEM));
    h->force_blocks = std::max(1, nb) * sms;
    return GBSPH_OK;
}

}  // namespace

namespace gbsph {

int fluid3d_access(gbsph_fluid3d_t h, FluidAccess* a, KParams* kp) {
    RC(validate_params(h));
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    RC(ensure_tables(h));
    a->pos = P4(h, 0);
    a->vel = P4(h, 1);
    a->force = P4(h, 2);
    a->spos = h->spos;
    a->svel = h->svel;
    a->index = h->index;
    a->keys = h->keys_c;
    a->n = h->n;
    a->has_hook = h->hook != nullptr;
    a->compiled = h->compiled;
    *kp = make_kparams(h);
    return GBSPH_OK;
}

void fluid3d_set_record(gbsph_fluid3d_t h, float4* rec, uint32_t* rec_nbr, uint32_t* rec_cnt, const uint32_t* rec_slot,
                        uint32_t rec_n4) {
    h->rec_force = rec;
    h->rec_nbr = rec_nbr;
    h->rec_cnt = rec_cnt;
    h->rec_slot = rec_slot;
    h->rec_n4 = rec_n4;
}

}  // namespace gbsph

extern "C" {

GBSPH_API int gbsph_fluid3d_params_derive(gbsph_fluid3d_params* p) {
    if (!p) return GBSPH_ERR_ARGUMENT;
    const double pi = (double)(float)M_PI;
    const double h = p->cellSize;
    if (p->dims == 2) {
        p->kernelConstant = (float)(4.0 / (pi * std::pow(h, 8.0)));
        p->pressureConstant = (float)(30.0 / (pi * std::pow(h, 5.0)));
        p->viscosityConstant = (float)((double)p->viscosity * 40.0 / (pi * std::pow(h, 5.0)));
    } else {
        // DensityConstant / PressureConstant / ViscosityConstant, libCL/phys/oclFluid3D.cl:123-128,
        // with OpenCL C's types: M_PI_F is a float, so 64.0*M_PI_F*pow(h, 9) is a double
        // product while M_PI_F * pow(h, 6.0f) is a float product, divided into -45.0 in double.
        const float pi_f = (float)M_PI;
        p->kernelConstant = (float)(315.0 / (64.0 * pi * (double)std::pow(p->cellSize, 9.0f)));
        p->viscosityConstant =
            (float)(-(double)p->viscosity * (-45.0 / (double)(pi_f * std::pow(p->cellSize, 6.0f))));
        p->pressureConstant = (float)(-(-45.0 / (double)(pi_f * std::pow(p->cellSize, 6.0f))));
    }
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_default_params(gbsph_fluid3d_params* p) {
    if (!p) return GBSPH_ERR_ARGUMENT;
    default_params(p);
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_create(gbsph_fluid3d_t* out) {
    if (!out) return GBSPH_ERR_ARGUMENT;
    *out = nullptr;
    H* h = new H();
    int rc = GBSPH_OK;
    if (cudaGetDevice(&h->device) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMalloc(&h->err, 256) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMemset(h->err, 0, 256) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaStreamCreateWithFlags(&h->cap_stream, cudaStreamNonBlocking) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMalloc(&h->dparams, sizeof(gbsph_fluid3d_params)) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc && cudaMemset(h->dparams, 0, sizeof(gbsph_fluid3d_params)) != cudaSuccess) rc = GBSPH_ERR_CUDA;
    if (!rc) rc = alloc_particle_arrays(h, h->n);
    for (int w = 0; w < 3 && !rc; w++) rc = alloc_owned(h, w, h->n);
    if (rc) {
        cudaGetLastError();
        gbsph_fluid3d_destroy(h);
        return rc;
    }
    default_params(&h->params);
    *out = h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_destroy(gbsph_fluid3d_t h) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    cudaSetDevice(h->device);
    invalidate_graph(h);
    for (auto& b : h->buf)
        if (b.owned && b.ptr) cudaFree(b.ptr);
    free_particle_arrays(h);
    if (h->hash_tables) cudaFree(h->hash_tables);
    if (h->xlist) cudaFree(h->xlist);
    if (h->table) cudaFree(h->table);
    if (h->err) cudaFree(h->err);
    if (h->dparams) cudaFree(h->dparams);
    if (h->cap_stream) cudaStreamDestroy(h->cap_stream);
    if (h->io_stream) cudaStreamDestroy(h->io_stream);
    if (h->io_grav) cudaFree(h->io_grav);
    for (auto e : h->io_ev)
        if (e) cudaEventDestroy(e);
    for (auto e : h->ev)
        if (e) cudaEventDestroy(e);
    delete h;
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_compile(gbsph_fluid3d_t h) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    default_params(&h->params);
    RC(setup_kernels(h));
    RC(refresh_param_buffer(h, nullptr));
    GBSPH_CUDA_TRY(&h->last_error, cudaStreamSynchronize(nullptr));
    h->compiled = true;
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_set_particle_count(gbsph_fluid3d_t h, size_t n) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (n == 0) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "particle count must be > 0");
    if (n > SORT_MAX_KEYS - SORT_TILE)
        return fail(&h->last_error, GBSPH_ERR_TOO_LARGE, "particle count above " + std::to_string(SORT_MAX_KEYS - SORT_TILE));
    for (int w = 0; w < 3; w++)
        if (!h->buf[w].owned && h->buf[w].count < n)
            return fail(&h->last_error, GBSPH_ERR_SIZE_MISMATCH,
                        "borrowed buffer " + std::to_string(w) + " holds fewer than " + std::to_string(n) + " float4");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    invalidate_graph(h);
    h->n = n;
    RC(alloc_particle_arrays(h, n));
    for (int w = 0; w < 3; w++)
        if (h->buf[w].owned) RC(alloc_owned(h, w, n));
    return GBSPH_OK;
}

GBSPH_API size_t gbsph_fluid3d_get_particle_count(gbsph_fluid3d_t h) { return h ? h->n : 0; }

GBSPH_API int gbsph_fluid3d_set_buffer(gbsph_fluid3d_t h, int which, void* device_ptr, size_t count) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (which < GBSPH_BUF_POSITION || which > GBSPH_BUF_FORCE)
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "only position, velocity and force buffers can be set");
    if (!device_ptr) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null buffer");
    if ((uintptr_t)device_ptr % 16 != 0) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "buffer not 16-byte aligned");
    if (which == GBSPH_BUF_POSITION ? count != h->n : count < h->n)
        return fail(&h->last_error, GBSPH_ERR_SIZE_MISMATCH,
                    "buffer holds " + std::to_string(count) + " float4, particle count is " + std::to_string(h->n));
    DevBuf& b = h->buf[which];
    if (b.owned && b.ptr) {
        cudaSetDevice(h->device);
        cudaFree(b.ptr);
    }
    b.ptr = device_ptr;
    b.count = count;
    b.owned = false;
    invalidate_graph(h);
    return GBSPH_OK;
}

GBSPH_API void* gbsph_fluid3d_get_buffer(gbsph_fluid3d_t h, int which, size_t* count) {
    if (!h) return nullptr;
    void* p = nullptr;
    switch (which) {
        case GBSPH_BUF_POSITION:
        case GBSPH_BUF_VELOCITY:
        case GBSPH_BUF_FORCE:
            if (count) *count = h->buf[which].count;
            return h->buf[which].ptr;
        case GBSPH_BUF_SORTED_POSITION: p = h->spos; break;
        case GBSPH_BUF_SORTED_VELOCITY: p = h->svel; break;
        case GBSPH_BUF_INDEX: p = h->index; break;
        case GBSPH_BUF_CELL: p = h->keys_c; break;
        case GBSPH_BUF_PARAMS:  // one record, brought up to date with the host struct first
            if (cudaSetDevice(h->device) != cudaSuccess || refresh_param_buffer(h, nullptr) != GBSPH_OK ||
                cudaStreamSynchronize(nullptr) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;
            }
            if (count) *count = 1;
            return h->dparams;
        default: return nullptr;
    }
    if (count) *count = h->n;
    return p;
}

GBSPH_API gbsph_fluid3d_params* gbsph_fluid3d_get_params(gbsph_fluid3d_t h) { return h ? &h->params : nullptr; }

GBSPH_API int gbsph_fluid3d_set_integrate_hook(gbsph_fluid3d_t h, gbsph_fluid3d_hook_fn fn, void* user) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    h->hook = fn;
    h->hook_user = user;
    invalidate_graph(h);
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_set_option(gbsph_fluid3d_t h, int option, int value) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    switch (option) {
        case GBSPH_OPT_FUSED: h->opt_fused = value ? 1 : 0; break;
        case GBSPH_OPT_CUDA_GRAPH: h->opt_graph = value ? 1 : 0; break;
        case GBSPH_OPT_BRICK_WIDTH:
            if (value < 1 || value > BRICK_W_MAX)
                return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "brick width must be in [1, 16]");
            h->opt_bw = value;
            break;
        case GBSPH_OPT_PROFILE: h->opt_profile = value ? 1 : 0; break;
        default: return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "unknown option");
    }
    invalidate_graph(h);
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_stage_times(gbsph_fluid3d_t h, float* ms, int max_stages) {
    if (!h || !ms) return GBSPH_ERR_ARGUMENT;
    if (!h->ev_valid) return fail(&h->last_error, GBSPH_ERR_STATE, "no profiled compute() recorded");
    GBSPH_CUDA_TRY(&h->last_error, cudaEventSynchronize(h->ev[5]));
    const int n = std::min(max_stages, 5);
    for (int i = 0; i < n; i++) GBSPH_CUDA_TRY(&h->last_error, cudaEventElapsedTime(&ms[i], h->ev[i], h->ev[i + 1]));
    return n;
}

namespace {

// One step on `s`; with `io` (compute_host) the upload and download are part of it. The
// default path replays a captured graph (one per kind: with and without host copies).
int compute_impl(H* h, cudaStream_t s, const HostIO* io, bool io_graph) {
    RC(validate_params(h));
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    RC(ensure_tables(h));
    RC(refresh_param_buffer(h, s));
    const KParams kp = make_kparams(h);
    const size_t bytes = (size_t)kp.n * 16;
    if (!h->opt_fused) {
        if (io)
            for (int w = 0; w < 3; w++)
                GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(P4(h, w), io->in[w], bytes, cudaMemcpyHostToDevice, s));
        RC(enqueue_staged(h, kp, s));
        if (io)
            for (int w = 0; w < 3; w++)
                GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(io->out[w], P4(h, w), bytes, cudaMemcpyDeviceToHost, s));
        return GBSPH_OK;
    }
    const bool steady = kp.key_mode != GBSPH_KEY_LINEAR_GRID || h->table_clean;
    if (h->hook || !h->opt_graph || !steady || h->opt_profile || (io && !io_graph)) {
        const int rc = enqueue_fused(h, kp, s, io);
        if (rc) h->table_clean = false;
        return rc;
    }
    std::vector<char> key = graph_key(h, kp);
    if (io) {
        const size_t o = key.size();
        key.resize(o + sizeof(HostIO) + sizeof(void*));
        std::memcpy(key.data() + o, io, sizeof(HostIO));
        std::memcpy(key.data() + o + sizeof(HostIO), &h->io_grav, sizeof(void*));
    }
    cudaGraphExec_t& gexec = io ? h->gexec_io : h->gexec;
    std::vector<char>& gkey = io ? h->gkey_io : h->gkey;
    if (!gexec || key != gkey) {
        if (gexec) cudaGraphExecDestroy(gexec);
        gexec = nullptr;
        gkey.clear();
        GBSPH_CUDA_TRY(&h->last_error, cudaStreamBeginCapture(h->cap_stream, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue_fused(h, kp, h->cap_stream, io);
        cudaGraph_t g = nullptr;
        const cudaError_t ce = cudaStreamEndCapture(h->cap_stream, &g);
        if (rc || ce != cudaSuccess) {
            if (g) cudaGraphDestroy(g);
            h->table_clean = false;
            return rc ? rc : fail(&h->last_error, GBSPH_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        }
        const cudaError_t ie = cudaGraphInstantiate(&gexec, g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            gexec = nullptr;
            h->table_clean = false;
            return fail(&h->last_error, GBSPH_ERR_CUDA, std::string("graph instantiate: ") + cudaGetErrorString(ie));
        }
        gkey = key;
    }
    const cudaError_t le = cudaGraphLaunch(gexec, s);
    if (le != cudaSuccess) {
        h->table_clean = false;
        return fail(&h->last_error, GBSPH_ERR_CUDA, std::string("graph launch: ") + cudaGetErrorString(le));
    }
    h->table_clean = true;
    return GBSPH_OK;
}

bool is_pinned_host(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

}  // namespace

GBSPH_API int gbsph_fluid3d_compute(gbsph_fluid3d_t h, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!h->compiled) return fail(&h->last_error, GBSPH_ERR_NOT_COMPILED, "compute() before compile()");
    return compute_impl(h, (cudaStream_t)stream, nullptr, false);
}

GBSPH_API int gbsph_fluid3d_compute_host(gbsph_fluid3d_t h, const float* position_in, const float* velocity_in,
                                         const float* force_in, float* position_out, float* velocity_out,
                                         float* force_out, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!h->compiled) return fail(&h->last_error, GBSPH_ERR_NOT_COMPILED, "compute() before compile()");
    if (!position_in || !velocity_in || !force_in || !position_out || !velocity_out || !force_out)
        return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null host buffer");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    if (!h->io_stream) {
        GBSPH_CUDA_TRY(&h->last_error, cudaStreamCreateWithFlags(&h->io_stream, cudaStreamNonBlocking));
        for (auto& e : h->io_ev) GBSPH_CUDA_TRY(&h->last_error, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    }
    if (h->io_grav_n < h->n) {
        if (h->io_grav) cudaFree(h->io_grav);
        h->io_grav = nullptr;
        h->io_grav_n = 0;
        GBSPH_CUDA_TRY(&h->last_error, cudaMalloc(&h->io_grav, h->n * sizeof(float4)));
        h->io_grav_n = h->n;
    }
    const HostIO io{{position_in, velocity_in, force_in}, {position_out, velocity_out, force_out}};
    bool pinned = true;
    for (int w = 0; w < 3; w++) pinned = pinned && is_pinned_host(io.in[w]) && is_pinned_host(io.out[w]);
    return compute_impl(h, (cudaStream_t)stream, &io, pinned);
}

GBSPH_API int gbsph_fluid3d_stage(gbsph_fluid3d_t h, int stage, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!h->compiled) return fail(&h->last_error, GBSPH_ERR_NOT_COMPILED, "stage before compile()");
    RC(validate_params(h));
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    RC(ensure_tables(h));
    RC(refresh_param_buffer(h, (cudaStream_t)stream));
    const KParams kp = make_kparams(h);
    cudaStream_t s = (cudaStream_t)stream;
    h->table_clean = false;
    switch (stage) {
        case GBSPH_STAGE_HASH: return st_hash(h, kp, s, false);
        case GBSPH_STAGE_SORT:
            GBSPH_CUDA_TRY(&h->last_error, onesweep_reset_progress(h->scratch, kp.n, sort_passes(0, kp.end_bit), s));
            return st_sort(h, kp, s, false);
        case GBSPH_STAGE_REORDER: return st_reorder(h, kp, s);
        case GBSPH_STAGE_BOUNDS: return st_bounds(h, kp, s, true);
        case GBSPH_STAGE_DENSITY: return st_density_exact(h, kp, s);
        case GBSPH_STAGE_FORCES: return st_forces_exact(h, kp, s);
        case GBSPH_STAGE_CLIP_BOX:
        case GBSPH_STAGE_INTEGRATE_FORCE:
        case GBSPH_STAGE_GRAVITY:
        case GBSPH_STAGE_INTEGRATE_VELOCITY: return st_post(h, kp, stage, s);
        default: return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "unknown stage");
    }
}

GBSPH_API int gbsph_fluid3d_emit(gbsph_fluid3d_t h, uint32_t emit, float emit_speed, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!h->compiled) return fail(&h->last_error, GBSPH_ERR_NOT_COMPILED, "emit before compile()");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    k_emitter<<<grid1((uint32_t)h->n), 256, 0, (cudaStream_t)stream>>>(P4(h, 0), P4(h, 1), (uint32_t)h->n, emit,
                                                                        emit_speed, h->params.particleRadius);
    GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_get_cell_bounds(gbsph_fluid3d_t h, uint32_t* cell_start, uint32_t* cell_end,
                                            size_t n_cells, void* stream) {
    if (!h) return GBSPH_ERR_ARGUMENT;
    if (!cell_start || !cell_end) return fail(&h->last_error, GBSPH_ERR_ARGUMENT, "null pointer");
    GBSPH_CUDA_TRY(&h->last_error, cudaSetDevice(h->device));
    cudaStream_t s = (cudaStream_t)stream;
    if (h->params.keyMode == GBSPH_KEY_LINEAR_GRID) {
        if (n_cells != h->table_cells || !h->table)
            return fail(&h->last_error, GBSPH_ERR_SIZE_MISMATCH, "n_cells must equal the grid's cell count");
        k_table_split<<<(unsigned)((n_cells + 255) / 256), 256, 0, s>>>(h->table, (uint32_t)n_cells, cell_start, cell_end);
        GBSPH_CUDA_TRY(&h->last_error, cudaGetLastError());
    } else {
        if (n_cells != REF_BUCKETS || !h->hash_tables)
            return fail(&h->last_error, GBSPH_ERR_SIZE_MISMATCH, "n_cells must be 262144");
        GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(cell_start, h->hash_tables, REF_BUCKETS * 4ull, cudaMemcpyDeviceToDevice, s));
        GBSPH_CUDA_TRY(&h->last_error, cudaMemcpyAsync(cell_end, h->hash_tables + REF_BUCKETS, REF_BUCKETS * 4ull, cudaMemcpyDeviceToDevice, s));
    }
    return GBSPH_OK;
}

GBSPH_API int gbsph_fluid3d_sync_status(gbsph_fluid3d_t h, void* stream) {
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

GBSPH_API const char* gbsph_fluid3d_last_error(gbsph_fluid3d_t h) { return h ? h->last_error.c_str() : "null handle"; }

}  // extern "C"
