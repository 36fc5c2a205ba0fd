/*
 * gbsph.h -- C ABI of the GB300 (sm_103a) SPH fluid step and the stable radix sort it uses.
 *
 * Every entry point takes plain pointers, sizes and an opaque CUDA stream (`void*`, a
 * cudaStream_t; NULL = the legacy default stream). Device pointers are CUDA device
 * addresses on the handle's device. Status codes are ints: 0 = success, negative = error.
 * No C++ exceptions cross this boundary. Handles are independent (no global mutable state
 * apart from the optional log sink), and each handle must be used from one host thread at
 * a time.
 *
 * The reference interface each entry point replaces is cited as `libCL/<file>:<line>`
 * (jochenstier/libcl, an OpenCL 1.x library).
 */
#ifndef GBSPH_H
#define GBSPH_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define GBSPH_API __attribute__((visibility("default")))
#else
#define GBSPH_API
#endif

/* ------------------------------------------------------------------------------------------
 * Status codes. Replace the reference's int/bool returns plus the global `sStatusCL`
 * (libCL/oclCommon.cpp:19, libCL/oclCommon.h:36-38).
 * ---------------------------------------------------------------------------------------- */
enum {
    GBSPH_OK = 0,
    GBSPH_ERR_ARGUMENT = -1,        /* null handle/pointer, bad enum, NaN parameter */
    GBSPH_ERR_SIZE_MISMATCH = -2,   /* key/value counts differ, borrowed buffer too small */
    GBSPH_ERR_TOO_LARGE = -3,       /* element count beyond what the kernels address */
    GBSPH_ERR_BIT_RANGE = -4,       /* (end_bit - start_bit) not a multiple of 4, or outside [0,32] */
    GBSPH_ERR_CUDA = -5,            /* a CUDA runtime call failed; see *_last_error() */
    GBSPH_ERR_DEVICE_TIMEOUT = -6,  /* a bounded device-side wait (look-back, mbarrier, grid
                                       barrier) gave up */
    GBSPH_ERR_NOT_COMPILED = -7,    /* compute() before compile() */
    GBSPH_ERR_OUT_OF_MEMORY = -8,
    GBSPH_ERR_DEVICE_RANGE = -9,    /* a key/cell index fell outside its table on the device */
    GBSPH_ERR_STATE = -10           /* call not valid in the current state */
};

/* Human-readable name of a status code (static storage). */
GBSPH_API const char* gbsph_status_string(int status);

/* Failure-detection self-test (no counterpart in the reference). Runs, on the current device,
 * a wait that nothing will complete and reports what the bound made of it:
 *   which = 0: a one-sweep sort pass whose first tile never runs (its tile counter starts at
 *              1), so the next tile's decoupled look-back waits on a status word nobody
 *              writes;
 *   which = 1: a kernel that waits on a shared-memory mbarrier expecting bytes that no copy
 *              delivers;
 *   which = 2: the pass of which = 0 run inside the allocation-free sort's static array: it
 *              returns without synchronising, and gbsph_radix_sort_noalloc_status reports
 *              the timeout;
 *   which = 3: two CTAs at the persistent batch step's grid-wide barrier, counting on a
 *              third CTA that does not exist.
 * Each wait gives up after about one second, sets its device error bit and the kernel ends;
 * for which = 0, 1 and 3 the call synchronises `stream` and returns GBSPH_ERR_DEVICE_TIMEOUT if
 * that happened (and the context stays usable), GBSPH_OK if the wait somehow completed, or
 * an argument/CUDA error. */
GBSPH_API int gbsph_selftest_bounded_wait(int which, void* stream);

/* ABI version: major*10000 + minor*100 + patch. */
GBSPH_API int gbsph_version(void);

/* Log sink. Replaces the reference's replaceable `ERR/WARN/INFO/KERNEL` function pointers
 * (libCL/oclCommon.h:40-44, libCL/oclCommon.cpp:82-85). level: 0=ERR 1=WARN 2=INFO. */
typedef void (*gbsph_log_fn)(int level, const char* message, void* user);
GBSPH_API void gbsph_set_logger(gbsph_log_fn fn, void* user);

/* ------------------------------------------------------------------------------------------
 * Radix sort. Replaces `oclRadixSort` (libCL/sort/oclRadixSort.h:22-49):
 *   oclRadixSort(oclContext&, oclProgram* parent)        -> gbsph_radix_sort_create
 *   int compute(oclDevice&, oclBuffer& key, oclBuffer& val, int startBit, int endBit)
 *                                                         -> gbsph_radix_sort_compute
 *                                          (libCL/sort/oclRadixSort.cpp:62-144)
 * Semantics kept: a stable LSD sort of (uint32 key, uint32 value) pairs on key bits
 * [start_bit, end_bit), in place; key and value counts must match; (end_bit - start_bit)
 * must be a multiple of 4. Deviation: the reference rejects n >= 4,194,304
 * (libCL/sort/oclRadixSort.cpp:24,70-74); this sort accepts n < 2^30.
 * The handle owns temporary buffers that grow to the largest n seen (the reference's
 * `fit()`, libCL/sort/oclRadixSort.cpp:50-59).
 * ---------------------------------------------------------------------------------------- */
typedef struct gbsph_radix_sort_s* gbsph_radix_sort_t;

GBSPH_API int gbsph_radix_sort_create(gbsph_radix_sort_t* out);
GBSPH_API int gbsph_radix_sort_destroy(gbsph_radix_sort_t h);
GBSPH_API int gbsph_radix_sort_compute(gbsph_radix_sort_t h, uint32_t* keys, uint32_t* values,
                                       size_t n_keys, size_t n_values, int start_bit,
                                       int end_bit, void* stream);
/* Cell start/end extraction over sorted keys: fills both tables with 0xFFFFFFFF, then
 * cell_start[k] = first index of key k, cell_end[k] = one past its last index.
 * Replaces the fill + `clFindBounds` pair (libCL/phys/oclFluid3D.cpp:309-315,
 * libCL/phys/oclFluid3D.cl:85-113). Keys >= n_cells are skipped on the device and reported
 * as GBSPH_ERR_DEVICE_RANGE by gbsph_radix_sort_sync_status. */
GBSPH_API int gbsph_radix_sort_cell_bounds(gbsph_radix_sort_t h, const uint32_t* sorted_keys,
                                           size_t n, uint32_t* cell_start, uint32_t* cell_end,
                                           size_t n_cells, void* stream);
/* Synchronises `stream`, then reports (and clears) the handle's device-side error word. */
GBSPH_API int gbsph_radix_sort_sync_status(gbsph_radix_sort_t h, void* stream);
GBSPH_API const char* gbsph_radix_sort_last_error(gbsph_radix_sort_t h);

/* Allocation-free sort (no counterpart in the reference): the same stable in-place sort as
 * gbsph_radix_sort_compute for callers that cannot allocate device memory (a host framework
 * that owns all device memory through its own allocator, real-time loops that must not stall
 * on cudaMalloc/cudaFree, plugins with a fixed memory footprint). Its scratch is a static
 * device array of about 5 MB that every GPU loading the library holds until exit.
 * Limits: at most 262,144 pairs (GBSPH_ERR_TOO_LARGE beyond); the first call on a device
 * looks up the array's address, so make it before any stream capture, and do not reset the
 * device (cudaDeviceReset) afterwards in the same process; all calls share the array, so
 * calls that overlap on the GPU race. A device-side fault (a look-back wait that ran out)
 * leaves the output undefined and is recorded in the array's error word until
 * gbsph_radix_sort_noalloc_status reads it. */
GBSPH_API int gbsph_radix_sort_noalloc(uint32_t* keys, uint32_t* values, size_t n_keys,
                                       size_t n_values, int start_bit, int end_bit, void* stream);
/* Status of the allocation-free sort (no counterpart in the reference): synchronises
 * `stream`, then returns GBSPH_OK if no gbsph_radix_sort_noalloc call on the current device
 * recorded a device-side fault since the last read, else that fault's status
 * (GBSPH_ERR_DEVICE_TIMEOUT, GBSPH_ERR_STATE), and clears the record. Allocates nothing. */
GBSPH_API int gbsph_radix_sort_noalloc_status(void* stream);

/* ------------------------------------------------------------------------------------------
 * 3D SPH fluid. Replaces `oclFluid3D` (libCL/phys/oclFluid3D.h:21-123,
 * libCL/phys/oclFluid3D.cpp:21-342).
 * ---------------------------------------------------------------------------------------- */

/* Key modes. REFERENCE_HASH reproduces `hashKey` (libCL/phys/oclFluid3D.cl:44-52): the
 * Teschner XOR hash of the integer cell, modulo 262144 buckets, including the double visits
 * of colliding buckets in the 27-cell loops. LINEAR_GRID keys a bounded grid as
 * x + nx*(y + ny*z) with cell coordinates clamped to the grid (no collisions). */
enum { GBSPH_KEY_REFERENCE_HASH = 0, GBSPH_KEY_LINEAR_GRID = 1 };

/* Mirrors `oclFluid3D::Params` (libCL/phys/oclFluid3D.h:48-63) field for field, followed by
 * the values the reference hard-codes as kernel arguments (gravity, clip box:
 * libCL/phys/oclFluid3D.cpp:256-268) and the key-grid description. */
typedef struct gbsph_fluid3d_params {
    float deltaTime;
    float particleRadius;
    float cellSize;
    float mass;
    float viscosity;
    float pressure;
    float density;
    float spacing;
    float stiffness;
    float viscosityConstant;
    float pressureConstant;
    float kernelConstant;
    float velocitylimit;
    /* extensions (not in the reference struct) */
    float gravity[4];    /* value the gravity stage writes into every force; the reference
                            writes -9.8f * (0,0,1,0) */
    float boxMin[4];     /* clip box, reference: (-1,-1,-1,0) */
    float boxMax[4];     /* clip box, reference: ( 1, 1, 1,0) */
    float gridOrigin[4]; /* LINEAR_GRID: cell = floor((pos - origin) / cellSize) */
    int32_t gridDim[4];  /* LINEAR_GRID: nx, ny, nz (w unused) */
    int32_t keyMode;     /* GBSPH_KEY_* */
    int32_t dims;        /* 3 (default) or 2: 9 neighbour cells, z ignored, x/y walls only */
    int32_t reserved[2];
} gbsph_fluid3d_params;

/* Buffers, by role. Position/velocity/force are float4[N] in particle order (settable,
 * `setPositionBuffer` etc., libCL/phys/oclFluid3D.cpp:131-165). The sorted buffers are
 * float4[N] in cell order: after compute(), sorted position .w = density and sorted
 * velocity .w = pressure (libCL/phys/oclFluid3D.cl:192-198). INDEX maps sorted slot ->
 * particle (uint32[N]); CELL holds the sorted keys (uint32[N]). */
enum {
    GBSPH_BUF_POSITION = 0,
    GBSPH_BUF_VELOCITY = 1,
    GBSPH_BUF_FORCE = 2,
    GBSPH_BUF_SORTED_POSITION = 3,
    GBSPH_BUF_SORTED_VELOCITY = 4,
    GBSPH_BUF_INDEX = 5,
    GBSPH_BUF_CELL = 6,
    GBSPH_BUF_PARAMS = 7  /* one gbsph_fluid3d_params record on the device (getParamBuffer) */
};

/* Stages of one step, in the order `oclFluid3D::compute` enqueues them
 * (libCL/phys/oclFluid3D.cpp:293-342). Each can be run alone through gbsph_fluid3d_stage;
 * an integrate hook typically runs the last four itself. */
enum {
    GBSPH_STAGE_HASH = 0,               /* clHash */
    GBSPH_STAGE_SORT = 1,               /* oclRadixSort::compute(cell, index, 0, 24) */
    GBSPH_STAGE_REORDER = 2,            /* clReorder */
    GBSPH_STAGE_BOUNDS = 3,             /* fill 0xFFFFFFFF + clFindBounds */
    GBSPH_STAGE_DENSITY = 4,            /* clCalculateDensity */
    GBSPH_STAGE_FORCES = 5,             /* clCalculateForces */
    GBSPH_STAGE_CLIP_BOX = 6,           /* clClipBox */
    GBSPH_STAGE_INTEGRATE_FORCE = 7,    /* clIntegrateForce */
    GBSPH_STAGE_GRAVITY = 8,            /* clGravity */
    GBSPH_STAGE_INTEGRATE_VELOCITY = 9  /* clIntegrateVelocity */
};

/* Options (gbsph_fluid3d_set_option). */
enum {
    GBSPH_OPT_FUSED = 0,      /* 1 (default): fused kernels; 0: one kernel per reference stage */
    GBSPH_OPT_CUDA_GRAPH = 1, /* 1 (default): replay the step as a captured CUDA graph */
    GBSPH_OPT_BRICK_WIDTH = 2, /* LINEAR_GRID neighbour bricks: cells per brick along x (1..16) */
    GBSPH_OPT_PROFILE = 3,     /* 1: compute() runs eagerly and records a CUDA event pair per
                                  stage (the reference's CL_QUEUE_PROFILING_ENABLE events,
                                  libCL/oclDevice.cpp:31, libCL/oclKernel.cpp:162-202) */
    GBSPH_OPT_RADIX_BITS = 4,  /* batches: key bits sorted per radix pass (5..8, default 8; at
                                  most four passes over the batch's key width) */
    GBSPH_OPT_SORT_TILE = 5,   /* batches: keys per thread of a sort tile (8 or 16; 0, the
                                  default: 8 up to 2^21 keys, else 16) */
    GBSPH_OPT_PERSISTENT = 6   /* batches: 1 = the whole step (hash, sort passes, cell bounds,
                                  density, forces and integration) as one cooperative kernel
                                  whose CTAs stay resident and meet at grid-wide barriers;
                                  0 (default) = one kernel per stage, replayed as a graph */
};

typedef struct gbsph_fluid3d_s* gbsph_fluid3d_t;

/* Called by compute() in place of the clip/integrate stages when set. Replaces
 * `addEventHandler(srtEvent&)` with `EVT_INTEGRATE` (libCL/phys/oclFluid3D.h:69-70,
 * libCL/phys/oclFluid3D.cpp:287-291,325-328). Return 0 on success. */
typedef int (*gbsph_fluid3d_hook_fn)(gbsph_fluid3d_t h, void* stream, void* user);

/* oclFluid3D(oclContext&, oclProgram*) -- libCL/phys/oclFluid3D.cpp:21-83. Allocates
 * zeroed float4 buffers for the default 256 particles on the current CUDA device. */
GBSPH_API int gbsph_fluid3d_create(gbsph_fluid3d_t* out);
/* ~oclFluid3D -- libCL/phys/oclFluid3D.cpp:85-90. Frees owned buffers only. */
GBSPH_API int gbsph_fluid3d_destroy(gbsph_fluid3d_t h);
/* compile() -- libCL/phys/oclFluid3D.cpp:273-285: loads the default parameters of
 * `clInitFluid` (libCL/phys/oclFluid3D.cl:130-148). */
GBSPH_API int gbsph_fluid3d_compile(gbsph_fluid3d_t h);
/* setParticleCount -- libCL/phys/oclFluid3D.cpp:92-124. Re-creates owned buffers (contents
 * are lost, zero-filled). A borrowed buffer smaller than n is an error (it cannot be
 * resized here). */
GBSPH_API int gbsph_fluid3d_set_particle_count(gbsph_fluid3d_t h, size_t n);
/* getParticleCount -- libCL/phys/oclFluid3D.cpp:126-129. */
GBSPH_API size_t gbsph_fluid3d_get_particle_count(gbsph_fluid3d_t h);
/* setPositionBuffer / setVelocityBuffer / setForceBuffer -- libCL/phys/oclFluid3D.cpp:131-165.
 * `device_ptr` is borrowed (never freed). Position needs count == N, velocity/force
 * count >= N. Only POSITION, VELOCITY and FORCE are settable. */
GBSPH_API int gbsph_fluid3d_set_buffer(gbsph_fluid3d_t h, int which, void* device_ptr,
                                       size_t count);
/* get*Buffer -- libCL/phys/oclFluid3D.cpp:171-201. Returns the device pointer, or NULL.
 * GBSPH_BUF_PARAMS is getParamBuffer (libCL/phys/oclFluid3D.cpp:198-201, a device buffer
 * over the host Params, libCL/phys/oclFluid3D.cpp:58): one gbsph_fluid3d_params record
 * (count = 1) whose first 13 fields are the reference's `System` block, so kernels written
 * for it can bind it. The copy is brought up to date with the host struct by this call and,
 * on the step's stream, by every compute() and stage() whose parameters changed; kernels an
 * integrate hook enqueues see the parameters of the step that calls it. */
GBSPH_API void* gbsph_fluid3d_get_buffer(gbsph_fluid3d_t h, int which, size_t* count);
/* getParameters -- libCL/phys/oclFluid3D.cpp:204-207. Host-side struct, read at every
 * compute(); edit it in place. */
GBSPH_API gbsph_fluid3d_params* gbsph_fluid3d_get_params(gbsph_fluid3d_t h);
/* Recomputes kernelConstant, pressureConstant and viscosityConstant from cellSize and
 * viscosity with the formulas of `clInitFluid` (libCL/phys/oclFluid3D.cl:123-128,145-147)
 * when dims == 3; when dims == 2 it uses the 2D normalisations of the same kernels
 * (poly6 4/(pi h^8), spiky gradient 30/(pi h^5), viscosity Laplacian 40/(pi h^5)). */
GBSPH_API int gbsph_fluid3d_params_derive(gbsph_fluid3d_params* p);
/* Fills `p` with the defaults compile() loads: `clInitFluid` (libCL/phys/oclFluid3D.cl:130-148)
 * plus the reference's hard-coded gravity and clip box. Host only; needs no device. */
GBSPH_API int gbsph_fluid3d_default_params(gbsph_fluid3d_params* p);
GBSPH_API int gbsph_fluid3d_set_integrate_hook(gbsph_fluid3d_t h, gbsph_fluid3d_hook_fn fn,
                                               void* user);
GBSPH_API int gbsph_fluid3d_set_option(gbsph_fluid3d_t h, int option, int value);
/* compute(oclDevice&) -- libCL/phys/oclFluid3D.cpp:293-342. Asynchronous on `stream`. */
GBSPH_API int gbsph_fluid3d_compute(gbsph_fluid3d_t h, void* stream);
/* One step on state held in host memory, for callers that keep it there between steps (the
 * reference's users map position/velocity/force to the host around compute(), e.g.
 * libCL/TEST/main.cpp:222-236): the three float4[n] inputs are uploaded into the fluid's
 * position/velocity/force buffers, the step runs, and the three buffers are downloaded into
 * the outputs (which may be the inputs). With page-locked host memory the uploads of velocity
 * and force overlap the hash, sort and density passes, the force output (the gravity vector
 * in every entry when no integrate hook is set) is downloaded while the step computes, and the
 * whole is one replayed graph; pageable memory works too, without the overlap. The handle
 * keeps one extra float4[n] device array for the force output. Asynchronous on `stream`. */
GBSPH_API int gbsph_fluid3d_compute_host(gbsph_fluid3d_t h, const float* position_in, const float* velocity_in,
                                         const float* force_in, float* position_out, float* velocity_out,
                                         float* force_out, void* stream);
/* One reference stage alone (GBSPH_STAGE_*), asynchronous on `stream`. */
GBSPH_API int gbsph_fluid3d_stage(gbsph_fluid3d_t h, int stage, void* stream);
/* Copies the cell table out as two uint32 arrays of n_cells entries (device pointers),
 * 0xFFFFFFFF for empty cells, as `clFindBounds` leaves bfCellStart/bfCellEnd. n_cells is
 * 262144 in REFERENCE_HASH mode and nx*ny*nz in LINEAR_GRID mode. */
GBSPH_API int gbsph_fluid3d_get_cell_bounds(gbsph_fluid3d_t h, uint32_t* cell_start,
                                            uint32_t* cell_end, size_t n_cells, void* stream);
GBSPH_API int gbsph_fluid3d_sync_status(gbsph_fluid3d_t h, void* stream);
/* clEmitter (libCL/phys/oclFluid3D.cl:273-282; the reference's compute() does not enqueue
 * it): particles emit+1 .. emit+99 of the position/velocity buffers are placed on a sheet at
 * y = 0.6 (10 per row, 2 particleRadius apart) with velocity (0, emit_speed, 0). */
GBSPH_API int gbsph_fluid3d_emit(gbsph_fluid3d_t h, uint32_t emit, float emit_speed, void* stream);
/* With GBSPH_OPT_PROFILE on: waits for the last profiled compute() and writes the duration
 * in milliseconds of each of its stages (front end = scratch clear + hash, sort passes incl.
 * the fused reorder, cell bounds, density, forces + integration) into ms[0..4]. Returns the
 * number of stages written (5) or a negative status. Replaces oclKernel::getStartTime /
 * getEndTime (libCL/oclKernel.cpp:167-202). */
GBSPH_API int gbsph_fluid3d_stage_times(gbsph_fluid3d_t h, float* ms, int max_stages);
GBSPH_API const char* gbsph_fluid3d_last_error(gbsph_fluid3d_t h);

/* ------------------------------------------------------------------------------------------
 * Batched 3D scenes (no counterpart in the reference, which advances one oclFluid3D per
 * compute()): many independent LINEAR_GRID scenes of uneven particle counts, each with its own
 * gas constant, viscosity, clip box and grid, advanced together by one launch per stage of the
 * step (hash, sort passes, bounds, density, forces + integration), replayed as one CUDA graph.
 * Scene s owns particles [first_s, first_s + n_s) of the concatenated float4 arrays (in the
 * order the scenes were given) and never interacts with another scene.
 * ---------------------------------------------------------------------------------------- */
typedef struct gbsph_scene3d_desc {
    uint32_t n_particles;
    float stiffness;      /* gas constant k of p = p0 + k (rho - rho0) */
    float viscosity;      /* mu; the viscosity constant is mu * 45 / (pi h^6) */
    float boxMin[3];
    float boxMax[3];
    float gridOrigin[3];
    int32_t gridDim[3];
} gbsph_scene3d_desc;

typedef struct gbsph_batch3d_s* gbsph_batch3d_t;

GBSPH_API int gbsph_batch3d_create(gbsph_batch3d_t* out);
GBSPH_API int gbsph_batch3d_destroy(gbsph_batch3d_t h);
/* Defines the scenes. `shared` supplies deltaTime, particleRadius, cellSize, mass, pressure,
 * density, kernelConstant, pressureConstant, velocitylimit, gravity and dims (3); stiffness,
 * viscosity, box and grid come from each scene. Allocates every buffer (zeroed). */
GBSPH_API int gbsph_batch3d_set_scenes(gbsph_batch3d_t h, const gbsph_fluid3d_params* shared,
                                       const gbsph_scene3d_desc* scenes, int n_scenes);
/* Concatenated buffers (GBSPH_BUF_*), `count` = total particles. */
GBSPH_API void* gbsph_batch3d_get_buffer(gbsph_batch3d_t h, int which, size_t* count);
/* First particle and particle count of scene `s`. */
GBSPH_API int gbsph_batch3d_scene_range(gbsph_batch3d_t h, int s, size_t* first, size_t* count);
/* GBSPH_OPT_CUDA_GRAPH, GBSPH_OPT_BRICK_WIDTH, GBSPH_OPT_RADIX_BITS, GBSPH_OPT_SORT_TILE,
 * GBSPH_OPT_PERSISTENT. A digit width that needs more than four passes over the batch's
 * keys is refused by compute() (GBSPH_ERR_ARGUMENT). */
GBSPH_API int gbsph_batch3d_set_option(gbsph_batch3d_t h, int option, int value);
/* Current value of one of the options above. */
GBSPH_API int gbsph_batch3d_get_option(gbsph_batch3d_t h, int option, int* value);
/* One step of every scene, asynchronous on `stream`. */
GBSPH_API int gbsph_batch3d_compute(gbsph_batch3d_t h, void* stream);
/* Times the step on the current state (which is saved and restored) for every combination
 * of brick width (4, 8, 16), sort digit width (6, 7, 8 bits, where four passes cover the
 * keys), sort tile (8 or 16 keys per thread) and step form (staged graph or persistent
 * kernel), keeps the fastest and returns its brick width through best_width (the others
 * through gbsph_batch3d_get_option). Synchronises `stream`. */
GBSPH_API int gbsph_batch3d_autotune(gbsph_batch3d_t h, void* stream, int* best_width);
GBSPH_API int gbsph_batch3d_sync_status(gbsph_batch3d_t h, void* stream);
GBSPH_API const char* gbsph_batch3d_last_error(gbsph_batch3d_t h);

/* ------------------------------------------------------------------------------------------
 * 2D SPH fluid: the reference's double-density relaxation model with an image-sampled wall
 * field. Replaces `oclFluid2D` (libCL/phys/oclFluid2D.h:22-138, libCL/phys/oclFluid2D.cpp:18-362,
 * libCL/phys/oclFluid2D.cl:14-443). The step is clAdvanceState -> clHash -> sort bits [0,24) ->
 * clReorder -> clInitBounds -> clFindBounds -> clComputePressure -> clComputePosition ->
 * clUpdateState (libCL/phys/oclFluid2D.cpp:256-362). The wall field is two W x H RGBA images
 * stored with half-float precision (libCL/phys/oclFluid2D.cpp:72-75), sampled bilinearly with
 * normalised, clamp-to-edge coordinates; here they are float4 arrays whose values are rounded
 * to half precision when written. As in the reference, no integrate hook is called.
 * ---------------------------------------------------------------------------------------- */

/* oclFluid2D::Params (libCL/phys/oclFluid2D.h:42-60), field for field. */
typedef struct gbsph_fluid2d_params {
    float dT;
    float h;
    float containerW;
    float containerH;
    float cellSize;
    int32_t cellCountX;
    int32_t cellCountY;
    float particleSize;
    float particleMass;
    float p0; /* restDensity in the kernels' System struct */
    float vmax;
    float B;
} gbsph_fluid2d_params;

/* oclFluid2D::Particle (libCL/phys/oclFluid2D.h:62-69): 24 bytes. */
typedef struct gbsph_particle2d {
    float pos[2];
    float vel[2];
    float mass;
    float unused;
} gbsph_particle2d;

enum {
    GBSPH2D_BUF_STATE = 0,         /* gbsph_particle2d[N], particle order (settable) */
    GBSPH2D_BUF_SORTED_STATE = 1,  /* gbsph_particle2d[N], cell order */
    GBSPH2D_BUF_INDEX = 2,         /* uint32[N] sorted slot -> particle */
    GBSPH2D_BUF_CELL = 3,          /* uint32[N] sorted keys */
    GBSPH2D_BUF_PRESSURE = 4,      /* float4[N] (density, near density, pressure, near pressure), cell order */
    GBSPH2D_BUF_RELAXED = 5,       /* float2[N] relaxed positions, cell order */
    GBSPH2D_BUF_PREVIOUS = 6,      /* float2[N] positions before the step, particle order */
    GBSPH2D_BUF_BORDER_STATE = 7,  /* float4[W*H] wall (density, near density, pressure, near pressure) */
    GBSPH2D_BUF_BORDER_VECTOR = 8  /* float4[W*H] wall (normal x, normal y, distance, 0) */
};

typedef struct gbsph_fluid2d_s* gbsph_fluid2d_t;

/* oclFluid2D(oclContext&, oclProgram*) -- libCL/phys/oclFluid2D.cpp:18-85: 128*128 particles,
 * zeroed state, 256x256 zeroed wall images. */
GBSPH_API int gbsph_fluid2d_create(gbsph_fluid2d_t* out);
GBSPH_API int gbsph_fluid2d_destroy(gbsph_fluid2d_t h);
/* compile() -- libCL/phys/oclFluid2D.cpp:230-248: clInitFluid's defaults
 * (libCL/phys/oclFluid2D.cl:136-151) and a cell table of
 * (cellCountX*cellCountY/256 + 1)*256 entries. */
GBSPH_API int gbsph_fluid2d_compile(gbsph_fluid2d_t h);
/* Fills `p` with clInitFluid's defaults (host only). */
GBSPH_API int gbsph_fluid2d_default_params(gbsph_fluid2d_params* p);
/* setParticleCount -- libCL/phys/oclFluid2D.cpp:92-112. */
GBSPH_API int gbsph_fluid2d_set_particle_count(gbsph_fluid2d_t h, size_t n);
GBSPH_API size_t gbsph_fluid2d_get_particle_count(gbsph_fluid2d_t h);
/* setStateBuffer -- libCL/phys/oclFluid2D.cpp:119-129: borrowed gbsph_particle2d[count],
 * count must equal the particle count. */
GBSPH_API int gbsph_fluid2d_set_state_buffer(gbsph_fluid2d_t h, void* device_ptr, size_t count);
/* getStateBuffer and the internal buffers (GBSPH2D_BUF_*). */
GBSPH_API void* gbsph_fluid2d_get_buffer(gbsph_fluid2d_t h, int which, size_t* count);
/* getParameters -- libCL/phys/oclFluid2D.cpp:163-166. Read at every compute(). */
GBSPH_API gbsph_fluid2d_params* gbsph_fluid2d_get_params(gbsph_fluid2d_t h);
/* computeBorder(oclImage2D*) -- libCL/phys/oclFluid2D.cpp:131-146, clComputeBorder
 * (libCL/phys/oclFluid2D.cl:358-443): `mask` is a device float4[width*height] RGBA image whose
 * .w == 1.0 marks wall pixels; the wall images are resized to width x height. */
GBSPH_API int gbsph_fluid2d_compute_border(gbsph_fluid2d_t h, const float* mask, int width, int height,
                                           void* stream);
/* compute(oclDevice&) -- libCL/phys/oclFluid2D.cpp:256-362. */
GBSPH_API int gbsph_fluid2d_compute(gbsph_fluid2d_t h, void* stream);
/* clEmitter (libCL/phys/oclFluid2D.cl:342-352; the reference's compute() does not enqueue
 * it): particle emit + 1 is placed at x = 1 with velocity (25, 1). */
GBSPH_API int gbsph_fluid2d_emit(gbsph_fluid2d_t h, uint32_t emit, void* stream);
/* The cell table as two uint32 arrays of n_cells (= the compiled table size) entries. */
GBSPH_API int gbsph_fluid2d_get_cell_bounds(gbsph_fluid2d_t h, uint32_t* cell_start, uint32_t* cell_end,
                                            size_t n_cells, void* stream);
GBSPH_API int gbsph_fluid2d_sync_status(gbsph_fluid2d_t h, void* stream);
GBSPH_API const char* gbsph_fluid2d_last_error(gbsph_fluid2d_t h);

/* ------------------------------------------------------------------------------------------
 * Linear BVH over a triangle mesh. Replaces `oclBvhTrimesh` (libCL/geom/oclBvhTrimesh.h:20-84,
 * libCL/geom/oclBvhTrimesh.cpp:56-178), the reference's other user of the radix sort: global
 * box of the vertices -> 30-bit Morton key per triangle centroid -> 32-bit sort -> internal
 * nodes split at the highest differing key bit, linked to the nearer higher-bit neighbour ->
 * leaves -> boxes. The node layout is the reference's BVHNode (libCL/geom/oclBvhTrimesh.h:
 * 31-39): nodes [0, n-1) are internal (left/right children), nodes [n-1, 2n-1) are leaves
 * (left == right == 0, bit = triangle index), internal nodes end with trav = 2. As in the
 * reference, the global box starts at zero (so it contains the origin) and grows over
 * builds; it is never reset. Sorted keys that repeat make the reference's linking race; here
 * the largest claimant of a child slot wins and the build stays deterministic.
 * ---------------------------------------------------------------------------------------- */
typedef struct gbsph_bvh_node {
    float bbMin[4];
    float bbMax[4];
    int32_t left;
    int32_t right;
    uint32_t bit;
    uint32_t trav;
} gbsph_bvh_node;

typedef struct gbsph_bvh_s* gbsph_bvh_t;

/* oclBvhTrimesh(oclContext&, oclProgram* parent) -- libCL/geom/oclBvhTrimesh.cpp:21-47. */
GBSPH_API int gbsph_bvh_create(gbsph_bvh_t* out);
GBSPH_API int gbsph_bvh_destroy(gbsph_bvh_t h);
/* compute(oclDevice&, oclBuffer& vertex, oclBuffer& index) -- libCL/geom/oclBvhTrimesh.cpp:
 * 56-143: `vertex` is a device float4[n_vertices], `index` a device uint32[n_indices] (three
 * per triangle, n_indices / 3 >= 2 triangles). Asynchronous on `stream`. */
GBSPH_API int gbsph_bvh_compute(gbsph_bvh_t h, const float* vertex, size_t n_vertices, const uint32_t* index,
                                size_t n_indices, void* stream);
/* getNodeBuffer / getNodeCount -- libCL/geom/oclBvhTrimesh.cpp:167-175: device nodes
 * (2n - 1 of them after a build of n triangles). */
GBSPH_API gbsph_bvh_node* gbsph_bvh_get_node_buffer(gbsph_bvh_t h, size_t* count);
GBSPH_API size_t gbsph_bvh_get_node_count(gbsph_bvh_t h);
/* getRootNode -- libCL/geom/oclBvhTrimesh.cpp:162-165 (the reference reads it back after the
 * build): synchronises `stream` and returns the root's node index. */
GBSPH_API int gbsph_bvh_get_root_node(gbsph_bvh_t h, uint32_t* root, void* stream);
/* The accumulated global box (bfAABB, libCL/geom/oclBvhTrimesh.cpp:40): box8 = min xyzw,
 * max xyzw. Synchronises `stream`. */
GBSPH_API int gbsph_bvh_get_bounds(gbsph_bvh_t h, float* box8, void* stream);
/* Synchronises `stream`; reports (and clears) device-side errors: a triangle index outside
 * the vertex buffer gives GBSPH_ERR_DEVICE_RANGE. */
GBSPH_API int gbsph_bvh_sync_status(gbsph_bvh_t h, void* stream);
GBSPH_API const char* gbsph_bvh_last_error(gbsph_bvh_t h);
/* clCollideBVH (libCL/phys/oclFluid3D.cl:365-550; the reference's step does not enqueue it, a
 * caller adds it, e.g. from the integrate hook): per particle, a breadth-first walk of the
 * last built BVH (256-entry circular queue, boxes tested along the velocity ray) stops at the
 * first triangle the particle's next displacement crosses within particleRadius; that
 * particle's position, velocity and force (device float4[n_particles]) are then updated as
 * the reference does. Uses deltaTime, particleRadius, pressureConstant, density, cellSize and
 * mass of `params`; `vertex` / `index` are the mesh the BVH was built from. Reads the root
 * back (synchronises `stream` once), then runs asynchronously. */
GBSPH_API int gbsph_bvh_collide(gbsph_bvh_t h, const gbsph_fluid3d_params* params, float* position,
                                float* velocity, float* force, size_t n_particles, const float* vertex,
                                size_t n_vertices, const uint32_t* index, void* stream);

/* ------------------------------------------------------------------------------------------
 * Linear BVH over 2D line segments. Replaces `oclBvhLines` (libCL/geom/oclBvhLines.h:20-77,
 * libCL/geom/oclBvhLines.cpp:18-132), the 2D sibling of oclBvhTrimesh: Morton key of each
 * segment's midpoint taken directly as 16-bit integer coordinates (no global box) -> 32-bit
 * sort -> internal nodes split at the highest differing key bit (31..0), linked to the nearer
 * higher-bit neighbour -> leaves -> boxes. The node layout is the reference's 32-byte BVHNode
 * (libCL/geom/oclBvhLines.h:28-36): nodes [0, n-1) internal, nodes [n-1, 2n-1) leaves
 * (left == right == 0, bit = segment index); internal nodes end with trav = 3 (the reference's
 * second visitor swaps the first visitor's 2 for 3). Midpoint coordinates are converted to
 * integers by truncation; the reference leaves negative coordinates and coordinates of 2^32
 * or more undefined, here they become 0 and 0xFFFFFFFF. Repeated keys: as gbsph_bvh.
 * ---------------------------------------------------------------------------------------- */
typedef struct gbsph_bvh2d_node {
    float bbMin[2];
    float bbMax[2];
    int32_t left;
    int32_t right;
    uint32_t bit;
    uint32_t trav;
} gbsph_bvh2d_node;

typedef struct gbsph_bvh_lines_s* gbsph_bvh_lines_t;

/* oclBvhLines(oclContext&, oclProgram* parent) -- libCL/geom/oclBvhLines.cpp:18-42. */
GBSPH_API int gbsph_bvh_lines_create(gbsph_bvh_lines_t* out);
GBSPH_API int gbsph_bvh_lines_destroy(gbsph_bvh_lines_t h);
/* compute(oclDevice&, oclBuffer& vertex) -- libCL/geom/oclBvhLines.cpp:48-115: `vertex` is a
 * device float2[n_vertices], two per segment (n_vertices / 2 >= 2 segments; an odd last
 * vertex is ignored, as the reference's integer division does). Asynchronous on `stream`. */
GBSPH_API int gbsph_bvh_lines_compute(gbsph_bvh_lines_t h, const float* vertex, size_t n_vertices, void* stream);
/* getNodeBuffer / getNodeCount -- libCL/geom/oclBvhLines.cpp:123-131. */
GBSPH_API gbsph_bvh2d_node* gbsph_bvh_lines_get_node_buffer(gbsph_bvh_lines_t h, size_t* count);
GBSPH_API size_t gbsph_bvh_lines_get_node_count(gbsph_bvh_lines_t h);
/* getRootNode -- libCL/geom/oclBvhLines.cpp:118-121: synchronises `stream`. */
GBSPH_API int gbsph_bvh_lines_get_root_node(gbsph_bvh_lines_t h, uint32_t* root, void* stream);
/* Synchronises `stream` and reports (and clears) device-side errors. */
GBSPH_API int gbsph_bvh_lines_sync_status(gbsph_bvh_lines_t h, void* stream);
GBSPH_API const char* gbsph_bvh_lines_last_error(gbsph_bvh_lines_t h);

/* ------------------------------------------------------------------------------------------
 * Adjoint of the 3D step (no counterpart in the reference, which has no derivatives):
 * reverse-mode gradients of a loss on the state after `steps` gbsph_fluid3d_compute() calls
 * with respect to the initial positions and velocities, the gas constant (stiffness) and the
 * viscosity. The sort permutation and neighbour sets of each step are held fixed (the integer
 * sort is not differentiated); the count > 2, max(1, rho), velocity clamp and wall branches are
 * differentiated on the side the forward step took. Memory: a checkpoint (position, velocity,
 * force) every `checkpoint_every` steps; backward() recomputes one segment at a time from its
 * checkpoint, recording 316 bytes per particle per step of that segment (sorted state, force,
 * permutation, keys and the density pass's neighbour list of up to 64 entries).
 * Requires keyMode GBSPH_KEY_LINEAR_GRID, dims 3 and no integrate hook.
 * ---------------------------------------------------------------------------------------- */
typedef struct gbsph_adjoint3d_s* gbsph_adjoint3d_t;

/* Sized for the fluid's current particle count; the fluid must outlive the adjoint. */
GBSPH_API int gbsph_adjoint3d_create(gbsph_adjoint3d_t* out, gbsph_fluid3d_t fluid, uint32_t steps,
                                     uint32_t checkpoint_every);
GBSPH_API int gbsph_adjoint3d_destroy(gbsph_adjoint3d_t a);
/* Advances the fluid `steps` steps from its current state (exactly `steps` compute() calls),
 * keeping the checkpoints. Asynchronous on `stream`. */
GBSPH_API int gbsph_adjoint3d_forward(gbsph_adjoint3d_t a, void* stream);
/* After forward(), with the fluid's parameters unchanged: given device float4[n] dL/dposition
 * and dL/dvelocity of the final state (.w ignored; grad_velocity may be NULL for zero), writes
 * dL/dposition and dL/dvelocity of the initial state (float4[n], .w = 0; either may be NULL)
 * and, if grad_params is not NULL, the device doubles grad_params[0] = dL/dstiffness and
 * grad_params[1] = dL/dviscosity. The fluid is left in the state forward() produced.
 * Asynchronous on `stream`. */
GBSPH_API int gbsph_adjoint3d_backward(gbsph_adjoint3d_t a, const float* grad_position,
                                       const float* grad_velocity, float* grad_position0,
                                       float* grad_velocity0, double* grad_params, void* stream);
GBSPH_API const char* gbsph_adjoint3d_last_error(gbsph_adjoint3d_t a);

#ifdef __cplusplus
}
#endif

#endif /* GBSPH_H */
