/*
 * nbody_cuda -- C ABI of the GB300 (sm_103a) N-body solver.
 *
 * This is the device layer a CUDA solver variant of stett/nbody binds. It stands where
 * the Vulkan device layer stands for the reference's GPU variants (source/gpu.h:72-353):
 * the reference's Solver implementations (source/solvers/gpu_solver*.h) call
 * GpuDevice::{reserve_bodies, map_bodies, step, accelerate, integrate, download}; the
 * CUDA solver (nbody_gb300/host/cuda_solver.h) calls the functions below instead.
 *
 * Conventions
 *   - Plain C: no exceptions cross this boundary; every call returns an nbody_status and
 *     nbody_cuda_last_error() describes the most recent failure on a context.
 *   - Host memory is caller-owned. Device memory belongs to the context, except for the
 *     nbody_cuda_dev_* entry points, which work on caller-owned device buffers.
 *   - Body records are the reference's 48-byte Body (include/nbody/body.h:6-19):
 *       float pos[3], radius, vel[3], mass, acc[3], pad.
 *     The split layout is the reference's three 16-byte streams (source/gpu.h:32-48):
 *       pos_mass {x, y, z, m}, vel_radius {vx, vy, vz, r}, acc {ax, ay, az, 0}.
 *   - One context is used from one host thread at a time (the reference's Sim is
 *     single-threaded, source/sim.cpp:86-90). Work is queued on the context's stream and
 *     only synchronised where a result must reach the host.
 */
#ifndef NBODY_CUDA_H
#define NBODY_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NBODY_CUDA_ABI_VERSION 1

typedef enum nbody_status
{
    NBODY_OK = 0,
    NBODY_ERR_INVALID = 1,      /* a bad argument; nothing was queued */
    NBODY_ERR_NO_DEVICE = 2,    /* no usable CUDA device */
    NBODY_ERR_CUDA = 3,         /* a CUDA runtime call failed */
    NBODY_ERR_ALLOC = 4,        /* device or pinned host allocation failed */
    NBODY_ERR_TIMEOUT = 5,      /* a bounded device-side wait gave up */
    NBODY_ERR_UNSUPPORTED = 6   /* a parameter combination this build does not provide */
} nbody_status;

/* Force summation mode; mirrors nbody::Mode (source/gpu.h:13). */
typedef enum nbody_mode
{
    NBODY_MODE_N2 = 0,          /* direct summation (the reference's brute force) */
    NBODY_MODE_NLOGN = 1,       /* Barnes-Hut tree */
    NBODY_MODE_BATCHED = 2      /* direct summation within each system of the context's
                                   system table (nbody_cuda_set_systems); no reference
                                   counterpart */
} nbody_mode;

/* Force law. CUTOFF is the reference's (source/detail/physics.h:21-42): a pair
 * contributes nothing when |d|^2 <= radius_target^2, else G*m*d/|d|^3.
 * SOFTENED is G*m*d/(|d|^2 + eps2)^(3/2) and needs eps2 > 0. */
typedef enum nbody_law
{
    NBODY_LAW_CUTOFF = 0,
    NBODY_LAW_SOFTENED = 1
} nbody_law;

/* Arithmetic of the force sum and the integrator.
 * FP32: FP32 throughout (the reference's arithmetic).
 * COMPENSATED: FP32 pair forces; per-tile FP32 partials Kahan-summed, chunk partials
 *   summed in FP64; positions kept as an FP64 origin plus FP32 offsets with Kahan
 *   compensation of the position and velocity updates.
 * FP64: FP64 throughout (direct summation only). */
typedef enum nbody_precision
{
    NBODY_PREC_FP32 = 0,
    NBODY_PREC_COMPENSATED = 1,
    NBODY_PREC_FP64 = 2
} nbody_precision;

/* Barnes-Hut traversal (nbody_step_params.walk). No reference counterpart beyond TARGET. */
typedef enum nbody_walk
{
    NBODY_WALK_TARGET = 0,      /* every target decides every cell itself with the reference's
                                   opening test, and applies exactly the cells the reference's
                                   walk accepts for it (bhtree.cpp:97-138) */
    NBODY_WALK_GROUP = 1        /* one walk per group of Morton-consecutive targets: a cell is
                                   accepted for the whole group when the group's bounding box
                                   lies beyond the cell's opening distance, and the accepted
                                   cells and leaves form an interaction list applied to every
                                   target of the group. Each target's sum refines the set the
                                   reference accepts for it (at least as accurate, more
                                   interactions, far fewer instructions per interaction) */
} nbody_walk;

/* Device-side body layout of a context: the reference's two GPU layouts. */
typedef enum nbody_layout
{
    NBODY_LAYOUT_SOA = 0,       /* split streams, as GpuSolverSplit (gpu_solver_split.h) */
    NBODY_LAYOUT_AOS = 1        /* interleaved Body, as GpuSolver (gpu_solver.h) */
} nbody_layout;

/* Which streams a download brings back; mirrors nbody::Readback (source/gpu.h:52-58). */
enum
{
    NBODY_READ_POSITIONS = 1u << 0,     /* pos and mass */
    NBODY_READ_VELOCITIES = 1u << 1,    /* vel and radius */
    NBODY_READ_ACCELERATIONS = 1u << 2,
    NBODY_READ_ALL = 7u
};

/* Per-step parameters; the fields of nbody::PushConstants (source/gpu.h:17-27) that a
 * step reads, plus the law/precision selection the reference does not have. */
typedef struct nbody_step_params
{
    float dt;           /* time step */
    float theta;        /* Barnes-Hut opening parameter, reference convention:
                           a cell is accepted when |com - x|^2 > size^2 * theta^2 */
    float G;            /* gravitational constant (State::gravity) */
    float eps2;         /* softening length squared (SOFTENED law only) */
    float size;         /* world edge (State::size): wrap period and Barnes-Hut root box */
    int32_t wrap;       /* nonzero: wrap positions into [-size/2, size/2] (State::wrap) */
    int32_t mode;       /* nbody_mode */
    int32_t law;        /* nbody_law */
    int32_t precision;  /* nbody_precision */
    int32_t tree_box;   /* Barnes-Hut root box: 0 = the reference's, centred at the origin
                           with edge `size` (source/detail/tree.h:20); 1 = the smallest
                           power-of-two cube around the bodies (FP64 bounding box).
                           0 with size <= 0 behaves as 1. */
    int32_t walk;       /* nbody_walk (Barnes-Hut only); zero is the reference's per-target walk */
    int32_t reserved;   /* zero */
} nbody_step_params;

typedef struct nbody_cuda nbody_cuda;

/* --- device discovery and lifetime ------------------------------------------------- */

/* Probe for a usable sm_103 device without creating a context. Returns NBODY_OK, or a
 * status with the reason written to `why`. Replaces GpuDevice::probe (source/gpu.cpp:115-149). */
int nbody_cuda_probe(char* why, size_t why_len);

/* Create a context on the current CUDA device with the given body layout. Replaces
 * constructing GpuDevice (source/gpu.cpp, via Context::require_gpu, source/sim.cpp:129-136). */
int nbody_cuda_create(nbody_cuda** out, int layout);
void nbody_cuda_destroy(nbody_cuda* ctx);

/* Copy the description of the last failure on `ctx` (or of the last failed create when
 * ctx is NULL) into buf. Returns the status of that failure. */
int nbody_cuda_last_error(const nbody_cuda* ctx, char* buf, size_t len);

/* Queue work on `stream` (a cudaStream_t) instead of the context's own stream. NULL
 * restores the context's own stream. */
int nbody_cuda_set_stream(nbody_cuda* ctx, void* stream);
void* nbody_cuda_stream(const nbody_cuda* ctx);
int nbody_cuda_layout(const nbody_cuda* ctx);

/* --- bodies ---------------------------------------------------------------------------- */

/* Grow device storage to hold at least n bodies. Replaces GpuDevice::reserve_bodies. */
int nbody_cuda_reserve(nbody_cuda* ctx, size_t n);
size_t nbody_cuda_count(const nbody_cuda* ctx);

/* Replace the device bodies with n host Body records (48 B each). The device copy is
 * split or kept interleaved per the context layout. Replaces the upload half of
 * GpuSolverSplit::upload_bodies / GpuSolver::upload (gpu_solver_split.h:155-177). */
int nbody_cuda_upload_bodies(nbody_cuda* ctx, const void* bodies, size_t n);

/* Write the streams selected by `mask` into n host Body records; fields not selected
 * are left untouched. Reads min(n, count) bodies (gpu_solver_split.h:202). Synchronous.
 * Replaces GpuDevice::download + the re-interleave in materialize(). */
int nbody_cuda_download_bodies(nbody_cuda* ctx, void* bodies, size_t n, unsigned mask);

/* Split-stream transfers (16 B per body per stream); NULL pointers are skipped. */
int nbody_cuda_upload_soa(nbody_cuda* ctx, const float* pos_mass, const float* vel_radius,
                          const float* acc, size_t n);
int nbody_cuda_download_soa(nbody_cuda* ctx, float* pos_mass, float* vel_radius, float* acc,
                            size_t n);

/* --- host transfer policy -------------------------------------------------------------- */

/* How nbody_cuda_upload_bodies / download_bodies move Body records between the caller's
 * host array and the device streams. The reference always goes through mapped staging
 * allocations and a host-side (de)interleave (gpu_solver_split.h:155-177, 188-221). */
typedef enum nbody_transfer
{
    NBODY_TRANSFER_AUTO = 0,    /* DIRECT where the device reaches pageable host memory
                                   through the host's page tables (a coherent host link,
                                   as NVLink-C2C), else MAPPED */
    NBODY_TRANSFER_STAGED = 1,  /* (de)interleave on the device, copy engine to/from pinned
                                   staging, host copy to/from the caller's array */
    NBODY_TRANSFER_MAPPED = 2,  /* a kernel writes/reads the records in page-locked mapped
                                   staging directly (zero-copy), host copy to/from the caller */
    NBODY_TRANSFER_DIRECT = 3   /* a kernel writes/reads the caller's own array: no staging
                                   and no host copy. Needs pageable memory access */
} nbody_transfer;

/* Select the transfer path. DIRECT on a device without pageable memory access returns
 * NBODY_ERR_UNSUPPORTED and leaves the policy unchanged. No reference counterpart. */
int nbody_cuda_set_transfer(nbody_cuda* ctx, int policy);

/* The policy selected, the path AUTO resolves to, whether the device accesses pageable
 * host memory (0/1; 2 = through the host's page tables), and how many downloads were
 * served from a predicted readback. Any pointer may be NULL. */
int nbody_cuda_transfer_info(const nbody_cuda* ctx, int* policy, int* resolved, int* pageable,
                             uint64_t* readback_hits);

/* Predicted readback: queue, behind the work already on the stream, a copy of the
 * streams in `mask` into the context's mapped staging, so that a later
 * nbody_cuda_download_bodies asking for no more than `mask` only waits for that copy and
 * takes the records from host memory. Valid until a call changes the device bodies. When
 * the resolved path is DIRECT the call queues nothing: a download then writes the
 * caller's array straight from the device, which moves the same bytes once. Replaces the
 * Readback argument of GpuDevice::step (source/gpu.cpp:842-875) chosen by
 * GpuSolverSplit::wanted_readback (gpu_solver_split.h:122-132). */
int nbody_cuda_prefetch(nbody_cuda* ctx, unsigned mask);

/* --- scene generators (queued) ---------------------------------------------------------- */

/* util::DiskArgs (include/nbody/util.h) as a plain struct; the reference's defaults are
 * center 0, vel 0, axis (0, 0, 1), inner 0, outer 250, thickness 1, central mass 4.1e6
 * (nbody::sagittarius_mass), star mass 1 (nbody::solar_mass). */
typedef struct nbody_disk_args
{
    float center[3];
    float vel[3];
    float axis[3];
    float inner_radius;
    float outer_radius;
    float thickness;
    float central_mass;
    float star_mass;
} nbody_disk_args;

/* util::CubeArgs: center (unused by the reference's generator, as here), edge `size`
 * (default 500), vel, star mass. */
typedef struct nbody_cube_args
{
    float center[3];
    float size;
    float vel[3];
    float star_mass;
} nbody_cube_args;

/* Fill device bodies [begin, begin + num) as util::disk (source/util.cpp:14-96) fills the
 * range [begin, end): a central body and num - 1 stars with circular speeds, from the
 * reference's own random stream (std::default_random_engine, seed 1, through
 * uniform_real_distribution<float> and normal_distribution<float> as libstdc++ draws
 * them). begin must not exceed the body count; the count grows to begin + num when that
 * is larger. The speeds use the centre of mass and mass of the generated bodies, which is
 * what the reference's theta = 0.5 walk of its own tree (util.cpp:81-95) folds together
 * for every body, up to its float rounding. Replaces util::disk for a device solver. */
int nbody_cuda_scene_disk(nbody_cuda* ctx, const nbody_disk_args* args, size_t begin, size_t num);

/* Fill device bodies [begin, begin + num) as util::cube (source/util.cpp:98-126) does. */
int nbody_cuda_scene_cube(nbody_cuda* ctx, const nbody_cube_args* args, size_t begin, size_t num);

/* --- stepping (queued, asynchronous) --------------------------------------------------- */

/* Accelerations for every body. Replaces GpuDevice::accelerate (source/gpu.cpp:799-841). */
int nbody_cuda_accelerate(nbody_cuda* ctx, const nbody_step_params* p);
/* Semi-implicit Euler v += a*dt; x += v*dt; optional wrap (physics.h:60-70).
 * Replaces GpuDevice::integrate. */
int nbody_cuda_integrate(nbody_cuda* ctx, const nbody_step_params* p);
/* `steps` x (accelerate; integrate), fused where possible. Replaces GpuDevice::step
 * (source/gpu.cpp:842-875) and Solver::update (source/solver.h:59). */
int nbody_cuda_update(nbody_cuda* ctx, const nbody_step_params* p, int steps);
/* Wait for queued work; reports a device-side error (e.g. NBODY_ERR_TIMEOUT). */
int nbody_cuda_synchronize(nbody_cuda* ctx);

/* --- caller-owned device buffers (no context storage, no allocation by the call
 *     beyond the context's scratch) ------------------------------------------------------ */

/* Direct-sum accelerations over split streams already resident on the device:
 * pos_mass, vel_radius (radius read for the CUTOFF law only), acc out; n bodies. Each
 * stream the kernel reads must be 16-byte aligned (NBODY_ERR_INVALID otherwise).
 * The device twin of accelerate_split.comp N2 mode (shaders/accelerate_split.comp:9-18). */
int nbody_cuda_dev_accel_soa(nbody_cuda* ctx, const void* pos_mass, const void* vel_radius,
                             void* acc, size_t n, const nbody_step_params* p);
/* Same over interleaved 48-byte Body records (shaders/accelerate.comp:9-17); writes
 * Body::acc. */
int nbody_cuda_dev_accel_aos(nbody_cuda* ctx, void* bodies, size_t n,
                             const nbody_step_params* p);
/* Semi-implicit Euler over split streams (shaders/integrate_split.comp). */
int nbody_cuda_dev_integrate_soa(nbody_cuda* ctx, void* pos_mass, void* vel_radius,
                                 const void* acc, size_t n, const nbody_step_params* p);

/* Direct-sum accelerate over caller-owned device buffers that allocates nothing. It has
 * no counterpart in the reference. It is for callers that cannot let a library call
 * cudaMalloc: a renderer or engine frame loop that must not stall on the device-wide
 * synchronisation cudaMalloc/cudaFree imply, or a plugin whose host application owns
 * every device allocation and its budget.
 *
 * Inputs, outputs and results are those of nbody_cuda_dev_accel_soa (direct sum, FP32),
 * without a context. The scratch for the source split is a fixed 16 MiB array inside the
 * library, which every GPU that loads the library holds until the process exits. Hence
 * n <= 1048576; a larger n returns NBODY_ERR_INVALID. Work is queued on `stream` (a
 * cudaStream_t; NULL is the default stream) and waited for before the call returns;
 * NBODY_ERR_TIMEOUT reports a device-side wait that gave up. The call is synchronous:
 * it returns after the kernel has finished. The first call in each CUDA context (the
 * device's primary context, also after cudaDeviceReset re-creates it, or any context
 * the caller made current) looks up the array's device address (cudaGetSymbolAddress)
 * and caches it under that context's id; make that first call before any stream
 * capture. All calls share the one array and its error word, so calls that overlap on
 * the GPU (from other host threads or streams) race: the caller must serialise them.
 * Every pointer the kernel reads as float4 must be 16-byte aligned: pos_mass, acc, and
 * vel_radius under the CUTOFF law; otherwise NBODY_ERR_INVALID before any launch. */
int nbody_cuda_dev_accel_soa_noalloc(const void* pos_mass, const void* vel_radius, void* acc,
                                     size_t n, const nbody_step_params* p, void* stream);

/* --- Barnes-Hut introspection ----------------------------------------------------------- */

/* Statistics of the last Barnes-Hut accelerate: out[0] = force interactions (accepted
 * cells + bodies applied), out[1] = cells visited (summed over warps), out[2] = octree
 * cells built. Synchronous. */
int nbody_cuda_bh_stats(nbody_cuda* ctx, uint64_t out[3]);

/* Device time of the last Barnes-Hut accelerate's two stages, in milliseconds, from CUDA
 * events on the context's stream: ms[0] = the tree build (root box, Morton codes, sort,
 * cell sums, octree records), ms[1] = the traversal. NBODY_ERR_INVALID when no accelerate
 * has been timed (none yet, or the last one was captured into a CUDA graph, where no
 * events are recorded). Synchronous. No reference counterpart. */
int nbody_cuda_bh_stage_ms(nbody_cuda* ctx, float ms[2]);

/* Build the Barnes-Hut tree keys for the current bodies and copy back the Morton codes in
 * sorted order (codes, n entries), the sorted body order (order: the body index at each
 * sorted position; equal codes keep index order) and the root box (box: lower corner
 * xyz, edge). Any output may be NULL. Synchronous. No reference counterpart: the
 * reference inserts bodies one by one (source/bhtree.cpp:14-85). */
int nbody_cuda_morton(nbody_cuda* ctx, const nbody_step_params* p, uint64_t* codes,
                      uint32_t* order, double box[4]);

/* The tree of the last Barnes-Hut accelerate in the reference's node layout: 48-byte
 * bh::Node records (include/nbody/bhtree.h:13-22), root at index 0, 8 contiguous children
 * per split node with child q in the reference's octant order (bounds.h:31-38), threaded
 * `next` links, empty octants as massless leaves. Writes min(count, max_nodes) nodes (none
 * when nodes is NULL) and the total into *count. This is what Solver::tree() returns for a
 * tree-building variant (source/solvers/cpu_barnes_hut.h:46, sim.cpp:329-335). */
int nbody_cuda_tree_export(nbody_cuda* ctx, void* nodes, size_t max_nodes, size_t* count);

/* When a ray query stops (the visitor's answer in Tree::query). */
enum
{
    NBODY_QUERY_ALL = 0,            /* visit every node the ray meets */
    NBODY_QUERY_FIRST_BODY = 1      /* stop after the first met leaf that holds mass (picking) */
};

/* Tree::query (source/bhtree.cpp:153-173) for nrays rays at once. rays: 6 floats per ray,
 * origin xyz then direction xyz (nbody::Ray, include/nbody/ray.h). The tree is `count`
 * bh::Node records at `nodes` (any reference tree, e.g. Tree::nodes()), or, when nodes is
 * NULL, the context's last Barnes-Hut tree as nbody_cuda_tree_export gives it. Per ray the
 * walk visits, in the reference's order, the nodes whose bounds the ray meets
 * (Bounds::ray_intersect, bounds.h:64-133), descending into each met node. Past a node the
 * ray misses it moves to that node's `next`: the reference's loop stays on such a node
 * and never ends, so the two agree wherever the reference's walk ends. hits[r * max_hits
 * ...] receives ray r's first max_hits visited node indices and counts[r] how many it
 * visited. A malformed node array (a link out of range, a cycle) stops the walk and
 * returns NBODY_ERR_CUDA. Synchronous. */
int nbody_cuda_tree_query(nbody_cuda* ctx, const void* nodes, size_t count, const float* rays, size_t nrays,
                          int stop, uint32_t* hits, size_t max_hits, uint32_t* counts);

/* --- direct-sum kernel shapes ---------------------------------------------------------------- */

/* Number of instantiated direct-sum kernel shapes; describe one (targets per thread, threads
 * per CTA, *packed: 0 scalar FP32, 1 packed FP32x2, 2 packed with each source tile first
 * rewritten as ready-made operand pairs); pin one for this context (index < 0 returns to the
 * size-based choice). */
int nbody_cuda_direct_variant_count(void);
int nbody_cuda_direct_variant(int index, int* targets_per_thread, int* block, int* packed);
int nbody_cuda_set_direct_variant(nbody_cuda* ctx, int index);

/* Time every direct-sum kernel shape on the current bodies (FP32, p->law), pin the fastest
 * and return its index in *best; times_ms (optional, ntimes entries) receives each shape's
 * accelerate time. Synchronous. */
int nbody_cuda_direct_autotune(nbody_cuda* ctx, const nbody_step_params* p, double* times_ms,
                               size_t ntimes, int* best);

/* --- batched systems and graphs (no reference counterpart) ------------------------------- */

/* Declare the context's bodies to be nsys independent systems: system s owns bodies
 * [offsets[s], offsets[s+1]); offsets[0] = 0 and offsets[nsys] = the body count. Used by
 * NBODY_MODE_BATCHED (one persistent launch sums every system) and by the energy
 * diagnostics. Upload the concatenated bodies first. */
int nbody_cuda_set_systems(nbody_cuda* ctx, const int64_t* offsets, size_t nsys);

/* Time every batched kernel configuration (threads per CTA, targets per thread, sources
 * per chunk) on the current bodies and system table, keep the fastest for later batched
 * steps and return its index in *best; times_ms (optional, ntimes entries) receives each
 * configuration's accelerate time. Synchronous. */
int nbody_cuda_batch_autotune(nbody_cuda* ctx, const nbody_step_params* p, double* times_ms,
                              size_t ntimes, int* best);
/* Number of batched configurations; describe one (index < 0: the active one); pin one. */
int nbody_cuda_batch_config_count(void);
int nbody_cuda_batch_config(const nbody_cuda* ctx, int index, int* threads_per_cta,
                            int* targets_per_thread, int* sources_per_chunk);
int nbody_cuda_batch_set_config(nbody_cuda* ctx, int index);

/* FP64 diagnostics per system (one system covering every body when no table is set):
 * out[5*s + 0..4] = kinetic energy, potential energy (softened with eps2 when p->law is
 * SOFTENED, else unsoftened), momentum xyz. O(sum of N_s^2) FP64 work. Synchronous. */
int nbody_cuda_system_energy(nbody_cuda* ctx, const nbody_step_params* p, double* out, size_t nsys);

/* Energy and momentum of all bodies at the direct sum's rate, for runs too large for the
 * FP64 diagnostics above: out[0] = kinetic energy, out[1] = potential energy (softened
 * with eps2 under the SOFTENED law, else unsoftened), out[2..4] = momentum. Pair terms
 * are FP32 (rsqrt on the SFU), summed in FP32 over 256-source tiles whose sums are folded
 * exactly, per body in FP64, over each pair once; every total is an FP64 sum in a fixed
 * order, so the result is deterministic and the potential is within about 1e-7 of the FP64
 * one. Pairs at zero separation are left out. O(N^2 / 2) FP32 work. Synchronous. No
 * reference counterpart. */
int nbody_cuda_energy(nbody_cuda* ctx, const nbody_step_params* p, double out[5]);

/* `steps` x update, with one step captured as a CUDA graph and replayed: the first step
 * runs eagerly (it sets up every buffer), the step is captured once per parameter set,
 * body count, stream and buffer generation, and replayed for the remaining steps. Results
 * equal nbody_cuda_update's. The context's stream must not be the legacy default stream. */
int nbody_cuda_update_graph(nbody_cuda* ctx, const nbody_step_params* p, int steps);

/* --- precision forms --------------------------------------------------------------------- */

/* Direct-sum accelerations of the listed bodies only (targets[k] in [0, count)), against all
 * bodies, with p->precision COMPENSATED or FP64; results in FP64, 3 per target, before the
 * rounding to float that nbody_cuda_accelerate applies. Synchronous. For error statistics
 * on sampled targets at full size. No reference counterpart (the reference is FP32 only). */
int nbody_cuda_accel_sampled(nbody_cuda* ctx, const nbody_step_params* p, const int64_t* targets,
                             size_t nt, double* acc_out);

/* The FP64 origin of the split-precision state (xyz) and the power-of-two edge it was
 * aligned to; valid after a COMPENSATED or FP64 step. Synchronous. */
int nbody_cuda_split_origin(nbody_cuda* ctx, double out[4]);

/* --- introspection ------------------------------------------------------------------- */

/* Kernel launches this context queued since creation (all entry points). */
uint64_t nbody_cuda_launch_count(const nbody_cuda* ctx);
/* Last direct-sum launch shape: targets per thread, threads per block, source tile,
 * j-split count and grid size (for the bench's roofline arithmetic and for tests). */
int nbody_cuda_last_direct_config(const nbody_cuda* ctx, int* targets_per_thread,
                                  int* block, int* tile, int* jsplit, int* grid);

/* Measured FP32 multiply-add throughput of this device in TFLOP/s (2 flop per lane per
 * FFMA), scalar FFMA and packed FFMA2 chains; the denominator of the direct-sum
 * roofline. Synchronous; takes well under a second. */
int nbody_cuda_calibrate_fp32(nbody_cuda* ctx, double* tflops_scalar, double* tflops_packed);

/* Measured FP64 DFMA throughput in TFLOP/s (2 flop per DFMA); the denominator of the FP64
 * form's roofline. Synchronous. */
int nbody_cuda_calibrate_fp64(nbody_cuda* ctx, double* tflops);

/* Failure-path self-test: one kernel waits, with the same bounded wait every TMA pipeline
 * uses, on an mbarrier phase that nothing completes, and gives up after limit_ns
 * (at most 0.1 s). Returns NBODY_ERR_TIMEOUT -- the status a stuck copy would produce --
 * and leaves the context usable. No reference counterpart (its fence waits are unbounded,
 * source/gpu.cpp:780). Synchronous. */
int nbody_cuda_selftest_wait(nbody_cuda* ctx, uint64_t limit_ns);

#ifdef __cplusplus
}
#endif
#endif
