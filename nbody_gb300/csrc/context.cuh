// The nbody_cuda context (opaque in the C ABI) and the internal calls the translation
// units make on it.
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>
#include <cuda_runtime.h>

#include "nbody_cuda.h"
#include "direct.cuh"

namespace nbg
{
    struct BhState;         // bh.cu
    struct PreciseState;    // direct_precise.cu
    struct BatchState;      // batch.cu
}

struct nbody_cuda
{
    int layout = NBODY_LAYOUT_SOA;
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;

    // Bodies: live count and capacity (bodies), grow-only.
    size_t count = 0;
    size_t cap = 0;
    float4* pm = nullptr;       // SoA: {x, y, z, m}
    float4* vr = nullptr;       // SoA: {vx, vy, vz, radius}
    float4* acc = nullptr;      // SoA: {ax, ay, az, 0}
    float* bodies = nullptr;    // AoS: 12 floats per body

    // Device staging for interleaved transfers into a split context.
    float* aos_stage = nullptr;
    size_t aos_stage_cap = 0;

    // Kernel scratch (j-split partials, sort buffers, ...), grow-only.
    void* scratch = nullptr;
    size_t scratch_bytes = 0;
    int pending_partials = 0;   // >1: scratch holds this many accelerate partials
    float pending_G = 1.f;      // the G those partials are to be scaled by

    // Pinned host staging for pageable transfers.
    void* pinned = nullptr;
    size_t pinned_bytes = 0;
    cudaEvent_t pinned_event = nullptr;

    // Transfer paths (transfer.cu). `mapped` is page-locked host memory the kernels write
    // and read directly over the host link; it also holds the predicted readback, which is
    // current while `body_version` has not moved since it was enqueued.
    int transfer = NBODY_TRANSFER_AUTO;
    int pageable_access = 0;        // cudaDevAttrPageableMemoryAccess
    int pageable_host_tables = 0;   // cudaDevAttrPageableMemoryAccessUsesHostPageTables
    void* mapped = nullptr;
    void* mapped_dev = nullptr;
    size_t mapped_bytes = 0;
    cudaEvent_t mapped_event = nullptr;   // the last device access to `mapped`
    uint64_t body_version = 0;      // bumped by every call that may change the device bodies
    bool readback_valid = false;
    uint64_t readback_version = 0;
    size_t readback_count = 0;
    unsigned readback_mask = 0;
    uint64_t readback_hits = 0;

    unsigned* dev_error = nullptr;  // device error word (nbg::DEV_ERR_*)

    // Split-precision state (direct_precise.cu): FP64 origin + FP32 offsets live on the
    // device while origin_valid; the float positions in pm/bodies are refreshed from
    // them before anything reads positions.
    bool origin_valid = false;
    nbg::PreciseState* precise = nullptr;
    nbg::BhState* bh = nullptr;

    nbg::BatchState* batch = nullptr;   // system table + batched work lists (batch.cu)

    // Bumped whenever a device buffer moves or a kernel argument baked into a captured
    // graph changes (uploads, growth, system tables, stream switches).
    uint64_t generation = 0;
    bool capturing = false;             // inside nbody_cuda_update_graph's capture: no allocation
    cudaGraphExec_t graph = nullptr;
    uint64_t graph_launches = 0;        // kernels in one replay of the captured step
    nbody_step_params graph_params{};
    uint64_t graph_generation = 0;
    size_t graph_count = 0;
    cudaStream_t graph_stream = nullptr;

    // The last tree in the reference's node layout (tree_export.cu), and the build it is of.
    std::vector<unsigned char> tree_export;
    uint64_t tree_export_id = 0;

    // Ray queries (query.cu): the node array on the device (the exported tree while
    // query_nodes_id matches its build) and the rays / hits / counts buffers.
    void* query_nodes = nullptr;
    size_t query_nodes_cap = 0;
    uint64_t query_nodes_id = 0;
    void* query_buf = nullptr;
    size_t query_buf_cap = 0;

    int force_variant = -1;     // pins the direct-sum (T, block) table entry when >= 0
    nbg::DirectPlan last_plan{};
    uint64_t launches = 0;

    std::string last_error;
    int last_status = NBODY_OK;
};

namespace nbg
{
    int ctx_fail(nbody_cuda* ctx, int status, const char* msg);
    int ctx_cuda_fail(nbody_cuda* ctx, cudaError_t e, const char* what);

    // Two timing events for host-side measurement loops, destroyed with the object.
    // `status` is the first creation error, if any.
    struct EventPair
    {
        cudaEvent_t start = nullptr, stop = nullptr;
        cudaError_t status = cudaSuccess;
        EventPair()
        {
            status = cudaEventCreate(&start);
            if (status == cudaSuccess)
                status = cudaEventCreate(&stop);
        }
        ~EventPair()
        {
            if (start)
                cudaEventDestroy(start);
            if (stop)
                cudaEventDestroy(stop);
        }
        EventPair(const EventPair&) = delete;
        EventPair& operator=(const EventPair&) = delete;
        // milliseconds between the two recorded events, after waiting for the second
        float elapsed_ms() const
        {
            float ms = 0.f;
            if (cudaEventSynchronize(stop) == cudaSuccess)
                cudaEventElapsedTime(&ms, start, stop);
            return ms;
        }
    };
    int ensure_scratch(nbody_cuda* ctx, size_t bytes);
    // Every growth of a device buffer goes through here: refused during graph capture (the
    // pointers a graph holds must stay valid), and it retires any captured graph.
    int before_allocation(nbody_cuda* ctx);
    int check_device_error(nbody_cuda* ctx);

    // context.cu: copies through the pinned staging buffer, and the device-side Body staging
    int staging(nbody_cuda* ctx, size_t bytes, void** out);
    int h2d(nbody_cuda* ctx, void* dst, const void* src, size_t bytes);
    int d2h(nbody_cuda* ctx, void* dst, const void* src, size_t bytes);
    int ensure_aos_stage(nbody_cuda* ctx, size_t n);
    bool is_pinned(const void* p);

    // transfer.cu
    void host_copy(void* dst, const void* src, size_t bytes);     // split across threads when large
    int download_records(nbody_cuda* ctx, void* bodies, size_t take, unsigned mask);
    int upload_records(nbody_cuda* ctx, const void* bodies, size_t n);
    int prefetch_records(nbody_cuda* ctx, unsigned mask);
    void release_transfer(nbody_cuda* ctx);

    // query.cu
    int tree_query(nbody_cuda* ctx, const void* nodes, size_t count, const float* rays, size_t nrays, int stop,
                   uint32_t* hits, size_t max_hits, uint32_t* counts);
    void release_query(nbody_cuda* ctx);

    // scenes.cu
    int scene_disk(nbody_cuda* ctx, const nbody_disk_args* a, size_t begin, size_t num);
    int scene_cube(nbody_cuda* ctx, const nbody_cube_args* a, size_t begin, size_t num);

    // direct_precise.cu
    int precise_accelerate(nbody_cuda* ctx, const nbody_step_params* p);
    int precise_integrate(nbody_cuda* ctx, const nbody_step_params* p);
    int sync_precise_positions(nbody_cuda* ctx);
    void release_precise(nbody_cuda* ctx);
    int precise_sampled(nbody_cuda* ctx, const nbody_step_params* p, const int64_t* targets, size_t nt,
                        double* out);
    int precise_origin(nbody_cuda* ctx, double out[4]);

    // bh.cu
    int bh_accelerate(nbody_cuda* ctx, const nbody_step_params* p);
    void release_bh(nbody_cuda* ctx);

    // energy.cu: kinetic, potential energy and momentum of all bodies (nbody_cuda_energy)
    int energy_all(nbody_cuda* ctx, const nbody_step_params* p, double out[5]);
}
