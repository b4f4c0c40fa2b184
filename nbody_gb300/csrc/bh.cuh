// Internal interface of the Barnes-Hut pipeline (bh.cu).
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "nbody_cuda.h"

struct nbody_cuda;

namespace nbg
{
    // Root box of the Morton grid, kept on the device between the build kernels.
    struct BoxParams
    {
        double lo[3];       // lower corner
        double center[3];   // centre
        double edge;        // cube edge
        double inv_cell;    // 2^21 / edge
        // When the edge is a power of two and the corner lies on the cell grid, the cell
        // index of x is floor(x / 2^cell_exp) - lo_cells exactly, in integers (see morton).
        int exact;
        int cell_exp;               // log2(edge / 2^21)
        long long lo_cells[3];      // lo / cell
        // Fixed-point cell sums: a body's mass is summed as the integer m 2^mass_shift and
        // its moment as m x 2^mom_shift, both rounded; the shifts keep every sum of all n
        // bodies below 2^61 (from the largest finite |m| and |x|, see box_final_kernel).
        int mass_shift;
        int mom_shift;
        float edge_f;       // the edge in float (exact: a float size or a power of two)
    };

    // One octree cell: 64 bytes, read whole by a warp (a broadcast load per field).
    struct __align__(16) OctNode
    {
        float4 com_mass;    // centre of mass (float) and mass
        float open_r2;      // (cell edge)^2 * theta^2: accepted when |com - x|^2 > open_r2
        int nchild;         // children listed below; -1 for a bucket of identical codes
        int first, last;    // sorted body range of the cell
        int child[8];       // >= 0: octree cell index; < 0: ~(sorted body index)
    };
    static_assert(sizeof(OctNode) == 64, "OctNode is one 64-byte record");

    // Host copy of the last device tree (tree_export.cu turns it into reference nodes).
    struct TreeSnapshot
    {
        size_t n = 0;                   // bodies
        uint64_t build_id = 0;
        BoxParams box{};
        std::vector<OctNode> cells;     // cell 0 is the root cell (n >= 2)
        std::vector<uint64_t> codes;    // sorted Morton codes
        std::vector<float4> bodies;     // pos + mass in Morton order
    };

    int bh_build(nbody_cuda* ctx, const nbody_step_params* p);
    int bh_download(nbody_cuda* ctx, TreeSnapshot* out);
    uint64_t bh_build_id(const nbody_cuda* ctx);    // 0 before the first build
    int bh_stats(nbody_cuda* ctx, unsigned long long out[3]);
    int bh_stage_ms(nbody_cuda* ctx, float ms[2]);
    int bh_morton(nbody_cuda* ctx, const nbody_step_params* p, uint64_t* codes, uint32_t* order, double box[4]);
}
