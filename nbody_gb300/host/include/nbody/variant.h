// Solver variants. The first six are stett/nbody's (include/nbody/variant.h:7-17), kept in
// their order so a Variant value means the same thing on both sides; the CUDA variants this
// library provides are appended before Count, where a maintainer adds them there too.
#pragma once
#include <string>

namespace nbody
{
    enum class Variant : int
    {
        CpuBarnesHut = 0,
        CpuBruteForce,
        GpuBarnesHut,
        GpuBruteForce,
        GpuBarnesHutSoA,
        GpuBruteForceSoA,

        CudaBruteForce,             // direct sum, split streams, the reference's force law, FP32
        CudaBruteForceAoS,          // direct sum over interleaved Body records
        CudaBarnesHut,              // device octree, the reference's opening test
        CudaBruteForceCompensated,  // direct sum, FP64 origin + FP32 offsets, Kahan sums

        Count
    };

    struct VariantInfo
    {
        Variant variant = Variant::CudaBruteForce;
        const char* name = "";
        const char* description = "";
        bool available = false;
        std::string unavailable_reason;
    };
}
