// One body as the solver boundary moves it: 48 bytes, {pos, radius}, {vel, mass},
// {acc, pad} -- the record layout of stett/nbody's include/nbody/body.h, which the CUDA
// library's C ABI (include/nbody_cuda.h) reads and writes directly.
#pragma once
#include "nbody/vector.h"

namespace nbody
{
    struct Body
    {
        Vector pos = { 0, 0, 0 };
        float radius = 0;
        Vector vel = { 0, 0, 0 };
        float mass = 0;
        Vector acc = { 0, 0, 0 };
        float __pad = 0;
    };
    static_assert(sizeof(Body) == 48, "Body must stay the 48-byte record the C ABI moves");
}
