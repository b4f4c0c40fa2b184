// Resources shared by the solvers a Sim runs (the part of stett/nbody's source/context.h
// this library needs: nothing, since every CUDA solver owns its own device context).
#pragma once

namespace nbody
{
    struct Context
    {
    };
}
