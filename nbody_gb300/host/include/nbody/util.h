// The argument records of stett/nbody's scene generators (include/nbody/util.h), with the
// reference's fields and defaults, so that Sim::disk / Sim::cube take what util::disk /
// util::cube take. The generation itself runs on the device (nbody_cuda_scene_disk /
// nbody_cuda_scene_cube in include/nbody_cuda.h).
#pragma once
#include "nbody/vector.h"

namespace nbody
{
    namespace util
    {
        struct DiskArgs
        {
            Vector center = { 0, 0, 0 };
            Vector vel = { 0, 0, 0 };
            Vector axis = { 0, 0, 1 };
            float inner_radius = 0.f;
            float outer_radius = 250.f;
            float thickness = 1.f;
            float central_mass = 4.1e6f;    // sagittarius_mass (constants.h:8)
            float star_mass = 1.0f;         // solar_mass (constants.h:9)
        };

        struct CubeArgs
        {
            Vector center = { 0, 0, 0 };
            float size = 500;
            Vector vel = { 0, 0, 0 };
            float star_mass = 1.0f;
        };
    }
}
