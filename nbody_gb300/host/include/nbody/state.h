// The canonical simulation state every solver variant speaks: the fields of stett/nbody's
// State (include/nbody/state.h) -- world size, opening parameter, G, wrap, the Body array
// and a revision counter that callers bump when they mutate the bodies.
#pragma once
#include <cstdint>
#include <memory>
#include <vector>
#include "nbody/body.h"

namespace nbody
{
    struct State
    {
        float size = 10000.f;   // world edge; wrap period and Barnes-Hut root box
        float theta = .5f;      // opening parameter (accept when |com - x| > size * theta)
        float gravity = 1.f;    // G
        bool wrap = true;
        std::vector<Body> bodies;
        uint64_t revision = 0;
        void touch() noexcept { ++revision; }
    };

    using StateRef = std::shared_ptr<State>;
}
