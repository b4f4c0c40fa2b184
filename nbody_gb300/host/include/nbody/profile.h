// Profiling hooks with the names stett/nbody uses (include/nbody/profile.h). They compile
// to nothing here; per-kernel timing comes from CUDA events and ncu instead.
#pragma once
#define NBODY_PROFILE_ZONE() ((void)0)
#define NBODY_PROFILE_ZONE_NAMED(name) ((void)0)
#define NBODY_PROFILE_PLOT(name, value) ((void)0)
