"""GB300-native (sm_103a) N-body solver for stett/nbody's Solver interface.

``nbody_gb300.native`` binds the C ABI (``include/nbody_cuda.h``) of the CUDA library
built by ``nbody_gb300.build``; ``nbody_gb300.scenes`` makes the seeded synthetic inputs.
"""
