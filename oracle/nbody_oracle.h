/*
 * CPU oracle for the N-body hot path -- TEST INFRASTRUCTURE ONLY.
 *
 * This is a plain-C restatement of the reference CPU solvers (stett/nbody) plus FP64
 * checkers that the reference lacks. It exists so the CUDA path can be checked; nothing
 * in the product (nbody_gb300/, include/) may link or call it. Only tests/, the smoke
 * check in __graft_entry__.py and the CPU-baseline leg of bench.py use it.
 *
 * Parity is pinned two ways (tests/test_oracle.py):
 *   - against the reference's own known answers (tests/source/test_bhtree.cpp:30-142,
 *     node counts 1/9/17 and hand-computed centres of mass), and
 *   - bit-for-bit against the reference itself, compiled from its sources into
 *     oracle/_ref/ by oracle/build_oracle.py, through golden fixtures in tests/golden/.
 *
 * Body layout (include/nbody/body.h:6-19): 12 floats per body,
 *   [0..2] pos, [3] radius, [4..6] vel, [7] mass, [8..10] acc, [11] pad.
 * Node layout (include/nbody/bhtree.h:13-22): 12 words per node,
 *   center xyz, size, com xyz, mass, next, children, pad, pad.
 */
#ifndef NBODY_ORACLE_H
#define NBODY_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { ORC_LAW_CUTOFF = 0, ORC_LAW_SOFTENED = 1 };

typedef struct
{
    float cx, cy, cz, size;     /* Bounds: centre and edge */
    float comx, comy, comz;     /* centre of mass */
    float mass;
    uint32_t next;              /* threaded link: next sibling or the parent's next */
    uint32_t children;          /* first of 8 contiguous children, 0 for a leaf */
    uint32_t pad0, pad1;
} orc_node;

typedef struct orc_tree orc_tree;

/* --- force law and integrator (source/detail/physics.h) --------------------------- */
void orc_gravity(const float pos[3], float radius, const float src[3], float src_mass,
                 float G, float out[3]);
float orc_wrap(float x, float size);
void orc_integrate(float* bodies, size_t n, float dt, float size, int wrap);

/* --- solvers (source/solvers/cpu_brute_force.h, cpu_barnes_hut.h) ----------------- */
void orc_brute_force(float* bodies, size_t n, float G, int nthreads);
/* Brute force for a subset of targets only; acc_out is 3 floats per listed target. */
void orc_brute_force_targets(const float* bodies, size_t n, float G,
                             const int64_t* targets, size_t ntargets, float* acc_out,
                             int nthreads);
void orc_barnes_hut(float* bodies, size_t n, float size, float theta, float G,
                    int nthreads, uint64_t* interactions);

/* The softened law G*m*d/(|d|^2 + eps2)^(3/2) in the reference law's operation order
 * (no cutoff), and the solvers above with the law chosen (ORC_LAW_CUTOFF: the
 * reference's own). No reference counterpart: the benchmark configurations soften. */
void orc_gravity_softened(const float pos[3], const float src[3], float src_mass, float G,
                          float eps2, float out[3]);
void orc_brute_force_targets_law(const float* bodies, size_t n, float G, int law, float eps2,
                                 const int64_t* targets, size_t ntargets, float* acc_out,
                                 int nthreads);
void orc_barnes_hut_law(float* bodies, size_t n, float size, float theta, float G, int law,
                        float eps2, int nthreads, uint64_t* interactions);

/* --- octree (source/bhtree.cpp, source/detail/tree.h) ----------------------------- */
orc_tree* orc_tree_new(float size);
void orc_tree_free(orc_tree* t);
void orc_tree_clear(orc_tree* t, float cx, float cy, float cz, float size);
void orc_tree_insert(orc_tree* t, float x, float y, float z, float mass);
void orc_tree_build(orc_tree* t, const float* bodies, size_t n, float size);
/* orc_tree_build on a root box centred at (cx, cy, cz) with edge size. */
void orc_tree_build_box(orc_tree* t, const float* bodies, size_t n, float cx, float cy, float cz,
                        float size);
/* Recompute each node's mass and centre of mass exactly (double sums over its bodies, one
 * rounding to float), keeping the reference's cells. bodies must be the ones the tree was
 * built from. Returns 0, or -1 when the scratch cannot be allocated. */
int orc_tree_exact_moments(orc_tree* t, const float* bodies, size_t n);
size_t orc_tree_size(const orc_tree* t);
const orc_node* orc_tree_nodes(const orc_tree* t);
/* Barnes-Hut acceleration for listed targets (or all bodies when targets is NULL). */
void orc_tree_accel(const orc_tree* t, const float* bodies, size_t n,
                    const int64_t* targets, size_t ntargets, float theta, float G,
                    float* acc_out, uint64_t* interactions, int nthreads);

/* Tree::apply over an arbitrary node array in the reference layout (root at index 0). */
void orc_nodes_accel(const orc_node* nodes, size_t count, const float* bodies, size_t n,
                     const int64_t* targets, size_t ntargets, float theta, float G,
                     float* acc_out, uint64_t* interactions, int nthreads);
/* The two walks above with the law chosen (the softened visitor applies
 * orc_gravity_softened to every accepted node; the walk is unchanged). */
void orc_tree_accel_law(const orc_tree* t, const float* bodies, size_t n,
                        const int64_t* targets, size_t ntargets, float theta, float G,
                        int law, float eps2, float* acc_out, uint64_t* interactions,
                        int nthreads);
void orc_nodes_accel_law(const orc_node* nodes, size_t count, const float* bodies, size_t n,
                         const int64_t* targets, size_t ntargets, float theta, float G,
                         int law, float eps2, float* acc_out, uint64_t* interactions,
                         int nthreads);

/* --- FP64 direct sum (no reference counterpart) ----------------------------------- */
/* pos_mass: 4 floats per body (x, y, z, m). radius: per-body cutoff radius for
 * ORC_LAW_CUTOFF (may be NULL: 0). Compensated (Neumaier) double accumulation.
 * acc_out: 3 doubles per target; scale_out (optional): sum over j of |a_ij|. */
void orc_direct_f64(const float* pos_mass, const float* radius, size_t n, double G,
                    double eps2, int law, const int64_t* targets, size_t ntargets,
                    double* acc_out, double* scale_out, int nthreads);
/* Same law with positions given in double (for the split-precision form). */
void orc_direct_f64_pos(const double* pos, const double* mass, size_t n, double G,
                        double eps2, const int64_t* targets, size_t ntargets,
                        double* acc_out, int nthreads);
/* Kinetic and potential energy, total momentum, in double. */
void orc_energy_f64(const double* pos, const double* vel, const double* mass, size_t n,
                    double G, double eps2, double* kinetic, double* potential,
                    double momentum[3], int nthreads);

/* --- Morton codes and sort order (no reference counterpart) ----------------------- */
/* Per axis q = floor((x - lo) * inv_cell) with both double operations rounded toward
 * -inf, clamped to [0, 2^21-1]; bits interleaved x -> bit 0, y -> bit 1, z -> bit 2. */
void orc_morton63(const float* xyz, size_t stride, size_t n, const double lo[3],
                  double inv_cell, uint64_t* codes);
/* Stable order by (code, index). */
void orc_sort_order(const uint64_t* codes, size_t n, uint32_t* order);

/* --- scene generators (source/util.cpp:9-126) ------------------------------------- */
/* The reference's random stream, restated: std::default_random_engine of libstdc++ (GCC 13)
 * is minstd_rand0, x <- 16807 x mod (2^31 - 1), seed 1; generate_canonical<float, 24>
 * takes one engine value (the range 2^31 - 2 holds >= 24 bits): float(x - 1) / 2^31,
 * clamped below 1; uniform_real_distribution<float>(a, b) = canonical * (b - a) + a;
 * normal_distribution<float> is the Marsaglia polar method with the second value saved. */
uint32_t orc_minstd_value(uint64_t j);      /* the j-th value (from 0) the engine returns */
float orc_compute_radius(float mass, float density);
/* util::disk over bodies[0, num): a[] = center[3], vel[3], axis[3], inner, outer,
 * thickness, central mass, star mass. Velocities from the reference's own walk: a tree
 * rooted at the centre with edge 2 * outer (before the clamp), theta 0.5, folding the
 * applied nodes into a running centre of mass (util.cpp:81-95). */
void orc_disk(float* bodies, size_t num, const float a[14]);
/* The star positions of util::disk for stars [first, last) only (last 0: all), with the
 * random stream drawn in full up to them and no velocity pass: a fast check of any tail
 * of a large disk. Writes only those bodies (velocities are the unit directions). */
void orc_disk_positions(float* bodies, size_t num, const float a[14], size_t first, size_t last);
/* util::cube over bodies[0, num): a[] = center[3], size, vel[3], star mass. */
void orc_cube(float* bodies, size_t num, const float a[8]);

/* --- ray query (source/bhtree.cpp:153-173) ------------------------------------------ */
/* Tree::query over a reference node array for one ray (origin xyz, direction xyz).
 * stop 0 visits every node the ray meets; stop 1 ends after the first met leaf with mass.
 * Writes the first max_hits visited indices, returns how many were visited. At a node the
 * ray misses the walk moves to its next and *missed is set: there the reference's loop
 * would not advance and never ends. */
size_t orc_tree_query(const orc_node* nodes, size_t count, const float ray[6], int stop,
                      uint32_t* hits, size_t max_hits, int* missed);

/* Threads this process would use by default (online CPUs). */
int orc_default_threads(void);

#ifdef __cplusplus
}
#endif
#endif
