/*
 * CPU oracle for the N-body hot path -- TEST INFRASTRUCTURE ONLY (see nbody_oracle.h).
 *
 * Built with -O2 -ffp-contract=off -frounding-math so every float operation is the one
 * written here, in the order written, on both x86-64 and aarch64: the FP32 restatement
 * of the reference then reproduces the reference (compiled with the same flags) bit for
 * bit, which tests/test_oracle.py checks against fixtures made from the reference.
 */
#include "nbody_oracle.h"

#include <fenv.h>
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#pragma STDC FENV_ACCESS ON

/* ------------------------------------------------------------------------------------
 * Fork-join helper: run fn(ctx, begin, end) over a block partition of [0, n).
 * Plays the part of detail::parallel_blocks (source/detail/parallel.h:16-22).
 * ---------------------------------------------------------------------------------- */
typedef void (*orc_block_fn)(void* ctx, size_t begin, size_t end);

typedef struct
{
    orc_block_fn fn;
    void* ctx;
    size_t begin, end;
} orc_job;

static void* orc_job_run(void* p)
{
    orc_job* j = (orc_job*)p;
    j->fn(j->ctx, j->begin, j->end);
    return NULL;
}

int orc_default_threads(void)
{
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

static void orc_parallel(size_t n, int nthreads, orc_block_fn fn, void* ctx)
{
    if (n == 0)
        return;
    if (nthreads <= 0)
        nthreads = orc_default_threads();
    if ((size_t)nthreads > n)
        nthreads = (int)n;
    if (nthreads == 1)
    {
        fn(ctx, 0, n);
        return;
    }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    orc_job* jobs = (orc_job*)malloc(sizeof(orc_job) * (size_t)nthreads);
    const size_t base = n / (size_t)nthreads, rem = n % (size_t)nthreads;
    size_t at = 0;
    for (int t = 0; t < nthreads; ++t)
    {
        const size_t len = base + ((size_t)t < rem ? 1 : 0);
        jobs[t].fn = fn;
        jobs[t].ctx = ctx;
        jobs[t].begin = at;
        jobs[t].end = at + len;
        at += len;
    }
    for (int t = 1; t < nthreads; ++t)
        pthread_create(&th[t], NULL, orc_job_run, &jobs[t]);
    orc_job_run(&jobs[0]);
    for (int t = 1; t < nthreads; ++t)
        pthread_join(th[t], NULL);
    free(jobs);
    free(th);
}

/* ------------------------------------------------------------------------------------
 * Force law: source/detail/physics.h:21-42.
 * delta = src - pos; |delta|^2 = (dx*dx + dy*dy) + dz*dz (Vector dot, source/vector.cpp:10-13);
 * zero when |delta|^2 <= radius^2; else ((G*m) * delta) / (sqrt(|delta|^2) * |delta|^2).
 * ---------------------------------------------------------------------------------- */
void orc_gravity(const float pos[3], const float radius, const float src[3],
                 const float src_mass, const float G, float out[3])
{
    const float dx = src[0] - pos[0];
    const float dy = src[1] - pos[1];
    const float dz = src[2] - pos[2];
    const float dsq = (dx * dx + dy * dy) + dz * dz;
    const float rsq = radius * radius;
    if (dsq <= rsq)
    {
        out[0] = out[1] = out[2] = 0.f;
        return;
    }
    const float s = G * src_mass;
    const float den = sqrtf(dsq) * dsq;
    out[0] = (s * dx) / den;
    out[1] = (s * dy) / den;
    out[2] = (s * dz) / den;
}

/* The softened law the benchmark configurations use, G*m*d/(|d|^2 + eps2)^(3/2), written
 * in the operation order of the reference's law above (physics.h:21-42) with eps2 added to
 * |d|^2 and no cutoff. No reference counterpart: the reference has only the cutoff law. */
void orc_gravity_softened(const float pos[3], const float src[3], const float src_mass, const float G,
                          const float eps2, float out[3])
{
    const float dx = src[0] - pos[0];
    const float dy = src[1] - pos[1];
    const float dz = src[2] - pos[2];
    const float dsq = ((dx * dx + dy * dy) + dz * dz) + eps2;
    const float s = G * src_mass;
    const float den = sqrtf(dsq) * dsq;
    out[0] = (s * dx) / den;
    out[1] = (s * dy) / den;
    out[2] = (s * dz) / den;
}

/* One pair under either law (the visitor of cpu_brute_force.h:31-39 and
 * cpu_barnes_hut.h:31-41, with the law chosen). */
static inline void orc_pair(const int law, const float pos[3], const float radius, const float src[3],
                            const float src_mass, const float G, const float eps2, float out[3])
{
    if (law == ORC_LAW_SOFTENED)
        orc_gravity_softened(pos, src, src_mass, G, eps2, out);
    else
        orc_gravity(pos, radius, src, src_mass, G, out);
}

/* Wrap into [-size/2, size/2]: physics.h:50-58 (double fmod, as the reference writes it). */
float orc_wrap(const float x, const float size)
{
    if (size <= 0.f)
        return x;
    const float half = size * .5f;
    return fmodf(fmodf(x + half, size) + size, size) - half;
}

/* Semi-implicit Euler: physics.h:60-70, run over all bodies as cpu_solver.h:29-42. */
void orc_integrate(float* b, const size_t n, const float dt, const float size, const int wrap)
{
    for (size_t i = 0; i < n; ++i)
    {
        float* p = b + 12 * i;
        for (int a = 0; a < 3; ++a)
            p[4 + a] = p[4 + a] + p[8 + a] * dt;
        for (int a = 0; a < 3; ++a)
            p[a] = p[a] + p[4 + a] * dt;
        if (!wrap)
            continue;
        for (int a = 0; a < 3; ++a)
            p[a] = orc_wrap(p[a], size);
    }
}

/* ------------------------------------------------------------------------------------
 * Brute force: source/solvers/cpu_brute_force.h:17-43. Sequential j loop from 0, j == i
 * skipped, FP32 accumulation acc += gravity(...).
 * ---------------------------------------------------------------------------------- */
typedef struct
{
    const float* bodies;
    size_t n;
    float G;
    const int64_t* targets;
    float* acc_out;     /* 3 per target, or NULL to write Body::acc in place */
    float* bodies_rw;
    int law;
    float eps2;
} orc_bf_ctx;

static void orc_bf_block(void* p, const size_t begin, const size_t end)
{
    orc_bf_ctx* c = (orc_bf_ctx*)p;
    for (size_t t = begin; t < end; ++t)
    {
        const size_t i = c->targets ? (size_t)c->targets[t] : t;
        const float* bi = c->bodies + 12 * i;
        float acc[3] = { 0.f, 0.f, 0.f };
        for (size_t j = 0; j < c->n; ++j)
        {
            if (j == i)
                continue;
            const float* bj = c->bodies + 12 * j;
            float g[3];
            orc_pair(c->law, bi, bi[3], bj, bj[7], c->G, c->eps2, g);
            acc[0] += g[0];
            acc[1] += g[1];
            acc[2] += g[2];
        }
        if (c->acc_out)
            memcpy(c->acc_out + 3 * t, acc, sizeof acc);
        else
            memcpy(c->bodies_rw + 12 * i + 8, acc, sizeof acc);
    }
}

void orc_brute_force(float* bodies, const size_t n, const float G, const int nthreads)
{
    /* Results land in a side buffer first: writing Body::acc in place while other
     * threads read the same bodies is harmless (acc is never read) but keep it simple. */
    orc_bf_ctx c = { bodies, n, G, NULL, NULL, bodies, ORC_LAW_CUTOFF, 0.f };
    orc_parallel(n, nthreads, orc_bf_block, &c);
}

void orc_brute_force_targets(const float* bodies, const size_t n, const float G,
                             const int64_t* targets, const size_t ntargets, float* acc_out,
                             const int nthreads)
{
    orc_brute_force_targets_law(bodies, n, G, ORC_LAW_CUTOFF, 0.f, targets, ntargets, acc_out, nthreads);
}

void orc_brute_force_targets_law(const float* bodies, const size_t n, const float G, const int law,
                                 const float eps2, const int64_t* targets, const size_t ntargets,
                                 float* acc_out, const int nthreads)
{
    orc_bf_ctx c = { bodies, n, G, targets, acc_out, NULL, law, eps2 };
    orc_parallel(targets ? ntargets : n, nthreads, orc_bf_block, &c);
}

/* ------------------------------------------------------------------------------------
 * Octree: source/bhtree.cpp:7-146, include/nbody/bounds.h:31-52, source/detail/tree.h.
 * ---------------------------------------------------------------------------------- */
struct orc_tree
{
    orc_node* nodes;
    size_t count, cap;
};

static void orc_tree_push(orc_tree* t, const orc_node* n)
{
    if (t->count == t->cap)
    {
        t->cap = t->cap ? t->cap * 2 : 64;
        t->nodes = (orc_node*)realloc(t->nodes, t->cap * sizeof(orc_node));
    }
    t->nodes[t->count++] = *n;
}

orc_tree* orc_tree_new(const float size)
{
    orc_tree* t = (orc_tree*)calloc(1, sizeof(orc_tree));
    orc_tree_clear(t, 0.f, 0.f, 0.f, size);
    return t;
}

void orc_tree_free(orc_tree* t)
{
    if (!t)
        return;
    free(t->nodes);
    free(t);
}

/* Tree::clear(bounds): bhtree.cpp:140-146 -- a lone root with the new bounds. */
void orc_tree_clear(orc_tree* t, const float cx, const float cy, const float cz, const float size)
{
    orc_node root;
    memset(&root, 0, sizeof root);
    root.cx = cx;
    root.cy = cy;
    root.cz = cz;
    root.size = size;
    t->count = 0;
    orc_tree_push(t, &root);
}

size_t orc_tree_size(const orc_tree* t) { return t->count; }
const orc_node* orc_tree_nodes(const orc_tree* t) { return t->nodes; }

/* Bounds::quadrant: bit0 = x < cx, bit1 = y < cy, bit2 = z < cz (bounds.h:31-38). */
static unsigned orc_quadrant(const orc_node* n, const float x, const float y, const float z)
{
    return (unsigned)(x < n->cx) | ((unsigned)(y < n->cy) << 1) | ((unsigned)(z < n->cz) << 2);
}

/* Tree::accumulate: running weighted mean, bhtree.cpp:87-95. */
static void orc_accumulate(orc_node* n, const float x, const float y, const float z, const float m)
{
    const float nm = n->mass;
    const float total = m + nm;
    const float px = (x * m) + (n->comx * nm);
    const float py = (y * m) + (n->comy * nm);
    const float pz = (z * m) + (n->comz * nm);
    n->mass = total;
    n->comx = px / total;
    n->comy = py / total;
    n->comz = pz / total;
}

/* Tree::insert: bhtree.cpp:14-85. */
void orc_tree_insert(orc_tree* t, const float x, const float y, const float z, const float mass)
{
    uint32_t idx = 0;
    while (t->nodes[idx].children != 0)
    {
        orc_accumulate(&t->nodes[idx], x, y, z, mass);
        const unsigned q = orc_quadrant(&t->nodes[idx], x, y, z);
        idx = t->nodes[idx].children + q;
    }

    if (t->nodes[idx].mass == 0)
    {
        t->nodes[idx].mass = mass;
        t->nodes[idx].comx = x;
        t->nodes[idx].comy = y;
        t->nodes[idx].comz = z;
        return;
    }

    for (;;)
    {
        if (t->nodes[idx].size < FLT_EPSILON)
        {
            t->nodes[idx].mass += mass;
            return;
        }

        /* Bounds::quadrant_bounds (bounds.h:40-52) for the 8 children, threaded so
         * that child q's next is child q+1 and the last child's next is the parent's. */
        const orc_node parent = t->nodes[idx];
        const uint32_t child = (uint32_t)t->count;
        t->nodes[idx].children = child;
        const float half = parent.size * .5f;
        const float quart = parent.size * .25f;
        for (unsigned q = 0; q < 8; ++q)
        {
            orc_node c;
            memset(&c, 0, sizeof c);
            c.cx = (q & 1u) ? (parent.cx - quart) : (parent.cx + quart);
            c.cy = (q & 2u) ? (parent.cy - quart) : (parent.cy + quart);
            c.cz = (q & 4u) ? (parent.cz - quart) : (parent.cz + quart);
            c.size = half;
            c.next = (q < 7) ? (child + q + 1) : parent.next;
            orc_tree_push(t, &c);
        }

        const unsigned new_q = orc_quadrant(&parent, x, y, z);
        const unsigned old_q = orc_quadrant(&parent, parent.comx, parent.comy, parent.comz);
        if (new_q == old_q)
        {
            const uint32_t c = t->nodes[idx].children + new_q;
            t->nodes[c].mass = t->nodes[idx].mass;
            t->nodes[c].comx = t->nodes[idx].comx;
            t->nodes[c].comy = t->nodes[idx].comy;
            t->nodes[c].comz = t->nodes[idx].comz;
            orc_accumulate(&t->nodes[idx], x, y, z, mass);
            idx = c;
        }
        else
        {
            const uint32_t ni = t->nodes[idx].children + new_q;
            const uint32_t oi = t->nodes[idx].children + old_q;
            t->nodes[ni].comx = x;
            t->nodes[ni].comy = y;
            t->nodes[ni].comz = z;
            t->nodes[ni].mass = mass;
            t->nodes[oi].comx = t->nodes[idx].comx;
            t->nodes[oi].comy = t->nodes[idx].comy;
            t->nodes[oi].comz = t->nodes[idx].comz;
            t->nodes[oi].mass = t->nodes[idx].mass;
            orc_accumulate(&t->nodes[idx], x, y, z, mass);
            return;
        }
    }
}

/* detail::build_tree: tree.h:14-29 -- root centred at the origin with edge `size`,
 * bodies inserted in index order. */
void orc_tree_build(orc_tree* t, const float* bodies, const size_t n, const float size)
{
    orc_tree_build_box(t, bodies, n, 0.f, 0.f, 0.f, size);
}

/* Replace every node's mass and centre of mass by the exact values over the bodies below
 * it, summed in double and rounded once to float. No reference counterpart: the reference
 * keeps an FP32 running mean per node (bhtree.cpp:87-95), whose total mass stalls once it
 * dwarfs the added masses (16.8M equal bodies lose 6 % of the root mass), while the cells
 * stay exactly the reference's. A body's path is the insert's descent: the quadrant test
 * at each split node (bounds.h:31-38), which is where bhtree.cpp:14-85 placed it. */
int orc_tree_exact_moments(orc_tree* t, const float* bodies, const size_t n)
{
    const size_t count = t->count;
    double* acc = (double*)calloc(4 * (count ? count : 1), sizeof(double));
    if (!acc)
        return -1;
    for (size_t i = 0; i < n; ++i)
    {
        const float* b = bodies + 12 * i;
        const double m = b[7];
        uint32_t idx = 0;
        for (;;)
        {
            double* a = acc + 4 * idx;
            a[0] += m;
            a[1] += m * b[0];
            a[2] += m * b[1];
            a[3] += m * b[2];
            const orc_node* nd = &t->nodes[idx];
            if (nd->children == 0)
                break;
            idx = nd->children + orc_quadrant(nd, b[0], b[1], b[2]);
        }
    }
    for (size_t k = 0; k < count; ++k)
    {
        const double* a = acc + 4 * k;
        orc_node* nd = &t->nodes[k];
        nd->mass = (float)a[0];
        if (a[0] != 0.0)
        {
            nd->comx = (float)(a[1] / a[0]);
            nd->comy = (float)(a[2] / a[0]);
            nd->comz = (float)(a[3] / a[0]);
        }
    }
    free(acc);
    return 0;
}

/* The same insertion sequence on a root box of any centre (the reference always centres
 * its root at the origin, tree.h:20; the device tree may fit a box around the bodies). */
void orc_tree_build_box(orc_tree* t, const float* bodies, const size_t n, const float cx, const float cy,
                        const float cz, const float size)
{
    orc_tree_clear(t, cx, cy, cz, size);
    for (size_t i = 0; i < n; ++i)
    {
        const float* b = bodies + 12 * i;
        orc_tree_insert(t, b[0], b[1], b[2], b[7]);
    }
}

/* Tree::apply with the gravity visitor: bhtree.cpp:97-138 and cpu_barnes_hut.h:31-41.
 * The visitor applies the reference's cutoff law, or the softened law with eps2 (the law
 * of the benchmark configurations); the walk and the opening test are the reference's
 * either way. */
typedef struct
{
    const orc_tree* tree;
    const float* bodies;
    const int64_t* targets;
    float theta, G;
    float* acc_out;
    uint64_t* counts;   /* per target interaction counts */
    int law;
    float eps2;
} orc_bh_ctx;

static void orc_bh_block(void* p, const size_t begin, const size_t end)
{
    orc_bh_ctx* c = (orc_bh_ctx*)p;
    const orc_node* nodes = c->tree->nodes;
    const size_t count = c->tree->count;
    const float theta_sq = c->theta * c->theta;
    for (size_t t = begin; t < end; ++t)
    {
        const size_t i = c->targets ? (size_t)c->targets[t] : t;
        const float* b = c->bodies + 12 * i;
        float acc[3] = { 0.f, 0.f, 0.f };
        uint64_t visits = 0;
        uint32_t idx = 0;
        do
        {
            const orc_node* nd = &nodes[idx];
            if (nd->mass == 0)
            {
                idx = nd->next;
                continue;
            }
            int apply = nd->children == 0;
            if (!apply)
            {
                const float node_size_sq = nd->size * nd->size;
                const float dx = nd->comx - b[0];
                const float dy = nd->comy - b[1];
                const float dz = nd->comz - b[2];
                const float dist_sq = (dx * dx + dy * dy) + dz * dz;
                apply = dist_sq > node_size_sq * theta_sq;
            }
            if (apply)
            {
                const float com[3] = { nd->comx, nd->comy, nd->comz };
                float g[3];
                orc_pair(c->law, b, b[3], com, nd->mass, c->G, c->eps2, g);
                acc[0] += g[0];
                acc[1] += g[1];
                acc[2] += g[2];
                ++visits;
                idx = nd->next;
                continue;
            }
            idx = nd->children;
        } while (0 < idx && idx < count);
        memcpy(c->acc_out + 3 * t, acc, sizeof acc);
        if (c->counts)
            c->counts[t] = visits;
    }
}

void orc_tree_accel(const orc_tree* t, const float* bodies, const size_t n,
                    const int64_t* targets, const size_t ntargets, const float theta,
                    const float G, float* acc_out, uint64_t* interactions, const int nthreads)
{
    orc_tree_accel_law(t, bodies, n, targets, ntargets, theta, G, ORC_LAW_CUTOFF, 0.f, acc_out, interactions,
                       nthreads);
}

void orc_tree_accel_law(const orc_tree* t, const float* bodies, const size_t n,
                        const int64_t* targets, const size_t ntargets, const float theta,
                        const float G, const int law, const float eps2, float* acc_out,
                        uint64_t* interactions, const int nthreads)
{
    const size_t nt = targets ? ntargets : n;
    uint64_t* counts = interactions ? (uint64_t*)calloc(nt ? nt : 1, sizeof(uint64_t)) : NULL;
    orc_bh_ctx c = { t, bodies, targets, theta, G, acc_out, counts, law, eps2 };
    orc_parallel(nt, nthreads, orc_bh_block, &c);
    if (interactions)
    {
        uint64_t total = 0;
        for (size_t i = 0; i < nt; ++i)
            total += counts[i];
        *interactions = total;
        free(counts);
    }
}

/* Tree::apply over a node array given from outside (e.g. a tree exported by the device
 * layer): the same walk as orc_tree_accel, bhtree.cpp:97-138. */
void orc_nodes_accel(const orc_node* nodes, const size_t count, const float* bodies, const size_t n,
                     const int64_t* targets, const size_t ntargets, const float theta, const float G,
                     float* acc_out, uint64_t* interactions, const int nthreads)
{
    orc_nodes_accel_law(nodes, count, bodies, n, targets, ntargets, theta, G, ORC_LAW_CUTOFF, 0.f, acc_out,
                        interactions, nthreads);
}

void orc_nodes_accel_law(const orc_node* nodes, const size_t count, const float* bodies, const size_t n,
                         const int64_t* targets, const size_t ntargets, const float theta, const float G,
                         const int law, const float eps2, float* acc_out, uint64_t* interactions,
                         const int nthreads)
{
    orc_tree t;
    t.nodes = (orc_node*)nodes;
    t.count = count;
    t.cap = count;
    orc_tree_accel_law(&t, bodies, n, targets, ntargets, theta, G, law, eps2, acc_out, interactions, nthreads);
}

/* CpuBarnesHutSolver::accelerate: cpu_barnes_hut.h:22-44 (acc written in place). */
void orc_barnes_hut(float* bodies, const size_t n, const float size, const float theta,
                    const float G, const int nthreads, uint64_t* interactions)
{
    orc_barnes_hut_law(bodies, n, size, theta, G, ORC_LAW_CUTOFF, 0.f, nthreads, interactions);
}

void orc_barnes_hut_law(float* bodies, const size_t n, const float size, const float theta,
                        const float G, const int law, const float eps2, const int nthreads,
                        uint64_t* interactions)
{
    orc_tree* t = orc_tree_new(size);
    orc_tree_build(t, bodies, n, size);
    float* acc = (float*)malloc(sizeof(float) * 3 * (n ? n : 1));
    orc_tree_accel_law(t, bodies, n, NULL, 0, theta, G, law, eps2, acc, interactions, nthreads);
    for (size_t i = 0; i < n; ++i)
        memcpy(bodies + 12 * i + 8, acc + 3 * i, 3 * sizeof(float));
    free(acc);
    orc_tree_free(t);
}

/* ------------------------------------------------------------------------------------
 * FP64 direct sum with Neumaier-compensated accumulation. No reference counterpart:
 * the checker every precision claim is stated against.
 * ---------------------------------------------------------------------------------- */
typedef struct { double s, c; } orc_ksum;

static inline void orc_kadd(orc_ksum* k, const double v)
{
    const double t = k->s + v;
    if (fabs(k->s) >= fabs(v))
        k->c += (k->s - t) + v;
    else
        k->c += (v - t) + k->s;
    k->s = t;
}

static inline double orc_kval(const orc_ksum* k) { return k->s + k->c; }

typedef struct
{
    const float* pm;
    const float* radius;
    const double* pos64;
    const double* mass64;
    size_t n;
    double G, eps2;
    int law;
    const int64_t* targets;
    double* acc_out;
    double* scale_out;
} orc_f64_ctx;

static void orc_f64_block(void* p, const size_t begin, const size_t end)
{
    orc_f64_ctx* c = (orc_f64_ctx*)p;
    for (size_t t = begin; t < end; ++t)
    {
        const size_t i = c->targets ? (size_t)c->targets[t] : t;
        double xi, yi, zi;
        if (c->pos64)
        {
            xi = c->pos64[3 * i]; yi = c->pos64[3 * i + 1]; zi = c->pos64[3 * i + 2];
        }
        else
        {
            xi = c->pm[4 * i]; yi = c->pm[4 * i + 1]; zi = c->pm[4 * i + 2];
        }
        const double r = (c->radius && c->law == ORC_LAW_CUTOFF) ? (double)c->radius[i] : 0.0;
        const double rsq = r * r;
        orc_ksum ax = { 0, 0 }, ay = { 0, 0 }, az = { 0, 0 }, sc = { 0, 0 };
        for (size_t j = 0; j < c->n; ++j)
        {
            double dx, dy, dz, m;
            if (c->pos64)
            {
                dx = c->pos64[3 * j] - xi; dy = c->pos64[3 * j + 1] - yi; dz = c->pos64[3 * j + 2] - zi;
                m = c->mass64[j];
            }
            else
            {
                dx = (double)c->pm[4 * j] - xi;
                dy = (double)c->pm[4 * j + 1] - yi;
                dz = (double)c->pm[4 * j + 2] - zi;
                m = c->pm[4 * j + 3];
            }
            const double d2 = dx * dx + dy * dy + dz * dz;
            double f;
            if (c->law == ORC_LAW_CUTOFF)
            {
                if (d2 <= rsq || d2 == 0.0)
                    continue;
                f = c->G * m / (sqrt(d2) * d2);
            }
            else
            {
                const double s2 = d2 + c->eps2;
                if (s2 == 0.0)
                    continue;
                f = c->G * m / (sqrt(s2) * s2);
            }
            orc_kadd(&ax, f * dx);
            orc_kadd(&ay, f * dy);
            orc_kadd(&az, f * dz);
            if (c->scale_out)
                orc_kadd(&sc, fabs(f) * sqrt(d2));
        }
        c->acc_out[3 * t] = orc_kval(&ax);
        c->acc_out[3 * t + 1] = orc_kval(&ay);
        c->acc_out[3 * t + 2] = orc_kval(&az);
        if (c->scale_out)
            c->scale_out[t] = orc_kval(&sc);
    }
}

void orc_direct_f64(const float* pos_mass, const float* radius, const size_t n, const double G,
                    const double eps2, const int law, const int64_t* targets,
                    const size_t ntargets, double* acc_out, double* scale_out, const int nthreads)
{
    orc_f64_ctx c = { pos_mass, radius, NULL, NULL, n, G, eps2, law, targets, acc_out, scale_out };
    orc_parallel(targets ? ntargets : n, nthreads, orc_f64_block, &c);
}

void orc_direct_f64_pos(const double* pos, const double* mass, const size_t n, const double G,
                        const double eps2, const int64_t* targets, const size_t ntargets,
                        double* acc_out, const int nthreads)
{
    orc_f64_ctx c = { NULL, NULL, pos, mass, n, G, eps2, ORC_LAW_SOFTENED, targets, acc_out, NULL };
    orc_parallel(targets ? ntargets : n, nthreads, orc_f64_block, &c);
}

typedef struct
{
    const double* pos;
    const double* vel;
    const double* mass;
    size_t n;
    double G, eps2;
    int nblocks;
    double* partial;    /* per block: kinetic, potential, px, py, pz */
} orc_en_ctx;

static void orc_en_block(void* p, const size_t begin, const size_t end)
{
    orc_en_ctx* c = (orc_en_ctx*)p;
    for (size_t blk = begin; blk < end; ++blk)
    {
        /* Rows are dealt round-robin so the triangular loop balances across blocks. */
        orc_ksum ke = { 0, 0 }, pe = { 0, 0 }, px = { 0, 0 }, py = { 0, 0 }, pz = { 0, 0 };
        for (size_t i = blk; i < c->n; i += (size_t)c->nblocks)
        {
            const double m = c->mass[i];
            const double* v = c->vel + 3 * i;
            orc_kadd(&ke, 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
            orc_kadd(&px, m * v[0]);
            orc_kadd(&py, m * v[1]);
            orc_kadd(&pz, m * v[2]);
            const double* xi = c->pos + 3 * i;
            orc_ksum row = { 0, 0 };
            for (size_t j = i + 1; j < c->n; ++j)
            {
                const double* xj = c->pos + 3 * j;
                const double dx = xj[0] - xi[0], dy = xj[1] - xi[1], dz = xj[2] - xi[2];
                const double s2 = dx * dx + dy * dy + dz * dz + c->eps2;
                if (s2 > 0.0)
                    orc_kadd(&row, c->mass[j] / sqrt(s2));
            }
            orc_kadd(&pe, -c->G * m * orc_kval(&row));
        }
        double* out = c->partial + 5 * blk;
        out[0] = orc_kval(&ke);
        out[1] = orc_kval(&pe);
        out[2] = orc_kval(&px);
        out[3] = orc_kval(&py);
        out[4] = orc_kval(&pz);
    }
}

void orc_energy_f64(const double* pos, const double* vel, const double* mass, const size_t n,
                    const double G, const double eps2, double* kinetic, double* potential,
                    double momentum[3], const int nthreads)
{
    const int nblocks = 64;
    double* partial = (double*)calloc(5 * (size_t)nblocks, sizeof(double));
    orc_en_ctx c = { pos, vel, mass, n, G, eps2, nblocks, partial };
    orc_parallel((size_t)nblocks, nthreads, orc_en_block, &c);
    orc_ksum s[5] = { { 0, 0 }, { 0, 0 }, { 0, 0 }, { 0, 0 }, { 0, 0 } };
    for (int b = 0; b < nblocks; ++b)
        for (int k = 0; k < 5; ++k)
            orc_kadd(&s[k], partial[5 * b + k]);
    *kinetic = orc_kval(&s[0]);
    *potential = orc_kval(&s[1]);
    momentum[0] = orc_kval(&s[2]);
    momentum[1] = orc_kval(&s[3]);
    momentum[2] = orc_kval(&s[4]);
    free(partial);
}

/* ------------------------------------------------------------------------------------
 * Morton codes (no reference counterpart). The quantisation rounds toward -inf in both
 * double operations so that, for a power-of-two box whose lower corner is exact, every
 * cell boundary compares exactly as the reference's float centre comparisons do
 * (bounds.h:31-38): floor(rd(v)) == floor(v) whenever the boundaries are representable.
 * ---------------------------------------------------------------------------------- */
static uint64_t orc_spread3(uint64_t v)
{
    v &= 0x1fffffull;
    v = (v | (v << 32)) & 0x001f00000000ffffull;
    v = (v | (v << 16)) & 0x001f0000ff0000ffull;
    v = (v | (v << 8)) & 0x100f00f00f00f00full;
    v = (v | (v << 4)) & 0x10c30c30c30c30c3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

void orc_morton63(const float* xyz, const size_t stride, const size_t n, const double lo[3],
                  const double inv_cell, uint64_t* codes)
{
    const int old = fegetround();
    fesetround(FE_DOWNWARD);
    for (size_t i = 0; i < n; ++i)
    {
        uint64_t code = 0;
        for (int a = 0; a < 3; ++a)
        {
            volatile double x = (double)xyz[stride * i + (size_t)a];
            volatile double t = x - lo[a];
            volatile double u = t * inv_cell;
            const double f = floor(u);
            uint64_t q;
            if (!(f >= 0.0))
                q = 0;
            else if (f > 2097151.0)
                q = 2097151;
            else
                q = (uint64_t)f;
            code |= orc_spread3(q) << a;
        }
        codes[i] = code;
    }
    fesetround(old);
}

static const uint64_t* orc_sort_keys;

static int orc_cmp_order(const void* a, const void* b)
{
    const uint32_t ia = *(const uint32_t*)a, ib = *(const uint32_t*)b;
    const uint64_t ka = orc_sort_keys[ia], kb = orc_sort_keys[ib];
    if (ka != kb)
        return ka < kb ? -1 : 1;
    return ia < ib ? -1 : (ia > ib ? 1 : 0);
}

void orc_sort_order(const uint64_t* codes, const size_t n, uint32_t* order)
{
    for (size_t i = 0; i < n; ++i)
        order[i] = (uint32_t)i;
    orc_sort_keys = codes;
    qsort(order, n, sizeof(uint32_t), orc_cmp_order);
    orc_sort_keys = NULL;
}

/* ------------------------------------------------------------------------------------
 * Scene generators: util::compute_radius, util::disk, util::cube (source/util.cpp:9-126)
 * and the libstdc++ (GCC 13) random machinery they draw from, restated.
 * ---------------------------------------------------------------------------------- */
#define ORC_MINSTD_M 2147483647u
#define ORC_PI 3.1415926535897932384626433832795028841971693993751058209749445923078164062f

typedef struct
{
    uint64_t x;                 /* minstd_rand0 state, seed 1 */
    int saved_available;        /* normal_distribution's cached second value */
    float saved;
} orc_rng;

static uint32_t orc_engine(orc_rng* g)
{
    g->x = (g->x * 16807u) % ORC_MINSTD_M;
    return (uint32_t)g->x;
}

uint32_t orc_minstd_value(const uint64_t j)
{
    /* 16807^(j+1) mod (2^31 - 1) by square-and-multiply */
    uint64_t e = (j + 1) % (ORC_MINSTD_M - 1), base = 16807u, r = 1;
    while (e)
    {
        if (e & 1)
            r = (r * base) % ORC_MINSTD_M;
        base = (base * base) % ORC_MINSTD_M;
        e >>= 1;
    }
    return (uint32_t)r;
}

/* generate_canonical<float, 24>: one engine value; sum / 2^31 where 2^31 is the engine's
 * range 2^31 - 2 rounded to float. */
static float orc_canonical(orc_rng* g)
{
    const float sum = (float)(orc_engine(g) - 1u) * 1.0f;
    const float tmp = (float)(1.0L * (long double)(ORC_MINSTD_M - 1u));
    float ret = sum / tmp;
    if (ret >= 1.0f)
        ret = nextafterf(1.0f, 0.0f);
    return ret;
}

static float orc_uniform(orc_rng* g, const float a, const float b)
{
    return (orc_canonical(g) * (b - a)) + a;
}

/* normal_distribution<float>::operator(): Marsaglia polar method. */
static float orc_normal(orc_rng* g, const float mean, const float stddev)
{
    float ret;
    if (g->saved_available)
    {
        g->saved_available = 0;
        ret = g->saved;
    }
    else
    {
        float x, y, r2;
        do
        {
            x = (float)((double)(2.0f * orc_canonical(g)) - 1.0);
            y = (float)((double)(2.0f * orc_canonical(g)) - 1.0);
            r2 = x * x + y * y;
        } while ((double)r2 > 1.0 || (double)r2 == 0.0);
        const float mult = sqrtf(-2 * logf(r2) / r2);
        g->saved = x * mult;
        g->saved_available = 1;
        ret = y * mult;
    }
    return ret * stddev + mean;
}

float orc_compute_radius(const float mass, const float density)
{
    return powf((3.f * ORC_PI * mass) / (4.f * density), 1.f / 3.f);
}

static void orc_put_body(float* b, const float p[3], const float radius, const float v[3], const float mass)
{
    b[0] = p[0]; b[1] = p[1]; b[2] = p[2]; b[3] = radius;
    b[4] = v[0]; b[5] = v[1]; b[6] = v[2]; b[7] = mass;
    b[8] = 0.f; b[9] = 0.f; b[10] = 0.f; b[11] = 0.f;
}

static void orc_norm3(float v[3])
{
    const float s = sqrtf((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
    v[0] = v[0] / s;
    v[1] = v[1] / s;
    v[2] = v[2] / s;
}

static void orc_cross3(const float a[3], const float b[3], float out[3])
{
    out[0] = (a[1] * b[2]) - (a[2] * b[1]);
    out[1] = (a[2] * b[0]) - (a[0] * b[2]);
    out[2] = (a[0] * b[1]) - (a[1] * b[0]);
}

/* The star loop of util::disk (util.cpp:52-79) for stars [1, num), writing bodies whose
 * index lies in [first, last) (all when last == 0) and inserting every star into `tree`
 * when one is given. */
static void orc_disk_stars(float* bodies, const size_t num, const float a[14], const size_t first,
                           const size_t last, orc_tree* tree)
{
    const float center[3] = { a[0], a[1], a[2] };
    const float axis[3] = { a[6], a[7], a[8] };
    float inner = a[9], outer = a[10];
    const float thickness = a[11], central_mass = a[12], star_mass = a[13];
    const float center_radius = orc_compute_radius(central_mass, 1e2f);
    outer = outer < center_radius ? center_radius : outer;      /* std::max */
    inner = inner < center_radius ? center_radius : inner;

    orc_rng g = { 1u, 0, 0.f };
    const float c0[3] = { copysignf(axis[2], axis[0]), copysignf(axis[2], axis[1]),
                          -copysignf(axis[0], axis[2]) - copysignf(axis[1], axis[2]) };
    float c1[3];
    orc_cross3(axis, c0, c1);

    for (size_t i = 1; i < num; ++i)
    {
        const float t = (float)i / (float)(num - 1);
        const float angle = t * 2.f * ORC_PI;
        /* the unqualified sqrt of a float is ::sqrt(double) */
        const float dist = (float)((double)inner + (sqrt((double)orc_uniform(&g, 0.f, 1.f)) * (double)(outer - inner)));
        const float disp = ((outer - dist) / outer) * (thickness * center_radius) * orc_normal(&g, 0.f, .5f);
        if (!tree && (i < first || (last && i >= last)))
            continue;
        const float s = sinf(angle), c = cosf(angle);
        float s0[3] = { (s * c0[0]) + (c * c1[0]), (s * c0[1]) + (c * c1[1]), (s * c0[2]) + (c * c1[2]) };
        orc_norm3(s0);
        float s1[3];
        orc_cross3(axis, s0, s1);
        orc_norm3(s1);
        const float p[3] = { (center[0] + (s0[0] * dist)) + (axis[0] * disp),
                             (center[1] + (s0[1] * dist)) + (axis[1] * disp),
                             (center[2] + (s0[2] * dist)) + (axis[2] * disp) };
        if (i >= first && (!last || i < last))
            orc_put_body(bodies + 12 * i, p, orc_compute_radius(star_mass, 1e2f), s1, star_mass);
        if (tree)
            orc_tree_insert(tree, p[0], p[1], p[2], star_mass);
    }
}

void orc_disk_positions(float* bodies, const size_t num, const float a[14], const size_t first, const size_t last)
{
    orc_disk_stars(bodies, num, a, first ? first : 1, last, NULL);
}

void orc_disk(float* bodies, const size_t num, const float a[14])
{
    if (num == 0)
        return;
    const float center[3] = { a[0], a[1], a[2] };
    const float vel[3] = { a[3], a[4], a[5] };
    const float outer = a[10], central_mass = a[12];

    /* the tree's edge is twice the outer radius as given, before the clamp */
    orc_tree* tree = orc_tree_new(1.f);
    orc_tree_clear(tree, center[0], center[1], center[2], 2.f * outer);

    const float center_radius = orc_compute_radius(central_mass, 1e2f);
    const float zero[3] = { 0.f, 0.f, 0.f };
    orc_put_body(bodies, center, center_radius, zero, central_mass);
    orc_tree_insert(tree, center[0], center[1], center[2], central_mass);

    orc_disk_stars(bodies, num, a, 1, 0, tree);

    /* circular speeds: Tree::apply(pos, visitor, 0.5) (bhtree.cpp:97-138) with the
     * running centre-of-mass visitor of util.cpp:84-90 */
    const orc_node* nodes = tree->nodes;
    const size_t count = tree->count;
    const float theta_sq = .5f * .5f;
    for (size_t k = 0; k < num; ++k)
    {
        float* b = bodies + 12 * k;
        float com[3] = { 0.f, 0.f, 0.f }, mass = 0.f;
        uint32_t idx = 0;
        do
        {
            const orc_node* nd = &nodes[idx];
            if (nd->mass == 0)
            {
                idx = nd->next;
                continue;
            }
            int apply = nd->children == 0;
            if (!apply)
            {
                const float node_size_sq = nd->size * nd->size;
                const float dx = nd->comx - b[0], dy = nd->comy - b[1], dz = nd->comz - b[2];
                apply = ((dx * dx + dy * dy) + dz * dz) > node_size_sq * theta_sq;
            }
            if (apply)
            {
                const float tot = mass + nd->mass;
                com[0] = ((com[0] * mass) + (nd->comx * nd->mass)) / tot;
                com[1] = ((com[1] * mass) + (nd->comy * nd->mass)) / tot;
                com[2] = ((com[2] * mass) + (nd->comz * nd->mass)) / tot;
                mass += nd->mass;
                idx = nd->next;
                continue;
            }
            idx = nd->children;
        } while (0 < idx && idx < count);
        const float d[3] = { com[0] - b[0], com[1] - b[1], com[2] - b[2] };
        const float dist = sqrtf((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
        const float speed = sqrtf(1.f * mass / dist);
        b[4] = vel[0] + (b[4] * speed);
        b[5] = vel[1] + (b[5] * speed);
        b[6] = vel[2] + (b[6] * speed);
    }
    orc_tree_free(tree);
}

void orc_cube(float* bodies, const size_t num, const float a[8])
{
    const float size = a[3];
    const float vel[3] = { a[4], a[5], a[6] };
    const float star_mass = a[7];
    orc_rng g = { 1u, 0, 0.f };
    const float lo = (float)(-.5 * (double)size), hi = (float)(.5 * (double)size);
    for (size_t i = 0; i < num; ++i)
    {
        float p[3];
        p[0] = orc_uniform(&g, lo, hi);
        p[1] = orc_uniform(&g, lo, hi);
        p[2] = orc_uniform(&g, lo, hi);
        orc_put_body(bodies + 12 * i, p, orc_compute_radius(star_mass, 1e2f), vel, star_mass);
    }
}

/* ------------------------------------------------------------------------------------
 * Tree::query (source/bhtree.cpp:153-173) with Bounds::ray_intersect
 * (include/nbody/bounds.h:64-133).
 * ---------------------------------------------------------------------------------- */

/* ray_intersect_coord<i> with length = FLT_MAX (only a hit lowers it, and ray_intersect
 * returns on the first hit). */
static int orc_face(const float o[3], const float d[3], const float c[3], const float s, const int i)
{
    const int j = (i + 1) % 3, k = (i + 2) % 3;
    float t;
    if (d[i] < -FLT_EPSILON)
        t = (c[i] + s - o[i]) / d[i];
    else if (d[i] > FLT_EPSILON)
        t = (c[i] - s - o[i]) / d[i];
    else
        return 0;
    if (!(t < FLT_MAX))
        return 0;
    const float p[3] = { o[0] + (d[0] * t), o[1] + (d[1] * t), o[2] + (d[2] * t) };
    return p[j] > c[j] - s && p[j] < c[j] + s && p[k] > c[k] - s && p[k] < c[k] + s;
}

static int orc_ray_meets(const orc_node* n, const float ray[6])
{
    const float c[3] = { n->cx, n->cy, n->cz };
    const float s = n->size;
    int inside = 1;
    for (int i = 0; i < 3; ++i)
        if (ray[i] < c[i] - s || ray[i] > c[i] + s)
        {
            inside = 0;
            break;
        }
    if (inside)
        return 1;
    return orc_face(ray, ray + 3, c, s, 0) || orc_face(ray, ray + 3, c, s, 1) || orc_face(ray, ray + 3, c, s, 2);
}

size_t orc_tree_query(const orc_node* nodes, const size_t count, const float ray[6], const int stop,
                      uint32_t* hits, const size_t max_hits, int* missed)
{
    size_t visited = 0, steps = 0;
    uint32_t idx = 0;
    if (missed)
        *missed = 0;
    if (!count)
        return 0;
    do
    {
        if (idx >= count || ++steps > count)
            break;      /* a malformed array */
        const orc_node* nd = &nodes[idx];
        if (orc_ray_meets(nd, ray))
        {
            if (visited < max_hits)
                hits[visited] = idx;
            ++visited;
            if (stop == 1 && nd->children == 0 && nd->mass != 0)
                break;
            idx = nd->children ? nd->children : nd->next;
        }
        else
        {
            if (missed)
                *missed = 1;
            idx = nd->next;
        }
    } while (idx != 0);
    return visited;
}
