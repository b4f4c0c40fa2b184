// C-ABI driver around the reference's own CPU solvers, compiled together with the
// reference sources (source/bhtree.cpp, source/vector.cpp, source/util.cpp and the
// header-only source/solvers/cpu_*.h) into oracle/_ref/libnbody_ref.so by
// oracle/build_oracle.py. Written for this repository; the reference code it calls is
// used unmodified, straight from where it lies.
//
// TEST INFRASTRUCTURE ONLY: used to pin the oracle restatement (tests/golden/) and as
// the CPU baseline where it can be built. Nothing in the product links it.
#include <cstdint>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "context.h"
#include "solvers/cpu_barnes_hut.h"
#include "solvers/cpu_brute_force.h"
#include "detail/physics.h"
#include "detail/tree.h"
#include "nbody/util.h"

namespace
{
    // Body is 12 floats on both sides: pos, radius, vel, mass, acc, pad (body.h:6-19).
    static_assert(sizeof(nbody::Body) == 48, "Body layout");
    static_assert(sizeof(nbody::bh::Node) == 48, "Node layout");

    std::shared_ptr<nbody::State> make_state(const float* bodies, const size_t n, const float size,
                                             const float theta, const float G, const int wrap)
    {
        auto s = std::make_shared<nbody::State>();
        s->size = size;
        s->theta = theta;
        s->gravity = G;
        s->wrap = wrap != 0;
        s->bodies.resize(n);
        if (n)
            std::memcpy(s->bodies.data(), bodies, n * sizeof(nbody::Body));
        return s;
    }

    void copy_out(const nbody::State& s, float* bodies)
    {
        if (!s.bodies.empty())
            std::memcpy(bodies, s.bodies.data(), s.bodies.size() * sizeof(nbody::Body));
    }

    std::shared_ptr<nbody::Context> context(const int threads)
    {
        auto c = std::make_shared<nbody::Context>();
        if (threads > 0)
            c->pool = std::make_shared<BS::thread_pool>(static_cast<size_t>(threads));
        return c;
    }

    template <typename SolverT>
    void run(float* bodies, const size_t n, const float size, const float theta, const float G,
             const int wrap, const float dt, const int steps, const int accelerate_only,
             const int threads)
    {
        auto state = make_state(bodies, n, size, theta, G, wrap);
        SolverT solver(context(threads), state);
        solver.adopt(state);
        if (accelerate_only)
            solver.accelerate();
        else
            for (int i = 0; i < steps; ++i)
                solver.update(dt);
        copy_out(*solver.state(), bodies);
    }
}

extern "C"
{
    int ref_hardware_threads() { return static_cast<int>(std::thread::hardware_concurrency()); }

    // CpuBruteForceSolver::accelerate (cpu_brute_force.h:17-43) or, with steps > 0 and
    // accelerate_only == 0, `steps` calls of Solver::update(dt) (solver.h:59).
    void ref_brute_force(float* bodies, size_t n, float G, float dt, int steps,
                         int accelerate_only, float size, int wrap, int threads)
    {
        run<nbody::CpuBruteForceSolver>(bodies, n, size, 0.5f, G, wrap, dt, steps, accelerate_only, threads);
    }

    // CpuBarnesHutSolver (cpu_barnes_hut.h:22-44), as above.
    void ref_barnes_hut(float* bodies, size_t n, float size, float theta, float G, float dt,
                        int steps, int accelerate_only, int wrap, int threads)
    {
        run<nbody::CpuBarnesHutSolver>(bodies, n, size, theta, G, wrap, dt, steps, accelerate_only, threads);
    }

    // CpuSolver::integrate (cpu_solver.h:29-42) alone.
    void ref_integrate(float* bodies, size_t n, float dt, float size, int wrap)
    {
        for (size_t i = 0; i < n; ++i)
        {
            nbody::Body b;
            std::memcpy(&b, bodies + 12 * i, sizeof b);
            nbody::detail::integrate_euler(b, dt, size, wrap != 0);
            std::memcpy(bodies + 12 * i, &b, sizeof b);
        }
    }

    // detail::build_tree (tree.h:14-29). Copies at most max_nodes nodes; returns the count.
    size_t ref_build_tree(const float* bodies, size_t n, float size, void* nodes_out, size_t max_nodes)
    {
        std::vector<nbody::Body> bs(n);
        if (n)
            std::memcpy(bs.data(), bodies, n * sizeof(nbody::Body));
        nbody::bh::Tree tree;
        nbody::detail::build_tree(tree, bs, size);
        const size_t count = tree.nodes().size();
        const size_t take = count < max_nodes ? count : max_nodes;
        if (take)
            std::memcpy(nodes_out, tree.nodes().data(), take * sizeof(nbody::bh::Node));
        return count;
    }

    // Tree::insert sequence from an explicit list (pos xyz, mass) into a tree of the given
    // root bounds, as the reference's own tree tests do (tests/source/test_bhtree.cpp).
    size_t ref_insert_points(const float* pts, size_t n, float cx, float cy, float cz, float size,
                             void* nodes_out, size_t max_nodes)
    {
        nbody::bh::Tree tree({ .center = { cx, cy, cz }, .size = size });
        for (size_t i = 0; i < n; ++i)
            tree.insert({ pts[4 * i], pts[4 * i + 1], pts[4 * i + 2] }, pts[4 * i + 3]);
        const size_t count = tree.nodes().size();
        const size_t take = count < max_nodes ? count : max_nodes;
        if (take)
            std::memcpy(nodes_out, tree.nodes().data(), take * sizeof(nbody::bh::Node));
        return count;
    }

    // util::disk (util.cpp:14-98) with the arguments the reference tests pass.
    void ref_disk(float* bodies, size_t n, float cx, float cy, float cz, float outer_radius)
    {
        std::vector<nbody::Body> bs(n);
        nbody::util::DiskArgs args{ .center = { cx, cy, cz } };
        args.outer_radius = outer_radius;
        nbody::util::disk(bs.begin(), bs.end(), args);
        if (n)
            std::memcpy(bodies, bs.data(), n * sizeof(nbody::Body));
    }

    // util::cube (util.cpp:100-126) with its defaults.
    void ref_cube(float* bodies, size_t n)
    {
        std::vector<nbody::Body> bs(n);
        nbody::util::cube(bs.begin(), bs.end());
        if (n)
            std::memcpy(bodies, bs.data(), n * sizeof(nbody::Body));
    }

    // Tree::query (bhtree.cpp:153-173) over the tree detail::build_tree makes of the bodies,
    // recording the visited node indices; stop 1: the visitor returns false at the first
    // leaf with mass. The reference's loop does not advance past a node the ray misses, so
    // callers pass only rays that meet every node the walk reaches.
    size_t ref_tree_query(const float* bodies, size_t n, float size, const float* ray, int stop, uint32_t* hits,
                          size_t max_hits)
    {
        std::vector<nbody::Body> bs(n);
        if (n)
            std::memcpy(bs.data(), bodies, n * sizeof(nbody::Body));
        nbody::bh::Tree tree;
        nbody::detail::build_tree(tree, bs, size);
        const nbody::bh::Node* base = tree.nodes().data();
        size_t visited = 0;
        const nbody::Ray r{ { ray[0], ray[1], ray[2] }, { ray[3], ray[4], ray[5] } };
        tree.query(r, [&](const nbody::bh::Node& node) {
            if (visited < max_hits)
                hits[visited] = static_cast<uint32_t>(&node - base);
            ++visited;
            return !(stop == 1 && node.children == 0 && node.mass != 0);
        });
        return visited;
    }

    // util::disk over bodies[begin, begin + num) of an n-body array, every DiskArgs field
    // given: center[3], vel[3], axis[3], inner, outer, thickness, central mass, star mass.
    void ref_disk_args(float* bodies, size_t n, size_t begin, size_t num, const float* a)
    {
        std::vector<nbody::Body> bs(n);
        if (n)
            std::memcpy(bs.data(), bodies, n * sizeof(nbody::Body));
        nbody::util::DiskArgs args{ .center = { a[0], a[1], a[2] }, .vel = { a[3], a[4], a[5] },
                                    .axis = { a[6], a[7], a[8] } };
        args.inner_radius = a[9];
        args.outer_radius = a[10];
        args.thickness = a[11];
        args.central_mass = a[12];
        args.star_mass = a[13];
        nbody::util::disk(bs.begin() + begin, bs.begin() + begin + num, args);
        if (n)
            std::memcpy(bodies, bs.data(), n * sizeof(nbody::Body));
    }

    // util::cube over bodies[begin, begin + num): center[3], size, vel[3], star mass.
    void ref_cube_args(float* bodies, size_t n, size_t begin, size_t num, const float* a)
    {
        std::vector<nbody::Body> bs(n);
        if (n)
            std::memcpy(bs.data(), bodies, n * sizeof(nbody::Body));
        nbody::util::CubeArgs args{ .center = { a[0], a[1], a[2] }, .size = a[3], .vel = { a[4], a[5], a[6] } };
        args.star_mass = a[7];
        nbody::util::cube(bs.begin() + begin, bs.begin() + begin + num, args);
        if (n)
            std::memcpy(bodies, bs.data(), n * sizeof(nbody::Body));
    }
}
