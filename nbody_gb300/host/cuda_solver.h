// CudaSolver: a Solver (source/solver.h:17-75) whose bodies live on a GB300 and whose steps
// run the sm_103a kernels through the C ABI in include/nbody_cuda.h.
//
// It follows the synchronisation contract of the reference's split-layout GPU solver
// (source/solvers/gpu_solver_split.h:34-52, 188-221):
//   - adopt() and ingest() only mark the host copy authoritative; the upload happens lazily,
//     before the next accelerate(), integrate() or update() -- including integrate() alone,
//     so a mutation is never stepped over (gpu_solver_split.h:100-108);
//   - steps leave their results on the device; state() materialises them into
//     State::bodies, reading only min(bodies.size(), device count) (gpu_solver_split.h:202);
//   - an empty body array launches nothing (gpu_solver_split.h:56-59);
//   - G, theta, size and wrap are read from the State at every step;
//   - update() predicts the next read as the reference does (wanted_readback,
//     gpu_solver_split.h:122-132): when a state() followed the previous step, the step
//     queues the readback behind itself (nbody_cuda_prefetch), and state() then only waits
//     for it. Where the library resolves the transfer to DIRECT (a coherent host link), the
//     prefetch queues nothing and state() has the device write State::bodies directly.
// Unlike the reference, the Barnes-Hut tree is built on the device; tree() exports it into
// the reference's node layout on demand.
//
// Compiles against this library's host headers (nbody_gb300/host/include) or, unchanged,
// against the reference's own (include/, source/): tree() uses bh::Tree::assign where the
// header provides it (NBODY_TREE_ASSIGN) and otherwise returns nullptr.
#pragma once
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "nbody_cuda.h"
#include "solver.h"

namespace nbody
{
    struct CudaSolverConfig
    {
        int layout = NBODY_LAYOUT_SOA;      // nbody_layout
        int mode = NBODY_MODE_N2;           // nbody_mode
        int law = NBODY_LAW_CUTOFF;         // nbody_law (the reference's physics by default)
        int precision = NBODY_PREC_FP32;    // nbody_precision
        float eps2 = 0.f;                   // softening^2 for NBODY_LAW_SOFTENED
        int tree_box = 0;                   // 0: the reference's root box; 1: fitted
        int walk = NBODY_WALK_TARGET;       // nbody_walk: the reference's per-target walk, or per group
    };

    class CudaSolver final : public Solver
    {
    public:
        // Throws std::runtime_error when no usable device exists; Sim turns that into an
        // unavailable variant with a reason (source/sim.cpp:226-239).
        CudaSolver(std::shared_ptr<Context> context, StateRef state, const CudaSolverConfig& config)
            : Solver(std::move(context), std::move(state)), _config(config)
        {
            if (nbody_cuda_create(&_dev, _config.layout) != NBODY_OK)
                throw std::runtime_error(last_error(nullptr));
        }

        ~CudaSolver() override { nbody_cuda_destroy(_dev); }

        [[nodiscard]] StateRef state() const override
        {
            materialize();
            return _state;
        }

        void adopt(StateRef state) override
        {
            _state = std::move(state);
            _host_dirty = true;
            _device_dirty = false;
            _tree_build = 0;
            _tree_valid = false;
        }

        void ingest() const override { _host_dirty = true; }

        void accelerate() override
        {
            if (!prepare())
                return;
            const nbody_step_params p = params(0.f);
            check(nbody_cuda_accelerate(_dev, &p), "accelerate");
            stepped();
        }

        void integrate(const float dt) override
        {
            if (!prepare())
                return;
            const nbody_step_params p = params(dt);
            check(nbody_cuda_integrate(_dev, &p), "integrate");
            _device_dirty = true;
        }

        // Both halves queued back to back on the device (the reference's split solver does the
        // same in one submission, gpu_solver_split.h:54-72).
        void update(const float dt) override
        {
            if (!prepare())
                return;
            const nbody_step_params p = params(dt);
            check(nbody_cuda_update(_dev, &p, 1), "update");
            stepped();
            if (const unsigned want = wanted_readback())
                check(nbody_cuda_prefetch(_dev, want), "readback");
        }

        [[nodiscard]] const bh::Tree* tree() const override
        {
            if (_config.mode != NBODY_MODE_NLOGN)
                return nullptr;
#ifdef NBODY_TREE_ASSIGN
            if (!_tree_valid)
            {
                if (_tree_build > 0)
                {
                    size_t count = 0;
                    check(nbody_cuda_tree_export(_dev, nullptr, 0, &count), "tree export");
                    std::vector<bh::Node> nodes(count);
                    check(nbody_cuda_tree_export(_dev, nodes.data(), count, &count), "tree export");
                    _tree.assign(std::move(nodes));
                }
                else
                    _tree.clear({ .center = {}, .size = _state->size });
                _tree_valid = true;
            }
            return &_tree;
#else
            return nullptr;
#endif
        }

        [[nodiscard]] const CudaSolverConfig& config() const { return _config; }

        // Change law, precision or softening between steps (not the layout).
        void configure(const CudaSolverConfig& config)
        {
            if (config.layout != _config.layout)
                throw std::invalid_argument("CudaSolver::configure cannot change the body layout");
            _config = config;
        }

        [[nodiscard]] nbody_cuda* device() const { return _dev; }

        // util::disk / util::cube (source/util.cpp:14-126) over State::bodies[begin, end),
        // generated on the device from the reference's own random stream; state()
        // materialises them. `args` is the reference's util::DiskArgs / CubeArgs, or any
        // type with their fields.
        template <class DiskArgs>
        void disk(const size_t begin, const size_t end, const DiskArgs& args)
        {
            nbody_disk_args a{};
            put3(a.center, args.center);
            put3(a.vel, args.vel);
            put3(a.axis, args.axis);
            a.inner_radius = args.inner_radius;
            a.outer_radius = args.outer_radius;
            a.thickness = args.thickness;
            a.central_mass = args.central_mass;
            a.star_mass = args.star_mass;
            generate(begin, end, [&] { return nbody_cuda_scene_disk(_dev, &a, begin, end - begin); });
        }

        template <class CubeArgs>
        void cube(const size_t begin, const size_t end, const CubeArgs& args)
        {
            nbody_cube_args a{};
            put3(a.center, args.center);
            a.size = args.size;
            put3(a.vel, args.vel);
            a.star_mass = args.star_mass;
            generate(begin, end, [&] { return nbody_cuda_scene_cube(_dev, &a, begin, end - begin); });
        }

    private:
        static std::string last_error(const nbody_cuda* dev)
        {
            char buf[512];
            nbody_cuda_last_error(dev, buf, sizeof buf);
            return std::string("CUDA solver: ") + buf;
        }

        void check(const int status, const char* what) const
        {
            if (status != NBODY_OK)
                throw std::runtime_error(std::string(what) + ": " + last_error(_dev));
        }

        [[nodiscard]] nbody_step_params params(const float dt) const
        {
            nbody_step_params p{};
            p.dt = dt;
            p.theta = _state->theta;
            p.G = _state->gravity;
            p.eps2 = _config.eps2;
            p.size = _state->size;
            p.wrap = _state->wrap ? 1 : 0;
            p.mode = _config.mode;
            p.law = _config.law;
            p.precision = _config.precision;
            p.tree_box = _config.tree_box;
            p.walk = _config.walk;
            return p;
        }

        // Upload a host-side change before anything runs on the device; false when there is
        // nothing to step.
        bool prepare()
        {
            if (_state->bodies.empty())
                return false;
            if (_host_dirty)
            {
                check(nbody_cuda_upload_bodies(_dev, _state->bodies.data(), _state->bodies.size()), "upload");
                _host_dirty = false;
            }
            return true;
        }

        template <class V>
        static void put3(float out[3], const V& v)
        {
            out[0] = v.x;
            out[1] = v.y;
            out[2] = v.z;
        }

        // Bring the device up to date with everything outside the range, then generate.
        template <class F>
        void generate(const size_t begin, const size_t end, F&& call)
        {
            if (begin > end || end > _state->bodies.size())
                throw std::out_of_range("CudaSolver: generated range outside the bodies");
            if (begin == end)
                return;
            if (_host_dirty || nbody_cuda_count(_dev) != _state->bodies.size())
            {
                check(nbody_cuda_upload_bodies(_dev, _state->bodies.data(), _state->bodies.size()), "upload");
                _host_dirty = false;
            }
            check(call(), "scene generator");
            _device_dirty = true;
            _tree_valid = false;
        }

        void stepped()
        {
            _device_dirty = true;
            if (_config.mode == NBODY_MODE_NLOGN)
            {
                ++_tree_build;
                _tree_valid = false;
            }
        }

        // Everything, if the last step was followed by a read: a caller that reads every
        // frame will read again. The device tree needs no positions on the host.
        [[nodiscard]] unsigned wanted_readback() const
        {
            const unsigned want = _materialize_expected ? NBODY_READ_ALL : 0u;
            _materialize_expected = false;
            return want;
        }

        void materialize() const
        {
            _materialize_expected = true;   // set even when there is nothing to fetch
            if (!_device_dirty || _host_dirty)
                return;
            const size_t n = _state->bodies.size();
            check(nbody_cuda_download_bodies(_dev, _state->bodies.data(), n, NBODY_READ_ALL), "download");
            _device_dirty = false;
        }

        nbody_cuda* _dev = nullptr;
        CudaSolverConfig _config;
        mutable bool _host_dirty = true;
        mutable bool _device_dirty = false;
        mutable bool _materialize_expected = false;
        mutable bh::Tree _tree;
        mutable bool _tree_valid = false;
        uint64_t _tree_build = 0;
    };
}
