// Sim: the facade that owns one interchangeable Solver and keeps the canonical State,
// with the API of stett/nbody's Sim (include/nbody/sim.h:23-117) -- variant discovery and
// switching with the state carried across, revision-tracked mutation, stepping, tree
// access. This build registers the CUDA variants; the reference's CPU and Vulkan variants
// are listed (so Variant values mean the same thing) but live in the reference library.
#pragma once
#include <cstdint>
#include <memory>
#include <span>
#include <string>
#include <vector>
#include "nbody/bhtree.h"
#include "nbody/body.h"
#include "nbody/state.h"
#include "nbody/util.h"
#include "nbody/variant.h"

namespace nbody
{
    class Solver;
    struct Context;

    class Sim
    {
    public:
        Sim();                      // the first available variant, CUDA Barnes-Hut first
        explicit Sim(Variant variant);
        ~Sim();
        Sim(Sim&&) noexcept;
        Sim& operator=(Sim&&) noexcept;
        Sim(const Sim&) = delete;
        Sim& operator=(const Sim&) = delete;

        [[nodiscard]] static std::span<const VariantInfo> variants();
        [[nodiscard]] static const VariantInfo& info(Variant v);
        [[nodiscard]] static bool available(Variant v);

        [[nodiscard]] Variant variant() const { return _variant; }
        bool set_variant(Variant v);
        [[nodiscard]] const std::string& last_error() const { return _last_error; }

        [[nodiscard]] std::shared_ptr<const State> state() const;
        [[nodiscard]] const std::vector<Body>& bodies() const;
        [[nodiscard]] std::vector<Body>& mutable_bodies();

        [[nodiscard]] float size() const;
        void set_size(float v);
        [[nodiscard]] float theta() const;
        void set_theta(float v);
        [[nodiscard]] float gravity() const;
        void set_gravity(float v);
        [[nodiscard]] bool wrap() const;
        void set_wrap(bool v);

        void update(float dt);
        void accelerate();
        void integrate(float dt);

        // util::disk / util::cube (source/util.cpp:14-126) over bodies()[begin, end),
        // generated by the active CUDA variant on the device; throws std::logic_error on a
        // variant without a device generator and std::out_of_range outside the bodies.
        void disk(size_t begin, size_t end, const util::DiskArgs& args = {});
        void cube(size_t begin, size_t end, const util::CubeArgs& args = {});

        [[nodiscard]] const bh::Tree* tree() const;
        [[nodiscard]] std::span<const bh::Node> nodes() const;

        // The active solver (for CUDA-specific configuration such as the softened law).
        [[nodiscard]] Solver* solver() const { return _solver.get(); }

    private:
        void sync_solver() const;

        std::shared_ptr<Context> _context;
        StateRef _state;
        std::unique_ptr<Solver> _solver;
        Variant _variant = Variant::CudaBarnesHut;
        std::string _last_error;
        mutable uint64_t _synced_revision = 0;
    };
}
