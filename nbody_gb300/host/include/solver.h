// The solver plug-in interface: stett/nbody's Solver (source/solver.h:17-75), the boundary
// the CUDA solver sits behind. Same members and contract:
//   state()     the canonical State, materialised from the solver's own representation;
//   adopt(s)    take on a State wholesale, keeping *that* shared_ptr;
//   ingest()    a caller mutated the bodies: re-converge before the next use;
//   accelerate(), integrate(dt), update(dt)   stepping;
//   tree()      the Barnes-Hut tree of the last accelerate, or nullptr.
#pragma once
#include <memory>
#include "nbody/bhtree.h"
#include "nbody/state.h"

namespace nbody
{
    struct Context;

    class Solver
    {
    public:
        virtual ~Solver() = default;
        Solver(const Solver&) = delete;
        Solver& operator=(const Solver&) = delete;

        [[nodiscard]] virtual StateRef state() const = 0;
        virtual void adopt(StateRef state) = 0;
        virtual void ingest() const {}

        virtual void accelerate() = 0;
        virtual void integrate(float dt) = 0;
        virtual void update(const float dt) { accelerate(); integrate(dt); }

        [[nodiscard]] virtual const bh::Tree* tree() const { return nullptr; }

    protected:
        Solver(std::shared_ptr<Context> context, StateRef state)
            : _context(std::move(context)), _state(std::move(state))
        {}

        std::shared_ptr<Context> _context;
        StateRef _state;
    };
}
