// Sim facade and variant registry for this library (API of stett/nbody's source/sim.cpp).
// The registry probes the CUDA device once, on first query; a variant whose solver fails
// to construct is demoted with the reason, the running solver keeps going, and a switch
// carries the canonical State across with its identity intact.
#include <array>
#include <stdexcept>

#include "context.h"
#include "cuda_solver.h"
#include "nbody/sim.h"
#include "solver.h"

using nbody::Sim;
using nbody::Variant;
using nbody::VariantInfo;

namespace
{
    constexpr size_t kVariants = static_cast<size_t>(Variant::Count);

    bool is_cuda(const Variant v)
    {
        return v == Variant::CudaBruteForce || v == Variant::CudaBruteForceAoS || v == Variant::CudaBarnesHut
               || v == Variant::CudaBruteForceCompensated;
    }

    nbody::CudaSolverConfig config_for(const Variant v)
    {
        nbody::CudaSolverConfig c;
        switch (v)
        {
        case Variant::CudaBruteForceAoS: c.layout = NBODY_LAYOUT_AOS; break;
        case Variant::CudaBarnesHut: c.mode = NBODY_MODE_NLOGN; break;
        case Variant::CudaBruteForceCompensated: c.precision = NBODY_PREC_COMPENSATED; break;
        default: break;
        }
        return c;
    }

    std::array<VariantInfo, kVariants>& infos()
    {
        static std::array<VariantInfo, kVariants> table = [] {
            std::array<VariantInfo, kVariants> t{};
            const char* ref = "provided by stett/nbody's own library; this build holds the CUDA variants";
            t[size_t(Variant::CpuBarnesHut)] = { Variant::CpuBarnesHut, "CPU Barnes-Hut", "O(n log n), multithreaded", false, ref };
            t[size_t(Variant::CpuBruteForce)] = { Variant::CpuBruteForce, "CPU brute force", "O(n^2) exact summation", false, ref };
            t[size_t(Variant::GpuBarnesHut)] = { Variant::GpuBarnesHut, "GPU Barnes-Hut", "Vulkan compute", false, ref };
            t[size_t(Variant::GpuBruteForce)] = { Variant::GpuBruteForce, "GPU brute force", "Vulkan compute", false, ref };
            t[size_t(Variant::GpuBarnesHutSoA)] = { Variant::GpuBarnesHutSoA, "GPU Barnes-Hut (SoA)", "Vulkan compute", false, ref };
            t[size_t(Variant::GpuBruteForceSoA)] = { Variant::GpuBruteForceSoA, "GPU brute force (SoA)", "Vulkan compute", false, ref };
            t[size_t(Variant::CudaBruteForce)] = { Variant::CudaBruteForce, "CUDA brute force",
                                                   "sm_103a direct sum, split streams", false, "not probed" };
            t[size_t(Variant::CudaBruteForceAoS)] = { Variant::CudaBruteForceAoS, "CUDA brute force (AoS)",
                                                      "sm_103a direct sum over interleaved bodies", false, "not probed" };
            t[size_t(Variant::CudaBarnesHut)] = { Variant::CudaBarnesHut, "CUDA Barnes-Hut",
                                                  "sm_103a device octree, the reference opening test", false, "not probed" };
            t[size_t(Variant::CudaBruteForceCompensated)] = { Variant::CudaBruteForceCompensated, "CUDA brute force (compensated)",
                                                              "FP64 origin + FP32 offsets, Kahan sums", false, "not probed" };
            return t;
        }();
        return table;
    }

    void probe_once()
    {
        static const bool probed = [] {
            char why[256] = { 0 };
            const int st = nbody_cuda_probe(why, sizeof why);
            for (size_t i = 0; i < kVariants; ++i)
                if (is_cuda(Variant(i)))
                {
                    infos()[i].available = st == NBODY_OK;
                    infos()[i].unavailable_reason = st == NBODY_OK ? "" : why;
                }
            return true;
        }();
        (void)probed;
    }

    bool valid(const Variant v) { return static_cast<size_t>(v) < kVariants; }
}

std::span<const VariantInfo> Sim::variants()
{
    probe_once();
    return infos();
}

const VariantInfo& Sim::info(const Variant v)
{
    probe_once();
    if (!valid(v))
    {
        static const VariantInfo invalid{ Variant::Count, "invalid", "", false, "not a valid variant" };
        return invalid;
    }
    return infos()[size_t(v)];
}

bool Sim::available(const Variant v) { return info(v).available; }

Sim::Sim() : Sim(Variant::CudaBarnesHut) {}

Sim::Sim(const Variant variant) : _context(std::make_shared<Context>()), _state(std::make_shared<State>())
{
    if (set_variant(variant))
        return;
    const std::string requested = _last_error;
    for (size_t i = 0; i < kVariants; ++i)
        if (Variant(i) != variant && available(Variant(i)) && set_variant(Variant(i)))
        {
            _last_error = requested;
            return;
        }
    throw std::runtime_error("no simulation variant could be constructed: " + requested);
}

Sim::~Sim() = default;
Sim::Sim(Sim&&) noexcept = default;
Sim& Sim::operator=(Sim&&) noexcept = default;

bool Sim::set_variant(const Variant v)
{
    if (!valid(v))
    {
        _last_error = "unknown variant";
        return false;
    }
    if (v == _variant && _solver)
        return true;
    const VariantInfo& want = info(v);
    if (!want.available)
    {
        _last_error = want.unavailable_reason;
        return false;
    }
    if (_solver)
        sync_solver();
    StateRef state = _solver ? _solver->state() : _state;
    std::unique_ptr<Solver> next;
    try
    {
        next = std::make_unique<CudaSolver>(_context, state, config_for(v));
        next->adopt(state);
    }
    catch (const std::exception& e)
    {
        _last_error = e.what();
        infos()[size_t(v)].available = false;
        infos()[size_t(v)].unavailable_reason = _last_error;
        return false;
    }
    _solver = std::move(next);
    _state = std::move(state);
    _variant = v;
    _synced_revision = _state->revision;
    _last_error.clear();
    return true;
}

void Sim::sync_solver() const
{
    if (_synced_revision == _state->revision)
        return;
    _solver->ingest();
    _synced_revision = _state->revision;
}

std::shared_ptr<const nbody::State> Sim::state() const
{
    sync_solver();
    return _solver->state();
}

const std::vector<nbody::Body>& Sim::bodies() const
{
    sync_solver();
    return _solver->state()->bodies;
}

std::vector<nbody::Body>& Sim::mutable_bodies()
{
    sync_solver();
    const StateRef s = _solver->state();
    s->touch();
    return s->bodies;
}

float Sim::size() const { return _state->size; }
void Sim::set_size(const float v) { _state->size = v; }
float Sim::theta() const { return _state->theta; }
void Sim::set_theta(const float v) { _state->theta = v; }
float Sim::gravity() const { return _state->gravity; }
void Sim::set_gravity(const float v) { _state->gravity = v; }
bool Sim::wrap() const { return _state->wrap; }
void Sim::set_wrap(const bool v) { _state->wrap = v; }

void Sim::update(const float dt)
{
    sync_solver();
    _solver->update(dt);
}

void Sim::accelerate()
{
    sync_solver();
    _solver->accelerate();
}

void Sim::integrate(const float dt)
{
    sync_solver();
    _solver->integrate(dt);
}

void Sim::disk(const size_t begin, const size_t end, const util::DiskArgs& args)
{
    sync_solver();
    auto* cuda = dynamic_cast<CudaSolver*>(_solver.get());
    if (!cuda)
        throw std::logic_error("Sim::disk: the active variant has no device generator");
    cuda->disk(begin, end, args);
}

void Sim::cube(const size_t begin, const size_t end, const util::CubeArgs& args)
{
    sync_solver();
    auto* cuda = dynamic_cast<CudaSolver*>(_solver.get());
    if (!cuda)
        throw std::logic_error("Sim::cube: the active variant has no device generator");
    cuda->cube(begin, end, args);
}

const nbody::bh::Tree* Sim::tree() const { return _solver->tree(); }

std::span<const nbody::bh::Node> Sim::nodes() const
{
    const bh::Tree* t = tree();
    return t ? std::span<const bh::Node>(t->nodes()) : std::span<const bh::Node>{};
}
