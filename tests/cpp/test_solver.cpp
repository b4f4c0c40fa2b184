// The CUDA solver variants driven through Sim and the Solver interface, with the checks of
// stett/nbody's own suite (tests/source/test_gpu.cpp, test_variant.cpp, test_wrap.cpp,
// test_sim.cpp) restated for the CUDA variants. CPU results come from the oracle's
// restatement of the reference's CPU solvers (oracle/nbody_oracle.h).
//
// Built and run by tests/test_solver_cpp.py; prints one PASS/FAIL line per case and exits
// non-zero if any case failed.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "cuda_solver.h"
#include "nbody/sim.h"
#include "nbody_oracle.h"

using nbody::Body;
using nbody::Sim;
using nbody::Variant;
using nbody::Vector;

namespace
{
    struct Case
    {
        const char* name;
        std::function<void()> fn;
    };
    std::vector<Case>& cases()
    {
        static std::vector<Case> c;
        return c;
    }
    struct Registrar
    {
        Registrar(const char* n, std::function<void()> f) { cases().push_back({ n, std::move(f) }); }
    };
    struct Failure
    {
        std::string what;
    };

#define TEST_CASE(name)                                \
    static void name();                                \
    static Registrar reg_##name(#name, name);          \
    static void name()

#define CHECK(cond)                                                                                     \
    do                                                                                                  \
    {                                                                                                   \
        if (!(cond))                                                                                    \
            throw Failure{ std::string(__FILE__) + ":" + std::to_string(__LINE__) + ": " + #cond };    \
    } while (0)

    const Variant kCuda[] = { Variant::CudaBruteForce, Variant::CudaBruteForceAoS, Variant::CudaBarnesHut,
                              Variant::CudaBruteForceCompensated };

    // A central mass with a disk of stars on near-circular orbits, in the spirit of the
    // reference's util::disk (source/util.cpp:14-98): deterministic, own generator.
    void seed_disk(Sim& sim, const size_t n, const Vector center = { 0, 0, 0 }, const float outer = 100.f)
    {
        std::vector<Body>& b = sim.mutable_bodies();
        const size_t first = b.size();
        b.resize(first + n);
        if (n == 0)
            return;
        const float M = 4.1e6f, inner = 45.88f;
        b[first] = Body{ .pos = center, .radius = inner, .mass = M };
        uint64_t s = 0x9e3779b97f4a7c15ull + first;
        auto u01 = [&] {
            s = s * 6364136223846793005ull + 1442695040888963407ull;
            return static_cast<float>((s >> 40) & 0xffffff) / 16777216.f;
        };
        for (size_t i = 1; i < n; ++i)
        {
            const float r = inner + std::sqrt(u01()) * (outer - inner);
            const float a = 6.2831853f * static_cast<float>(i) / static_cast<float>(n > 1 ? n - 1 : 1);
            const float z = (u01() - .5f) * 2.f;
            const float v = std::sqrt(M / r);
            b[first + i] = Body{ .pos = { center.x + r * std::cos(a), center.y + r * std::sin(a), center.z + z },
                                 .radius = 0.2867f,
                                 .vel = { -v * std::sin(a), v * std::cos(a), 0 },
                                 .mass = 1.f };
        }
    }

    float rel_acc_error(const std::vector<Body>& a, const std::vector<Body>& b)
    {
        float worst = 0.f;
        for (size_t i = 0; i < a.size(); ++i)
        {
            const float mag = a[i].acc.size();
            if (mag <= 0.f)
                continue;
            worst = std::max(worst, (b[i].acc - a[i].acc).size() / mag);
        }
        return worst;
    }

    std::vector<Body> cpu(const std::vector<Body>& in, const bool barnes_hut, const float size, const float theta,
                          const float G)
    {
        std::vector<Body> out = in;
        float* f = reinterpret_cast<float*>(out.data());
        if (barnes_hut)
            orc_barnes_hut(f, out.size(), size, theta, G, 0, nullptr);
        else
            orc_brute_force(f, out.size(), G, 0);
        return out;
    }
}

TEST_CASE(every_variant_reports_itself_consistently)
{
    const auto all = Sim::variants();
    CHECK(all.size() == size_t(Variant::Count));
    for (size_t i = 0; i < all.size(); ++i)
    {
        CHECK(size_t(all[i].variant) == i);
        CHECK(std::strlen(all[i].name) > 0);
        if (!all[i].available)
            CHECK(!all[i].unavailable_reason.empty());
        else
        {
            Sim sim(all[i].variant);
            CHECK(sim.variant() == all[i].variant);
            seed_disk(sim, 32);
            sim.update(1.f / 120.f);
        }
    }
    for (const Variant v : kCuda)
        CHECK(Sim::available(v));
    CHECK(!Sim::available(Variant::Count));
    Sim sim;
    CHECK(!sim.set_variant(Variant::Count));
}

TEST_CASE(state_survives_a_variant_round_trip)
{
    Sim sim(Variant::CudaBarnesHut);
    seed_disk(sim, 512);
    for (int i = 0; i < 10; ++i)
        sim.update(1.f / 120.f);
    const auto before = sim.state();
    const std::vector<Body> snapshot = before->bodies;
    CHECK(sim.set_variant(Variant::CudaBruteForce));
    CHECK(sim.state() == before);
    CHECK(sim.bodies().size() == snapshot.size());
    for (size_t i = 0; i < snapshot.size(); ++i)
        CHECK(sim.bodies()[i].pos == snapshot[i].pos);
    CHECK(sim.tree() == nullptr);
    CHECK(sim.nodes().empty());
    CHECK(sim.set_variant(Variant::CudaBarnesHut));
    sim.accelerate();
    CHECK(sim.tree() != nullptr);
    CHECK(sim.nodes().size() > 1);
    float total = 0.f;
    for (const Body& b : sim.bodies())
        total += b.mass;
    CHECK(std::abs(sim.nodes()[0].mass - total) <= 1e-6f * total);
}

TEST_CASE(settings_carry_across_a_variant_switch)
{
    Sim sim(Variant::CudaBarnesHut);
    sim.set_size(1234.f);
    sim.set_theta(.25f);
    sim.set_gravity(2.f);
    sim.set_wrap(false);
    CHECK(sim.set_variant(Variant::CudaBruteForceAoS));
    CHECK(sim.size() == 1234.f && sim.theta() == .25f && sim.gravity() == 2.f && !sim.wrap());
}

TEST_CASE(switching_to_an_unavailable_variant_is_a_no_op_with_a_reason)
{
    Sim sim(Variant::CudaBruteForce);
    CHECK(!sim.set_variant(Variant::CpuBarnesHut));
    CHECK(sim.variant() == Variant::CudaBruteForce);
    CHECK(!sim.last_error().empty());
    seed_disk(sim, 64);
    sim.update(1.f / 120.f);
    CHECK(sim.bodies().size() == 64);
}

TEST_CASE(every_variant_picks_up_bodies_added_after_a_step)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        seed_disk(sim, 128);
        sim.update(1.f / 120.f);
        const size_t first = sim.bodies().size();
        seed_disk(sim, 64, { 400.f, 0.f, 0.f }, 50.f);
        sim.update(1.f / 120.f);
        CHECK(sim.bodies().size() == first + 64);
        size_t accelerated = 0;
        for (size_t i = first + 1; i < sim.bodies().size(); ++i)
            if (sim.bodies()[i].acc.size_sq() > 0.f)
                ++accelerated;
        CHECK(accelerated == 63);
    }
}

TEST_CASE(every_variant_tolerates_bodies_with_no_radius)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        auto& b = sim.mutable_bodies();
        b.resize(3);
        b[0] = Body{ .pos = { 0, 0, 0 }, .mass = 1000.f };
        b[1] = Body{ .pos = { 100, 0, 0 }, .mass = 1.f };
        b[2] = Body{ .pos = { 0, 100, 0 }, .mass = 1.f };
        sim.update(1.f / 120.f);
        for (const Body& x : sim.bodies())
            CHECK(std::isfinite(x.acc.x) && std::isfinite(x.acc.y) && std::isfinite(x.acc.z) &&
                  std::isfinite(x.pos.x) && std::isfinite(x.pos.y) && std::isfinite(x.pos.z));
        CHECK(sim.bodies()[1].acc.x < 0.f);
        CHECK(sim.bodies()[2].acc.y < 0.f);
    }
}

TEST_CASE(every_variant_steps_with_no_bodies)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        CHECK(sim.bodies().empty());
        sim.update(1.f / 120.f);
        CHECK(sim.bodies().empty());
        seed_disk(sim, 32);
        sim.update(1.f / 120.f);
        CHECK(sim.bodies().size() == 32);
    }
}

static void setup_drifting(Sim& sim)
{
    sim.set_size(1000.f);
    sim.set_gravity(0.f);
    sim.mutable_bodies().resize(1);
    sim.mutable_bodies()[0] = Body{ .pos = { 499.f, 0.f, 0.f }, .radius = 1.f, .vel = { 10.f, 0.f, 0.f }, .mass = 1.f };
}

TEST_CASE(every_variant_wraps_and_agrees_on_where)
{
    std::vector<Body> ref(1);
    ref[0] = Body{ .pos = { 499.f, 0.f, 0.f }, .radius = 1.f, .vel = { 10.f, 0.f, 0.f }, .mass = 1.f };
    orc_integrate(reinterpret_cast<float*>(ref.data()), 1, 1.f, 1000.f, 1);
    for (const Variant v : { Variant::CudaBruteForce, Variant::CudaBruteForceAoS, Variant::CudaBarnesHut })
    {
        Sim sim(v);
        setup_drifting(sim);
        sim.update(1.f);
        const Vector p = sim.bodies()[0].pos;
        CHECK(std::abs(p.x) <= 500.f && std::abs(p.y) <= 500.f && std::abs(p.z) <= 500.f);
        CHECK(p == ref[0].pos);
        Sim off(v);
        setup_drifting(off);
        off.set_wrap(false);
        off.update(1.f);
        CHECK(off.bodies()[0].pos.x > 500.f);
    }
}

TEST_CASE(integrating_first_thing_works)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        seed_disk(sim, 256);
        const Vector from = sim.bodies()[3].pos;
        sim.mutable_bodies()[3].vel = { 10.f, 0.f, 0.f };
        sim.mutable_bodies()[3].acc = { 0.f, 0.f, 0.f };
        sim.set_wrap(false);
        sim.integrate(.1f);
        const Vector expected = from + Vector{ 1.f, 0.f, 0.f };
        CHECK((sim.bodies()[3].pos - expected).size() < 1e-2f);
    }
}

TEST_CASE(stepping_blind_agrees_with_stepping_while_reading)
{
    for (const Variant v : { Variant::CudaBarnesHut, Variant::CudaBruteForce })
    {
        Sim seed(v);
        seed_disk(seed, 8192);
        const std::vector<Body> initial = seed.bodies();
        auto run = [&](const bool reading) {
            Sim sim(v);
            sim.mutable_bodies() = initial;
            for (int i = 0; i < 64; ++i)
            {
                sim.update(.02f);
                if (reading)
                    CHECK(sim.bodies().size() == 8192);
            }
            return sim.bodies();
        };
        const auto blind = run(false);
        const auto reading = run(true);
        float worst = 0.f;
        for (size_t i = 0; i < blind.size(); ++i)
            worst = std::max({ worst, (blind[i].pos - reading[i].pos).size(), (blind[i].vel - reading[i].vel).size() });
        CHECK(worst < 1e-3f);
    }
}

TEST_CASE(reading_bodies_materializes_the_device_work)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        seed_disk(sim, 1024);
        sim.accelerate();
        size_t moving = 0;
        for (size_t i = 1; i < sim.bodies().size(); ++i)
            if (sim.bodies()[i].acc.size_sq() > 0.f)
                ++moving;
        CHECK(moving > 0);
    }
}

TEST_CASE(a_mutation_reaches_the_device_on_the_integrate_only_path)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        seed_disk(sim, 256);
        sim.update(1.f / 120.f);
        const Vector marker = { 4000.f, 0.f, 0.f };
        sim.mutable_bodies()[7].pos = marker;
        sim.mutable_bodies()[7].vel = {};
        sim.mutable_bodies()[7].acc = {};
        sim.integrate(1.f / 120.f);
        const Vector p = sim.bodies()[7].pos;
        CHECK(std::abs(p.x - marker.x) < 1e-2f && std::abs(p.y) < 1e-2f && std::abs(p.z) < 1e-2f);
    }
}

TEST_CASE(a_mutation_is_visible_through_the_read_path_and_survives_a_switch)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        seed_disk(sim, 256);
        sim.update(1.f / 120.f);
        const Vector marker = { 12.f, -34.f, 56.f };
        sim.mutable_bodies()[7].pos = marker;
        CHECK(sim.bodies()[7].pos == marker);
        sim.mutable_bodies()[5].pos = { 1.f, 2.f, 3.f };
        const Variant other = v == Variant::CudaBarnesHut ? Variant::CudaBruteForce : Variant::CudaBarnesHut;
        CHECK(sim.set_variant(other));
        CHECK(sim.bodies()[5].pos == (Vector{ 1.f, 2.f, 3.f }));
        CHECK(sim.bodies()[7].pos == marker);
    }
}

TEST_CASE(cuda_barnes_hut_agrees_with_cpu_barnes_hut)
{
    Sim sim(Variant::CudaBarnesHut);
    seed_disk(sim, 2048);
    const std::vector<Body> in = sim.bodies();
    sim.accelerate();
    const auto dev = sim.bodies();
    const auto ref = cpu(in, true, sim.size(), sim.theta(), sim.gravity());
    CHECK(dev[1].acc.size_sq() > 0.f && ref[1].acc.size_sq() > 0.f);
    CHECK(rel_acc_error(ref, dev) < 1e-2f);
}

TEST_CASE(cuda_brute_force_agrees_with_cpu_brute_force)
{
    for (const Variant v : { Variant::CudaBruteForce, Variant::CudaBruteForceAoS, Variant::CudaBruteForceCompensated })
    {
        Sim sim(v);
        seed_disk(sim, 1024);
        const std::vector<Body> in = sim.bodies();
        CHECK(sim.tree() == nullptr);
        sim.accelerate();
        const auto dev = sim.bodies();
        const auto ref = cpu(in, false, sim.size(), sim.theta(), sim.gravity());
        CHECK(rel_acc_error(ref, dev) < 1e-4f);
    }
}

TEST_CASE(every_variant_honors_the_gravitational_constant)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        seed_disk(sim, 256);
        sim.set_gravity(1.f);
        sim.accelerate();
        const float base = sim.bodies()[1].acc.size();
        CHECK(base > 0.f);
        sim.set_gravity(4.f);
        sim.accelerate();
        CHECK(std::abs(sim.bodies()[1].acc.size() / base - 4.f) < 0.01f);
    }
}

TEST_CASE(shrinking_the_body_count_does_not_corrupt_memory)
{
    for (const Variant v : kCuda)
    {
        Sim sim(v);
        seed_disk(sim, 4096);
        sim.update(1.f / 60.f);
        sim.mutable_bodies().resize(16);
        sim.update(1.f / 60.f);
        CHECK(sim.bodies().size() == 16);
    }
}

TEST_CASE(switching_between_cuda_variants_repeatedly)
{
    Sim sim(Variant::CudaBarnesHut);
    seed_disk(sim, 512);
    sim.update(1.f / 120.f);
    for (int i = 0; i < 3; ++i)
    {
        CHECK(sim.set_variant(Variant::CudaBruteForce));
        sim.update(1.f / 120.f);
        CHECK(sim.set_variant(Variant::CudaBarnesHut));
        sim.update(1.f / 120.f);
    }
    CHECK(sim.bodies().size() == 512);
}

TEST_CASE(orbits_neither_decay_nor_escape)
{
    Sim sim(Variant::CudaBarnesHut);
    sim.set_wrap(false);
    seed_disk(sim, 16);
    std::vector<float> initial;
    std::vector<Vector> prev;
    for (const Body& b : sim.bodies())
    {
        initial.push_back(b.pos.size());
        prev.push_back(b.pos);
    }
    std::vector<float> path(16, 0.f);
    for (int s = 0; s < 400; ++s)
    {
        sim.update(1.f / 120.f);
        for (size_t i = 0; i < 16; ++i)
        {
            path[i] += (sim.bodies()[i].pos - prev[i]).size();
            prev[i] = sim.bodies()[i].pos;
        }
    }
    float drift = 0.f, least = 1e30f;
    for (size_t i = 1; i < 16; ++i)
    {
        drift = std::max(drift, std::abs(sim.bodies()[i].pos.size() - initial[i]) / initial[i]);
        least = std::min(least, path[i] / initial[i]);
    }
    CHECK(least > 3.14f);
    CHECK(drift < 0.10f);
}

TEST_CASE(every_body_is_integrated_regardless_of_body_count)
{
    for (const size_t n : { 2, 3, 5, 16, 129 })
    {
        Sim sim(Variant::CudaBarnesHut);
        seed_disk(sim, n);
        std::vector<Vector> before;
        for (const Body& b : sim.bodies())
            before.push_back(b.pos);
        for (int i = 0; i < 10; ++i)
            sim.update(1.f / 120.f);
        for (size_t i = 1; i < n; ++i)
            CHECK(sim.bodies()[i].pos.dist_sq(before[i]) > 0.f);
    }
}

TEST_CASE(the_exported_tree_walks_like_the_reference)
{
    Sim sim(Variant::CudaBarnesHut);
    seed_disk(sim, 2048);
    sim.accelerate();
    const auto nodes = sim.nodes();
    const auto bodies = sim.bodies();
    std::vector<float> acc(3 * bodies.size());
    uint64_t inter = 0;
    orc_nodes_accel(reinterpret_cast<const orc_node*>(nodes.data()), nodes.size(),
                    reinterpret_cast<const float*>(bodies.data()), bodies.size(), nullptr, 0, sim.theta(),
                    sim.gravity(), acc.data(), &inter, 0);
    float worst = 0.f;
    for (size_t i = 1; i < bodies.size(); ++i)
    {
        const Vector a = { acc[3 * i], acc[3 * i + 1], acc[3 * i + 2] };
        worst = std::max(worst, (a - bodies[i].acc).size() / bodies[i].acc.size());
    }
    CHECK(inter > 0 && worst < 1e-2f);
}

// util::disk appended after existing bodies, as test_variant.cpp:150-160 grows a scene:
// generated on the device by every CUDA variant, against the oracle's util::disk.
TEST_CASE(every_variant_generates_the_reference_disk_on_the_device)
{
    const size_t keep = 257, added = 3001;
    const float args14[14] = { 1.f, 2.f, 3.f, 0.f, 0.5f, 0.f, 0.f, 0.f, 1.f, 0.f, 100.f, 1.f, 4.1e6f, 1.f };
    std::vector<float> want(12 * added);
    orc_disk(want.data(), added, args14);
    for (Variant v : kCuda)
    {
        Sim sim(v);
        seed_disk(sim, keep);
        const std::vector<Body> before = sim.bodies();
        sim.mutable_bodies().resize(keep + added);
        nbody::util::DiskArgs args{ .center = { 1.f, 2.f, 3.f }, .vel = { 0.f, 0.5f, 0.f } };
        args.outer_radius = 100.f;
        sim.disk(keep, keep + added, args);
        const std::vector<Body>& got = sim.bodies();
        CHECK(got.size() == keep + added);
        CHECK(std::memcmp(got.data(), before.data(), keep * sizeof(Body)) == 0);
        size_t exact = 0;
        float worst_pos = 0.f, worst_vel = 0.f;
        for (size_t i = 0; i < added; ++i)
        {
            const Body& g = got[keep + i];
            Body w;
            std::memcpy(&w, want.data() + 12 * i, sizeof w);
            CHECK(g.mass == w.mass && g.radius == w.radius);
            exact += g.pos == w.pos;
            worst_pos = std::max(worst_pos, (g.pos - w.pos).size());
            if (w.vel.size() > 0.f)
                worst_vel = std::max(worst_vel, (g.vel - w.vel).size() / w.vel.size());
        }
        CHECK(worst_pos <= 1e-6f * 103.f);
        CHECK(exact * 10 >= added * 9);
        CHECK(worst_vel <= 1e-5f);
        // and it steps from there like any other scene
        sim.update(1.f / 120.f);
        CHECK(std::isfinite(sim.bodies()[keep + added - 1].pos.x));
    }
}

TEST_CASE(every_variant_generates_the_reference_cube_on_the_device)
{
    const size_t n = 4096;
    const float args8[8] = { 0.f, 0.f, 0.f, 500.f, 0.f, 0.f, 0.f, 1.f };
    std::vector<float> want(12 * n);
    orc_cube(want.data(), n, args8);
    for (Variant v : kCuda)
    {
        Sim sim(v);
        sim.mutable_bodies().resize(n);
        sim.cube(0, n);
        const std::vector<Body>& got = sim.bodies();
        for (size_t i = 0; i < n; ++i)
            CHECK(std::memcmp(&got[i], want.data() + 12 * i, 44) == 0);
    }
}

TEST_CASE(a_generated_range_outside_the_bodies_throws)
{
    Sim sim(Variant::CudaBruteForce);
    sim.mutable_bodies().resize(10);
    bool threw = false;
    try
    {
        sim.disk(5, 11);
    }
    catch (const std::out_of_range&)
    {
        threw = true;
    }
    CHECK(threw);
}

TEST_CASE(a_solver_constructed_without_a_device_throws_a_reason)
{
    // The probe result, not a fault: with the injected no-device fault the constructor throws
    // and Sim demotes the variant with the message (source/sim.cpp:226-239).
    setenv("NBODY_CUDA_FAULT", "nodevice", 1);
    bool threw = false;
    std::string msg;
    try
    {
        auto state = std::make_shared<nbody::State>();
        nbody::CudaSolver s(nullptr, state, {});
    }
    catch (const std::runtime_error& e)
    {
        threw = true;
        msg = e.what();
    }
    unsetenv("NBODY_CUDA_FAULT");
    CHECK(threw && msg.find("injected") != std::string::npos);
}

int main(int argc, char** argv)
{
    int failed = 0, run = 0;
    for (const Case& c : cases())
    {
        if (argc > 1 && std::string(argv[1]) != c.name)
            continue;
        ++run;
        try
        {
            c.fn();
            std::printf("PASS %s\n", c.name);
        }
        catch (const Failure& f)
        {
            ++failed;
            std::printf("FAIL %s: %s\n", c.name, f.what.c_str());
        }
        catch (const std::exception& e)
        {
            ++failed;
            std::printf("FAIL %s: exception %s\n", c.name, e.what());
        }
        std::fflush(stdout);
    }
    std::printf("%d of %d passed\n", run - failed, run);
    return failed ? 1 : 0;
}
