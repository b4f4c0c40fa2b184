"""The oracle pinned against the reference (CPU only).

Two kinds of pin: the reference's own known answers (tests/source/test_bhtree.cpp) and
bit-for-bit agreement with fixtures produced by the reference itself
(tests/golden/make_golden.py). When the reference was also built here (oracle/_ref), the
restatement is additionally compared with it live on fresh inputs.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O


def node_array(raw):
    return np.frombuffer(raw.tobytes(), dtype=O.NODE_DTYPE)


def restated_nodes(points, size=100.0):
    t = O.Tree(size)
    for p in np.asarray(points, np.float32):
        t.insert(p[:3], p[3])
    return t.nodes()


# --- reference known answers (test_bhtree.cpp) -------------------------------------------

def test_tree_known_answers_two_quadrants():
    # test_bhtree.cpp:40-71: 1 node, then 9; root mass 3 and COM the weighted mean
    t = O.Tree(100.0)
    t.insert((1, 1, 1), 1)
    n = t.nodes()
    assert len(n) == 1 and n[0]["mass"] == 1 and tuple(n[0]["com"]) == (1, 1, 1)
    t.insert((-1, -1, -1), 2)
    n = t.nodes()
    assert len(n) == 9 and n[0]["mass"] == 3
    np.testing.assert_allclose(n[0]["com"], (-1 / 3, -1 / 3, -1 / 3), rtol=1e-5, atol=1e-5)
    # child slot = 1 + quadrant, quadrant bit set when the coordinate is below centre
    assert n[1 + 0]["mass"] == 1 and n[1 + 7]["mass"] == 2


def test_tree_known_answers_same_quadrant():
    # test_bhtree.cpp:73-113: 17 nodes, intermediate cell holds both
    n = restated_nodes([[1, 1, 1, 1], [99, 99, 99, 1]])
    assert len(n) == 17 and n[0]["mass"] == 2
    np.testing.assert_allclose(n[0]["com"], (50, 50, 50), rtol=1e-5)
    c = n[0]["children"]
    assert n[c]["mass"] == 2


def test_tree_known_answers_eight():
    # test_bhtree.cpp:115-142: exact COMs {0,50,50} etc.
    t = O.Tree(100.0)
    t.insert((50, 50, 50), 1)
    t.insert((-50, 50, 50), 1)
    n = t.nodes()
    assert len(n) == 9 and n[0]["mass"] == 2
    assert tuple(n[0]["com"]) == (0, 50, 50)
    assert tuple(n[1]["com"]) == (50, 50, 50) and tuple(n[2]["com"]) == (-50, 50, 50)
    t.insert((50, -50, 50), 1)
    n = t.nodes()
    assert len(n) == 9 and n[0]["mass"] == 3
    assert tuple(n[3]["com"]) == (50, -50, 50)


def test_tree_coincident_terminates():
    # test_bhtree.cpp:148-167
    n = restated_nodes([[1, 1, 1, 1], [1, 1, 1, 1]])
    assert len(n) > 1 and n[0]["mass"] == 2
    n = restated_nodes([[1, 1, 1, 1], [1 + np.finfo(np.float32).eps, 1, 1, 1]])
    assert len(n) > 1 and n[0]["mass"] == 2


def test_tree_mass_conserved_100k():
    # test_bhtree.cpp:169-212 (normal(0, .5) clamped, x100, in a 200 box)
    g = np.random.default_rng(5)
    p = np.clip(g.normal(0, 0.5, (100000, 3)), -1, 1).astype(np.float32) * 100
    b = np.zeros((len(p), 12), np.float32)
    b[:, :3] = p
    b[:, 7] = 1
    t = O.Tree(200.0)
    t.build(b, 200.0)
    assert t.nodes()[0]["mass"] == 100000.0


def test_apply_far_particles_one_visit():
    # test_bhtree.cpp:218-257: one visit for one far body and for a far pair
    b = np.zeros((2, 12), np.float32)
    b[0, :3] = (100, 100, 100)
    b[0, 7] = 1
    b[1, :3] = (99, 99, 99)
    b[1, 7] = 1
    t = O.Tree(200.0)
    t.build(b[:1], 200.0)
    tgt = np.zeros((1, 12), np.float32)
    _, inter = t.accel(tgt, 0.5, 1.0)
    assert inter == 1
    t.build(b, 200.0)
    _, inter = t.accel(tgt, 0.5, 1.0)
    assert inter == 1


def test_theta_convention_accuracy():
    # test_bhtree.cpp:259-367: larger theta is more accurate (inverted convention)
    g = np.random.default_rng(11)
    p = np.clip(g.normal(0, 0.5, (100, 3)), -1, 1).astype(np.float32) * 100
    b = np.zeros((100, 12), np.float32)
    b[:, :3] = p
    b[:, 7] = 1
    exact = O.brute_force(b, 1.0)[:, 8:11].astype(np.float64)
    mean_force = np.linalg.norm(exact, axis=1).mean()
    t = O.Tree(200.0)
    t.build(b, 200.0)
    loose, li = t.accel(b, 0.5, 1.0)
    tight, ti = t.accel(b, 8.0, 1.0)
    el = np.linalg.norm(loose - exact, axis=1).max() / mean_force
    et = np.linalg.norm(tight - exact, axis=1).max() / mean_force
    assert et < el and et < 0.05 and el < 3.0
    assert ti > li > 0 and ti < 100 * 100


# --- the softened law (the benchmark configurations' law; no reference counterpart) ------------

def test_softened_pair_against_fp64():
    """orc_gravity_softened is G*m*d/(|d|^2 + eps2)^(3/2) to FP32 rounding."""
    g = np.random.default_rng(21)
    for _ in range(200):
        x, s = g.normal(0, 1, 3).astype(np.float32), g.normal(0, 1, 3).astype(np.float32)
        m, eps2 = np.float32(g.uniform(0.1, 2)), np.float32(10.0 ** g.uniform(-6, 0))
        got = O.gravity_softened(x, s, m, 1.5, eps2)
        d = s.astype(np.float64) - x
        want = 1.5 * float(m) * d / (d @ d + float(eps2)) ** 1.5
        assert np.linalg.norm(got - want) <= 4e-7 * np.linalg.norm(want)


@pytest.mark.parametrize("fixture", ["disk_1024.npz", "cube_4096.npz"])
def test_softened_visitor_at_vanishing_eps_is_the_reference_walk(fixture):
    """The softened visitor follows the reference's walk and opening test unchanged: with
    eps2 far below every |d|^2 (and radii 0, so the cutoff only drops d = 0) it adds exactly
    the terms of the reference-law walk, which the fixtures pin to the reference bit for
    bit, and so gives the same bits and the same interaction count."""
    b = golden(fixture)["bodies"].copy()
    b[:, 3] = 0.0
    t = O.Tree(10000.0)
    t.build(b, 10000.0)
    for theta in (0.5, 2.0):
        ref, ri = t.accel(b, theta, 1.0)
        soft, si = t.accel(b, theta, 1.0, law=O.LAW_SOFTENED, eps2=1e-30)
        assert si == ri
        assert np.array_equal(soft.view(np.uint32), ref.view(np.uint32))
    bh, _ = O.barnes_hut(b, 10000.0, 0.5, 1.0, law=O.LAW_SOFTENED, eps2=1e-30)
    assert np.array_equal(bh[:, 8:11], t.accel(b, 0.5, 1.0)[0])


def test_softened_brute_force_against_fp64():
    """The softened brute force (the reference's loop, cpu_brute_force.h:17-43, with the
    softened pair) sits within FP32 summation error of the FP64 softened sum."""
    from nbody_gb300 import scenes
    b = scenes.plummer(2048, seed=77)
    eps2 = 1e-4
    tg = np.arange(0, 2048, 7)
    a = O.brute_force_targets(b, 1.0, tg, law=O.LAW_SOFTENED, eps2=eps2)
    a64, scale = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(eps2)), O.LAW_SOFTENED, targets=tg,
                              with_scale=True)
    err = np.linalg.norm(a - a64, axis=1) / scale
    assert err.max() < 5e-6 and np.median(err) < 1e-6


def test_softened_theta_convention_accuracy():
    """test_bhtree.cpp:259-367 with the softened visitor (eps = 1 on a 100-unit cloud):
    reference theta 8 is accurate (< 0.05 of the mean force), 0.5 loose (< 3.0)."""
    g = np.random.default_rng(11)
    p = np.clip(g.normal(0, 0.5, (100, 3)), -1, 1).astype(np.float32) * 100
    b = np.zeros((100, 12), np.float32)
    b[:, :3] = p
    b[:, 7] = 1
    exact = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, 1.0, O.LAW_SOFTENED)
    mean_force = np.linalg.norm(exact, axis=1).mean()
    t = O.Tree(200.0)
    t.build(b, 200.0)
    loose, li = t.accel(b, 0.5, 1.0, law=O.LAW_SOFTENED, eps2=1.0)
    tight, ti = t.accel(b, 8.0, 1.0, law=O.LAW_SOFTENED, eps2=1.0)
    el = np.linalg.norm(loose - exact, axis=1).max() / mean_force
    et = np.linalg.norm(tight - exact, axis=1).max() / mean_force
    assert et < el and et < 0.05 and el < 3.0
    assert ti > li > 0


# --- bit-for-bit against the reference's own outputs ---------------------------------------

@pytest.mark.parametrize("n", [512, 1024, 2048])
def test_restatement_matches_reference_fixtures(n):
    g = golden(f"disk_{n}.npz")
    b = g["bodies"]
    assert np.array_equal(O.brute_force(b, 1.0)[:, 8:11], g["bf_acc"])
    bh, _ = O.barnes_hut(b, 10000.0, 0.5, 1.0)
    assert np.array_equal(bh[:, 8:11], g["bh_acc"])
    s = b.copy()
    for _ in range(5):
        s = O.integrate(O.brute_force(s, 1.0), 1.0 / 120.0, 10000.0, True)
    assert np.array_equal(s, g["steps"])


def test_restatement_matches_reference_cube():
    g = golden("cube_4096.npz")
    b = g["bodies"]
    assert np.array_equal(O.brute_force(b, 1.0)[:, 8:11], g["bf_acc"])
    bh, _ = O.barnes_hut(b, 10000.0, 0.5, 1.0)
    assert np.array_equal(bh[:, 8:11], g["bh_acc"])
    t = O.Tree(10000.0)
    t.build(b, 10000.0)
    assert t.nodes().tobytes() == g["nodes"].tobytes()


def test_restatement_matches_reference_tree_cases():
    g = golden("bhtree_cases.npz")
    names = sorted({k.rsplit("_", 1)[0] for k in g})
    assert len(names) == 5
    for name in names:
        assert restated_nodes(g[f"{name}_points"]).tobytes() == g[f"{name}_nodes"].tobytes(), name


@pytest.mark.skipif(not O.ref_available(), reason="reference sources not present on this machine")
def test_restatement_matches_reference_live():
    g = np.random.default_rng(3)
    b = O.ref_cube(3000)
    b[:, 4:7] = g.normal(0, 1, (3000, 3))
    assert np.array_equal(O.ref_brute_force(b, 2.0), O.brute_force(b, 2.0))
    r = O.ref_barnes_hut(b, 10000.0, 0.75, 2.0)
    o, _ = O.barnes_hut(b, 10000.0, 0.75, 2.0)
    assert np.array_equal(r, o)
    assert np.array_equal(O.ref_integrate(b, 0.37, 300.0, True), O.integrate(b, 0.37, 300.0, True))


# --- the FP64 checker and the integrator ------------------------------------------------------

def test_wrap_known_answer():
    # test_wrap.cpp:17-56: x=499, v=10, dt=1, size=1000 lands inside the box
    b = np.zeros((1, 12), np.float32)
    b[0, 0] = 499
    b[0, 4] = 10
    out = O.integrate(b, 1.0, 1000.0, True)
    assert abs(out[0, 0]) <= 500 and out[0, 0] == np.float32(-491.0)
    out = O.integrate(b, 1.0, 1000.0, False)
    assert out[0, 0] > 500


def test_f64_matches_fp32_reference_law():
    g = golden("disk_1024.npz")
    b = g["bodies"]
    pm = b[:, [0, 1, 2, 7]]
    a64, scale = O.direct_f64(pm, 1.0, law=O.LAW_CUTOFF, radius=b[:, 3], with_scale=True)
    # The reference's own FP32 sequential sum sits up to ~1.9e-5 (in units of the sum of
    # pair magnitudes) from the FP64 sum on this input: a 4.1e6 central mass swamps the
    # 1023 unit-mass terms added after it.
    err = np.linalg.norm(a64 - g["bf_acc"], axis=1) / scale
    assert err.max() < 5e-5 and np.median(err) < 1e-5


def test_f64_energy_two_body():
    pos = np.array([[0.0, 0, 0], [1.0, 0, 0]])
    vel = np.array([[0.0, 1, 0], [0.0, -1, 0]])
    m = np.array([2.0, 3.0])
    ke, pe, mom = O.energy_f64(pos, vel, m, 1.0, 0.0)
    assert ke == pytest.approx(0.5 * 2 + 0.5 * 3)
    assert pe == pytest.approx(-6.0)
    np.testing.assert_allclose(mom, [0, -1, 0])


# --- Morton codes: exact cells of the reference octree -------------------------------------

def test_morton_cells_match_reference_octants():
    """For a power-of-two box at the origin the Morton digits are the reference's octants
    (bounds.h:31-38) with bits flipped: reference bit set means below the centre."""
    g = np.random.default_rng(9)
    size = 64.0
    p = g.uniform(-32, 32, (2000, 3)).astype(np.float32)
    p[:10] = 0.0                      # exactly on every centre plane
    p[10:20] = -np.float32(1e-30)     # tiny negatives: below the centre
    codes = O.morton63(p, np.array([-32.0] * 3), 2.0 ** 21 / size)
    for i in range(len(p)):
        cx = cy = cz = 0.0
        s = size
        for level in range(12):
            ref_q = int(p[i, 0] < cx) | (int(p[i, 1] < cy) << 1) | (int(p[i, 2] < cz) << 2)
            digit = int(codes[i] >> np.uint64(3 * (20 - level))) & 7
            assert digit == ref_q ^ 7, (i, level)
            q = s * 0.25
            cx += -q if ref_q & 1 else q
            cy += -q if ref_q & 2 else q
            cz += -q if ref_q & 4 else q
            s *= 0.5


def test_sort_order_stable():
    codes = np.array([5, 3, 5, 1, 3, 3], np.uint64)
    assert list(O.sort_order(codes)) == [3, 1, 4, 5, 0, 2]


# --- properties of the reference semantics (the ones the GPU tests check at full size) ----

def test_reference_semantics_scale_exactly_with_mass():
    """Doubling every mass doubles every acceleration bit for bit in the reference's brute
    force and in its octree (the running-mean centres of mass of bhtree.cpp:87-95 are
    unchanged by a power-of-two factor), both in the restatement and, where it was built,
    in the reference itself."""
    from nbody_gb300 import scenes
    b = scenes.plummer(2048, seed=11)
    b2 = b.copy()
    b2[:, 7] *= 2.0
    bf = [O.brute_force(x, 1.0)[:, 8:11] for x in (b, b2)]
    assert np.array_equal(bf[1], 2.0 * bf[0])
    bh = [O.barnes_hut(x, 64.0, 0.5, 1.0)[0][:, 8:11] for x in (b, b2)]
    assert np.array_equal(bh[1], 2.0 * bh[0])
    if O.ref_available():
        rb = [O.ref_barnes_hut(x, 64.0, 0.5, 1.0)[:, 8:11] for x in (b, b2)]
        assert np.array_equal(rb[1], 2.0 * rb[0])
        assert np.array_equal(rb[0], bh[0])


def test_reference_brute_force_momentum_residual():
    """With every radius 0 the reference's force law is antisymmetric, so sum_i m_i a_i = 0
    up to FP32 rounding. Its own sequential FP32 sum leaves under 1e-7 of sum_i m_i |a_i|
    (about 3e-8 measured): the GPU property tests bound the same residual by 1e-6."""
    from nbody_gb300 import scenes
    b = scenes.plummer(4096, seed=12)
    a = O.brute_force(b, 1.0)[:, 8:11].astype(np.float64)
    m = b[:, 7].astype(np.float64)
    res = np.linalg.norm((m[:, None] * a).sum(0)) / (m * np.linalg.norm(a, axis=1)).sum()
    assert res < 1e-7
