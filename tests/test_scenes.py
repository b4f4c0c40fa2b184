"""Scene generators on the CPU: the oracle's util::disk / util::cube restatement pinned to
the reference (fixtures and, where it is built, the reference itself), the random stream
pinned to the C++ standard's known answer, and the slot recurrence the device generator
parses the stream with, checked against a sequential replay of the reference's draws.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

CASES = golden("scenes.npz")


def case_names(kind):
    return sorted({k.split("_", 1)[1].rsplit("_", 1)[0] for k in CASES if k.startswith(kind + "_")})


def kwargs_from(kind, arr):
    a = [float(x) for x in arr]
    if kind == "disk":
        return dict(center=a[0:3], vel=a[3:6], axis=a[6:9], inner_radius=a[9], outer_radius=a[10],
                    thickness=a[11], central_mass=a[12], star_mass=a[13])
    return dict(center=a[0:3], size=a[3], vel=a[4:7], star_mass=a[7])


def test_engine_known_answer():
    """[rand.predef]: the 10000th value of a default-constructed minstd_rand0 is 1043618065."""
    assert O.minstd_value(9999) == 1043618065
    assert O.minstd_value(0) == 16807 and O.minstd_value(1) == 282475249


@pytest.mark.parametrize("name", case_names("disk"))
def test_disk_restatement_matches_reference_fixture(name):
    total, begin, num = CASES[f"disk_{name}_range"]
    kw = kwargs_from("disk", CASES[f"disk_{name}_args"])
    got = O.disk(int(num), **kw)
    want = CASES[f"disk_{name}_bodies"]
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("name", case_names("cube"))
def test_cube_restatement_matches_reference_fixture(name):
    total, begin, num = CASES[f"cube_{name}_range"]
    kw = kwargs_from("cube", CASES[f"cube_{name}_args"])
    got = O.cube(int(num), **kw)
    assert np.array_equal(got.view(np.uint32), CASES[f"cube_{name}_bodies"].view(np.uint32))


def test_disk_positions_only_matches_full():
    d = O.disk(5000, outer_radius=100.0)
    t = O.disk_positions(5000, 4000, 5000, outer_radius=100.0)
    assert np.array_equal(t[:, [0, 1, 2, 3, 7]], d[4000:, [0, 1, 2, 3, 7]])


@pytest.mark.skipif(O.ref_lib() is None, reason="the reference could not be built here")
@pytest.mark.parametrize("n", [65537, 200000])
def test_disk_restatement_matches_reference_live(n):
    kw = dict(outer_radius=120.0, axis=(0.3, -0.4, 0.866), inner_radius=5.0, thickness=0.5)
    want = O.ref_disk_range(np.zeros((n, 12), np.float32), 0, n, **kw)
    assert np.array_equal(O.disk(n, **kw).view(np.uint32), want.view(np.uint32))


# --- the device's stream parse, restated in numpy ------------------------------------------

def engine_values(count):
    x, out = 1, np.empty(count, np.uint64)
    for j in range(count):
        x = (x * 16807) % 2147483647
        out[j] = x
    return out


def canonical(x):
    f = (x.astype(np.int64) - 1).astype(np.float32) * np.float32(2.0 ** -31)
    return np.where(f >= 1, np.float32(np.nextafter(np.float32(1), np.float32(0))), f).astype(np.float32)


def accepted(u1, u2):
    x = np.float32(2) * u1 - np.float32(1)
    y = np.float32(2) * u2 - np.float32(1)
    r2 = x * x + y * y
    return ~((r2 > 1) | (r2 == 0))


def sequential_parse(stars, vals):
    """Replay the reference's draw order: per star one uniform, then one normal (a fresh
    polar pair for odd stars, the saved half for even ones). Returns, per star, the draw
    index of its uniform and the draw index of its pair's first value."""
    u = canonical(vals)
    at, uni, pair = 0, [], []
    saved_pair = None
    for i in range(1, stars + 1):
        uni.append(at)
        at += 1
        if saved_pair is None:
            while not accepted(u[at:at + 1], u[at + 1:at + 2])[0]:
                at += 2
            pair.append(at)
            saved_pair = at
            at += 2
        else:
            pair.append(saved_pair)
            saved_pair = None
    return np.array(uni), np.array(pair)


def slot_parse(stars, vals):
    """What the device computes: slot j = draws (2j+1, 2j+2); chosen_j = accepted_j and not
    chosen_{j-1}; chosen slot a_k serves stars 2k+1 (uniform at 2 a_{k-1} + 4, a_{-1} = -2)
    and 2k+2 (uniform at 2 a_k + 3)."""
    u = canonical(vals)
    slots = (len(vals) - 1) // 2
    acc = accepted(u[1:2 * slots:2], u[2:2 * slots + 1:2])
    chosen = np.zeros(slots, bool)
    prev = False
    for j in range(slots):      # the one-bit recurrence (the device resolves it per 64-slot word)
        chosen[j] = acc[j] and not prev
        prev = chosen[j]
    a = np.flatnonzero(chosen)[: (stars + 1) // 2]
    uni, pair = [], []
    for k, ak in enumerate(a):
        prev_a = a[k - 1] if k else -2
        uni.append(2 * prev_a + 4)
        pair.append(2 * ak + 1)
        if 2 * k + 2 <= stars:
            uni.append(2 * ak + 3)
            pair.append(2 * ak + 1)
    return np.array(uni[:stars]), np.array(pair[:stars])


@pytest.mark.parametrize("stars", [1, 2, 3, 10, 999, 4000])
def test_slot_recurrence_reproduces_the_draw_order(stars):
    vals = engine_values(3 * stars + 200)
    su, sp = sequential_parse(stars, vals)
    du, dp = slot_parse(stars, vals)
    assert np.array_equal(su, du) and np.array_equal(sp, dp)


def test_words_without_rejection_pass_the_carry():
    """A 64-slot word with every slot accepted flips the carry 64 times: it passes through."""
    for carry in (False, True):
        prev = carry
        for _ in range(64):
            prev = (not prev)
        assert prev == carry
