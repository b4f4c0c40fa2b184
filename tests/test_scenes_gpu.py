"""Device scene generators against the reference (fixtures) and the oracle, on the GPU.

Bars:
  * util::cube: bit-exact (the arithmetic is only the engine, one int -> float conversion,
    a power-of-two scaling and a multiply-add, all correctly rounded on both sides).
  * util::disk positions, radius, mass: radius and mass bit-exact; positions within
    1e-6 x (outer radius + |center|) for all bodies and bit-exact for at least 90 % of
    them. The rest trace back to sinf / cosf / logf: the device evaluates them in double
    and rounds once (correctly rounded), while glibc's float versions are accurate to
    0.82 ulp (logf) and so round the other way for a few percent of arguments; one logf
    serves the two stars of a polar pair.
  * util::disk velocities: relative error <= 1e-5. The reference folds a running FP32
    centre of mass over the nodes its own tree walk applies, which differs from the exact
    centre of mass by rounding only.
  * bodies outside the generated range: untouched, bit for bit.
"""
import numpy as np
import pytest

from oracle import oracle as O
from test_scenes import CASES, case_names, kwargs_from

pytestmark = pytest.mark.gpu


def prefix(n):
    return (np.arange(n * 12, dtype=np.float32).reshape(n, 12) % 97.0) - 48.0


def generate(native, kind, total, begin, num, kw, layout=0):
    with native.Context(layout) as ctx:
        before = prefix(total)
        if begin:
            ctx.upload_bodies(before[:begin])
        getattr(ctx, f"scene_{kind}")(num, begin, **kw)
        assert ctx.count() == begin + num
        out = ctx.download_bodies()
    return out


def check_disk(got, want, kw):
    scale = float(kw.get("outer_radius", 250.0)) + float(np.abs(kw.get("center", (0, 0, 0))).max())
    assert np.array_equal(got[:, [3, 7]].view(np.uint32), want[:, [3, 7]].view(np.uint32)), "radius / mass"
    dp = np.abs(got[:, :3].astype(np.float64) - want[:, :3])
    exact = np.all(got[:, :3].view(np.uint32) == want[:, :3].view(np.uint32), axis=1)
    assert dp.max() <= 1e-6 * scale, dp.max()
    assert exact.mean() >= 0.90, exact.mean()
    v_ref = want[:, 4:7].astype(np.float64)
    v = got[:, 4:7].astype(np.float64)
    finite = np.all(np.isfinite(v_ref), axis=1)
    assert np.array_equal(finite, np.all(np.isfinite(v), axis=1))
    if finite.any():
        rel = np.linalg.norm(v[finite] - v_ref[finite], axis=1) / np.maximum(np.linalg.norm(v_ref[finite], axis=1), 1e-30)
        assert rel.max() <= 1e-5, rel.max()
    assert np.all(got[:, 8:12] == 0)


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
@pytest.mark.parametrize("name", case_names("cube"))
def test_cube_matches_reference_bit_exact(gpu, name, layout):
    total, begin, num = (int(x) for x in CASES[f"cube_{name}_range"])
    kw = kwargs_from("cube", CASES[f"cube_{name}_args"])
    out = generate(gpu, "cube", total, begin, num, kw, layout)
    assert np.array_equal(out[begin:begin + num, :11].view(np.uint32),
                          CASES[f"cube_{name}_bodies"][:, :11].view(np.uint32))
    assert np.array_equal(out[:begin, :11], prefix(total)[:begin, :11])


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
@pytest.mark.parametrize("name", case_names("disk"))
def test_disk_matches_reference(gpu, name, layout):
    total, begin, num = (int(x) for x in CASES[f"disk_{name}_range"])
    kw = kwargs_from("disk", CASES[f"disk_{name}_args"])
    out = generate(gpu, "disk", total, begin, num, kw, layout)
    check_disk(out[begin:begin + num], CASES[f"disk_{name}_bodies"], kw)
    assert np.array_equal(out[:begin, :11], prefix(total)[:begin, :11])


def test_central_body_alone_matches_the_reference_nan(gpu):
    """One body: the reference divides by a zero distance and its velocity is NaN."""
    out = generate(gpu, "disk", 1, 0, 1, {})
    assert np.all(np.isnan(out[0, 4:7])) and out[0, 7] == np.float32(4.1e6)


@pytest.mark.parametrize("n", [1 << 20, (1 << 20) + 1])
def test_disk_1m_matches_oracle(gpu, n):
    kw = dict(outer_radius=100.0)
    want = O.disk(n, **kw)
    with gpu.Context() as ctx:
        ctx.scene_disk(n, **kw)
        got = ctx.download_bodies()
    check_disk(got, want, kw)


def test_cube_4m_matches_oracle(gpu):
    n = 1 << 22
    want = O.cube(n, size=1000.0, vel=(0.0, 1.0, 0.0))
    with gpu.Context() as ctx:
        ctx.scene_cube(n, size=1000.0, vel=(0.0, 1.0, 0.0))
        got = ctx.download_bodies()
    assert np.array_equal(got[:, :11].view(np.uint32), want[:, :11].view(np.uint32))


def test_disk_16m_tail_and_invariants(gpu):
    """Full size: the last 20,000 stars against the oracle's replay of the whole stream,
    and size-independent properties of all 16,777,216 bodies."""
    n = 1 << 24
    kw = dict(outer_radius=250.0)
    with gpu.Context() as ctx:
        ctx.scene_disk(n, **kw)
        got = ctx.download_bodies()
    tail = O.disk_positions(n, n - 20000, n, **kw)
    g = got[n - 20000:]
    assert np.array_equal(g[:, [3, 7]].view(np.uint32), tail[:, [3, 7]].view(np.uint32))
    dp = np.abs(g[:, :3].astype(np.float64) - tail[:, :3])
    assert dp.max() <= 1e-6 * 250.0
    assert np.mean(np.all(g[:, :3] == tail[:, :3], axis=1)) >= 0.90
    # every star between the clamped radii from the axis, unit-speed directions scaled
    r_xy = np.hypot(got[1:, 0].astype(np.float64), got[1:, 1])
    crad = O.lib().orc_compute_radius(4.1e6, 1e2)
    assert r_xy.min() >= crad * (1 - 1e-6) and r_xy.max() <= 250.0 * (1 + 1e-6)
    assert np.all(np.isfinite(got[:, :7]))
    assert float(got[:, 7].astype(np.float64).sum()) == 4.1e6 + (n - 1)


def test_range_past_the_count_is_rejected(gpu):
    with gpu.Context() as ctx:
        ctx.upload_bodies(prefix(10))
        with pytest.raises(gpu.NbodyError) as e:
            ctx.scene_disk(100, begin=11)
        assert e.value.status == gpu.ERR_INVALID
        ctx.scene_cube(0, begin=10)     # an empty range is fine
        assert ctx.count() == 10
