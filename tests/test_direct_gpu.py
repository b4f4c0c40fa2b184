"""Direct-sum parity on the GPU, through the C ABI.

Tolerances (stated once, used throughout):
  * scale_i = sum_j |a_ij| from the FP64 oracle; an FP32 sum of N terms in any order sits
    within a few 1e-5 * scale_i of the exact sum -- the reference's own CPU solver is
    1.9e-5 * scale_i from FP64 on the 1024-body disk (tests/test_oracle.py).
  * FP32 direct sum vs the reference (and vs FP64): max |da_i| / scale_i <= 5e-5 and
    median <= 1e-5 (the stated direct-sum tolerance: <= 1e-5 relative).
  * the plain relative bar against FP64 at configs 1 and 3: median and p99 of
    |a - a_fp64| / |a_fp64| <= 1e-5.
  * launch shapes: every kernel shape gives the same bits (tile sums folded exactly).
  * integrate: bit-identical to the reference's CPU integrator.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL_MAX = 5e-5
TOL_MEDIAN = 1e-5


def scaled_err(acc, bodies, law, eps2=0.0, G=1.0, ref=None, targets=None):
    pm = bodies[:, [0, 1, 2, 7]]
    a64, scale = O.direct_f64(pm, G, eps2, law, radius=bodies[:, 3], targets=targets, with_scale=True)
    ref = a64 if ref is None else ref
    scale = np.maximum(scale, 1e-30)
    return np.linalg.norm(np.asarray(acc, np.float64) - ref, axis=1) / scale


def run_accel(native, bodies, layout, **kw):
    with native.Context(layout) as ctx:
        ctx.upload_bodies(bodies)
        ctx.accelerate(native.params(**kw))
        out = ctx.download_bodies()
    return out


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
@pytest.mark.parametrize("fixture", ["disk_1024.npz", "disk_2048.npz", "cube_4096.npz"])
def test_bf_matches_reference(gpu, fixture, layout):
    """GPU brute force vs CpuBruteForceSolver (test_gpu.cpp:256-283 asks < 1e-2)."""
    g = golden(fixture)
    b = g["bodies"]
    out = run_accel(gpu, b, layout, law=gpu.LAW_CUTOFF, G=1.0)
    assert np.array_equal(out[:, :8], b[:, :8]), "accelerate must not move bodies"
    err_ref = scaled_err(out[:, 8:11], b, O.LAW_CUTOFF, ref=g["bf_acc"].astype(np.float64))
    err_64 = scaled_err(out[:, 8:11], b, O.LAW_CUTOFF)
    assert err_ref.max() <= TOL_MAX and np.median(err_ref) <= TOL_MEDIAN
    assert err_64.max() <= TOL_MAX and np.median(err_64) <= TOL_MEDIAN
    # the reference test's own metric: max relative error < 1e-2
    a_ref = g["bf_acc"].astype(np.float64)
    mag = np.linalg.norm(a_ref, axis=1)
    rel = np.linalg.norm(out[:, 8:11] - a_ref, axis=1)[mag > 0] / mag[mag > 0]
    assert rel.max() < 1e-2


def test_aos_and_soa_bit_identical(gpu):
    b = golden("cube_4096.npz")["bodies"]
    a = run_accel(gpu, b, gpu.LAYOUT_SOA, law=gpu.LAW_CUTOFF)
    c = run_accel(gpu, b, gpu.LAYOUT_AOS, law=gpu.LAW_CUTOFF)
    assert np.array_equal(a[:, 8:11], c[:, 8:11])


@pytest.mark.parametrize("n", [1, 2, 3, 31, 33, 255, 257, 1000, 4097])
def test_small_and_ragged_sizes(gpu, n):
    from nbody_gb300 import scenes
    b = scenes.plummer(n, seed=77 + n)
    b[:, 3] = 0.0
    for law, eps2 in ((gpu.LAW_CUTOFF, 0.0), (gpu.LAW_SOFTENED, 1e-4)):
        out = run_accel(gpu, b, gpu.LAYOUT_SOA, law=law, eps2=eps2)
        assert np.isfinite(out).all()
        if n == 1:
            assert np.all(out[:, 8:11] == 0)
            continue
        err = scaled_err(out[:, 8:11], b, law, eps2=eps2)
        assert err.max() <= TOL_MAX and np.median(err) <= TOL_MEDIAN, (law, err.max())


def test_empty_is_a_no_op(gpu):
    with gpu.Context() as ctx:
        ctx.upload_bodies(np.zeros((0, 12), np.float32))
        ctx.update(gpu.params(dt=0.01), steps=3)
        ctx.synchronize()
        assert ctx.launches() == 0
        assert ctx.download_bodies().shape == (0, 12)


def test_plummer_softened_vs_fp64(gpu):
    """Config 1 (N=4096 Plummer, eps=0.01): FP32 softened law vs the FP64 oracle."""
    from nbody_gb300 import scenes
    b = scenes.plummer(4096, seed=1001)
    out = run_accel(gpu, b, gpu.LAYOUT_SOA, law=gpu.LAW_SOFTENED, eps2=1e-4)
    err = scaled_err(out[:, 8:11], b, O.LAW_SOFTENED, eps2=1e-4)
    assert err.max() <= TOL_MAX and np.median(err) <= TOL_MEDIAN
    pm = b[:, [0, 1, 2, 7]]
    a64 = O.direct_f64(pm, 1.0, 1e-4, O.LAW_SOFTENED)
    rel = np.linalg.norm(out[:, 8:11] - a64, axis=1) / np.linalg.norm(a64, axis=1)
    assert np.median(rel) <= 1e-5


@pytest.mark.parametrize("n", [65536, 200003])
def test_jsplit_path_sampled(gpu, n):
    """Sizes whose launch splits the sources into chunks summed in a fixed order."""
    from nbody_gb300 import scenes
    b = scenes.uniform_cube(n, seed=5 + n)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        p = gpu.params(law=gpu.LAW_SOFTENED, eps2=1e-6)
        ctx.accelerate(p)
        cfg = ctx.last_direct_config()
        out = ctx.download_bodies()
        ctx.accelerate(p)
        again = ctx.download_bodies()
    assert np.array_equal(out, again), "the sum order is fixed, so results repeat exactly"
    tg = np.random.default_rng(1).choice(n, 512, replace=False)
    err = scaled_err(out[tg, 8:11], b, O.LAW_SOFTENED, eps2=1e-6, targets=tg)
    assert err.max() <= TOL_MAX and np.median(err) <= TOL_MEDIAN, cfg
    assert cfg["jsplit"] >= 1


def test_full_size_1m_sampled(gpu):
    """Config 3 size (N=1,048,576) FP32: sampled targets against FP64."""
    from nbody_gb300 import scenes
    n = 1 << 20
    b = scenes.uniform_cube(n, seed=1003)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.accelerate(gpu.params(law=gpu.LAW_SOFTENED, eps2=1e-6))
        out = ctx.download_bodies()
        cfg = ctx.last_direct_config()
    assert cfg["jsplit"] > 1
    tg = np.random.default_rng(2).choice(n, 128, replace=False)
    err = scaled_err(out[tg, 8:11], b, O.LAW_SOFTENED, eps2=1e-6, targets=tg)
    assert np.median(err) <= TOL_MEDIAN and err.max() <= 1e-4


def test_integrate_bit_exact_with_reference(gpu):
    """integrate.comp / physics.h:60-70: the same bits as the CPU integrator, wrap on."""
    g = golden("disk_2048.npz")
    b = g["bodies"].copy()
    b[:, 8:11] = g["bf_acc"]
    b[:, 0] *= 60.0        # push some bodies across the 10000 box edge
    b[:, 4:7] *= 3.0
    for layout in (0, 1):
        for wrap in (True, False):
            with gpu.Context(layout) as ctx:
                ctx.upload_bodies(b)
                ctx.integrate(gpu.params(dt=1.7, size=10000.0, wrap=wrap))
                out = ctx.download_bodies()
            expect = O.integrate(b, 1.7, 10000.0, wrap)
            assert np.array_equal(out[:, :11], expect[:, :11]), (layout, wrap)


def test_wrap_lands_where_reference_does(gpu):
    """test_wrap.cpp:32-110: x=499, v=10, dt=1, size=1000, G=0."""
    b = np.zeros((1, 12), np.float32)
    b[0, :8] = (499, 0, 0, 1, 10, 0, 0, 1)
    for layout in (0, 1):
        for wrap in (True, False):
            with gpu.Context(layout) as ctx:
                ctx.upload_bodies(b)
                ctx.update(gpu.params(dt=1.0, G=0.0, size=1000.0, wrap=wrap))
                p = ctx.download_bodies()[0, :3]
            ref = O.integrate(b, 1.0, 1000.0, wrap)[0, :3]
            assert np.array_equal(p, ref)
            assert (abs(p[0]) <= 500) if wrap else (p[0] > 500)


def test_update_matches_reference_steps(gpu):
    """5 x Solver::update(1/120) of the 512-body disk vs the reference's brute force."""
    g = golden("disk_512.npz")
    with gpu.Context() as ctx:
        ctx.upload_bodies(g["bodies"])
        ctx.update(gpu.params(dt=1.0 / 120.0, size=10000.0, wrap=True, law=gpu.LAW_CUTOFF), steps=5)
        out = ctx.download_bodies()
    ref = g["steps"]
    dpos = np.abs(out[:, :3] - ref[:, :3]).max()
    dvel = np.abs(out[:, 4:7] - ref[:, 4:7]).max()
    assert dpos < 1e-3 and dvel < 1e-2, (dpos, dvel)


def test_gravity_constant_scales(gpu):
    """test_gpu.cpp:285-315: scaling G scales the accelerations (exactly: G is applied once)."""
    b = golden("disk_1024.npz")["bodies"]
    a1 = run_accel(gpu, b, 0, law=gpu.LAW_CUTOFF, G=1.0)[:, 8:11]
    a4 = run_accel(gpu, b, 0, law=gpu.LAW_CUTOFF, G=4.0)[:, 8:11]
    assert np.array_equal(a4, a1 * np.float32(4.0))


def test_shrinking_count(gpu):
    """test_gpu.cpp:317-338: shrinking N reads back only the live bodies."""
    b = O.ref_cube(4096) if O.ref_available() else golden("cube_4096.npz")["bodies"]
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.update(gpu.params(dt=1 / 60, law=gpu.LAW_CUTOFF))
        ctx.upload_bodies(b[:16])
        ctx.update(gpu.params(dt=1 / 60, law=gpu.LAW_CUTOFF))
        out = ctx.download_bodies(4096)
    assert out.shape == (4096, 12)
    assert np.all(out[16:] == 0)
    ref = O.integrate(O.brute_force(b[:16], 1.0), 1 / 60, 10000.0, False)
    assert np.abs(out[:16, :3] - ref[:, :3]).max() < 1e-3


def test_radius_zero_finite(gpu):
    """test_variant.cpp:218-264: radius-0 bodies stay finite and still attract."""
    b = np.zeros((3, 12), np.float32)
    b[0, 7] = 1000
    b[1, [0, 7]] = (100, 1)
    b[2, [1, 7]] = (100, 1)
    for layout in (0, 1):
        with gpu.Context(layout) as ctx:
            ctx.upload_bodies(b)
            ctx.update(gpu.params(dt=1 / 120, law=gpu.LAW_CUTOFF))
            out = ctx.download_bodies()
        assert np.isfinite(out).all()
        assert out[1, 8] < 0 and out[2, 9] < 0


def test_masked_download_and_soa_round_trip(gpu):
    b = golden("disk_512.npz")["bodies"].copy()
    b[:, 11] = 0
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        host = np.full_like(b, -7.0)
        ctx.download_bodies(mask=gpu.READ_POSITIONS, into=host)
        assert np.array_equal(host[:, [0, 1, 2, 7]], b[:, [0, 1, 2, 7]])
        assert np.all(host[:, [3, 4, 5, 6, 8, 9, 10]] == -7.0)
        pm, vr, acc = ctx.download_soa()
        assert np.array_equal(pm, b[:, [0, 1, 2, 7]]) and np.array_equal(vr, b[:, [4, 5, 6, 3]])
        ctx.upload_soa(pm * 2, vr, acc)
        assert np.array_equal(ctx.download_bodies()[:, 0:3], b[:, 0:3] * 2)


def test_invalid_parameters_rejected(gpu):
    with gpu.Context() as ctx:
        ctx.upload_bodies(golden("disk_512.npz")["bodies"])
        with pytest.raises(gpu.NbodyError) as e:
            ctx.accelerate(gpu.params(law=gpu.LAW_SOFTENED, eps2=0.0))
        assert e.value.status == gpu.ERR_INVALID and "eps2" in str(e.value)
        with pytest.raises(gpu.NbodyError):
            ctx.accelerate(gpu.params(law=9))
        ctx.accelerate(gpu.params(law=gpu.LAW_CUTOFF))     # still usable
        ctx.synchronize()


def test_caller_owned_device_buffers(gpu):
    """nbody_cuda_dev_*: caller device memory (torch tensors as plain allocations)."""
    torch = pytest.importorskip("torch")
    b = golden("cube_4096.npz")["bodies"]
    pm = torch.from_numpy(np.ascontiguousarray(b[:, [0, 1, 2, 7]])).cuda()
    vr = torch.from_numpy(np.ascontiguousarray(b[:, [4, 5, 6, 3]])).cuda()
    acc = torch.zeros_like(pm)
    aos = torch.from_numpy(b.copy()).cuda()
    with gpu.Context() as ctx:
        ctx.set_stream(torch.cuda.current_stream().cuda_stream)
        p = gpu.params(law=gpu.LAW_CUTOFF)
        ctx.dev_accel_soa(pm.data_ptr(), vr.data_ptr(), acc.data_ptr(), len(b), p)
        ctx.dev_accel_aos(aos.data_ptr(), len(b), p)
        ctx.synchronize()
        ref = run_accel(gpu, b, 0, law=gpu.LAW_CUTOFF)[:, 8:11]
        assert np.array_equal(acc.cpu().numpy()[:, :3], ref)
        assert np.array_equal(aos.cpu().numpy()[:, 8:11], ref)
        ctx.dev_integrate_soa(pm.data_ptr(), vr.data_ptr(), acc.data_ptr(), len(b), gpu.params(dt=0.5))
        ctx.synchronize()
        bb = b.copy()
        bb[:, 8:11] = ref
        expect = O.integrate(bb, 0.5, 10000.0, False)
        assert np.array_equal(pm.cpu().numpy()[:, :3], expect[:, :3])


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
@pytest.mark.parametrize("law", [0, 1], ids=["cutoff", "softened"])
def test_every_kernel_shape(gpu, law, layout):
    """Each instantiated direct-sum shape (the ones the autotuner may pin: targets per
    thread x threads, scalar, packed, and packed with pre-paired source tiles), pinned in
    turn, on a ragged size whose launch splits the sources: within the direct-sum
    tolerance of the FP64 oracle, and each repeats exactly."""
    from nbody_gb300 import scenes
    n = 9001
    b = scenes.uniform_cube(n, seed=77)
    b[:, 3] = np.float32(1e-3)                       # target radius for the cutoff law
    eps2 = 1e-6 if law == gpu.LAW_SOFTENED else 0.0
    p = gpu.params(law=law, eps2=eps2)
    count = gpu.Context.direct_variant_count()
    assert count >= 10
    first = None
    with gpu.Context(layout) as ctx:
        ctx.upload_bodies(b)
        for i in range(count):
            ctx.set_direct_variant(i)
            ctx.accelerate(p)
            out = ctx.download_bodies()[:, 8:11].copy()
            ctx.accelerate(p)
            assert np.array_equal(out, ctx.download_bodies()[:, 8:11]), gpu.Context.direct_variant(i)
            err = scaled_err(out, b, law, eps2=eps2)
            assert err.max() <= TOL_MAX and np.median(err) <= TOL_MEDIAN, (gpu.Context.direct_variant(i), err.max())
            # the same 256-source tile sums, folded exactly: every shape gives the same
            # bits (a differing last bit needs the sum within ~2^-48 of a rounding tie)
            if first is None:
                first = out
            assert np.count_nonzero(out.view(np.uint32) != first.view(np.uint32)) <= 1, gpu.Context.direct_variant(i)


def test_fp32_result_independent_of_launch_shape_at_1m(gpu):
    """Config 3 (N = 2^20 uniform cube, eps = 1e-3): the three size-planned shapes (which
    split the sources into different numbers of chunks) give the same accelerations bit
    for bit on at least 99.999 % of components, so the FP32 error no longer depends on
    the launch shape. Also the plain bar of the direct sum: median |a - a_fp64| / |a_fp64|
    <= 1e-5 (and p99 <= 1e-5) on 4096 sampled targets, against the GPU's FP64 form, which
    is itself within 1e-12 of the CPU FP64 oracle on 32 of them."""
    from nbody_gb300 import scenes
    n = 1 << 20
    b = scenes.uniform_cube(n, seed=1003)
    eps2 = 1e-6
    p = gpu.params(law=gpu.LAW_SOFTENED, eps2=eps2)
    tg = np.random.default_rng(3).choice(n, 4096, replace=False)
    outs, splits = [], []
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        for v in range(3):
            ctx.set_direct_variant(v)
            ctx.accelerate(p)
            outs.append(ctx.download_bodies()[:, 8:11].copy())
            splits.append(ctx.last_direct_config()["jsplit"])
        a64 = ctx.accel_sampled(gpu.params(law=gpu.LAW_SOFTENED, eps2=eps2, precision=gpu.PREC_FP64), tg)
    chk = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(eps2)), O.LAW_SOFTENED, targets=tg[:32])
    assert (np.linalg.norm(a64[:32] - chk, axis=1) / np.linalg.norm(chk, axis=1)).max() < 1e-12
    assert len(set(splits)) > 1, splits           # the shapes really split differently
    for o in outs[1:]:
        assert np.count_nonzero(o.view(np.uint32) != outs[0].view(np.uint32)) <= 1e-5 * o.size, splits
    rel = np.linalg.norm(outs[0][tg] - a64, axis=1) / np.linalg.norm(a64, axis=1)
    assert np.median(rel) <= 1e-5 and np.percentile(rel, 99) <= 1e-5, (np.median(rel), np.percentile(rel, 99),
                                                                          rel.max())


def test_plain_relative_bar_config1(gpu):
    """Config 1 (N = 4096 Plummer, eps = 0.01): median |a - a_fp64| / |a_fp64| <= 1e-5 and
    p99 <= 1e-5 against the CPU FP64 oracle over every body."""
    from nbody_gb300 import scenes
    b = scenes.plummer(4096, seed=1001)
    out = run_accel(gpu, b, gpu.LAYOUT_SOA, law=gpu.LAW_SOFTENED, eps2=1e-4)
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(1e-4)), O.LAW_SOFTENED)
    rel = np.linalg.norm(out[:, 8:11] - a64, axis=1) / np.linalg.norm(a64, axis=1)
    assert np.median(rel) <= 1e-5 and np.percentile(rel, 99) <= 1e-5, (np.median(rel), np.percentile(rel, 99),
                                                                          rel.max())
