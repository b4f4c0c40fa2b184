"""The group walk (NBODY_WALK_GROUP) on the GPU, through the C ABI.

A warp walks the tree once for a group of Morton-consecutive targets and accepts a cell for
the whole group when the group's bounding box lies beyond the reference's opening distance
(bhtree.cpp:117-125); accepted cells and leaves go to an interaction list applied to every
target of the group. Each target's sources therefore refine the cells the reference's walk
accepts for it alone.

Bars (stated once, used throughout):
  * accuracy against the FP64 direct sum: median and p99 of |a - a_fp64| / |a_fp64| no worse
    than the per-target walk's (the reference's own accepted sets) on the same targets
    (x 1.05, plus 1e-7 median / 1e-6 p99 for FP32 rounding when the theta error vanishes);
  * the interaction count is at least the per-target walk's (a refinement);
  * coincident bodies, massless bodies and tiny systems give finite sums within the same bar.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def accel(native, bodies, walk, layout=0, **kw):
    kw.setdefault("mode", native.MODE_NLOGN)
    with native.Context(layout) as ctx:
        ctx.upload_bodies(bodies)
        ctx.accelerate(native.params(walk=walk, **kw))
        out = ctx.download_bodies()[:, 8:11].astype(np.float64)
        stats = ctx.bh_stats()
    return out, stats


def rel_err(acc, exact):
    return np.linalg.norm(acc - exact, axis=1) / np.maximum(np.linalg.norm(exact, axis=1), 1e-300)


def assert_no_worse(e_group, e_target, what):
    assert np.median(e_group) <= 1.05 * np.median(e_target) + 1e-7, (what, np.median(e_group), np.median(e_target))
    assert np.percentile(e_group, 99) <= 1.05 * np.percentile(e_target, 99) + 1e-6, \
        (what, np.percentile(e_group, 99), np.percentile(e_target, 99))


@pytest.mark.parametrize("theta", [0.5, 2.0], ids=["ref-theta-0.5", "ref-theta-2"])
@pytest.mark.parametrize("tree_box", [1, 0], ids=["fitted-box", "reference-box"])
def test_group_walk_config2(gpu, tree_box, theta):
    """Config 2 (two Plummer spheres of 131,072, eps = 0.01), softened law, 4096 sampled
    targets against the FP64 oracle."""
    from nbody_gb300 import scenes
    b = scenes.two_plummer(131072)
    kw = dict(theta=theta, law=gpu.LAW_SOFTENED, eps2=1e-4, size=64.0, tree_box=tree_box)
    ag, sg = accel(gpu, b, gpu.WALK_GROUP, **kw)
    at, st = accel(gpu, b, gpu.WALK_TARGET, **kw)
    assert np.all(np.isfinite(ag))
    assert sg["interactions"] >= st["interactions"]
    tg = np.random.default_rng(9).choice(len(b), 4096, replace=False)
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(1e-4)), O.LAW_SOFTENED, targets=tg)
    assert_no_worse(rel_err(ag[tg], a64), rel_err(at[tg], a64), (tree_box, theta))


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
@pytest.mark.parametrize("law", [0, 1], ids=["cutoff", "softened"])
def test_group_walk_laws_and_layouts(gpu, law, layout):
    """Both laws, both layouts, on a Plummer sphere with radii (the cutoff law's target
    radius), every body checked against the FP64 oracle."""
    from nbody_gb300 import scenes
    b = scenes.plummer(20000, seed=3, rmax=10.0)
    b[:, 3] = np.float32(1e-3)
    eps2 = 1e-4 if law == 1 else 0.0
    kw = dict(theta=1.0, law=law, eps2=eps2, size=0.0, tree_box=1)
    ag, _ = accel(gpu, b, gpu.WALK_GROUP, layout, **kw)
    at, _ = accel(gpu, b, gpu.WALK_TARGET, layout, **kw)
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(eps2)), law, radius=b[:, 3])
    assert np.all(np.isfinite(ag))
    assert_no_worse(rel_err(ag, a64), rel_err(at, a64), (law, layout))


def test_group_walk_soa_aos_identical(gpu):
    from nbody_gb300 import scenes
    b = scenes.two_plummer(5000)
    kw = dict(theta=2.0, law=gpu.LAW_SOFTENED, eps2=1e-4, size=0.0, tree_box=1)
    a, _ = accel(gpu, b, gpu.WALK_GROUP, 0, **kw)
    c, _ = accel(gpu, b, gpu.WALK_GROUP, 1, **kw)
    assert np.array_equal(a, c)


@pytest.mark.parametrize("n", [2, 3, 5, 33, 257, 4097])
def test_group_walk_small_sizes(gpu, n):
    """Tiny systems (fewer targets than one group; ragged last group): with few bodies the
    walk opens nearly everything, so the sum is the direct sum to FP32 rounding."""
    from nbody_gb300 import scenes
    b = scenes.plummer(n, seed=50 + n, rmax=10.0)
    ag, _ = accel(gpu, b, gpu.WALK_GROUP, theta=0.5, law=gpu.LAW_SOFTENED, eps2=1e-4, size=0.0, tree_box=1)
    at, _ = accel(gpu, b, gpu.WALK_TARGET, theta=0.5, law=gpu.LAW_SOFTENED, eps2=1e-4, size=0.0, tree_box=1)
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(1e-4)), O.LAW_SOFTENED)
    assert np.all(np.isfinite(ag))
    assert_no_worse(rel_err(ag, a64), rel_err(at, a64), n)


@pytest.mark.parametrize("tree_box", [1, 0], ids=["fitted-box", "reference-box"])
def test_group_walk_buckets_massless_and_outliers(gpu, tree_box):
    """Coincident bodies (a bucket of identical codes, opened as a body range), massless
    bodies, masses over twelve decades and a far outlier."""
    from nbody_gb300 import scenes
    b = scenes.two_plummer(10000).copy()
    rng = np.random.default_rng(12)
    b[:, 7] = (10.0 ** rng.uniform(-8, 4, len(b))).astype(np.float32)
    b[:40, 7] = 0.0
    b[100:160, :3] = b[99, :3]                      # 61 coincident bodies: one bucket
    b[5, :3] = (3000.0, -2000.0, 1500.0)
    kw = dict(theta=1.0, law=gpu.LAW_SOFTENED, eps2=1e-4, size=8192.0, tree_box=tree_box)
    ag, _ = accel(gpu, b, gpu.WALK_GROUP, **kw)
    at, _ = accel(gpu, b, gpu.WALK_TARGET, **kw)
    assert np.all(np.isfinite(ag))
    tg = np.concatenate([np.arange(90, 170), rng.choice(len(b), 1500, replace=False)])
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(1e-4)), O.LAW_SOFTENED, targets=tg)
    assert_no_worse(rel_err(ag[tg], a64), rel_err(at[tg], a64), tree_box)


@pytest.mark.parametrize("law", [0, 1], ids=["cutoff", "softened"])
def test_group_walk_all_bodies_at_one_point(gpu, law):
    """Every body at one position: one bucket; every pair has d = 0 and adds exactly 0."""
    b = np.zeros((300, 12), np.float32)
    b[:, :3] = (1.5, -2.25, 0.75)
    b[:, 3] = 0.01
    b[:, 7] = 1.0
    a, _ = accel(gpu, b, gpu.WALK_GROUP, theta=0.5, law=law, eps2=1e-4 if law == 1 else 0.0, size=64.0,
                 tree_box=1)
    assert np.all(a == 0)


@pytest.mark.parametrize("group", ["64", "128", "256"])
def test_group_sizes(gpu, group, monkeypatch):
    """Every group size (NBODY_CUDA_BH_GROUP) meets the bar; a larger group opens more cells
    for its targets and so applies at least as many interactions."""
    from nbody_gb300 import scenes
    b = scenes.two_plummer(50000)
    kw = dict(theta=2.0, law=gpu.LAW_SOFTENED, eps2=1e-4, size=0.0, tree_box=1)
    monkeypatch.setenv("NBODY_CUDA_BH_GROUP", group)
    ag, sg = accel(gpu, b, gpu.WALK_GROUP, **kw)
    at, st = accel(gpu, b, gpu.WALK_TARGET, **kw)
    tg = np.random.default_rng(4).choice(len(b), 2048, replace=False)
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(1e-4)), O.LAW_SOFTENED, targets=tg)
    assert sg["interactions"] >= st["interactions"]
    assert_no_worse(rel_err(ag[tg], a64), rel_err(at[tg], a64), group)


def test_group_walk_config5(gpu):
    """Config 5 (16,777,216-body disk + halo, eps = 0.005) at reference theta 2 (the
    conventional 0.5) and 4/3 (conventional 0.75): 4096 sampled targets against the GPU's
    FP64 direct sum (itself pinned to the CPU oracle in test_bh_gpu.py)."""
    from nbody_gb300 import scenes
    b = scenes.disk_halo()
    eps2 = 0.005 ** 2
    tg = np.random.default_rng(5).choice(len(b), 4096, replace=False)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        a64 = ctx.accel_sampled(gpu.params(law=gpu.LAW_SOFTENED, eps2=eps2, precision=gpu.PREC_FP64), tg)
        for theta in (2.0, 4.0 / 3.0):
            res = {}
            for walk in (gpu.WALK_TARGET, gpu.WALK_GROUP):
                ctx.accelerate(gpu.params(mode=gpu.MODE_NLOGN, theta=theta, law=gpu.LAW_SOFTENED, eps2=eps2,
                                          size=0.0, tree_box=1, walk=walk))
                res[walk] = (ctx.download_bodies()[tg, 8:11].astype(np.float64), ctx.bh_stats())
            assert np.all(np.isfinite(res[gpu.WALK_GROUP][0]))
            assert res[gpu.WALK_GROUP][1]["interactions"] >= res[gpu.WALK_TARGET][1]["interactions"]
            assert_no_worse(rel_err(res[gpu.WALK_GROUP][0], a64), rel_err(res[gpu.WALK_TARGET][0], a64), theta)


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32", "compensated"])
def test_group_walk_graph_replay_equals_eager(gpu, precision):
    from nbody_gb300 import scenes
    b = scenes.two_plummer(10000)
    p = gpu.params(mode=gpu.MODE_NLOGN, theta=2.0, dt=5e-4, eps2=1e-4, law=gpu.LAW_SOFTENED, size=0.0, tree_box=1,
                   precision=precision, walk=gpu.WALK_GROUP)
    out = []
    for graph in (False, True):
        with gpu.Context() as ctx:
            ctx.upload_bodies(b)
            (ctx.update_graph if graph else ctx.update)(p, 12)
            out.append(ctx.download_bodies())
    assert np.array_equal(out[0], out[1])


def test_unknown_walk_rejected(gpu):
    from nbody_gb300 import scenes
    with gpu.Context() as ctx:
        ctx.upload_bodies(scenes.plummer(100, seed=1))
        with pytest.raises(gpu.NbodyError) as e:
            ctx.accelerate(gpu.params(mode=gpu.MODE_NLOGN, walk=7))
        assert e.value.status == gpu.ERR_INVALID
