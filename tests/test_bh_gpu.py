"""Barnes-Hut on the GPU against the reference's CPU octree solver, through the C ABI.

Bars:
  * Morton codes and sort order: bit-exact against the oracle (oracle/nbody_oracle.c).
  * Accelerations: the device tree has the reference's cells and applies the reference's
    opening test per target, so a body's sum covers the same cells; only the centre-of-mass
    rounding (FP64 sums here, an FP32 running mean in the reference, bhtree.cpp:87-95) and
    the summation order differ. Per body |a_gpu - a_ref| <= 5e-5 * sum|terms| for all but
    a handful of bodies (where a rounding difference flips one borderline acceptance), and
    every body within the reference's own bound: max relative error < 1e-2
    (tests/source/test_gpu.cpp:226-254).
"""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = 5e-5


def bh_accel(native, bodies, layout=0, **kw):
    kw.setdefault("mode", native.MODE_NLOGN)
    with native.Context(layout) as ctx:
        ctx.upload_bodies(bodies)
        ctx.accelerate(native.params(**kw))
        out = ctx.download_bodies()
        stats = ctx.bh_stats()
    return out[:, 8:11], stats


def term_scale(bodies, targets=None):
    """sum_j |a_ij| over all bodies (FP64): the natural scale of an FP32 sum's rounding."""
    _, scale = O.direct_f64(bodies[:, [0, 1, 2, 7]], 1.0, 0.0, O.LAW_CUTOFF, radius=bodies[:, 3],
                            targets=targets, with_scale=True)
    return np.maximum(scale, 1e-30)


def compare_to_reference(acc, ref, bodies, allowed_outliers):
    err = np.linalg.norm(acc.astype(np.float64) - ref, axis=1) / term_scale(bodies)
    bad = np.flatnonzero(err > TOL)
    assert len(bad) <= allowed_outliers, (len(bad), err.max())
    mag = np.linalg.norm(ref, axis=1)
    ok = mag > 0
    rel = np.linalg.norm(acc[ok] - ref[ok], axis=1) / mag[ok]
    assert rel.max() < 1e-2, rel.max()
    return err


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
@pytest.mark.parametrize("fixture", ["disk_1024.npz", "disk_2048.npz", "cube_4096.npz"])
def test_bh_matches_reference_cpu_barnes_hut(gpu, fixture, layout):
    g = golden(fixture)
    b = g["bodies"]
    acc, stats = bh_accel(gpu, b, layout, theta=0.5, size=10000.0, law=gpu.LAW_CUTOFF)
    compare_to_reference(acc, g["bh_acc"].astype(np.float64), b, allowed_outliers=max(2, len(b) // 500))
    # the same cells are accepted, so the interaction count matches the reference's
    t = O.Tree(10000.0)
    t.build(b, 10000.0)
    _, inter = t.accel(b, 0.5, 1.0)
    assert abs(stats["interactions"] - inter) <= 0.01 * inter, (stats, inter)


def test_bh_soa_aos_identical(gpu):
    b = golden("cube_4096.npz")["bodies"]
    a, _ = bh_accel(gpu, b, 0, theta=0.5, size=10000.0)
    c, _ = bh_accel(gpu, b, 1, theta=0.5, size=10000.0)
    assert np.array_equal(a, c)


def test_morton_and_sort_order_bit_exact(gpu):
    from nbody_gb300 import scenes
    b = scenes.plummer(20000, seed=31, rmax=15.0)
    b[:50, :3] = 0.0                        # exactly on the centre planes
    b[50:60, :3] = -np.float32(1e-30)       # tiny negatives: below every centre
    b[60:70, :3] = b[70:80, :3]             # duplicated codes (ties by index)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        for tree_box in (0, 1):
            p = gpu.params(mode=gpu.MODE_NLOGN, size=64.0, tree_box=tree_box)
            codes, order, box = ctx.morton(p)
            if tree_box == 0:
                assert list(box) == [-32.0, -32.0, -32.0, 64.0]
            ref_codes = O.morton63(b[:, :3], box[:3], 2.0 ** 21 / box[3])
            ref_order = O.sort_order(ref_codes)
            assert np.array_equal(order, ref_order)
            assert np.array_equal(codes, ref_codes[ref_order])


@pytest.mark.parametrize("n", [2, 3, 1023, 1024, 1025, 4095, 4096, 4097, 12289, 1 << 20, (1 << 22) - 1, (1 << 22) + 1])
def test_sort_order_at_tile_edges(gpu, n):
    """The radix sort (one kernel per digit pass, decoupled look-back between 4096-key
    tiles) against the oracle's stable order, at sizes on and next to multiples of a tile
    and of a warp's share of one, with runs of equal codes (ties keep index order)."""
    rng = np.random.default_rng(n)
    b = np.zeros((n, 12), np.float32)
    b[:, :3] = rng.uniform(-30, 30, (n, 3)).astype(np.float32)
    b[:, 7] = 1.0
    dup = rng.choice(n, n // 3, replace=True)
    b[dup, :3] = b[rng.choice(n, 1), :3]        # a third of the bodies share one position
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        codes, order, box = ctx.morton(gpu.params(mode=gpu.MODE_NLOGN, size=0.0, tree_box=1))
    ref_codes = O.morton63(b[:, :3], box[:3], 2.0 ** 21 / box[3])
    ref_order = O.sort_order(ref_codes)
    assert np.array_equal(order, ref_order)
    assert np.array_equal(codes, ref_codes[ref_order])


@pytest.mark.parametrize("max_run", [32, 33])
def test_sort_order_with_runs_in_one_fine_cell(gpu, max_run):
    """The Morton sort orders the top 45 code bits by radix passes and then each run of
    codes that agree on them by the low 18 bits; a run longer than 32 sorts everything again
    by all bits. Clusters of 2 .. max_run bodies inside one level-15 cell (codes that differ
    only in their low bits, some identical) take the first path at 32 and the second at 33."""
    rng = np.random.default_rng(max_run)
    sizes = rng.integers(2, max_run + 1, 3000)
    sizes[0] = max_run
    n = int(sizes.sum()) + 2
    b = np.zeros((n, 12), np.float32)
    b[:, 7] = 1.0
    b[0, :3], b[1, :3] = -30.0, 30.0         # fitted box: edge 64, corner -32 on every axis
    cell = 64.0 / 2 ** 15                    # level 15
    k = 2
    for s in sizes:
        c = -32.0 + (rng.integers(2 ** 10, 2 ** 15 - 2 ** 10, 3) + 0.5) * cell
        b[k:k + s, :3] = (c + rng.uniform(-0.45, 0.45, (s, 3)) * cell).astype(np.float32)
        b[k + s - 1, :3] = b[k, :3]          # one identical pair per cluster
        k += s
    b = b[rng.permutation(n)]                # clusters spread over the index range
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        codes, order, box = ctx.morton(gpu.params(mode=gpu.MODE_NLOGN, size=0.0, tree_box=1))
    assert list(box) == [-32.0, -32.0, -32.0, 64.0]
    ref_codes = O.morton63(b[:, :3], box[:3], 2.0 ** 21 / box[3])
    ref_order = O.sort_order(ref_codes)
    runs = np.diff(np.flatnonzero(np.r_[True, np.diff(ref_codes[ref_order] >> np.uint64(18)) != 0, True]))
    assert runs.max() == max_run
    assert np.array_equal(order, ref_order)
    assert np.array_equal(codes, ref_codes[ref_order])


def test_sort_order_at_16m(gpu):
    """The sort of the 16.8M disk + halo codes: 4096 tiles per pass, most of them waiting on
    their predecessors' counts, against the oracle's stable order."""
    from nbody_gb300 import scenes
    b = scenes.disk_halo()
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        codes, order, box = ctx.morton(gpu.params(mode=gpu.MODE_NLOGN, size=0.0, tree_box=1))
    ref_codes = O.morton63(b[:, :3], box[:3], 2.0 ** 21 / box[3])
    ref_order = O.sort_order(ref_codes)
    assert np.array_equal(order, ref_order)
    assert np.array_equal(codes, ref_codes[ref_order])


@pytest.mark.parametrize("size,tree_box", [(64.0, 0), (100.0, 0), (0.0, 1)],
                         ids=["pow2-box-integer-path", "other-box-fp64-path", "fitted-box"])
def test_morton_codes_at_special_values(gpu, size, tree_box):
    """The integer quantisation (power-of-two cells on a cell-aligned corner) and the FP64
    directed-rounding one agree with the oracle bit for bit on signed zeros, subnormals,
    values on and next to cell boundaries, values far outside the box and infinities."""
    rng = np.random.default_rng(5)
    special = np.array([0.0, -0.0, 1e-45, -1e-45, 1e-39, -1e-39, 1e-30, -1e-30, 31.999998, 32.0, -32.0,
                        -32.000004, 1e30, -1e30, np.inf, -np.inf, 2.0 ** -19, -2.0 ** -19,
                        np.nextafter(np.float32(2.0 ** -15), np.float32(0))], np.float32)
    n = 4096
    b = np.zeros((n, 12), np.float32)
    b[:, :3] = rng.uniform(-30, 30, (n, 3)).astype(np.float32)
    b[:, 7] = 1.0
    k = len(special)
    b[:k, 0] = special
    b[k:2 * k, 1] = special
    b[2 * k:3 * k, 2] = special
    if tree_box == 1:           # keep the fitted box finite: no infinities for the bounding box
        b[:, :3] = np.where(np.isfinite(b[:, :3]) & (np.abs(b[:, :3]) < 1e20), b[:, :3], 7.0)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        codes, order, box = ctx.morton(gpu.params(mode=gpu.MODE_NLOGN, size=size, tree_box=tree_box))
    ref_codes = O.morton63(b[:, :3], box[:3], 2.0 ** 21 / box[3])
    ref_order = O.sort_order(ref_codes)
    assert np.array_equal(order, ref_order)
    assert np.array_equal(codes, ref_codes[ref_order])


def test_morton_cells_are_reference_cells(gpu):
    """Every body's level-L Morton digit is its reference octant (bits flipped) in the
    reference's own tree (golden node array of the 4096-body cube)."""
    g = golden("cube_4096.npz")
    b = g["bodies"]
    nodes = np.frombuffer(g["nodes"].tobytes(), dtype=O.NODE_DTYPE)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        codes, order, box = ctx.morton(gpu.params(mode=gpu.MODE_NLOGN, size=10000.0))
    inv = np.empty_like(order)
    inv[order] = np.arange(len(order))
    for i in range(0, len(b), 37):
        code = int(codes[inv[i]])
        idx, level = 0, 0
        while nodes[idx]["children"] != 0:
            c = nodes[idx]["center"]
            q = int(b[i, 0] < c[0]) | (int(b[i, 1] < c[1]) << 1) | (int(b[i, 2] < c[2]) << 2)
            assert ((code >> (3 * (20 - level))) & 7) == q ^ 7
            idx = nodes[idx]["children"] + q
            level += 1


@pytest.mark.parametrize("n", [100, 2000])
def test_bh_theta_convention(gpu, n):
    """test_bhtree.cpp:259-367 on the GPU: larger theta is more accurate and does more work.
    The reference pins the loose error below 3.0 at its N = 100; at N = 2000 the GPU's
    errors are pinned to the oracle octree's errors for the same inputs instead."""
    g = np.random.default_rng(11)
    p = np.clip(g.normal(0, 0.5, (n, 3)), -1, 1).astype(np.float32) * 100
    b = np.zeros((n, 12), np.float32)
    b[:, :3] = p
    b[:, 7] = 1
    exact = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, 0.0, O.LAW_CUTOFF)
    mean_force = np.linalg.norm(exact, axis=1).mean()
    loose, sl = bh_accel(gpu, b, theta=0.5, size=200.0)
    tight, st = bh_accel(gpu, b, theta=8.0, size=200.0)
    el = np.linalg.norm(loose - exact, axis=1).max() / mean_force
    et = np.linalg.norm(tight - exact, axis=1).max() / mean_force
    assert et < el and et < 0.05
    assert st["interactions"] > sl["interactions"] > 0
    assert st["interactions"] < n * n
    t = O.Tree(200.0)
    t.build(b, 200.0)
    ol, _ = t.accel(b, 0.5, 1.0)
    ot, _ = t.accel(b, 8.0, 1.0)
    assert el <= 1.01 * np.linalg.norm(ol - exact, axis=1).max() / mean_force + 1e-6
    assert et <= 1.01 * np.linalg.norm(ot - exact, axis=1).max() / mean_force + 1e-6
    if n == 100:
        assert el < 3.0


@pytest.mark.parametrize("n", [2, 3, 5, 33, 257])
def test_bh_small_sizes(gpu, n):
    from nbody_gb300 import scenes
    b = scenes.plummer(n, seed=5 + n, rmax=10.0)
    acc, _ = bh_accel(gpu, b, theta=0.5, size=64.0)
    ref, _ = O.barnes_hut(b, 64.0, 0.5, 1.0)
    err = np.linalg.norm(acc - ref[:, 8:11], axis=1) / term_scale(b)
    assert np.all(np.isfinite(acc)) and err.max() <= TOL


def test_bh_one_body_and_empty(gpu):
    b = np.zeros((1, 12), np.float32)
    b[0, 7] = 5.0
    acc, _ = bh_accel(gpu, b, theta=0.5, size=64.0)
    assert np.all(acc == 0)
    with gpu.Context() as ctx:
        ctx.upload_bodies(np.zeros((0, 12), np.float32))
        ctx.update(gpu.params(mode=gpu.MODE_NLOGN, dt=0.1), steps=2)
        ctx.synchronize()


def test_bh_coincident_and_outside_bodies(gpu):
    """Coincident bodies (a bucket of identical codes) and bodies outside the root box
    (placed in edge cells, as the reference's quadrant test does)."""
    from nbody_gb300 import scenes
    b = scenes.plummer(3000, seed=8, rmax=10.0)
    b[100:110, :3] = b[99, :3]              # 11 coincident bodies
    b[200:205, 0] = 80.0                    # outside a 64 box
    b[205:210, 1] = -90.0
    acc, _ = bh_accel(gpu, b, theta=0.5, size=64.0)
    ref, _ = O.barnes_hut(b, 64.0, 0.5, 1.0)
    assert np.all(np.isfinite(acc))
    err = np.linalg.norm(acc - ref[:, 8:11], axis=1) / term_scale(b)
    # coincident bodies sit below the reference's FLT_EPSILON merge size and are merged
    # there (bhtree.cpp:36-42); here they are one bucket applied body by body. The median
    # body sits ~3e-6 from the reference: its FP32 running-mean centres of mass
    # (bhtree.cpp:87-95) against the FP64 sums here.
    assert np.median(err) <= 1e-5 and (err > TOL).sum() <= 15


def test_bh_two_plummer_sampled(gpu):
    """Config 2 inputs (two Plummer spheres, 2 x 131072) under the reference's cutoff law on
    the reference's fixed 64 box, against the oracle's restated octree on 2048 sampled
    targets (same root box). The softened law on the same inputs is
    test_bh_softened_config2_against_oracle_octree."""
    from nbody_gb300 import scenes
    b = scenes.two_plummer(131072)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        p = gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, law=gpu.LAW_CUTOFF, size=64.0)
        _, _, box = ctx.morton(p)
        ctx.accelerate(p)
        acc = ctx.download_bodies()[:, 8:11]
    assert list(box) == [-32.0, -32.0, -32.0, 64.0]
    assert np.all(np.isfinite(acc))
    tg = np.random.default_rng(4).choice(len(b), 2048, replace=False)
    t = O.Tree(64.0)
    t.build(b, 64.0)
    ref, _ = t.accel(b, 0.5, 1.0, targets=tg)
    err = np.linalg.norm(acc[tg] - ref, axis=1) / term_scale(b, tg)
    assert np.median(err) <= 1e-5 and (err > TOL).sum() <= 10, err.max()


def test_bh_update_steps(gpu):
    """BH update vs the reference's CPU Barnes-Hut stepping (5 steps, wrap on)."""
    g = golden("disk_512.npz")
    b = g["bodies"]
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.update(gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, dt=1 / 120, size=10000.0, wrap=True), steps=5)
        out = ctx.download_bodies()
    ref = b.copy()
    for _ in range(5):
        ref, _ = O.barnes_hut(ref, 10000.0, 0.5, 1.0)
        ref = O.integrate(ref, 1 / 120, 10000.0, True)
    assert np.abs(out[:, :3] - ref[:, :3]).max() < 1e-3


def _cells(nodes):
    """Non-empty nodes keyed by (centre, size): the tree's cells, independent of order."""
    return {(tuple(n["center"]), float(n["size"])): (float(n["mass"]), tuple(n["com"]), int(n["children"] != 0))
            for n in nodes if n["mass"] != 0}


@pytest.mark.parametrize("fixture", ["cube_4096.npz", "disk_2048.npz"])
def test_tree_export_is_the_reference_tree(gpu, fixture):
    """nbody_cuda_tree_export gives the reference's octree: the same cells, node count,
    masses, centres of mass (to rounding), and Tree::apply over it (oracle) gives the
    reference's accelerations."""
    g = golden(fixture)
    b = g["bodies"]
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.accelerate(gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, size=10000.0))
        nodes = ctx.tree_export()
    ref = O.ref_build_tree(b, 10000.0) if O.ref_available() else np.frombuffer(
        golden("cube_4096.npz")["nodes"].tobytes(), dtype=O.NODE_DTYPE) if fixture == "cube_4096.npz" else None
    if ref is None:
        t = O.Tree(10000.0)
        t.build(b, 10000.0)
        ref = t.nodes()
    assert len(nodes) == len(ref)
    ours, theirs = _cells(nodes), _cells(ref)
    assert ours.keys() == theirs.keys()
    for k, (m, com, split) in theirs.items():
        m2, com2, split2 = ours[k]
        assert split == split2 and abs(m - m2) <= 1e-6 * abs(m)
        assert np.allclose(com, com2, rtol=1e-5, atol=1e-3)
    # links: every node's children block and next pointer are in range, root next = 0
    assert nodes[0]["next"] == 0
    assert np.all(nodes["children"] < len(nodes)) and np.all(nodes["next"] < len(nodes))
    acc, inter = O.nodes_accel(nodes.view(O.NODE_DTYPE), b, 0.5, 1.0)
    racc, rinter = O.nodes_accel(ref.view(O.NODE_DTYPE), b, 0.5, 1.0)
    assert abs(inter - rinter) <= 0.01 * rinter
    scale = term_scale(b)
    err = np.linalg.norm(acc.astype(np.float64) - racc, axis=1) / scale
    assert np.median(err) <= 1e-5 and (err > TOL).sum() <= len(b) // 500 + 2


@pytest.mark.parametrize("per_warp", ["256", "128", "64"])
@pytest.mark.parametrize("law", [0, 1], ids=["cutoff", "softened"])
@pytest.mark.parametrize("n", [1000, 4097, 100000])
def test_two_targets_per_lane_walk_is_bit_identical(gpu, n, law, per_warp, monkeypatch):
    """The walks with 4 (the default) and 2 targets per lane and the 32-target walk accept
    the same nodes per target in the same depth-first order, so every acceleration and the
    interaction count agree bit for bit."""
    from nbody_gb300 import scenes
    b = scenes.two_plummer(n // 2 + 1)[:n]
    b[:, 3] = np.float32(1e-3)
    kw = dict(theta=0.6, law=law, eps2=1e-4 if law == 1 else 0.0, size=0.0, tree_box=1)
    monkeypatch.setenv("NBODY_CUDA_BH_TARGETS", per_warp)
    a64, s64 = bh_accel(gpu, b, **kw)
    monkeypatch.setenv("NBODY_CUDA_BH_TARGETS", "32")
    a32, s32 = bh_accel(gpu, b, **kw)
    assert np.array_equal(a64.view(np.uint32), a32.view(np.uint32))
    assert s64["interactions"] == s32["interactions"] and s64["cells"] == s32["cells"]


def test_two_targets_per_lane_walk_is_bit_identical_at_16m(gpu, monkeypatch):
    """The same identity over the full 16.8M disk + halo workload. A borderline acceptance
    flips for a few bodies in ten million when the distance test's roundings change, so
    only the full size tests it."""
    from nbody_gb300 import scenes
    b = scenes.disk_halo()
    kw = dict(mode=gpu.MODE_NLOGN, theta=0.5, law=gpu.LAW_SOFTENED, eps2=0.005 ** 2, size=0.0, tree_box=1)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.accelerate(gpu.params(**kw))
        a64 = ctx.download_bodies()[:, 8:11].copy()
        s64 = ctx.bh_stats()
        monkeypatch.setenv("NBODY_CUDA_BH_TARGETS", "32")
        ctx.accelerate(gpu.params(**kw))
        a32 = ctx.download_bodies()[:, 8:11]
        s32 = ctx.bh_stats()
    assert s64["interactions"] == s32["interactions"]
    assert np.array_equal(a64.view(np.uint32), a32.view(np.uint32))


def test_bh_stage_ms(gpu):
    """nbody_cuda_bh_stage_ms: refused before any Barnes-Hut accelerate; afterwards the build
    and traversal times are positive and no longer than the whole accelerate."""
    import time
    from nbody_gb300 import scenes
    b = scenes.two_plummer(50000)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        with pytest.raises(gpu.NbodyError):
            ctx.bh_stage_ms()
        p = gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, size=0.0, tree_box=1)
        ctx.accelerate(p)
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.accelerate(p)
        ctx.synchronize()
        wall_ms = (time.perf_counter() - t0) * 1e3
        build, walk = ctx.bh_stage_ms()
    assert 0 < build and 0 < walk and build + walk <= wall_ms


@pytest.mark.parametrize("tree_box", [1, 0], ids=["fitted-box", "reference-box"])
def test_bh_wide_mass_range_and_outlier(gpu, tree_box):
    """Masses over twelve decades, a body far outside the cluster and massless bodies: the
    cell sums' fixed-point scale comes from the largest |m| and |x|. The GPU tree's force
    error against an FP64 direct sum is no worse than the reference Barnes-Hut's own at the
    same theta (the oracle's restated octree, built on the same root box)."""
    from nbody_gb300 import scenes
    b = scenes.two_plummer(10000).copy()
    rng = np.random.default_rng(12)
    b[:, 7] = (10.0 ** rng.uniform(-8, 4, len(b))).astype(np.float32)
    b[:40, 7] = 0.0                                 # massless bodies
    b[5, :3] = (3000.0, -2000.0, 1500.0)            # far outside the cluster
    size = 8192.0
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        p = gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, law=gpu.LAW_CUTOFF, size=size, tree_box=tree_box)
        _, _, box = ctx.morton(p)
        ctx.accelerate(p)
        acc = ctx.download_bodies()[:, 8:11].astype(np.float64)
    assert np.all(np.isfinite(acc))
    tg = rng.choice(len(b), 2048, replace=False)
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, 0.0, O.LAW_CUTOFF, radius=b[:, 3], targets=tg)
    # the reference's octree on the same root box (bhtree.cpp:14-85, body by body)
    t = O.Tree(float(box[3]), center=box[:3] + 0.5 * box[3])
    for row in b:
        t.insert(row[:3], row[7])
    ref, _ = t.accel(b, 0.5, 1.0, targets=tg)
    mag = np.maximum(np.linalg.norm(a64, axis=1), 1e-30)
    err_gpu = np.linalg.norm(acc[tg] - a64, axis=1) / mag
    err_ref = np.linalg.norm(ref - a64, axis=1) / mag
    assert np.median(err_gpu) <= 1.05 * np.median(err_ref) + 1e-7, (np.median(err_gpu), np.median(err_ref))
    assert np.percentile(err_gpu, 99) <= 1.5 * np.percentile(err_ref, 99) + 1e-6


def oracle_bh_on_box(bodies, box, theta, targets=None):
    """The reference's octree (bhtree.cpp:14-138, restated) built body by body on the given
    root box (lower corner xyz, edge), and its accelerations."""
    t = O.Tree(float(box[3]), center=np.asarray(box[:3]) + 0.5 * box[3])
    for row in bodies:
        t.insert(row[:3], row[7])
    acc, inter = t.accel(bodies, theta, 1.0, targets=targets)
    return acc.astype(np.float64), inter


@pytest.mark.parametrize("n", [2, 3, 5, 33, 4097])
def test_bh_small_sizes_fitted_box(gpu, n):
    """Tiny systems on the fitted power-of-two box (tree_box = 1), against the reference's
    octree on the same box."""
    from nbody_gb300 import scenes
    b = scenes.plummer(n, seed=50 + n, rmax=10.0)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        p = gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, size=0.0, tree_box=1)
        _, _, box = ctx.morton(p)
        ctx.accelerate(p)
        acc = ctx.download_bodies()[:, 8:11]
    ref, _ = oracle_bh_on_box(b, box, 0.5)
    err = np.linalg.norm(acc - ref, axis=1) / term_scale(b)
    assert np.all(np.isfinite(acc)) and err.max() <= TOL


@pytest.mark.parametrize("tree_box", [1, 0], ids=["fitted-box", "reference-box"])
@pytest.mark.parametrize("law", [0, 1], ids=["cutoff", "softened"])
def test_bh_all_bodies_at_one_point(gpu, law, tree_box):
    """Every body at the same position: a zero-extent bounding box and one bucket of
    identical codes. Each pair has d = 0, which the cutoff removes and the softened law
    multiplies out, so every acceleration is exactly zero, as in the reference."""
    n = 100
    b = np.zeros((n, 12), np.float32)
    b[:, :3] = (1.5, -2.25, 0.75)
    b[:, 3] = 0.01
    b[:, 7] = 1.0
    acc, stats = bh_accel(gpu, b, theta=0.5, law=law, eps2=1e-4 if law == 1 else 0.0, size=64.0, tree_box=tree_box)
    assert np.all(acc == 0), acc[:3]
    assert stats["cells"] >= 1


@pytest.mark.parametrize("precision", [0, 1], ids=["fp32", "compensated"])
def test_bh_graph_replay_equals_eager(gpu, precision):
    """A Barnes-Hut step captured as a CUDA graph (nbody_cuda_update_graph) replays the whole
    build and walk on the device with no host round trip, and gives the same bits as eager
    steps."""
    from nbody_gb300 import scenes
    b = scenes.two_plummer(10000)
    p = gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, dt=5e-4, eps2=1e-4, law=gpu.LAW_SOFTENED, size=0.0, tree_box=1,
                   precision=precision)
    out = []
    for graph in (False, True):
        with gpu.Context() as ctx:
            ctx.upload_bodies(b)
            (ctx.update_graph if graph else ctx.update)(p, 12)
            out.append(ctx.download_bodies())
    assert np.array_equal(out[0], out[1])


def softened_scale(bodies, eps2, targets):
    """sum_j |a_ij| under the softened law (FP64): the scale of an FP32 sum's rounding."""
    _, scale = O.direct_f64(bodies[:, [0, 1, 2, 7]], 1.0, float(np.float32(eps2)), O.LAW_SOFTENED, targets=targets,
                            with_scale=True)
    return np.maximum(scale, 1e-30)


def error_vs(acc, exact):
    """Per target |a - a_exact| / |a_exact|."""
    return np.linalg.norm(np.asarray(acc, np.float64) - exact, axis=1) / np.maximum(np.linalg.norm(exact, axis=1),
                                                                                   1e-300)


@pytest.mark.parametrize("theta", [0.5, 2.0], ids=["ref-theta-0.5", "ref-theta-2"])
@pytest.mark.parametrize("tree_box", [1, 0], ids=["fitted-box", "reference-box"])
def test_bh_softened_config2_against_oracle_octree(gpu, tree_box, theta):
    """Config 2 (two Plummer spheres of 131,072, eps = 0.01) under the softened law, the law
    every benchmark Barnes-Hut number runs, on 4096 sampled targets:
      * against the oracle's octree (bhtree.cpp:14-138 restated, softened visitor) on the
        same root box: per target |a_gpu - a_oracle| <= 5e-5 * sum_j |a_ij| for all but 10
        targets (a rounding-flipped borderline acceptance), median <= 1e-5;
      * against the FP64 direct sum: the GPU's median and p99 relative error are no worse
        than the oracle octree's own (x 1.05), i.e. within the reference's theta error.
    theta is in the reference's convention (2.0 is the conventional 0.5)."""
    from nbody_gb300 import scenes
    b = scenes.two_plummer(131072)
    eps2 = 1e-4
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        p = gpu.params(mode=gpu.MODE_NLOGN, theta=theta, law=gpu.LAW_SOFTENED, eps2=eps2, size=64.0,
                       tree_box=tree_box)
        _, _, box = ctx.morton(p)
        ctx.accelerate(p)
        acc = ctx.download_bodies()[:, 8:11].astype(np.float64)
        stats = ctx.bh_stats()
    if tree_box == 0:
        assert list(box) == [-32.0, -32.0, -32.0, 64.0]
    assert np.all(np.isfinite(acc))
    tg = np.random.default_rng(2).choice(len(b), 4096, replace=False)
    t = O.Tree(1.0)
    t.build_on_box(b, box)
    ref, inter = t.accel(b, theta, 1.0, targets=tg, law=O.LAW_SOFTENED, eps2=float(np.float32(eps2)))
    err = np.linalg.norm(acc[tg] - ref, axis=1) / softened_scale(b, eps2, tg)
    assert np.median(err) <= 1e-5 and (err > TOL).sum() <= 10, (np.median(err), err.max())
    # interactions per body agree with the oracle's on the sampled targets
    assert abs(stats["interactions"] / len(b) - inter / len(tg)) <= 0.05 * inter / len(tg)
    a64 = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(eps2)), O.LAW_SOFTENED, targets=tg)
    e_gpu, e_ref = error_vs(acc[tg], a64), error_vs(ref, a64)
    assert np.median(e_gpu) <= 1.05 * np.median(e_ref) + 1e-7, (np.median(e_gpu), np.median(e_ref))
    assert np.percentile(e_gpu, 99) <= 1.05 * np.percentile(e_ref, 99) + 1e-6


def test_bh_softened_config5_sampled(gpu):
    """Config 5 (16,777,216 bodies: exponential disk + Hernquist halo, eps = 0.005, fitted
    power-of-two root box) under the softened law at reference theta 0.5 and 2 (the
    conventional 0.5), on 4096 sampled targets. The FP64 reference is the GPU's FP64 direct
    sum (nbody_cuda_accel_sampled), itself within 1e-12 of the CPU FP64 oracle on 48 of the
    targets. Two oracle trees, both with the reference's cells and walk:
      * the reference's own octree (FP32 running-mean moments, bhtree.cpp:87-95): the GPU's
        median and p99 error against FP64 are no worse than its own (x 1.05). At this size
        its total mass stalls 6 % low, so it bounds the GPU only loosely;
      * the same cells with exact (FP64-summed) moments, which is what the GPU's
        fixed-point cell sums compute: median |a_gpu - a_oracle| / |a_fp64| <= 1e-5, at
        most 2 % of targets above 1e-4 (a centre of mass one rounding apart flips a
        borderline acceptance), and the GPU's median and p99 error against FP64 within
        5 % of this oracle's."""
    from nbody_gb300 import scenes
    b = scenes.disk_halo()
    eps2 = 0.005 ** 2
    e2 = float(np.float32(eps2))
    thetas = (0.5, 2.0)
    tg = np.random.default_rng(5).choice(len(b), 4096, replace=False)
    accs = {}
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        for theta in thetas:
            p = gpu.params(mode=gpu.MODE_NLOGN, theta=theta, law=gpu.LAW_SOFTENED, eps2=eps2, size=0.0, tree_box=1)
            _, _, box = ctx.morton(p)
            ctx.accelerate(p)
            accs[theta] = ctx.download_bodies()[tg, 8:11].astype(np.float64)
        a64 = ctx.accel_sampled(gpu.params(law=gpu.LAW_SOFTENED, eps2=eps2, precision=gpu.PREC_FP64), tg)
    chk = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, e2, O.LAW_SOFTENED, targets=tg[:48])
    assert error_vs(a64[:48], chk).max() < 1e-12
    t = O.Tree(1.0)
    t.build_on_box(b, box)
    ref32 = {th: t.accel(b, th, 1.0, targets=tg, law=O.LAW_SOFTENED, eps2=e2)[0] for th in thetas}
    t.exact_moments(b)
    for theta, acc in accs.items():
        assert np.all(np.isfinite(acc))
        e_gpu = error_vs(acc, a64)
        e_ref32 = error_vs(ref32[theta], a64)
        assert np.median(e_gpu) <= 1.05 * np.median(e_ref32) + 1e-7, (theta, np.median(e_gpu), np.median(e_ref32))
        assert np.percentile(e_gpu, 99) <= 1.05 * np.percentile(e_ref32, 99) + 1e-6, theta
        exact, _ = t.accel(b, theta, 1.0, targets=tg, law=O.LAW_SOFTENED, eps2=e2)
        diff = np.linalg.norm(acc - exact, axis=1) / np.linalg.norm(a64, axis=1)
        e_ex = error_vs(exact, a64)
        stats = (theta, np.median(diff), np.mean(diff > 1e-4), np.median(e_gpu), np.median(e_ex))
        assert np.median(diff) <= 1e-5 and np.mean(diff > 1e-4) <= 0.02, stats
        assert abs(np.median(e_gpu) - np.median(e_ex)) <= 0.05 * np.median(e_ex), stats
        assert abs(np.percentile(e_gpu, 99) - np.percentile(e_ex, 99)) <= 0.05 * np.percentile(e_ex, 99), stats
