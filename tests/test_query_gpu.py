"""The device ray query against the reference and the oracle, on the GPU.

The bar is exact: the walk's arithmetic (Bounds::ray_intersect, include/nbody/bounds.h:
64-133) is a handful of correctly rounded float operations on both sides, so every ray
must visit the same node indices in the same order, with the same count.
"""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O
from nbody_gb300 import scenes

pytestmark = pytest.mark.gpu

Q = golden("query_cases.npz")


def test_reference_cases(gpu):
    """The cases where the reference's own walk ends, over the reference's tree."""
    with gpu.Context() as ctx:
        for i in range(len(Q["rays"])):
            nodes = O.tree_nodes(Q[f"bodies_{i}"], float(Q["size"][0]))
            hits, counts = ctx.tree_query(Q["rays"][i:i + 1], int(Q["stops"][i]), 128, nodes=nodes)
            c = int(Q[f"count_{i}"][0])
            assert counts[0] == c
            assert np.array_equal(hits[0, :c], Q[f"hits_{i}"])


def random_rays(n, seed, spread=3.0, scale=1.0):
    g = np.random.default_rng(seed)
    o = g.normal(0, spread * scale, (n, 3))
    d = g.normal(0, 1, (n, 3))
    d[: n // 8, 1:] = 0.0           # some axis-aligned rays (the epsilon branches)
    return np.concatenate([o, d], 1).astype(np.float32)


@pytest.mark.parametrize("stop", [0, 1])
@pytest.mark.parametrize("n", [1, 2, 1000, 100000])
def test_exported_tree_matches_oracle(gpu, n, stop):
    b = scenes.plummer(n, seed=11)
    rays = random_rays(4096 if n > 1 else 64, seed=n + stop)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.accelerate(gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, law=gpu.LAW_SOFTENED, eps2=1e-4, size=0.0,
                                  tree_box=1))
        nodes = ctx.tree_export()
        max_hits = 256
        hits, counts = ctx.tree_query(rays, stop, max_hits)           # the device's own exported tree
        hits2, counts2 = ctx.tree_query(rays, stop, max_hits, nodes=nodes)
    assert np.array_equal(hits, hits2) and np.array_equal(counts, counts2)
    missed_any = False
    for r in range(len(rays)):
        h, c, missed = O.tree_query(nodes, rays[r], stop, max_hits)
        missed_any |= missed
        assert counts[r] == c, r
        assert np.array_equal(hits[r, :min(c, max_hits)], h), r
    assert missed_any or n <= 2, "the rays should exercise the skipped-subtree rule"


def test_picking_returns_a_body_leaf(gpu):
    b = scenes.plummer(50000, seed=3)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        ctx.accelerate(gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, law=gpu.LAW_SOFTENED, eps2=1e-4, size=0.0,
                                  tree_box=1))
        nodes = ctx.tree_export()
        # rays from outside aimed at bodies
        tgt = b[:256, :3]
        origin = tgt + np.array([0, 0, 50], np.float32)
        rays = np.concatenate([origin, np.tile([0, 0, -1], (256, 1))], 1).astype(np.float32)
        hits, counts = ctx.tree_query(rays, gpu.QUERY_FIRST_BODY, 512)
    for r in range(256):
        last = nodes[hits[r, min(counts[r], 512) - 1]]
        assert counts[r] <= 512 and last["children"] == 0 and last["mass"] != 0


def test_malformed_node_array_is_an_error_not_a_hang(gpu):
    nodes = np.zeros(9, O.NODE_DTYPE)
    nodes["size"] = 100.0
    nodes[0]["children"] = 1
    for q in range(8):
        nodes[1 + q]["next"] = 1       # a cycle among the children
    rays = np.array([[0, 0, 0, 0, 0, 1]], np.float32)
    with gpu.Context() as ctx:
        with pytest.raises(gpu.NbodyError) as e:
            ctx.tree_query(rays, gpu.QUERY_ALL, 16, nodes=nodes)
        assert e.value.status == gpu.ERR_CUDA
        nodes[1]["next"] = 50          # an index past the array
        with pytest.raises(gpu.NbodyError):
            ctx.tree_query(rays, gpu.QUERY_ALL, 16, nodes=nodes)
        # the context stays usable
        ok = O.tree_nodes(np.array([[1, 1, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0]], np.float32), 100.0)
        h, c = ctx.tree_query(rays, gpu.QUERY_ALL, 16, nodes=ok)
        assert c[0] == 1 and h[0, 0] == 0


def test_empty_inputs(gpu):
    with gpu.Context() as ctx:
        h, c = ctx.tree_query(np.zeros((0, 6), np.float32), gpu.QUERY_ALL, 8,
                              nodes=np.zeros(1, O.NODE_DTYPE))
        assert h.shape == (0, 8) and c.shape == (0,)
        h, c = ctx.tree_query(np.zeros((3, 6), np.float32), gpu.QUERY_ALL, 8, nodes=np.zeros(0, O.NODE_DTYPE))
        assert np.all(c == 0)
        with pytest.raises(gpu.NbodyError):
            ctx.tree_query(np.zeros((1, 6), np.float32), 7, 8, nodes=np.zeros(1, O.NODE_DTYPE))
