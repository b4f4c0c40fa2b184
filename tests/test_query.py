"""The ray query's oracle on the CPU: Tree::query (source/bhtree.cpp:153-173) restated,
pinned to the node lists the reference's own walk visits (tests/golden/query_cases.npz),
and the one place the two must differ -- a node the ray misses, where the reference's loop
does not advance -- shown on a small tree."""
import numpy as np
import pytest

from conftest import golden
from oracle import oracle as O

Q = golden("query_cases.npz")


@pytest.mark.parametrize("i", range(len(Q["rays"])))
def test_query_restatement_matches_reference(i):
    # the restated tree build, itself pinned to the reference's node arrays
    nodes = O.tree_nodes(Q[f"bodies_{i}"], float(Q["size"][0]))
    hits, count, missed = O.tree_query(nodes, Q["rays"][i], int(Q["stops"][i]))
    assert not missed
    assert count == int(Q[f"count_{i}"][0])
    assert np.array_equal(hits, Q[f"hits_{i}"])


def test_a_missed_node_is_skipped_not_revisited():
    """A ray that misses one child: the walk visits the root, skips that child's subtree
    and goes on (the reference would stay on the missed child forever)."""
    b = np.zeros((2, 12), np.float32)
    b[0, :3] = (-30, -30, -30)
    b[1, :3] = (30, 30, 30)
    b[:, 7] = 1
    nodes = O.tree_nodes(b, 100.0)
    assert len(nodes) == 9
    ray = np.array([60, -60, 200, 0, 0, -1], np.float32)     # down through the +x, -y column
    hits, count, missed = O.tree_query(nodes, ray, 0)
    assert missed and hits[0] == 0 and 1 <= count < 9
