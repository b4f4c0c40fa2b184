"""Generate the golden fixtures in this directory from the reference itself.

Runs the reference's own CPU code (compiled from its sources into oracle/_ref/ by
oracle/build_oracle.py) and records its inputs and outputs:

* ``disk_{512,1024,2048}.npz`` -- util::disk (source/util.cpp:14-98) with the arguments
  the reference tests use (outer_radius = 100), and for each:
  ``bf_acc``  CpuBruteForceSolver::accelerate (cpu_brute_force.h:17-43), G = 1;
  ``bh_acc``  CpuBarnesHutSolver::accelerate (cpu_barnes_hut.h:22-44), size 10000, theta 0.5;
  ``steps``   bodies after 5 x Solver::update(1/120) of the brute-force solver, wrap on.
* ``cube_4096.npz`` -- util::cube (util.cpp:100-126) and its brute-force / Barnes-Hut
  accelerations and the octree node array (detail::build_tree, tree.h:14-29).
* ``bhtree_cases.npz`` -- the insertion sequences of tests/source/test_bhtree.cpp:30-142
  and the node arrays the reference builds for them.

Usage: ``python tests/golden/make_golden.py`` (needs the reference checkout; the
fixtures are committed so the tests never need it).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

from oracle import oracle as O  # noqa: E402


def main() -> None:
    if not O.ref_available():
        raise SystemExit("the reference could not be built here; fixtures unchanged")
    for n in (512, 1024, 2048):
        b = O.ref_disk(n)
        bf = O.ref_brute_force(b, 1.0)[:, 8:11]
        bh = O.ref_barnes_hut(b, 10000.0, 0.5, 1.0)[:, 8:11]
        steps = O.ref_brute_force(b, 1.0, steps=5, dt=1.0 / 120.0, size=10000.0, do_wrap=True)
        np.savez_compressed(HERE / f"disk_{n}.npz", bodies=b, bf_acc=bf, bh_acc=bh, steps=steps)
    c = O.ref_cube(4096)
    np.savez_compressed(HERE / "cube_4096.npz", bodies=c,
                        bf_acc=O.ref_brute_force(c, 1.0)[:, 8:11],
                        bh_acc=O.ref_barnes_hut(c, 10000.0, 0.5, 1.0)[:, 8:11],
                        nodes=O.ref_build_tree(c, 10000.0).view(np.uint8))
    cases = {
        "diff_quadrants": ([1, 1, 1, 1], [-1, -1, -1, 2]),
        "same_quadrant": ([1, 1, 1, 1], [99, 99, 99, 1]),
        "eight": ([50, 50, 50, 1], [-50, 50, 50, 1], [50, -50, 50, 1]),
        "same_location": ([1, 1, 1, 1], [1, 1, 1, 1]),
        "very_close": ([1, 1, 1, 1], [1 + np.finfo(np.float32).eps, 1, 1, 1]),
    }
    out = {}
    for name, pts in cases.items():
        pts = np.asarray(pts, np.float32)
        out[f"{name}_points"] = pts
        out[f"{name}_nodes"] = O.ref_insert_points(pts, (0, 0, 0), 100.0).view(np.uint8)
    np.savez_compressed(HERE / "bhtree_cases.npz", **out)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
