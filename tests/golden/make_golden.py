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
* ``scenes.npz`` -- util::disk and util::cube (util.cpp:14-126) over body ranges of
  arrays with other bodies around them, for the argument sets in DISK_CASES / CUBE_CASES.
* ``query_cases.npz`` -- Tree::query (bhtree.cpp:153-173) on small random trees and rays,
  visiting every met node or stopping at the first body, with the nodes the reference
  visits (only cases where its walk ends: see query_fixtures).

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
    np.savez_compressed(HERE / "scenes.npz", **scene_fixtures())
    np.savez_compressed(HERE / "query_cases.npz", **query_fixtures())
    print("fixtures written to", HERE)


def query_fixtures(per_stop: int = 40) -> dict:
    """Tree::query (bhtree.cpp:153-173) on random small trees and rays. The reference's loop
    never ends once the walk reaches a node the ray misses, so only cases whose walk (per
    the oracle) meets every node it reaches are kept, and the reference runs them in a
    child process with a time limit."""
    import subprocess
    import tempfile
    rng = np.random.default_rng(77)
    cases = []
    counts = {0: 0, 1: 0}
    while min(counts.values()) < per_stop:
        n = int(rng.integers(1, 48))
        b = np.zeros((n, 12), np.float32)
        b[:, :3] = rng.normal(0, 20, (n, 3)).astype(np.float32)
        b[:, 7] = rng.uniform(0.5, 2.0, n).astype(np.float32)
        nodes = O.ref_build_tree(b, 100.0)
        ray = np.r_[rng.normal(0, 30, 3), rng.normal(0, 1, 3)].astype(np.float32)
        for stop in (0, 1):
            if counts[stop] >= per_stop:
                continue
            _, _, missed = O.tree_query(nodes, ray, stop)
            if not missed:
                cases.append((b, ray, stop))
                counts[stop] += 1
    with tempfile.TemporaryDirectory() as tmp:
        src = Path(tmp) / "cases.npz"
        dst = Path(tmp) / "hits.npz"
        np.savez(src, **{f"b{i}": c[0] for i, c in enumerate(cases)},
                 rays=np.stack([c[1] for c in cases]), stops=np.array([c[2] for c in cases]))
        script = (
            "import sys, numpy as np; sys.path.insert(0, %r)\n"
            "from oracle import oracle as O\n"
            "z = np.load(%r); out = {}\n"
            "for i, (r, s) in enumerate(zip(z['rays'], z['stops'])):\n"
            "    h, c = O.ref_tree_query(z[f'b{i}'], 100.0, r, int(s))\n"
            "    out[f'h{i}'] = h; out[f'c{i}'] = np.array([c])\n"
            "np.savez(%r, **out)\n" % (str(HERE.parent.parent), str(src), str(dst)))
        subprocess.run([sys.executable, "-c", script], check=True, timeout=120)
        res = np.load(dst)
        out = {"rays": np.stack([c[1] for c in cases]), "stops": np.array([c[2] for c in cases], np.int32),
               "size": np.array([100.0], np.float32)}
        for i, c in enumerate(cases):
            out[f"bodies_{i}"] = c[0]
            out[f"hits_{i}"] = res[f"h{i}"]
            out[f"count_{i}"] = res[f"c{i}"]
    return out


# util::disk / util::cube argument sets: (total bodies, begin, num, keyword arguments)
DISK_CASES = {
    "defaults": (4097, 0, 4097, {}),
    "tilted": (1000, 0, 1000, dict(center=(10.0, -5.0, 3.0), vel=(1.0, 2.0, 3.0), axis=(0.0, 0.6, 0.8),
                                   inner_radius=50.0, outer_radius=300.0, thickness=2.0, central_mass=1e5,
                                   star_mass=2.0)),
    "one_star": (2, 0, 2, dict(outer_radius=100.0)),
    "central_only": (1, 0, 1, {}),
    "appended": (1001, 300, 701, dict(outer_radius=100.0, axis=(1.0, 0.0, 0.0))),
    "clamped_radii": (777, 0, 777, dict(outer_radius=10.0, axis=(0.0, 0.0, -1.0))),
}
CUBE_CASES = {
    "defaults": (3000, 0, 3000, {}),
    "moving": (500, 100, 300, dict(center=(5.0, 5.0, 5.0), size=100.0, vel=(0.5, 0.0, -1.0), star_mass=3.0)),
}


def scene_fixtures() -> dict:
    out = {}
    for kind, cases, run, args in (("disk", DISK_CASES, O.ref_disk_range, O.disk_arg_array),
                                   ("cube", CUBE_CASES, O.ref_cube_range, O.cube_arg_array)):
        for name, (n, begin, num, kw) in cases.items():
            before = scene_prefix(n)
            after = run(before, begin, num, **kw)
            out[f"{kind}_{name}_bodies"] = after[begin:begin + num]
            out[f"{kind}_{name}_args"] = args(**kw)
            out[f"{kind}_{name}_range"] = np.array([n, begin, num], np.int64)
            assert np.array_equal(np.delete(after, np.s_[begin:begin + num], 0),
                                  np.delete(before, np.s_[begin:begin + num], 0)), "bodies outside the range moved"
    return out


def scene_prefix(n: int) -> np.ndarray:
    """The bodies around a generated range: a fixed pattern the generators must not touch."""
    return (np.arange(n * 12, dtype=np.float32).reshape(n, 12) % 97.0) - 48.0


if __name__ == "__main__":
    main()
