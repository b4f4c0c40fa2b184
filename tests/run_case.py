"""Run one workload a fixed number of times and exit -- the target for profiler captures.

    python tests/run_case.py direct --n 262144 --steps 1
    python tests/run_case.py direct-aos --n 262144
    python tests/run_case.py integrate --n 16777216

Inputs are the seeded scenes of :mod:`nbody_gb300.scenes`; nothing is timed or checked.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent.parent))


def main(argv=None) -> int:
    from nbody_gb300 import native, scenes

    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["direct", "direct-aos", "direct-cutoff", "integrate", "update",
                                     "compensated", "fp64", "bh", "bh-disk", "batched"])
    ap.add_argument("--n", type=int, default=1 << 18)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--walk", type=int, default=0, help="Barnes-Hut walk: 0 per target, 1 per group")
    ap.add_argument("--variant", type=int, default=-1,
                    help="pin a direct-sum kernel shape (batched: the batched configuration)")
    a = ap.parse_args(argv)

    layout = native.LAYOUT_AOS if a.case == "direct-aos" else native.LAYOUT_SOA
    if a.case == "batched":
        # 512 Plummer systems, log-uniform sizes in [64, 8192]; one autotuned step per --steps
        bodies, off = scenes.batch_plummer()
        p = native.params(mode=native.MODE_BATCHED, law=native.LAW_SOFTENED, eps2=1e-4, dt=1e-3, size=0.0)
        with native.Context() as ctx:
            ctx.upload_bodies(bodies)
            ctx.set_systems(off)
            ctx.batch_set_config(a.variant if a.variant >= 0 else 0)
            ctx.update(p, a.steps)
            ctx.synchronize()
            print(f"batched: bodies={len(bodies)} steps={a.steps} launches={ctx.launches()}")
        return 0
    if a.case == "bh-disk":
        # the 16.8M disk + halo workload, scaled to --n bodies (same 12 : 4.777 split)
        n_disk = int(round(a.n * 12_000_000 / 16_777_216))
        bodies = scenes.disk_halo(n_disk=n_disk, n_halo=a.n - n_disk)
        p = native.params(mode=native.MODE_NLOGN, theta=a.theta, law=native.LAW_SOFTENED, eps2=0.005 ** 2,
                          dt=2.5e-4, size=0.0, tree_box=1, precision=native.PREC_COMPENSATED, walk=a.walk)
        with native.Context() as ctx:
            ctx.upload_bodies(bodies)
            ctx.update(p, a.steps)
            ctx.synchronize()
            print(f"bh-disk: n={a.n} steps={a.steps} launches={ctx.launches()} stats={ctx.bh_stats()}")
        return 0
    if a.case == "bh":
        bodies = scenes.two_plummer(a.n // 2)
    else:
        bodies = scenes.uniform_cube(a.n, seed=1003)
    law = native.LAW_CUTOFF if a.case == "direct-cutoff" else native.LAW_SOFTENED
    prec = {"compensated": native.PREC_COMPENSATED, "fp64": native.PREC_FP64}.get(a.case, native.PREC_FP32)
    mode = native.MODE_NLOGN if a.case == "bh" else native.MODE_N2
    p = native.params(dt=1e-3, G=1.0, eps2=1e-6, law=law, precision=prec, mode=mode, theta=a.theta,
                      size=64.0)
    with native.Context(layout) as ctx:
        ctx.upload_bodies(bodies)
        if a.variant >= 0:
            ctx.set_direct_variant(a.variant)
        for _ in range(a.steps):
            if a.case == "integrate":
                ctx.integrate(p)
            elif a.case == "update":
                ctx.update(p, 1)
            else:
                ctx.accelerate(p)
        ctx.synchronize()
        print(f"{a.case}: n={a.n} steps={a.steps} launches={ctx.launches()}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
