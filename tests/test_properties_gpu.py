"""Size-independent properties at full workload sizes, through the C ABI.

These need no oracle run, so they hold at the sizes where an FP64 or CPU sum over all pairs
would take too long.

Tolerances (stated once, used throughout):
  * Mass scaling: doubling every mass doubles every acceleration bit for bit. A power-of-two
    factor commutes with every rounding in m * r^-3 and in the sums of the direct forms
    (FP32 and compensated). In Barnes-Hut it shifts the fixed-point exponents of the cell
    sums by one, leaving their integers, the cells' centres of mass and every opening
    decision unchanged, so only the cell masses double.
  * Momentum: for the softened law, sum_i m_i a_i = 0 exactly. In FP32 the residual
    |sum_i m_i a_i| stays <= 1e-6 * sum_i m_i |a_i|. The reference's own FP32 brute force
    leaves about 3e-8 of it on the uniform cube at 8192 to 131072 bodies. A dropped source
    chunk or tile leaves orders of magnitude more.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_MOMENTUM = 1e-6


def accel(native, bodies, p):
    with native.Context() as ctx:
        ctx.upload_bodies(bodies)
        ctx.accelerate(p)
        return ctx.download_bodies()[:, 8:11].copy()


def momentum_residual(bodies, acc):
    m = bodies[:, 7].astype(np.float64)
    a = np.asarray(acc, np.float64)
    return np.linalg.norm((m[:, None] * a).sum(0)) / (m * np.linalg.norm(a, axis=1)).sum()


@pytest.mark.parametrize("precision,n", [("fp32", 1 << 20), ("compensated", 1 << 18)])
def test_direct_mass_scaling_and_momentum(gpu, precision, n):
    """The direct sum at the 1M-body bench size (FP32) and at 262,144 bodies (compensated):
    a(2m) == 2 a(m) bit for bit, and the momentum residual stays within TOL_MOMENTUM."""
    from nbody_gb300 import scenes
    b = scenes.uniform_cube(n, seed=1003)
    prec = gpu.PREC_FP32 if precision == "fp32" else gpu.PREC_COMPENSATED
    p = gpu.params(G=1.0, eps2=1e-6, law=gpu.LAW_SOFTENED, size=0.0, precision=prec)
    a1 = accel(gpu, b, p)
    b2 = b.copy()
    b2[:, 7] *= 2.0
    a2 = accel(gpu, b2, p)
    assert np.all(np.isfinite(a1))
    assert np.array_equal(a2, 2.0 * a1)
    assert momentum_residual(b, a1) <= TOL_MOMENTUM


def test_bh_mass_scaling_at_16m(gpu):
    """Barnes-Hut on the 16.8M-body disk + halo (softened, theta 0.5, fitted root box):
    a(2m) == 2 a(m) bit for bit."""
    from nbody_gb300 import scenes
    b = scenes.disk_halo()
    p = gpu.params(mode=gpu.MODE_NLOGN, theta=0.5, law=gpu.LAW_SOFTENED, eps2=0.005 ** 2, size=0.0,
                   tree_box=1)
    a1 = accel(gpu, b, p)
    b[:, 7] *= 2.0
    a2 = accel(gpu, b, p)
    assert np.all(np.isfinite(a1))
    assert np.array_equal(a2, 2.0 * a1)


def test_batched_mass_scaling_and_momentum(gpu):
    """The batched form on the 512 Plummer systems of log-uniform size in [64, 8192]
    (773,681 bodies): a(2m) == 2 a(m) bit for bit, and every system's own momentum
    residual stays within TOL_MOMENTUM (systems never interact)."""
    from nbody_gb300 import scenes
    b, off = scenes.batch_plummer()
    p = gpu.params(mode=gpu.MODE_BATCHED, law=gpu.LAW_SOFTENED, eps2=1e-4)
    out = []
    for scale in (1.0, 2.0):
        bb = b.copy()
        bb[:, 7] *= scale
        with gpu.Context() as ctx:
            ctx.upload_bodies(bb)
            ctx.set_systems(off)
            ctx.accelerate(p)
            out.append(ctx.download_bodies()[:, 8:11].copy())
    a1, a2 = out
    assert np.all(np.isfinite(a1))
    assert np.array_equal(a2, 2.0 * a1)
    m = b[:, 7].astype(np.float64)
    a = a1.astype(np.float64)
    mom = np.add.reduceat(m[:, None] * a, off[:-1], axis=0)
    mag = np.add.reduceat(m * np.linalg.norm(a, axis=1), off[:-1])
    assert np.all(np.linalg.norm(mom, axis=1) <= TOL_MOMENTUM * mag)
