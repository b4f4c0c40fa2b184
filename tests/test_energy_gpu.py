"""nbody_cuda_energy: energy and momentum of all bodies at the direct sum's rate.

Bars: against the FP64 oracle (orc_energy_f64, Neumaier-compensated FP64 over every pair)
and the GPU's FP64 per-system diagnostics (nbody_cuda_system_energy):
  * potential energy within 1e-7 relative (FP32 pair terms; tile sums folded exactly);
  * kinetic energy and momentum within 1e-12 relative (FP64 sums of the same floats);
  * the same result in the split and interleaved layouts, and bit-identical on repeat.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def oracle_energy(b, eps2):
    return O.energy_f64(b[:, :3].astype(np.float64), b[:, 4:7].astype(np.float64), b[:, 7].astype(np.float64),
                        1.0, float(np.float32(eps2)))


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
@pytest.mark.parametrize("law", [0, 1], ids=["unsoftened", "softened"])
@pytest.mark.parametrize("n", [4096, 3001])
def test_energy_matches_fp64_oracle(gpu, law, layout, n):
    """Config 1's Plummer sphere, and a ragged size whose last block row is short."""
    from nbody_gb300 import scenes
    b = scenes.plummer(n, seed=1001)
    eps2 = 1e-4 if law == 1 else 0.0
    p = gpu.params(law=law, eps2=eps2)
    with gpu.Context(layout) as ctx:
        ctx.upload_bodies(b)
        e = ctx.energy(p)
        again = ctx.energy(p)
    ke, pe, mom = oracle_energy(b, eps2)
    assert abs(e["potential"] - pe) <= 1e-7 * abs(pe), (e["potential"], pe)
    assert abs(e["kinetic"] - ke) <= 1e-12 * ke
    assert np.abs(e["momentum"] - mom).max() <= 1e-12 * np.abs(b[:, 7] * np.linalg.norm(b[:, 4:7], axis=1)).sum()
    assert e["potential"] == again["potential"] and e["kinetic"] == again["kinetic"]


def test_energy_matches_gpu_fp64_diagnostics(gpu):
    """A 131,073-body cube (the ragged last block included) against the FP64 per-system
    diagnostics on the same device state, with G applied."""
    from nbody_gb300 import scenes
    b = scenes.uniform_cube(131073, seed=7)
    b[:, 4:7] = np.random.default_rng(2).normal(0, 0.1, (len(b), 3)).astype(np.float32)
    p = gpu.params(law=gpu.LAW_SOFTENED, eps2=1e-6, G=2.5)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        e = ctx.energy(p)
        ref = ctx.system_energy(p)[0]
    assert abs(e["kinetic"] - ref[0]) <= 1e-12 * ref[0]
    assert abs(e["potential"] - ref[1]) <= 1e-7 * abs(ref[1]), (e["potential"], ref[1])
    assert np.abs(e["momentum"] - ref[2:5]).max() <= 1e-10 * np.abs(ref[2:5]).max() + 1e-15


def test_energy_tracks_a_run(gpu):
    """Over a short softened run the diagnostics see the same energy drift as the FP64
    per-system ones."""
    from nbody_gb300 import scenes
    b = scenes.plummer(8192, seed=3)
    p = gpu.params(law=gpu.LAW_SOFTENED, eps2=1e-4, dt=1e-3, size=0.0)
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        e0, r0 = ctx.energy(p), ctx.system_energy(p)[0]
        ctx.update(p, 50)
        e1, r1 = ctx.energy(p), ctx.system_energy(p)[0]
    d = (e1["kinetic"] + e1["potential"]) / (e0["kinetic"] + e0["potential"]) - 1
    dr = (r1[0] + r1[1]) / (r0[0] + r0[1]) - 1
    assert abs(d - dr) <= 2e-7, (d, dr)
    assert abs(d) < 1e-3


def test_energy_empty_and_rejects(gpu):
    with gpu.Context() as ctx:
        e = ctx.energy(gpu.params(law=gpu.LAW_SOFTENED, eps2=1e-4))
        assert e["kinetic"] == 0 and e["potential"] == 0
        with pytest.raises(gpu.NbodyError):
            ctx.energy(gpu.params(law=gpu.LAW_SOFTENED, eps2=0.0))
