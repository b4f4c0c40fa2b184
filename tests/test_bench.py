"""The bench's reference arm on the CPU: its arithmetic from a measured pair rate to the
reported body-steps/s, with the CPU measurement replaced by a known rate, and one short
real run of it."""
import json
import subprocess
import sys
import types

import numpy as np
import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def test_reference_arm_reports_what_it_timed(monkeypatch):
    """Each step of the reference arm is a bounded sample of k bodies of the workload: the
    line's value is those bodies' steps over the time the steps took, and ms_per_step is
    the measured time of one step, so steps x ms_per_step is the timed region."""
    from oracle import oracle as O
    calls = []

    def fake_bf(bodies, G, targets, nthreads=0, law=O.LAW_CUTOFF, eps2=0.0, timing=False):
        calls.append((len(targets), law, eps2, timing))
        return np.zeros((len(targets), 3), np.float32)

    monkeypatch.setattr(O, "brute_force_targets", fake_bf)
    args = types.SimpleNamespace(warmup=1, steps=3, cpu_seconds=1.0)
    line = bench.bench_reference(args)
    k = line["config"]["bodies_per_step"]
    assert line["value"] == pytest.approx(k / (line["ms_per_step"] * 1e-3))
    assert line["cpu_baseline"]["value"] == line["value"] and line["e2e"]["value"] == line["value"]
    assert line["impl"] == "reference" and line["unit"] == "body-steps/s"
    assert line["config"]["same_config"] and line["config"]["law"] == "softened"
    # the GPU arm's law, in the speed build, every step
    assert all(c[1] == O.LAW_SOFTENED and c[2] == pytest.approx(bench.EPS ** 2) and c[3] for c in calls)
    assert calls[-1][0] == k


def test_reference_arm_runs():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-seconds", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    # a CPU direct sum of 2^20 sources: well under 1e5 body-steps/s on any host
    assert 0 < line["value"] < 1e5
    assert line["ms_per_step"] > 0 and line["config"]["bodies_per_step"] >= 1


def test_config1_cpu_timing_runs():
    """The config-1 CPU leg: all steps of the restated brute force (softened law, speed
    build) and integrator, timed on the same bodies."""
    from nbody_gb300 import scenes
    b = scenes.plummer(256, seed=1001)
    s, cores, kind = bench.cpu_config1_seconds(b, 3, 1e-3, 1e-4)
    assert s > 0 and cores >= 1
    assert kind.startswith("port")


def test_cpu_baselines_use_the_gpu_law():
    """The CPU brute force the bench times is the softened law the GPU arm runs: on a small
    system its sums agree with the FP64 softened oracle."""
    from nbody_gb300 import scenes
    from oracle import oracle as O
    b = scenes.plummer(512, seed=4)
    tg = np.arange(512)
    a = O.brute_force_targets(b, 1.0, tg, law=O.LAW_SOFTENED, eps2=1e-4, timing=True)
    a64, scale = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, float(np.float32(1e-4)), O.LAW_SOFTENED, with_scale=True)
    assert (np.linalg.norm(a - a64, axis=1) / scale).max() < 1e-5
