"""The bench's reference arm on the CPU: its arithmetic from a measured pair rate to the
reported body-steps/s, with the CPU measurement replaced by a known rate, and one short
real run of it."""
import json
import subprocess
import sys
import types

import pytest

from conftest import ROOT

sys.path.insert(0, str(ROOT))
import bench  # noqa: E402


def test_reference_arm_converts_pairs_per_second_to_body_steps(monkeypatch):
    rate = 4.0e9        # pairs/s
    monkeypatch.setattr(bench, "cpu_brute_force_rate", lambda bodies, seconds: (rate, 16, "port", "sample"))
    args = types.SimpleNamespace(warmup=1, steps=3, cpu_seconds=1.0)
    line = bench.bench_reference(args)
    n = bench.N
    assert line["value"] == pytest.approx(rate / n)                 # N^2 pairs per body-step of N bodies
    assert line["ms_per_step"] == pytest.approx(n * n / rate * 1e3)
    assert line["cpu_baseline"]["value"] == line["value"] and line["e2e"]["value"] == line["value"]
    assert line["impl"] == "reference" and line["unit"] == "body-steps/s"


def test_reference_arm_runs():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1", "--cpu-seconds", "1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    # a CPU direct sum of 2^20 bodies takes minutes per step on any host: well under 1e5 body-steps/s
    assert 0 < line["value"] < 1e5
    assert line["ms_per_step"] > 1e3


@pytest.mark.parametrize("use_ref", [True, False], ids=["reference", "port"])
def test_config1_cpu_timing_runs_both_paths(monkeypatch, use_ref):
    """The config-1 CPU leg: all steps of the reference brute force where its build loads,
    else the restated solver and integrator, timed on the same bodies."""
    from nbody_gb300 import scenes
    from oracle import oracle as O
    if use_ref and not O.ref_available():
        pytest.skip("the reference's own CPU build is not present here")
    if not use_ref:
        monkeypatch.setattr(O, "ref_available", lambda: False)
    b = scenes.plummer(256, seed=1001)
    s, cores, kind = bench.cpu_config1_seconds(b, 3, 1e-3)
    assert s > 0 and cores >= 1
    assert kind.startswith("reference" if use_ref else "port")
