"""Shared test set-up: repo root on sys.path, the `gpu` marker, built libraries."""
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


@pytest.fixture(scope="session")
def cuda_lib():
    """The CUDA library, built in-tree if stale. Never a fallback."""
    from nbody_gb300 import build, native
    build.build()
    return native.lib()


@pytest.fixture(scope="session")
def gpu(cuda_lib):
    """Skip-free guard for GPU tests: fail loudly if the device is not usable."""
    from nbody_gb300 import native
    st, why = native.probe()
    assert st == native.OK, f"GPU test on a machine without a usable GB300: {why}"
    return native


def golden(name):
    with np.load(GOLDEN / name) as z:
        return {k: z[k] for k in z.files}
