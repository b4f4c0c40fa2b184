"""Failure detection on the GPU without faulting it: a bounded device wait that is made to
run out reports NBODY_ERR_TIMEOUT through the device error word and the context keeps
working; host-side injected failures surface as statuses with reasons, as the reference's
probe / constructor failures do (source/gpu.cpp:115-149, source/sim.cpp:226-239)."""
import ctypes as C

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_the_context_survives(gpu):
    b = golden("disk_512.npz")["bodies"]
    with gpu.Context() as ctx:
        ctx.upload_bodies(b)
        st = gpu.lib().nbody_cuda_selftest_wait(ctx.h, C.c_uint64(1_000_000))     # 1 ms
        assert st == gpu.ERR_TIMEOUT, st
        assert "timed out" in ctx.error()
        # the error word was consumed; the context steps normally afterwards
        ctx.accelerate(gpu.params(law=gpu.LAW_CUTOFF))
        ctx.synchronize()
        acc = ctx.download_bodies()[:, 8:11]
        assert np.isfinite(acc).all() and np.abs(acc).sum() > 0
        assert gpu.lib().nbody_cuda_selftest_wait(ctx.h, C.c_uint64(0)) == gpu.ERR_INVALID


def test_injected_allocation_failure_is_reported(gpu, monkeypatch):
    b = golden("disk_512.npz")["bodies"]
    with gpu.Context() as ctx:
        monkeypatch.setenv("NBODY_CUDA_FAULT", "alloc")
        with pytest.raises(gpu.NbodyError) as e:
            ctx.upload_bodies(b)
        assert e.value.status == gpu.ERR_ALLOC and "injected" in str(e.value)
        monkeypatch.delenv("NBODY_CUDA_FAULT")
        ctx.upload_bodies(b)
        ctx.accelerate(gpu.params(law=gpu.LAW_CUTOFF))
        ctx.synchronize()
    monkeypatch.setenv("NBODY_CUDA_FAULT", "alloc")
    with pytest.raises(gpu.NbodyError) as e:
        gpu.Context()
    assert e.value.status == gpu.ERR_ALLOC
