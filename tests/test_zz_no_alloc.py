"""The accelerate entry point that allocates nothing (nbody_cuda_dev_accel_soa_noalloc).

It serves callers that cannot let the library call cudaMalloc -- a frame loop that must
not stall on the device-wide synchronisation of cudaMalloc/cudaFree, or a plugin host
that owns every device allocation -- by keeping its scratch in a fixed array inside the
library. This file sorts last so that a run stopping at the first failure has already
run every other test. It must pass alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu

# The direct-sum tolerance used throughout tests/test_direct_gpu.py: per body
# |a - a_ref| <= 5e-5 * sum_j |a_ij|, median <= 1e-5.
TOL_MAX = 5e-5
TOL_MEDIAN = 1e-5


def _scaled(a, ref, scale):
    return np.linalg.norm(a.astype(np.float64) - ref.astype(np.float64), axis=1) / scale


@pytest.mark.parametrize("n,law,eps2", [(4096, 0, 0.0), (200003, 1, 1e-6), (1 << 20, 1, 1e-6)])
def test_noalloc_matches_context_entry_point(gpu, n, law, eps2):
    torch = pytest.importorskip("torch")
    from nbody_gb300 import native, scenes
    from oracle import oracle as O

    b = golden("cube_4096.npz")["bodies"] if n == 4096 else scenes.uniform_cube(n, seed=17 + n)
    pm = torch.from_numpy(np.ascontiguousarray(b[:, [0, 1, 2, 7]])).cuda()
    vr = torch.from_numpy(np.ascontiguousarray(b[:, [4, 5, 6, 3]])).cuda()
    ref_acc = torch.zeros_like(pm)
    p = native.params(law=law, eps2=eps2)
    stream = torch.cuda.current_stream().cuda_stream

    with native.Context() as ctx:
        ctx.set_stream(stream)
        ctx.dev_accel_soa(pm.data_ptr(), vr.data_ptr(), ref_acc.data_ptr(), n, p)
        ctx.synchronize()
    expect = ref_acc.cpu().numpy()[:, :3]

    tg = np.random.default_rng(n).choice(n, min(n, 256), replace=False)
    _, scale = O.direct_f64(b[:, [0, 1, 2, 7]], 1.0, eps2, law, radius=b[:, 3], targets=tg, with_scale=True)
    scale = np.maximum(scale, 1e-30)

    L = native.lib()
    for call in range(2):
        acc = torch.full_like(pm, float("nan"))
        st = L.nbody_cuda_dev_accel_soa_noalloc(C.c_void_p(pm.data_ptr()), C.c_void_p(vr.data_ptr()),
                                                C.c_void_p(acc.data_ptr()), n, C.byref(p), C.c_void_p(stream))
        assert st == native.OK, (call, st)
        got = acc.cpu().numpy()[:, :3]
        assert np.isfinite(got).all()
        err = _scaled(got[tg], expect[tg], scale)
        assert err.max() <= TOL_MAX and np.median(err) <= TOL_MEDIAN, (call, err.max())


def test_noalloc_runs_while_allocation_is_refused(gpu, monkeypatch):
    """The entry point's one promise: it allocates nothing. With every library allocation
    made to fail (NBODY_CUDA_FAULT=alloc, the host-side injector), a context cannot grow its
    scratch, yet two allocation-free calls in a row still succeed and agree bit for bit.
    Device free memory is unchanged across the two calls."""
    torch = pytest.importorskip("torch")
    from nbody_gb300 import native, scenes

    n = 200003
    b = scenes.uniform_cube(n, seed=99)
    pm = torch.from_numpy(np.ascontiguousarray(b[:, [0, 1, 2, 7]])).cuda()
    vr = torch.from_numpy(np.ascontiguousarray(b[:, [4, 5, 6, 3]])).cuda()
    p = native.params(law=1, eps2=1e-6)
    stream = torch.cuda.current_stream().cuda_stream
    L = native.lib()
    outs = [torch.full_like(pm, float("nan")) for _ in range(2)]
    torch.cuda.synchronize()
    with native.Context() as ctx:        # the context path refuses to grow its scratch
        ctx.set_stream(stream)
        monkeypatch.setenv("NBODY_CUDA_FAULT", "alloc")
        with pytest.raises(native.NbodyError) as e:
            ctx.dev_accel_soa(pm.data_ptr(), vr.data_ptr(), outs[0].data_ptr(), n, p)
        assert e.value.status == native.ERR_ALLOC
    free = []
    for acc in outs:
        free.append(torch.cuda.mem_get_info()[0])
        st = L.nbody_cuda_dev_accel_soa_noalloc(C.c_void_p(pm.data_ptr()), C.c_void_p(vr.data_ptr()),
                                                C.c_void_p(acc.data_ptr()), n, C.byref(p), C.c_void_p(stream))
        assert st == native.OK, st
    free.append(torch.cuda.mem_get_info()[0])
    a0, a1 = outs[0].cpu().numpy(), outs[1].cpu().numpy()
    assert np.isfinite(a0[:, :3]).all()
    assert np.array_equal(a0.view(np.uint32), a1.view(np.uint32))
    assert free[1] == free[2], free


def test_noalloc_rejects_oversize_and_bad_arguments(gpu):
    from nbody_gb300 import native
    L = native.lib()
    p = native.params(law=1, eps2=1e-6)
    st = L.nbody_cuda_dev_accel_soa_noalloc(C.c_void_p(16), C.c_void_p(16), C.c_void_p(16),
                                            (1 << 20) + 1, C.byref(p), None)
    assert st == native.ERR_INVALID
    bad = native.params(law=1, eps2=0.0)
    assert L.nbody_cuda_dev_accel_soa_noalloc(None, None, None, 10, C.byref(bad), None) == native.ERR_INVALID
    assert L.nbody_cuda_dev_accel_soa_noalloc(None, None, None, 0, C.byref(p), None) == native.OK
