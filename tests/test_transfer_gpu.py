"""Host transfer paths and the predicted readback, on the GPU, through the C ABI.

The bar is bit-exact throughout: a transfer moves bytes, so every path (STAGED, MAPPED,
DIRECT where the device reaches pageable memory) must deliver exactly the records the
copy-engine path delivers, write only the fields a mask selects (Readback,
source/gpu.h:52-58), read min(n, count) records (gpu_solver_split.h:202), and never serve
a predicted readback (gpu_solver_split.h:122-132) that a later call made stale.
"""
import numpy as np
import pytest

from nbody_gb300 import scenes

pytestmark = pytest.mark.gpu

SENTINEL = np.float32(-12345.5)
FIELDS = {1: [0, 1, 2, 7], 2: [3, 4, 5, 6], 4: [8, 9, 10]}     # READ_* bit -> Body floats


def policies(native):
    with native.Context() as ctx:
        pageable = ctx.transfer_info()["pageable"]
    out = [native.TRANSFER_STAGED, native.TRANSFER_MAPPED]
    if pageable:
        out.append(native.TRANSFER_DIRECT)
    return out


def bodies_for(n, seed=7):
    b = scenes.plummer(n, seed=seed)
    b[:, 8:11] = np.random.default_rng(seed).normal(size=(n, 3)).astype(np.float32)
    b[:, 3] = np.random.default_rng(seed + 1).uniform(0, 1e-3, n).astype(np.float32)
    return b


def stepped(native, layout, policy, b, steps=2, **kw):
    with native.Context(layout) as ctx:
        ctx.set_transfer(policy)
        ctx.upload_bodies(b)
        p = native.params(dt=1e-3, eps2=1e-4, law=native.LAW_SOFTENED, **kw)
        ctx.update(p, steps)
        return ctx.download_bodies()


def test_info_and_policy_validation(gpu):
    with gpu.Context() as ctx:
        info = ctx.transfer_info()
        assert info["policy"] == gpu.TRANSFER_AUTO
        assert info["pageable"] in (0, 1, 2)
        expect = gpu.TRANSFER_DIRECT if info["pageable"] == 2 else gpu.TRANSFER_MAPPED
        assert info["resolved"] == expect
        with pytest.raises(gpu.NbodyError) as e:
            ctx.set_transfer(9)
        assert e.value.status == gpu.ERR_INVALID
        if info["pageable"] == 0:
            with pytest.raises(gpu.NbodyError) as e:
                ctx.set_transfer(gpu.TRANSFER_DIRECT)
            assert e.value.status == gpu.ERR_UNSUPPORTED


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
@pytest.mark.parametrize("n", [1, 255, 4099, 1 << 17])
def test_round_trip_is_exact_on_every_path(gpu, layout, n):
    b = bodies_for(n)
    expect = b.copy()
    if layout == gpu.LAYOUT_SOA:
        expect[:, 11] = 0.0     # the split streams do not carry Body::pad
    for up in policies(gpu):
        for down in policies(gpu):
            with gpu.Context(layout) as ctx:
                ctx.set_transfer(up)
                ctx.upload_bodies(b)
                ctx.set_transfer(down)
                out = ctx.download_bodies()
            assert np.array_equal(out.view(np.uint32), expect.view(np.uint32)), (up, down)


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
def test_paths_agree_after_steps(gpu, layout):
    b = bodies_for(3000)
    outs = [stepped(gpu, layout, pol, b) for pol in policies(gpu)]
    for o in outs[1:]:
        assert np.array_equal(o.view(np.uint32), outs[0].view(np.uint32))
    assert not np.array_equal(outs[0][:, :3], b[:, :3]), "the steps must move the bodies"


@pytest.mark.parametrize("mask", [1, 2, 4, 3, 5, 6])
def test_masked_download_writes_only_the_selected_fields(gpu, mask):
    b = bodies_for(5000)
    for pol in policies(gpu):
        with gpu.Context() as ctx:
            ctx.set_transfer(pol)
            ctx.upload_bodies(b)
            ctx.update(gpu.params(dt=1e-3, eps2=1e-4, law=gpu.LAW_SOFTENED), 1)
            full = ctx.download_bodies()
            out = np.full_like(b, SENTINEL)
            ctx.download_bodies(mask=mask, into=out)
        chosen = sorted(sum((FIELDS[k] for k in FIELDS if mask & k), []))
        rest = [c for c in range(12) if c not in chosen]
        assert np.array_equal(out[:, chosen], full[:, chosen]), pol
        assert np.all(out[:, rest] == SENTINEL), pol


def test_download_reads_min_of_n_and_count(gpu):
    b = bodies_for(1000)
    for pol in policies(gpu):
        with gpu.Context() as ctx:
            ctx.set_transfer(pol)
            ctx.upload_bodies(b)
            short = ctx.download_bodies(n=600)
            assert np.array_equal(short[:, :11], b[:600, :11])
            long = np.full((1500, 12), SENTINEL, np.float32)
            ctx.download_bodies(n=1500, into=long)
            assert np.array_equal(long[:1000, :11], b[:, :11])
            assert np.all(long[1000:] == SENTINEL)
            # the count shrinks: a stale, larger readback must not be served
            ctx.set_transfer(gpu.TRANSFER_MAPPED)
            ctx.prefetch(gpu.READ_ALL)
            ctx.upload_bodies(b[:10])
            out = np.full((1000, 12), SENTINEL, np.float32)
            ctx.download_bodies(n=1000, into=out)
            assert np.array_equal(out[:10, :11], b[:10, :11]) and np.all(out[10:] == SENTINEL)


def test_pinned_caller_memory(gpu):
    torch = pytest.importorskip("torch")
    b = bodies_for(4096)
    for pol in policies(gpu):
        host = torch.empty((4096, 12), dtype=torch.float32, pin_memory=True).numpy()
        host[:] = b
        with gpu.Context() as ctx:
            ctx.set_transfer(pol)
            ctx.upload_bodies(host)
            host[:] = SENTINEL
            ctx.download_bodies(into=host)
        assert np.array_equal(host[:, :11], b[:, :11]), pol


@pytest.mark.parametrize("layout", [0, 1], ids=["soa", "aos"])
def test_predicted_readback_is_served_and_exact(gpu, layout):
    b = bodies_for(20000)
    p = gpu.params(dt=1e-3, eps2=1e-4, law=gpu.LAW_SOFTENED)
    with gpu.Context(layout) as ctx:
        ctx.set_transfer(gpu.TRANSFER_MAPPED)
        ctx.upload_bodies(b)
        ctx.update(p, 1)
        ctx.prefetch(gpu.READ_ALL)
        hits0 = ctx.transfer_info()["readback_hits"]
        got = ctx.download_bodies()
        assert ctx.transfer_info()["readback_hits"] == hits0 + 1
        ctx.set_transfer(gpu.TRANSFER_STAGED)
        fresh = ctx.download_bodies()
        assert np.array_equal(got.view(np.uint32), fresh.view(np.uint32))


def test_predicted_readback_goes_stale(gpu):
    b = bodies_for(20000)
    p = gpu.params(dt=1e-3, eps2=1e-4, law=gpu.LAW_SOFTENED)
    with gpu.Context() as ctx:
        ctx.set_transfer(gpu.TRANSFER_MAPPED)
        ctx.upload_bodies(b)
        ctx.update(p, 1)
        ctx.prefetch(gpu.READ_ALL)
        ctx.update(p, 1)                     # moves the bodies past the readback
        hits = ctx.transfer_info()["readback_hits"]
        got = ctx.download_bodies()
        assert ctx.transfer_info()["readback_hits"] == hits
        ctx.set_transfer(gpu.TRANSFER_STAGED)
        assert np.array_equal(got.view(np.uint32), ctx.download_bodies().view(np.uint32))
        # accelerate alone changes the accelerations: also stale
        ctx.set_transfer(gpu.TRANSFER_MAPPED)
        ctx.prefetch(gpu.READ_ALL)
        ctx.accelerate(gpu.params(eps2=4e-4, law=gpu.LAW_SOFTENED))
        got = ctx.download_bodies()
        ctx.set_transfer(gpu.TRANSFER_STAGED)
        assert np.array_equal(got.view(np.uint32), ctx.download_bodies().view(np.uint32))


def test_masked_readback_holds_whole_records(gpu):
    """A readback predicted for positions holds whole records (one pass writes whole lines
    whatever the mask), so both a positions read and a full read are served, exactly."""
    b = bodies_for(8000)
    p = gpu.params(dt=1e-3, eps2=1e-4, law=gpu.LAW_SOFTENED)
    with gpu.Context() as ctx:
        ctx.set_transfer(gpu.TRANSFER_MAPPED)
        ctx.upload_bodies(b)
        ctx.update(p, 1)
        ctx.prefetch(gpu.READ_POSITIONS)
        hits = ctx.transfer_info()["readback_hits"]
        pos = np.full_like(b, SENTINEL)
        ctx.download_bodies(mask=gpu.READ_POSITIONS, into=pos)
        full = ctx.download_bodies()
        assert ctx.transfer_info()["readback_hits"] == hits + 2
        assert np.array_equal(pos[:, FIELDS[1]], full[:, FIELDS[1]])
        assert np.all(pos[:, FIELDS[2] + FIELDS[4]] == SENTINEL)
        ctx.set_transfer(gpu.TRANSFER_STAGED)
        assert np.array_equal(full.view(np.uint32), ctx.download_bodies().view(np.uint32))


def test_misaligned_caller_array_takes_a_staged_path(gpu):
    """The record kernels move 16-byte chunks; an array that is not 16-byte aligned must be
    served through staging, with the same bytes."""
    b = bodies_for(3000)
    raw = np.zeros(3000 * 12 + 2, np.float32)
    view = raw[1:1 + 3000 * 12].reshape(3000, 12)       # 4-byte offset
    assert view.ctypes.data % 16 != 0
    for pol in policies(gpu):
        with gpu.Context() as ctx:
            ctx.set_transfer(pol)
            view[:] = b
            ctx.upload_bodies(view)
            view[:] = SENTINEL
            ctx.download_bodies(into=view)
            assert np.array_equal(view[:, :11], b[:, :11]), pol
            view[:] = SENTINEL
            ctx.download_bodies(mask=gpu.READ_VELOCITIES, into=view)
            assert np.array_equal(view[:, FIELDS[2]], b[:, FIELDS[2]]) and np.all(view[:, FIELDS[1]] == SENTINEL)


def test_prefetch_under_direct_queues_nothing(gpu):
    if gpu.TRANSFER_DIRECT not in policies(gpu):
        pytest.skip("the device does not access pageable host memory")
    b = bodies_for(4000)
    with gpu.Context() as ctx:
        ctx.set_transfer(gpu.TRANSFER_DIRECT)
        ctx.upload_bodies(b)
        ctx.prefetch(gpu.READ_ALL)
        ctx.download_bodies()
        assert ctx.transfer_info()["readback_hits"] == 0


def test_compensated_state_downloads_alike(gpu):
    b = bodies_for(4000)
    outs = [stepped(gpu, 0, pol, b, steps=3, precision=gpu.PREC_COMPENSATED, size=0.0) for pol in policies(gpu)]
    for o in outs[1:]:
        assert np.array_equal(o.view(np.uint32), outs[0].view(np.uint32))
