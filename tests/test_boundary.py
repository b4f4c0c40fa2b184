"""The C-ABI boundary without compute: the library builds, loads, exports every symbol
include/*.h declares, and reports failures the reference's way (a probe that returns a
reason, source/gpu.cpp:115-149; a constructor failure turned into a status)."""
import re

from conftest import ROOT


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(nbody_\w+)\s*\(", text))
    return names


def test_header_declares_and_library_exports_everything(cuda_lib):
    from nbody_gb300 import native
    names = declared_symbols()
    assert names, "no declarations found"
    missing = [n for n in sorted(names) if not hasattr(cuda_lib, n)]
    assert not missing, missing
    assert set(native.EXPORTS) <= names


def test_probe_reports_a_reason(cuda_lib):
    from nbody_gb300 import native
    st, why = native.probe()
    if st != native.OK:
        assert why, "an unavailable device must say why"


def test_injected_no_device(cuda_lib, monkeypatch):
    from nbody_gb300 import native
    monkeypatch.setenv("NBODY_CUDA_FAULT", "nodevice")
    st, why = native.probe()
    assert st == native.ERR_NO_DEVICE and "injected" in why
    try:
        native.Context()
    except native.NbodyError as e:
        assert e.status == native.ERR_NO_DEVICE and "injected" in str(e)
    else:
        raise AssertionError("context creation must fail when the probe fails")


def test_bad_layout_rejected(cuda_lib):
    from nbody_gb300 import native
    try:
        native.Context(layout=7)
    except native.NbodyError as e:
        assert e.status in (native.ERR_INVALID, native.ERR_NO_DEVICE, native.ERR_UNSUPPORTED)
    else:
        raise AssertionError("an unknown layout must be rejected")


def test_noalloc_rejects_misaligned_streams_before_any_cuda_call(cuda_lib):
    """The allocation-free accelerate checks its arguments before it touches CUDA: a stream
    it would read as float4 from an address that is not 16-byte aligned is NBODY_ERR_INVALID
    (the radii only under the CUTOFF law, where the kernel reads them). No device is needed."""
    import ctypes as C
    from nbody_gb300 import native
    f = cuda_lib.nbody_cuda_dev_accel_soa_noalloc
    cut = native.params(law=native.LAW_CUTOFF)
    soft = native.params(law=native.LAW_SOFTENED, eps2=1e-4)
    ok, off = C.c_void_p(1 << 20), C.c_void_p((1 << 20) + 4)
    assert f(ok, off, ok, 100, C.byref(cut), None) == native.ERR_INVALID
    assert f(off, ok, ok, 100, C.byref(soft), None) == native.ERR_INVALID
    assert f(ok, ok, off, 100, C.byref(soft), None) == native.ERR_INVALID
    assert f(ok, None, ok, 100, C.byref(cut), None) == native.ERR_INVALID


def test_step_params_layout():
    import ctypes
    from nbody_gb300 import native
    assert ctypes.sizeof(native.StepParams) == 12 * 4
