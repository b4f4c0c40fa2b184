"""Build recipe for the oracle -- TEST INFRASTRUCTURE ONLY.

Two shared libraries:

* ``oracle/_build/libnbody_oracle.so`` -- the plain-C restatement in ``nbody_oracle.c``.
  Built everywhere (this machine and the GPU host).
* ``oracle/_ref/libnbody_ref.so`` -- the reference's own CPU solvers compiled from their
  sources where they lie (``source/bhtree.cpp``, ``source/vector.cpp``,
  ``source/util.cpp`` and the header-only ``source/solvers/cpu_*.h``), with the stand-in
  thread pool in ``ref_shim/`` and the C-ABI driver ``ref_shim/ref_driver.cpp``. Built
  only when the reference checkout is present; nothing is copied out of it.

Both use ``-ffp-contract=off`` so every float operation is the one written in the
source on x86-64 and aarch64 alike (GCC contracts a*b+c into an FMA by default in GNU
mode, which would make results depend on the host ISA).

Timing builds (``*_timing.so``) compile the same sources for speed: ``-O2`` with GCC's
default FMA contraction and no errno from the math functions, for the host's baseline ISA
(no ``-march=native``). ``-O2`` is the reference's fastest build: on an x86-64 host its
brute force ran at 1.14 G pairs/s at ``-O2`` and 0.23 at ``-O3``. Only the CPU baselines
are timed on these builds; their results are not checked (contraction changes the last
bits).
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("NBODY_REFERENCE_DIR", "/root/reference"))

ORACLE_LIB = BUILD / "libnbody_oracle.so"
ORACLE_TIMING_LIB = BUILD / "libnbody_oracle_timing.so"
REF_LIB = REF_OUT / "libnbody_ref.so"
REF_TIMING_LIB = REF_OUT / "libnbody_ref_timing.so"

FP_FLAGS = ["-ffp-contract=off", "-fno-fast-math"]
TIMING_FLAGS = ["-O2", "-ffp-contract=fast", "-fno-math-errno"]


def _stale(out: Path, inputs: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"oracle build failed: {cmd[0]} exited {r.returncode}")


def build_oracle(force: bool = False) -> Path:
    srcs = [HERE / "nbody_oracle.c", HERE / "nbody_oracle.h"]
    if force or _stale(ORACLE_LIB, srcs):
        BUILD.mkdir(exist_ok=True)
        tmp = ORACLE_LIB.with_suffix(f".so.tmp{os.getpid()}")
        _run(["gcc", "-std=c11", "-O3", "-fPIC", "-shared", *FP_FLAGS, "-frounding-math",
              "-D_GNU_SOURCE", "-o", str(tmp), str(HERE / "nbody_oracle.c"), "-lm", "-lpthread"])
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_oracle_timing(force: bool = False) -> Path:
    srcs = [HERE / "nbody_oracle.c", HERE / "nbody_oracle.h"]
    if force or _stale(ORACLE_TIMING_LIB, srcs):
        BUILD.mkdir(exist_ok=True)
        tmp = ORACLE_TIMING_LIB.with_suffix(f".so.tmp{os.getpid()}")
        _run(["gcc", "-std=c11", "-fPIC", "-shared", *TIMING_FLAGS, "-D_GNU_SOURCE", "-o", str(tmp),
              str(HERE / "nbody_oracle.c"), "-lm", "-lpthread"])
        os.replace(tmp, ORACLE_TIMING_LIB)
    return ORACLE_TIMING_LIB


def reference_available() -> bool:
    return (REFERENCE / "source" / "bhtree.cpp").exists()


def build_ref(force: bool = False, timing: bool = False) -> Path | None:
    if not reference_available():
        return None
    shim = HERE / "ref_shim"
    srcs = [REFERENCE / "source" / f for f in ("bhtree.cpp", "vector.cpp", "util.cpp")]
    deps = srcs + [shim / "ref_driver.cpp", shim / "BS_thread_pool.hpp"]
    out = REF_TIMING_LIB if timing else REF_LIB
    flags = TIMING_FLAGS if timing else ["-O2", *FP_FLAGS]
    if force or _stale(out, deps):
        REF_OUT.mkdir(exist_ok=True)
        tmp = out.with_suffix(f".so.tmp{os.getpid()}")
        _run(["g++", "-std=c++20", "-fPIC", "-shared", *flags,
              "-I", str(shim), "-I", str(REFERENCE / "include"), "-I", str(REFERENCE / "source"),
              "-o", str(tmp), str(shim / "ref_driver.cpp"), *map(str, srcs), "-lpthread"])
        os.replace(tmp, out)
    return out


def build(force: bool = False) -> None:
    build_oracle(force)
    build_oracle_timing(force)
    build_ref(force)
    build_ref(force, timing=True)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
    print(ORACLE_LIB, REF_LIB if REF_LIB.exists() else "(reference not built)")
