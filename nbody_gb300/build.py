"""In-tree build of the native libraries (sm_103a only; no CMake).

``nbody_gb300/lib/libnbody_cuda.so``
    The CUDA kernels and the C ABI declared in ``include/nbody_cuda.h`` plus the C++
    host layer (``host/``: the CudaSolver behind the reference's Solver interface and the
    ``nbody_sim_*`` C entry points over it).

Each translation unit compiles in its own nvcc/g++ process, in parallel, and the link
step runs once at the end. Only the stale units rebuild.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
INCLUDE = ROOT / "include"
OBJ = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libnbody_cuda.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"]
CXX_FLAGS = ["-O2", "-std=c++20", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found (CUDA 13 toolkit required)")


def cuda_include() -> Path:
    return Path(nvcc()).resolve().parent.parent / "include"


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h")) + sorted(HOST.glob("**/*.h"))


def _units() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(HOST.glob("*.cpp"))


def _compile(src: Path, hdr_mtime: float) -> Path:
    out = OBJ / (src.name + ".o")
    if out.exists() and out.stat().st_mtime >= max(src.stat().st_mtime, hdr_mtime):
        return out
    if src.suffix == ".cu":
        cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", str(INCLUDE), "-I", str(CSRC), "-c", str(src), "-o", str(out)]
    else:
        cmd = ["g++", *CXX_FLAGS, "-I", str(INCLUDE), "-I", str(HOST / "include"), "-I", str(HOST),
               "-I", str(cuda_include()), "-c", str(src), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError(f"compile failed: {src.name}")
    if r.stderr.strip() and os.environ.get("NBODY_BUILD_VERBOSE"):
        sys.stderr.write(r.stderr)
    return out


def build(force: bool = False, jobs: int | None = None) -> Path:
    OBJ.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    if force:
        for o in OBJ.glob("*.o"):
            o.unlink()
    hdr_mtime = max((h.stat().st_mtime for h in _headers()), default=0.0)
    units = _units()
    with ThreadPoolExecutor(max_workers=jobs or min(len(units), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, hdr_mtime), units))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lstdc++"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
            raise RuntimeError("link failed")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
