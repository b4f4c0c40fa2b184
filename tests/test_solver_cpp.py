"""The C++ host layer: CudaSolver behind the Solver interface, driven through Sim.

* CPU: cuda_solver.h compiles unchanged against the reference's own Solver/State headers
  (when the reference checkout is present), i.e. it is a drop-in for source/solver.h.
* GPU: tests/cpp/test_solver.cpp -- the reference's Catch2 checks for GPU variants
  (tests/source/test_gpu.cpp, test_variant.cpp, test_wrap.cpp, test_sim.cpp) restated for
  the CUDA variants -- built against libnbody_cuda.so and the oracle, and run.
"""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from conftest import ROOT

REFERENCE = Path(os.environ.get("NBODY_REFERENCE_DIR", "/root/reference"))
CXX = shutil.which("g++")


def cuda_include():
    from nbody_gb300 import build
    return str(build.cuda_include())


@pytest.mark.skipif(not (REFERENCE / "source" / "solver.h").exists() or CXX is None,
                    reason="reference checkout not present on this machine")
def test_cuda_solver_compiles_against_the_reference_headers(tmp_path, cuda_lib):
    """The same cuda_solver.h, with the reference's include/ and source/ ahead of this
    library's host headers: Solver, State, Body and bh::Tree are the reference's."""
    src = tmp_path / "probe.cpp"
    src.write_text('#include "cuda_solver.h"\n'
                   'static_assert(!std::is_abstract_v<nbody::CudaSolver>);\n'
                   'int main() { return 0; }\n')
    shim = ROOT / "oracle" / "ref_shim"
    # this library's own mirror headers (nbody_gb300/host/include) are deliberately absent
    cmd = [CXX, "-std=c++20", "-fsyntax-only", "-include", "type_traits",
           "-I", str(REFERENCE / "include"), "-I", str(REFERENCE / "source"), "-I", str(shim),
           "-I", str(ROOT / "include"), "-I", str(ROOT / "nbody_gb300" / "host"),
           "-I", cuda_include(), str(src)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.fixture(scope="module")
def solver_test_binary(cuda_lib, tmp_path_factory):
    from nbody_gb300 import build
    from oracle import build_oracle
    oracle_lib = build_oracle.build_oracle()
    out = tmp_path_factory.mktemp("cpp") / "test_solver"
    lib = build.LIB
    cmd = [CXX or "g++", "-std=c++20", "-O1", "-o", str(out), str(ROOT / "tests" / "cpp" / "test_solver.cpp"),
           "-I", str(ROOT / "include"), "-I", str(ROOT / "nbody_gb300" / "host" / "include"),
           "-I", str(ROOT / "nbody_gb300" / "host"), "-I", str(ROOT / "oracle"), "-I", cuda_include(),
           str(lib), str(oracle_lib), f"-Wl,-rpath,{lib.parent}", f"-Wl,-rpath,{oracle_lib.parent}", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("transfer", ["auto", "staged", "mapped"])
def test_cuda_solver_suite(solver_test_binary, transfer):
    """The whole suite once per host transfer path: the state the reference's read path
    sees must not depend on how the bytes travel, nor on the predicted readback."""
    env = dict(os.environ, NBODY_CUDA_TRANSFER=transfer)
    r = subprocess.run([str(solver_test_binary)], capture_output=True, text=True, timeout=600, env=env)
    print(r.stdout)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert "FAIL" not in r.stdout
