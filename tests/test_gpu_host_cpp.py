"""The reference's own unit tests re-expressed in C++ against the host API
(tests/cpp/test_host_api.cpp: TestLinAlgebraInterfaces.cpp ordering/identity/
triangular, TestHDGSolver.cpp setup sequence + constant Dirichlet, TestHDF5Io.cpp write/load)."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_host_api(hfx_lib, tmp_path):
    exe = str(tmp_path / "test_host_api")
    lib = os.path.join(ROOT, "hyperfox_gb300", "_lib")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(ROOT, "hyperfox_gb300", "host"),
                           os.path.join(ROOT, "tests", "cpp", "test_host_api.cpp"), "-L", lib, "-lhfx_gb300",
                           "-Wl,-rpath," + lib, "-o", exe])
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout
