"""hfx::gpu::MeshUnion (the C++ host API's batch of independent problems) on the CPU:
tests/cpp/test_mesh_union.cpp calls host entry points only (topology, high-order nodes)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_cpp_mesh_union(hfx_lib, tmp_path):
    exe = str(tmp_path / "test_mesh_union")
    lib = os.path.join(ROOT, "hyperfox_gb300", "_lib")
    subprocess.check_call(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(ROOT, "hyperfox_gb300", "host"),
                           os.path.join(ROOT, "tests", "cpp", "test_mesh_union.cpp"), "-L", lib, "-lhfx_gb300",
                           "-Wl,-rpath," + lib, "-o", exe])
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "OK" in r.stdout
