"""Build the CUDA library in-tree: hyperfox_gb300/_lib/libhfx_gb300.so.

Every translation unit is compiled by nvcc for sm_103a only, in parallel, and
linked into one shared library with a plain C ABI (include/hfx_gb300.h).
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libhfx_gb300.so")

SOURCES = ["hdg_local.cu", "hdg_burgers.cu", "hdg_trace.cu", "krylov.cu", "trace_gmres.cu", "la_gmres.cu", "noalloc_solve.cu", "hdg_residual.cu", "mixed_kernels.cu", "coarse.cu", "hdg_affine.cu", "tc_assembly.cu", "cg_operators.cu", "rk.cu", "capi.cpp", "refel.cpp", "mesh.cpp", "mesh_io.cpp", "h5io.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-O3", "-I", CSRC, "-I", os.path.join(ROOT, "include")]


def nvcc():
    exe = shutil.which("nvcc")
    if exe is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        exe = "/usr/local/cuda/bin/nvcc"
    if exe is None:
        raise RuntimeError("nvcc not found")
    return exe


def _deps_newer(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".inc"))]
    deps.append(os.path.join(ROOT, "include", "hfx_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, extra):
    path = os.path.join(CSRC, src)
    obj = os.path.join(BUILD, src + ".o")
    if not _deps_newer(obj, path):
        return obj, ""
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc()] + COMMON + extra + ["-x", "c++", "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose=False, extra=None, jobs=None):
    extra = list(extra or [])
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    jobs = jobs or min(len(SOURCES), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for o, log in results:
            if log.strip():
                print(o, log)
    if (not os.path.exists(LIB)) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, extra=[a for a in sys.argv[1:] if a != "-v"]))
