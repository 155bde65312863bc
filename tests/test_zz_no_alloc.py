"""The allocation-free trace solve, through the C ABI (needs a GPU).

hfx_trace_solve_noalloc serves callers that cannot allocate device memory
(stream capture, frameworks whose allocator owns the device memory, real-time
loops): they pass their own device buffers and the solver works in a fixed
__device__ array inside the library. This test is the caller: torch allocates
the system in device memory, the entry point solves it twice in a row, and
both answers must equal hfx_solve's (same CG + block-Jacobi method) within the
solver tolerance. Collected last so that a run stopping at its first failure
has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from helpers import manufactured, mesh

pytestmark = pytest.mark.gpu


def face_block_pattern(rowptr, col, nfaces, nf):
    browptr = np.zeros(nfaces + 1, np.int64)
    bcol = []
    for f in range(nfaces):
        r0, r1 = rowptr[f * nf], rowptr[f * nf + 1]
        nb = (r1 - r0) // nf
        browptr[f + 1] = browptr[f] + nb
        bcol.extend(col[r0:r1:nf] // nf)
    return browptr, np.asarray(bcol, np.int32)


@pytest.mark.parametrize("dim,n,order", [(2, 8, 2), (3, 2, 3)])
def test_noalloc_solve_matches_hfx_solve(hfx_lib, dim, n, order):
    import torch
    from hyperfox_gb300 import capi
    re, coords, cells = mesh(dim, n, order, jitter=0.1, seed=4)
    ctx = capi.Context(0)
    ctx.upload_mesh(dim, order, coords, cells)
    _, _, faces, bnd = ctx.topology()
    ctx.set_source(capi.SRC_SINPROD, param=dim * np.pi ** 2)
    ctx.set_dirichlet(manufactured(coords, faces))
    ctx.assemble()
    ref, info_ref = ctx.solve(method=capi.KSP_CG, precond=capi.PC_BLOCK_JACOBI, rtol=1e-12)
    assert ctx.ndofs <= capi.NOALLOC_MAX_DOFS
    nf = ctx.re["nNodesFace"]
    rowptr, col, val, rhs = ctx.csr()
    browptr, bcol = face_block_pattern(rowptr, col, ctx.nFaces, nf)
    is_bnd = np.zeros(ctx.nFaces, np.uint8)
    is_bnd[bnd] = 1
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    d_browptr, d_bcol, d_bnd, d_val, d_rhs = t(browptr), t(bcol), t(is_bnd), t(val), t(rhs)
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = hfx_lib
    for call in range(2):  # two calls in a row: the shared scratch is reused
        x = torch.full((ctx.ndofs,), float(call + 7), dtype=torch.float64, device=dev)
        info = capi.SolveInfo()
        rc = L.hfx_trace_solve_noalloc(dim, nf, ctx.nFaces, d_browptr.data_ptr(), d_bcol.data_ptr(),
                                       d_bnd.data_ptr(), d_val.data_ptr(), d_rhs.data_ptr(), x.data_ptr(),
                                       1e-12, 20000, ctypes.c_void_p(stream), ctypes.byref(info))
        torch.cuda.synchronize()
        assert rc == capi.HFX_OK, (call, rc, info.status)
        xs = x.cpu().numpy()
        assert np.linalg.norm(xs - ref) / np.linalg.norm(ref) < 1e-9, call
        assert info.rel_residual < 1e-11
        assert abs(info.iterations - info_ref.iterations) <= 2


def test_noalloc_refuses_oversized_system(hfx_lib):
    from hyperfox_gb300 import capi
    info = capi.SolveInfo()
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    too_many_faces = capi.NOALLOC_MAX_DOFS // 3 + 1
    rc = hfx_lib.hfx_trace_solve_noalloc(2, 3, too_many_faces, dummy, dummy, dummy, dummy, dummy, dummy,
                                         1e-10, 100, None, ctypes.byref(info))
    assert rc == capi.HFX_ERR_ARG and info.status == capi.HFX_ERR_ARG
    rc = hfx_lib.hfx_trace_solve_noalloc(3, capi.NOALLOC_MAX_NF + 1, 10, dummy, dummy, dummy, dummy, dummy, dummy,
                                         1e-10, 100, None, ctypes.byref(info))
    assert rc == capi.HFX_ERR_ARG
