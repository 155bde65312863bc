"""The allocation-free trace solve, through the C ABI (needs a GPU).

hfx_trace_solve_noalloc serves callers that cannot allocate device memory: code
under a framework whose caching allocator owns the device memory, and
real-time loops that cannot take an allocation in the middle of a step. They
pass their own device buffers and the solver works in a fixed __device__ array
inside the library. Here torch plays that caller: it allocates the system in
device memory, and the entry point solves it twice in a row. Both answers must
equal hfx_solve's (same CG + block-Jacobi method) within the solver tolerance,
and the oracle's direct FP64 solve of the same system to 1e-8. The iteration
cap, a caller's non-default stream, a non-symmetric system and a pattern row
without its diagonal block are covered too. Collected last, so that a run
stopping at its first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import _oracle as O
from helpers import fields, manufactured, mesh

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


def _system(dim, n, order, kappa="none"):
    from hyperfox_gb300 import capi
    re, coords, cells = mesh(dim, n, order, jitter=0.1, seed=4)
    ctx = capi.Context(0)
    ctx.upload_mesh(dim, order, coords, cells)
    _, _, faces, bnd = ctx.topology()
    ctx.set_source(capi.SRC_SINPROD, param=dim * np.pi ** 2)
    ctx.set_dirichlet(manufactured(coords, faces))
    kap = None
    if kappa != "none":
        _, kap, _ = fields(dim, order, coords, cells, faces, ctx.nFaces, np.random.default_rng(5), kappa=kappa)
        ctx.set_kappa(kap)
    ctx.assemble()
    return ctx, coords, cells, faces, bnd, kap


def _device_system(ctx, bnd):
    import torch
    nf = ctx.re["nNodesFace"]
    rowptr, col, val, rhs = ctx.csr()
    browptr, bcol = face_block_pattern(rowptr, col, ctx.nFaces, nf)
    is_bnd = np.zeros(ctx.nFaces, np.uint8)
    is_bnd[bnd] = 1
    dev = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(dev)
    return dict(nf=nf, browptr=t(browptr), bcol=t(bcol), bnd=t(is_bnd), val=t(val), rhs=t(rhs),
                rowptr=rowptr, col=col, hval=val, hrhs=rhs)


def _call(L, dim, D, nfaces, x, rtol, maxits, stream):
    from hyperfox_gb300 import capi
    info = capi.SolveInfo()
    rc = L.hfx_trace_solve_noalloc(dim, D["nf"], nfaces, D["browptr"].data_ptr(), D["bcol"].data_ptr(),
                                   D["bnd"].data_ptr(), D["val"].data_ptr(), D["rhs"].data_ptr(), x.data_ptr(),
                                   rtol, maxits, ctypes.c_void_p(stream), ctypes.byref(info))
    return rc, info


@pytest.mark.parametrize("dim,n,order", [(2, 8, 2), (3, 2, 3)])
def test_noalloc_solve_matches_hfx_solve_and_oracle(hfx_lib, dim, n, order):
    import torch
    from hyperfox_gb300 import capi
    ctx, coords, cells, faces, bnd, _ = _system(dim, n, order)
    ref, info_ref = ctx.solve(method=capi.KSP_CG, precond=capi.PC_BLOCK_JACOBI, rtol=1e-12)
    assert ctx.ndofs <= capi.NOALLOC_MAX_DOFS
    D = _device_system(ctx, bnd)
    # the oracle's direct FP64 solve of the same problem
    P = O.Problem(dim, order, coords, cells)
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=manufactured(coords, faces).ravel())
    P.assemble()
    x_direct = P.solve_direct()
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for call in range(2):  # two calls in a row: the shared scratch is reused
        x = torch.full((ctx.ndofs,), float(call + 7), dtype=torch.float64, device=dev)
        rc, info = _call(hfx_lib, dim, D, ctx.nFaces, x, 1e-12, 20000, stream)
        torch.cuda.synchronize()
        assert rc == capi.HFX_OK, (call, rc, info.status)
        xs = x.cpu().numpy()
        assert np.linalg.norm(xs - ref) / np.linalg.norm(ref) < 1e-9, call
        assert np.linalg.norm(xs - x_direct) / np.linalg.norm(x_direct) < 1e-8, call
        assert info.rel_residual < 1e-11
        assert abs(info.iterations - info_ref.iterations) <= 2


def test_noalloc_iteration_cap_and_caller_stream(hfx_lib):
    import torch
    from hyperfox_gb300 import capi
    dim = 2
    ctx, _, _, _, bnd, _ = _system(dim, 8, 2)
    ref, _ = ctx.solve(method=capi.KSP_CG, precond=capi.PC_BLOCK_JACOBI, rtol=1e-12)
    D = _device_system(ctx, bnd)
    dev = torch.device("cuda", 0)
    # the cap ends the solve after exactly maxits iterations
    x = torch.zeros(ctx.ndofs, dtype=torch.float64, device=dev)
    rc, info = _call(hfx_lib, dim, D, ctx.nFaces, x, 1e-12, 3, torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize()
    assert rc == capi.HFX_ERR_NOT_CONVERGED and info.status == capi.HFX_ERR_NOT_CONVERGED
    assert info.iterations == 3
    assert info.rel_residual > 1e-12
    # a non-default stream of the caller's: the result is ready when the call returns on it
    side = torch.cuda.Stream(dev)
    with torch.cuda.stream(side):
        x2 = torch.full((ctx.ndofs,), 3.0, dtype=torch.float64, device=dev)
        side.synchronize()
        rc, info = _call(hfx_lib, dim, D, ctx.nFaces, x2, 1e-12, 20000, side.cuda_stream)
        assert rc == capi.HFX_OK
        xs = x2.cpu().numpy()
    assert np.linalg.norm(xs - ref) / np.linalg.norm(ref) < 1e-9


def test_noalloc_refuses_nonsymmetric_and_malformed(hfx_lib):
    import torch
    from hyperfox_gb300 import capi
    dim = 2
    # a diffusion tensor that varies inside the cells makes the trace system non-symmetric
    ctx, _, _, _, bnd, _ = _system(dim, 6, 2, kappa="scalar")
    D = _device_system(ctx, bnd)
    dev = torch.device("cuda", 0)
    x = torch.zeros(ctx.ndofs, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream(dev).cuda_stream
    rc, info = _call(hfx_lib, dim, D, ctx.nFaces, x, 1e-10, 100, s)
    assert rc == capi.HFX_ERR_ARG and info.status == capi.HFX_ERR_ARG
    # a symmetric system whose first interior row lost its diagonal block (its
    # column index points at another face of the system): refused
    ctx2, _, _, _, bnd2, _ = _system(dim, 6, 2)
    D2 = _device_system(ctx2, bnd2)
    bcol = D2["bcol"].cpu().numpy().copy()
    browptr = D2["browptr"].cpu().numpy()
    f = int(np.setdiff1d(np.arange(ctx2.nFaces), bnd2)[0])
    row = bcol[browptr[f]:browptr[f + 1]]
    k = int(np.nonzero(row == f)[0][0])
    other = int(np.setdiff1d(np.arange(ctx2.nFaces), row)[0])
    bcol[browptr[f] + k] = other
    D2["bcol"] = torch.from_numpy(bcol).to(dev)
    x = torch.zeros(ctx2.ndofs, dtype=torch.float64, device=dev)
    rc, info = _call(hfx_lib, dim, D2, ctx2.nFaces, x, 1e-10, 100, s)
    assert rc == capi.HFX_ERR_ARG
    # the same call on the intact pattern still solves (nothing of the refused calls stays behind)
    D2 = _device_system(ctx2, bnd2)
    rc, info = _call(hfx_lib, dim, D2, ctx2.nFaces, x, 1e-10, 20000, s)
    assert rc == capi.HFX_OK and info.rel_residual < 1e-9


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
