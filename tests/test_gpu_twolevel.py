"""Two-level trace preconditioner (block Jacobi + vertex coarse space), through the C ABI.

The coarse operator is checked against the Galerkin product P^T A' P formed here
from the oracle's trace CSR and a prolongation built independently from the face
geometry (barycentric coordinates of every face node w.r.t. its face's vertices);
FP32 coarse values, so the bar is 1e-5 of the largest entry. Solves with the
two-level preconditioner must match the oracle's direct solve like every other
solve (1e-8 relative L2) and need fewer iterations than block Jacobi.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from test_gpu_parity import build_pair, relerr

pytestmark = pytest.mark.gpu


def galerkin_coarse(P, coords, rowptr, col, val, vertex_node):
    """P^T A' P with A' = -A on interior rows/cols (Dirichlet rows/cols dropped)."""
    dim = coords.shape[1]
    nF, Nf = P.faces.shape
    A = sp.csr_matrix((val, col, rowptr), shape=(nF * Nf, nF * Nf))
    bnd = np.zeros(nF, bool)
    bnd[P.boundary] = True
    interior = np.repeat(~bnd, Nf)
    V = coords[P.faces[:, :dim]]                     # [nF, dim, dim] face vertices
    X = coords[P.faces]                              # [nF, Nf, dim] face nodes
    E = np.stack([V[:, k] - V[:, 0] for k in range(1, dim)], axis=-1)   # [nF, dim, dim-1]
    lam = np.einsum("fij,fnj->fni", np.linalg.pinv(E), X - V[:, None, 0])
    bary = np.concatenate([1 - lam.sum(-1, keepdims=True), lam], axis=-1)  # [nF, Nf, dim]
    cid = -np.ones(coords.shape[0], int)
    cid[vertex_node] = np.arange(len(vertex_node))
    fv = cid[P.faces[:, :dim]]
    assert (fv >= 0).all()
    rows = np.repeat(np.arange(nF * Nf), dim)
    cols = np.broadcast_to(fv[:, None, :], (nF, Nf, dim)).reshape(-1)
    w = (bary * interior.reshape(nF, Nf, 1)).reshape(-1)
    Pm = sp.csr_matrix((w, (rows, cols)), shape=(nF * Nf, len(vertex_node)))
    Ai = sp.diags(interior.astype(float)) @ A @ sp.diags(interior.astype(float))
    return (Pm.T @ (-Ai) @ Pm).toarray()


@pytest.mark.parametrize("dim,n,order,tau2", [(2, 5, 2, True), (2, 3, 4, False), (3, 2, 2, True), (3, 2, 3, False)])
def test_coarse_operator_is_galerkin_product(hfx_lib, dim, n, order, tau2):
    P, ctx, (coords, cells) = build_pair(hfx_lib, dim, n, order, tau2=tau2, kappa="cell")
    P.assemble()
    ctx.assemble()
    rowptr, col, val, vn = ctx.coarse_operator()
    nV = len(vn)
    # one coarse DOF per distinct cell vertex
    assert sorted(vn) == sorted(np.unique(cells[:, :dim + 1]))
    G = np.zeros((nV, nV))
    for v in range(nV):
        G[v, col[rowptr[v]:rowptr[v + 1]]] = val[rowptr[v]:rowptr[v + 1]]
    orow, ocol, oval, _ = P.csr()
    R = galerkin_coarse(P, coords, orow, ocol, oval, vn)
    assert np.abs(G - R).max() <= 1e-5 * np.abs(R).max()
    assert np.allclose(G, G.T, atol=1e-5 * np.abs(R).max())
    # the pattern holds every non-zero of the product
    mask = np.zeros((nV, nV), bool)
    for v in range(nV):
        mask[v, col[rowptr[v]:rowptr[v + 1]]] = True
    assert np.abs(R[~mask]).max(initial=0.0) <= 1e-12 * np.abs(R).max()


def scaled_coarse(ctx):
    """D^-1/2 A_c D^-1/2 on the rows with a positive diagonal, FP64 from the exported FP32 values."""
    rowptr, col, val, vn = ctx.coarse_operator()
    nV = len(vn)
    A = sp.csr_matrix((val.astype(np.float64), col, rowptr), shape=(nV, nV))
    d = A.diagonal()
    act = d > 0
    s = np.zeros(nV)
    s[act] = 1.0 / np.sqrt(d[act])
    return (sp.diags(s) @ A @ sp.diags(s)).tocsr()[act][:, act]


def bounds_case(hfx_lib, case):
    from hyperfox_gb300 import batch, capi, meshgen
    if case == "cube":
        _, ctx, _ = build_pair(hfx_lib, 3, 6, 2, tau2=False, kappa="cell")
        return ctx, None
    if case == "union":
        # one group of 24 small problems (one order, lognormal kappa per cell): a union of
        # spectra, where the Lanczos bounds first went wrong
        probs = batch.uneven_batch(count=24, seed=4, min_elements=200, max_elements=2000, orders=(2,))
        B = batch.Batch(probs, 0, capi.SRC_SINPROD, 2 * np.pi ** 2)
        return next(iter(B.groups.values())).ctx, B
    # 720,000 triangles p = 1: several coarse rows per thread of the Lanczos launch
    re = capi.refel(2, 1)
    v, s = meshgen.square_simplices(600)
    coords, cells = meshgen.high_order(v, s, re["nodes"])
    ctx = capi.Context(0)
    ctx.upload_mesh(2, 1, coords, cells)
    _, _, faces, _ = ctx.topology()
    ctx.set_source(capi.SRC_SINPROD, param=2 * np.pi ** 2)
    ctx.set_dirichlet(np.prod(np.sin(np.pi * coords[faces]), axis=-1))
    return ctx, None


@pytest.mark.parametrize("case", ["cube", "union", "large"])
def test_coarse_bounds_bracket_the_spectrum(hfx_lib, case):
    """The Chebyshev interval of the coarse solve comes from 30 FP32 Lanczos steps on
    D^-1/2 A_c D^-1/2. Its Ritz values must lie inside the operator's spectrum (scipy, FP64
    on the exported operator), the largest within 10% of the spectral radius, and lmax must
    cover the spectrum. (A Lanczos whose next beta assumed a unit Krylov vector let the
    vector's norm error grow about four-fold per step: Ritz values of -0.68, and of 2.5
    times the spectral radius, on such unions.)"""
    import scipy.sparse.linalg as sla
    ctx, keep = bounds_case(hfx_lib, case)
    ctx.assemble()
    b = ctx.coarse_bounds()
    S = scaled_coarse(ctx)
    lmax = sla.eigsh(S, k=1, which="LA", tol=1e-10, return_eigenvectors=False)[0]
    assert b["ritz_max"] <= lmax * (1 + 1e-4), (b, lmax)
    assert b["ritz_max"] >= 0.9 * lmax, (b, lmax)
    assert b["row_bound"] >= lmax * (1 - 1e-5), (b, lmax)
    assert b["lmax"] >= lmax * (1 - 1e-4), (b, lmax)
    assert 0 < b["lmin"] < b["lmax"]
    assert b["ritz_min"] > 0, b
    if S.shape[0] <= 60000:
        lmin = sla.eigsh(S.tocsc(), k=1, sigma=0, which="LM", return_eigenvectors=False)[0]
        assert b["ritz_min"] >= lmin * (1 - 1e-3), (b, lmin)
    # the two-level solve on these bounds converges
    from hyperfox_gb300 import capi
    _, info = ctx.solve(precision=1, rtol=1e-8, precond=capi.PC_TWOLEVEL, maxits=200000)
    assert info.status == 0 and info.fallback == 0
    if keep is not None:
        keep.close()
    else:
        ctx.close()


@pytest.mark.parametrize("dim,n,order", [(2, 8, 2), (2, 6, 3), (3, 3, 2), (3, 2, 3)])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("coarse_guess", [0, 1])
def test_twolevel_solve_matches_direct(hfx_lib, dim, n, order, precision, coarse_guess):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, dim, n, order, tau2=True, kappa="cell")
    P.assemble()
    ctx.assemble()
    x_ref = P.solve_direct()
    trace, info = ctx.solve(precision=precision, rtol=1e-13, precond=capi.PC_TWOLEVEL, coarse_guess=coarse_guess)
    assert info.status == 0 and info.fallback == 0
    assert info.coarse_degree >= 1
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
    assert info.rel_residual < 1e-12
    sol, flux = ctx.recover()
    osol, oflux = P.recover(trace)
    assert relerr(sol, osol) < 1e-12
    assert relerr(flux, oflux) < 1e-12


@pytest.mark.parametrize("precision", [0, 1])
def test_twolevel_iterations_grow_slower_than_block_jacobi(hfx_lib, precision):
    """Block-Jacobi CG iterations grow like 1/h; the coarse space removes most of that growth."""
    from hyperfox_gb300 import capi
    its = {}
    for n in (5, 10):
        P, ctx, _ = build_pair(hfx_lib, 3, n, 2, tau2=False, kappa="none", jitter=0.0)
        ctx.assemble()
        _, bj = ctx.solve(precision=precision, rtol=1e-10, precond=capi.PC_BLOCK_JACOBI)
        _, tl = ctx.solve(precision=precision, rtol=1e-10, precond=capi.PC_TWOLEVEL)
        assert bj.status == 0 and tl.status == 0 and tl.fallback == 0
        its[n] = (bj.iterations, tl.iterations)
    (bj5, tl5), (bj10, tl10) = its[5], its[10]
    assert tl10 < 0.6 * bj10, its
    assert tl10 - tl5 < 0.5 * (bj10 - bj5), its


def test_twolevel_refused_for_gmres_and_mixed_assembly(hfx_lib):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 2, 4, 2, tau2=False, kappa="cell")
    ctx.assemble()
    with pytest.raises(capi.HfxError) as ei:
        ctx.solve(method=capi.KSP_GMRES, precond=capi.PC_TWOLEVEL)
    assert ei.value.code == capi.HFX_ERR_UNSUPPORTED
    ctx.assemble(capi.PREC_MIXED)
    with pytest.raises(capi.HfxError) as ei:
        ctx.solve(precond=capi.PC_TWOLEVEL)
    assert ei.value.code == capi.HFX_ERR_UNSUPPORTED


def test_twolevel_falls_back_to_block_jacobi(hfx_lib):
    """A two-level solve that stops short (maxits) hands over to block Jacobi and says so."""
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 2, 6, 2, tau2=False, kappa="cell")
    ctx.assemble()
    o = capi.solve_opts(precond=capi.PC_TWOLEVEL, rtol=1e-12, maxits=2)
    info = capi.SolveInfo()
    rc = ctx.L.hfx_solve(ctx.h, ctypes.byref(o), None, ctypes.byref(info))
    assert rc == capi.HFX_ERR_NOT_CONVERGED
    assert info.fallback == 1


@pytest.mark.parametrize("precision", [0, 1])
def test_coarse_barrier_wait_runs_out_and_falls_back(hfx_lib, precision):
    """The one-launch coarse solve's grid barrier waits a bounded time: with one block's
    arrival withheld (test hook) the wait runs out (about a second), the kernel sets its
    error flag and returns, the host discards the two-level iterates and block-Jacobi CG
    finishes the solve (info.fallback = 1) with the right answer; the context stays
    usable and later solves run the one-cluster or launch-per-step coarse solve."""
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 3, 4, 2, tau2=False, kappa="cell")
    P.assemble()
    ctx.assemble()
    x_ref = P.solve_direct()
    trace, info = ctx.solve(precision=precision, precond=capi.PC_TWOLEVEL, rtol=1e-12)
    assert info.status == 0 and info.fallback == 0
    ctx._chk(ctx.L.hfx_test_coarse_barrier(ctx.h), "test_coarse_barrier")
    trace, info = ctx.solve(precision=precision, precond=capi.PC_TWOLEVEL, rtol=1e-12)
    assert info.status == 0 and info.fallback == 1
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
    trace, info = ctx.solve(precision=precision, precond=capi.PC_TWOLEVEL, rtol=1e-12)
    assert info.status == 0 and info.fallback == 0
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
