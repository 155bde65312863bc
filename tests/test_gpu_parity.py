"""CUDA path vs the CPU oracle, through the C ABI (needs a GPU).

Bars (FP64 path): element blocks S, S0, U, Q, U0, Q0 and the trace CSR values
within 1e-12 relative (max-norm, scaled by the largest entry), CSR pattern and
DOF numbering bit-exact, trace solution within 1e-8 relative L2 of a direct
FP64 solve, recovery within 1e-12 of the oracle's recovery of the same trace.
"""
import numpy as np
import pytest

import _oracle as O
from helpers import fields, manufactured, mesh

pytestmark = pytest.mark.gpu

REL = 1e-12

CASES = [(2, 4, 1), (2, 4, 2), (2, 3, 3), (2, 3, 4), (2, 2, 5), (3, 2, 1), (3, 2, 2), (3, 1, 3)]


def relerr(a, b):
    scale = max(np.abs(b).max(), 1e-300)
    return np.abs(a - b).max() / scale


def build_pair(hfx_lib, dim, n, order, tau2, kappa, src=True, jitter=0.15, seed=1, dt=0.0):
    from hyperfox_gb300 import capi
    rng = np.random.default_rng(seed)
    re, coords, cells = mesh(dim, n, order, jitter=jitter, seed=seed)
    P = O.Problem(dim, order, coords, cells)
    tau, kap, g = fields(dim, order, coords, cells, P.faces, P.nFaces, rng, tau2=tau2, kappa=kappa)
    u_old = rng.normal(size=cells.shape) if dt > 0 else None
    P.set_fields(tau.ravel(), kappa=None if kap is None else kap.ravel(), src_mode=2 if src else 0,
                 dirichlet=g.ravel(), dt=dt, u_old=u_old)
    ctx = capi.Context(0)
    ctx.upload_mesh(dim, order, coords, cells)
    ctx.set_tau(tau)
    if kap is not None:
        ctx.set_kappa(kap, layout=1)
    if src:
        ctx.set_source(capi.SRC_SINPROD, param=dim * np.pi ** 2)
    ctx.set_dirichlet(g)
    if dt > 0:
        ctx.set_time_scheme(dt, u_old)
    return P, ctx, (coords, cells)


@pytest.mark.parametrize("dim,n,order", CASES)
def test_condensed_blocks(hfx_lib, dim, n, order):
    P, ctx, _ = build_pair(hfx_lib, dim, n, order, tau2=True, kappa="tensor")
    P.assemble()
    ctx.assemble()
    o = P.condensed()
    g = ctx.condensed()
    for k in ("S", "S0", "U", "Q", "U0", "Q0"):
        assert relerr(g[k], o[k]) < REL, (k, relerr(g[k], o[k]))


@pytest.mark.parametrize("dim,n,order", CASES)
def test_csr_pattern_and_values(hfx_lib, dim, n, order):
    P, ctx, _ = build_pair(hfx_lib, dim, n, order, tau2=False, kappa="scalar")
    P.assemble()
    ctx.assemble()
    orow, ocol, oval, orhs = P.csr()
    grow, gcol, gval, grhs = ctx.csr()
    assert np.array_equal(orow, grow)
    assert np.array_equal(ocol, gcol)
    assert relerr(gval, oval) < REL
    assert relerr(grhs, orhs) < REL


def test_topology_matches_oracle(hfx_lib):
    P, ctx, _ = build_pair(hfx_lib, 3, 2, 2, tau2=False, kappa="none")
    c2f, f2c, faces, bnd = ctx.topology()
    assert np.array_equal(c2f, P.cell2face)
    assert np.array_equal(f2c, P.face2cell)
    assert np.array_equal(faces, P.faces)
    assert np.array_equal(bnd, P.boundary)


@pytest.mark.parametrize("dim,n,order", [(2, 8, 2), (2, 4, 4), (3, 2, 2), (3, 2, 3)])
@pytest.mark.parametrize("precision", [0, 1])
@pytest.mark.parametrize("kappa", ["cell", "scalar"])
def test_solve_and_recover(hfx_lib, dim, n, order, precision, kappa):
    """kappa constant per cell: CG (symmetric system); nodal kappa: GMRES."""
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, dim, n, order, tau2=False, kappa=kappa)
    P.assemble()
    ctx.assemble()
    x_ref = P.solve_direct()
    trace, info = ctx.solve(precision=precision, rtol=1e-13, precond=capi.PC_BLOCK_JACOBI)
    assert info.status == 0
    err = np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref)
    assert err < 1e-8, err
    assert info.rel_residual < 1e-12
    sol, flux = ctx.recover()
    osol, oflux = P.recover(trace)
    assert relerr(sol, osol) < REL
    assert relerr(flux, oflux) < REL


def test_cg_refused_on_nonsymmetric_system(hfx_lib):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 2, 4, 2, tau2=False, kappa="scalar")
    ctx.assemble()
    with pytest.raises(capi.HfxError) as ei:
        ctx.solve(method=capi.KSP_CG)
    assert ei.value.code == capi.HFX_ERR_ARG


@pytest.mark.parametrize("method", [0, 1])
@pytest.mark.parametrize("precision", [0, 1])
def test_gmres_and_cg_agree_on_symmetric_system(hfx_lib, method, precision):
    P, ctx, _ = build_pair(hfx_lib, 3, 2, 3, tau2=True, kappa="cell")
    P.assemble()
    ctx.assemble()
    x_ref = P.solve_direct()
    trace, info = ctx.solve(method=method, precision=precision, rtol=1e-13, restart=40)
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
    assert info.rel_residual < 1e-12


@pytest.mark.parametrize("pc", [0, 1, 2])
def test_preconditioners_agree(hfx_lib, pc):
    P, ctx, _ = build_pair(hfx_lib, 2, 6, 3, tau2=False, kappa="none")
    P.assemble()
    ctx.assemble()
    x_ref = P.solve_direct()
    trace, info = ctx.solve(precond=pc, rtol=1e-13)
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8


def test_constant_dirichlet(hfx_lib):
    """TestHDGSolver.cpp:88-100: Dirichlet = 3 gives Solution = 3, Flux = 0, Trace = 3 (1e-12)."""
    from hyperfox_gb300 import capi
    re, coords, cells = mesh(2, 6, 2, jitter=0.2, seed=3)
    ctx = capi.Context(0)
    ctx.upload_mesh(2, 2, coords, cells)
    ctx.set_dirichlet(np.full(ctx.ndofs, 3.0))
    ctx.assemble()
    trace, info = ctx.solve(rtol=1e-15, maxits=5000)
    sol, flux = ctx.recover()
    assert np.abs(trace - 3).max() < 1e-12
    assert np.abs(sol - 3).max() < 1e-12
    assert np.abs(flux).max() < 1e-11


def test_implicit_euler(hfx_lib):
    P, ctx, _ = build_pair(hfx_lib, 2, 4, 2, tau2=False, kappa="scalar", dt=1e-2)
    P.assemble()
    ctx.assemble()
    o = P.condensed()
    g = ctx.condensed()
    for k in ("S", "S0", "U", "Q", "U0", "Q0"):
        assert relerr(g[k], o[k]) < REL, k


def test_source_values_mode(hfx_lib):
    """Caller-supplied source values at the integration points (Source.h:36 callback)."""
    from hyperfox_gb300 import capi
    P, ctx, (coords, cells) = build_pair(hfx_lib, 2, 4, 3, tau2=False, kappa="none", src=False)
    x = ctx.ip_coords()
    assert relerr(x, P.ip_coords()) < 1e-14
    f = np.exp(x[..., 0]) * np.cos(x[..., 1])
    P.set_fields(np.ones(P.ndofs), src_mode=1, src=f.ravel(), dirichlet=manufactured(coords, P.faces).ravel())
    ctx.set_tau(np.ones(P.ndofs))
    ctx.set_source(capi.SRC_VALUES, f)
    P.assemble()
    ctx.assemble()
    o = P.condensed()
    g = ctx.condensed()
    assert relerr(g["S0"], o["S0"]) < REL
    assert relerr(g["U0"], o["U0"]) < REL


def test_manufactured_convergence(hfx_lib):
    """TestHDGLaplace.cpp:110-150 in spirit: the HDG solution converges at the expected rate."""
    from hyperfox_gb300 import capi
    errs = []
    for n in (4, 8, 16):
        re, coords, cells = mesh(2, n, 2)
        ctx = capi.Context(0)
        ctx.upload_mesh(2, 2, coords, cells)
        _, _, faces, _ = ctx.topology()
        ctx.set_source(capi.SRC_SINPROD, param=2 * np.pi ** 2)
        ctx.set_dirichlet(manufactured(coords, faces))
        ctx.assemble()
        ctx.solve(rtol=1e-13)
        sol, _ = ctx.recover()
        u = np.prod(np.sin(np.pi * coords[cells]), axis=-1)
        errs.append(np.abs(sol - u).max())
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert errs[-1] < 1e-3
    assert rates.min() > 2.5, (errs, rates)


@pytest.mark.parametrize("dim,n,order", [(2, 8, 2), (2, 4, 4), (3, 2, 2), (3, 2, 3)])
@pytest.mark.parametrize("kappa", ["cell", "scalar"])
def test_mixed_precision_solve(hfx_lib, dim, n, order, kappa):
    """FP32 condensation + FP32 Krylov as corrections of the FP64 full-system
    residual: the refined trace, Solution and Flux equal the FP64 direct solution
    to 1e-8 relative."""
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, dim, n, order, tau2=True, kappa=kappa)
    P.assemble()
    x_ref = P.solve_direct()
    osol, oflux = P.recover(x_ref)
    ctx.assemble(precision=capi.PREC_MIXED)
    trace, info = ctx.solve(rtol=1e-12, inner_rtol=1e-5, restart=40)
    assert info.status == 0 and info.refinements >= 2
    assert info.rel_residual < 1e-12
    sol, flux = ctx.recover()
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
    assert np.linalg.norm(sol - osol) / np.linalg.norm(osol) < 1e-8
    assert np.linalg.norm(flux - oflux) / np.linalg.norm(oflux) < 1e-8


def test_mixed_precision_time_scheme_and_values_source(hfx_lib):
    from hyperfox_gb300 import capi
    P, ctx, (coords, cells) = build_pair(hfx_lib, 2, 4, 3, tau2=False, kappa="cell", dt=1e-2)
    P.assemble()
    x_ref = P.solve_direct()
    ctx.assemble(precision=capi.PREC_MIXED)
    trace, info = ctx.solve(rtol=1e-12)
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8


def test_mixed_assembly_refuses_fp64_exports(hfx_lib):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 2, 3, 2, tau2=False, kappa="none")
    ctx.assemble(precision=capi.PREC_MIXED)
    with pytest.raises(capi.HfxError):
        ctx.condensed()


@pytest.mark.parametrize("kernel", [0, 1, 2, 3])
@pytest.mark.parametrize("dim,n,order", [(3, 3, 3), (3, 3, 2), (2, 8, 3)])
def test_mixed_cg_both_fp32_operator_kernels(hfx_lib, kernel, dim, n, order):
    """Every kernel of the FP32 half-storage trace operator (row per lane, blocks staged in
    shared memory by bulk copies, row per lane with paired loads, the same with float4
    reads of the gathered x), fixed through hfx_set_tuning, gives the direct solution to 1e-8 with the
    two-level mixed CG at Nf = 10, 6 and 4; the tuner, when left to choose, picks one of
    them and reports their times."""
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, dim, n, order, tau2=False, kappa="cell")
    P.assemble()
    ctx.assemble()
    x_ref = P.solve_direct()
    ctx._chk(ctx.L.hfx_set_tuning(ctx.h, kernel), "set_tuning")
    for precond in (capi.PC_BLOCK_JACOBI, capi.PC_TWOLEVEL):
        trace, info = ctx.solve(precision=capi.PREC_MIXED, rtol=1e-12, precond=precond)
        assert info.status == 0
        assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
        assert ctx.tuning_info()[0] == kernel
    ctx._chk(ctx.L.hfx_set_tuning(ctx.h, -1), "set_tuning")
    ctx.solve(precision=capi.PREC_MIXED, rtol=1e-12, precond=capi.PC_TWOLEVEL)
    k, ms = ctx.tuning_info()
    assert k in (0, 1, 2, 3) and min(ms[:3]) > 0
