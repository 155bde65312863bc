"""Affine element kernel (reference operators) vs the oracle and vs the quadrature kernel.

Straight-sided cells with a symmetric diffusion tensor constant inside every
cell take the affine path; its condensed blocks (Q, Q0 formed on demand), CSR,
solve and recovery must meet the same 1e-12 bars as the quadrature kernel.
"""
import numpy as np
import pytest

import _oracle as O
from helpers import fields, mesh
from test_gpu_parity import CASES, relerr

pytestmark = pytest.mark.gpu


def cell_tensor(rng, nCells, N, dim):
    A = rng.normal(size=(nCells, dim, dim)) * 0.3
    K = np.einsum("eij,ekj->eik", A, A) + np.eye(dim)
    return np.repeat(K.transpose(0, 2, 1).reshape(nCells, 1, dim * dim), N, axis=1)  # column-major


def build(dim, n, order, kappa, dt=0.0, seed=1, perturb=0.0):
    from hyperfox_gb300 import capi
    rng = np.random.default_rng(seed)
    re, coords, cells = mesh(dim, n, order, jitter=0.15, seed=seed)
    if perturb:
        coords = coords.copy()
        coords[cells[0, -1]] += perturb  # bend one cell: no longer straight-sided
    P = O.Problem(dim, order, coords, cells)
    tau, _, g = fields(dim, order, coords, cells, P.faces, P.nFaces, rng, tau2=True, kappa="none")
    if kappa == "tensor":
        kap = cell_tensor(rng, cells.shape[0], cells.shape[1], dim)
    elif kappa == "scalar":
        kap = np.repeat(rng.uniform(0.5, 3.0, size=(cells.shape[0], 1, 1)), cells.shape[1], axis=1)
    else:
        kap = None
    u_old = rng.normal(size=cells.shape) if dt > 0 else None
    P.set_fields(tau.ravel(), kappa=None if kap is None else kap.ravel(), src_mode=2, dirichlet=g.ravel(), dt=dt,
                 u_old=u_old)
    ctx = capi.Context(0)
    ctx.upload_mesh(dim, order, coords, cells)
    ctx.set_tau(tau)
    if kap is not None:
        ctx.set_kappa(kap, layout=1)
    ctx.set_source(capi.SRC_SINPROD, param=dim * np.pi ** 2)
    ctx.set_dirichlet(g)
    if dt > 0:
        ctx.set_time_scheme(dt, u_old)
    return P, ctx


def affine_used(ctx):
    import ctypes
    v = ctypes.c_int()
    ctx._chk(ctx.L.hfx_assembly_info(ctx.h, ctypes.byref(v)), "assembly_info")
    return v.value


@pytest.mark.parametrize("dim,n,order", CASES)
@pytest.mark.parametrize("kappa", ["tensor", "scalar", "none"])
def test_affine_blocks_match_oracle(hfx_lib, dim, n, order, kappa):
    P, ctx = build(dim, n, order, kappa)
    P.assemble()
    ctx.assemble()
    assert affine_used(ctx) == 1
    o = P.condensed()
    g = ctx.condensed()
    for k in ("S", "S0", "U", "Q", "U0", "Q0"):
        assert relerr(g[k], o[k]) < 1e-12, (k, relerr(g[k], o[k]))
    orow, ocol, oval, orhs = P.csr()
    grow, gcol, gval, grhs = ctx.csr()
    assert np.array_equal(orow, grow) and np.array_equal(ocol, gcol)
    assert relerr(gval, oval) < 1e-12 and relerr(grhs, orhs) < 1e-12


@pytest.mark.parametrize("dim,n,order", [(2, 3, 3), (3, 2, 2)])
def test_affine_time_scheme(hfx_lib, dim, n, order):
    P, ctx = build(dim, n, order, "tensor", dt=0.01)
    P.assemble()
    ctx.assemble()
    assert affine_used(ctx) == 1
    o, g = P.condensed(), ctx.condensed()
    for k in ("S", "S0", "U", "Q", "U0", "Q0"):
        assert relerr(g[k], o[k]) < 1e-12, k


@pytest.mark.parametrize("dim,n,order", [(2, 6, 3), (3, 2, 3)])
def test_affine_solve_and_recover(hfx_lib, dim, n, order):
    P, ctx = build(dim, n, order, "tensor")
    P.assemble()
    ctx.assemble()
    x_ref = P.solve_direct()
    trace, info = ctx.solve(rtol=1e-13)
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
    sol, flux = ctx.recover()
    osol, oflux = P.recover(trace)
    assert relerr(sol, osol) < 1e-12
    assert relerr(flux, oflux) < 1e-12


def test_affine_equals_quadrature_kernel(hfx_lib):
    P, ctx = build(3, 2, 3, "tensor")
    ctx.assemble()
    a = ctx.condensed()
    ctx.L.hfx_set_assembly_path(ctx.h, 1)
    ctx.assemble()
    assert affine_used(ctx) == 0
    q = ctx.condensed()
    for k in ("S", "S0", "U", "Q", "U0", "Q0"):
        assert relerr(a[k], q[k]) < 1e-12, k


def test_curved_cell_uses_quadrature(hfx_lib):
    P, ctx = build(2, 3, 3, "tensor", perturb=0.01)
    P.assemble()
    ctx.assemble()
    assert affine_used(ctx) == 0
    o, g = P.condensed(), ctx.condensed()
    for k in ("S", "U", "Q"):
        assert relerr(g[k], o[k]) < 1e-12, k
