"""Explicit HDG modes (WEXPLICIT / SEXPLICIT, HDGSolver.cpp:349-354,709-729) vs the oracle.

S = Sll and S0 = -Slu Solution - Slq Flux from the current state; WEXPLICIT solves
the (face-block diagonal) trace system with the Krylov solver, SEXPLICIT face by
face. Blocks 1e-12, traces and recovery 1e-12 (SEXPLICIT) / 1e-10 (WEXPLICIT).
"""
import numpy as np
import pytest

from test_gpu_parity import build_pair, relerr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,n,order,kappa", [(2, 4, 2, "cell"), (2, 3, 3, "scalar"), (3, 2, 2, "cell"),
                                               (3, 2, 3, "tensor")])
@pytest.mark.parametrize("mode", [1, 2])
def test_explicit_modes_match_oracle(hfx_lib, dim, n, order, kappa, mode):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, dim, n, order, tau2=True, kappa=kappa)
    rng = np.random.default_rng(11)
    sol = rng.normal(size=(P.nCells, P.lenU))
    flux = rng.normal(size=(P.nCells, P.lenQ))
    P.set_solver(mode, sol, flux)
    P.assemble()
    ctx.set_solver_type(mode)
    ctx.set_state(sol, flux)
    ctx.assemble()
    o, g = P.condensed(), ctx.condensed()
    for k in ("S", "S0", "U", "Q", "U0", "Q0"):
        assert relerr(g[k], o[k]) < 1e-12, k
    x_ref = P.solve_faces()
    if mode == 2:
        trace, info = ctx.solve()
        assert info.status == 0 and info.iterations == 0
        assert relerr(trace, x_ref) < 1e-12
    else:
        trace, info = ctx.solve(method=capi.KSP_GMRES, rtol=1e-14)
        assert relerr(trace, x_ref) < 1e-10
    sol2, flux2 = ctx.recover()
    osol, oflux = P.recover(trace)
    assert relerr(sol2, osol) < 1e-12 and relerr(flux2, oflux) < 1e-12


def test_explicit_steps_follow_the_oracle(hfx_lib):
    """Three SEXPLICIT steps, each assembling from the state the previous recovery left."""
    P, ctx, _ = build_pair(hfx_lib, 2, 4, 2, tau2=False, kappa="cell")
    sol = np.zeros((P.nCells, P.lenU))
    flux = np.zeros((P.nCells, P.lenQ))
    ctx.set_solver_type(2)
    for _ in range(3):
        P.set_solver(2, sol, flux)
        P.assemble()
        ctx.assemble()
        x = P.solve_faces()
        trace, _ = ctx.solve()
        assert relerr(trace, x) < 1e-12
        sol, flux = P.recover(x)
        gs, gf = ctx.recover()
        assert relerr(gs, sol) < 1e-12 and relerr(gf, flux) < 1e-12


def test_explicit_refused_for_mixed_assembly(hfx_lib):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 2, 3, 2, tau2=False, kappa="cell")
    ctx.set_solver_type(1)
    with pytest.raises(capi.HfxError) as ei:
        ctx.assemble(capi.PREC_MIXED)
    assert ei.value.code == capi.HFX_ERR_UNSUPPORTED
