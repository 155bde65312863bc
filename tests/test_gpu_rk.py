"""Runge-Kutta time integration on the device vs the oracle's restated RungeKutta.

Each stage assembles the U rows modified as RungeKutta::apply does, solves the
trace system, recovers Solution/Flux and runs computeStage on the device; after
the last stage computeSolution. Two steps of explicit, diagonally implicit and
Crank-Nicolson tableaux from a nonzero start, on both element kernels (affine:
cell-constant tensor; quadrature: nodal tensor), must match the oracle to 1e-9
(relative L2; the trace solve runs at rtol 1e-13 and errors carry across stages).
"""
import numpy as np
import pytest

import _oracle as O
from test_gpu_parity import build_pair, relerr

pytestmark = pytest.mark.gpu


def oracle_steps(P, table, dt, steps, fields):
    rk = O.RungeKutta(table, dt)
    for _ in range(steps):
        rk.begin_step(fields)
        for _s in range(rk.S):
            rk.apply(P)
            P.assemble()
            x = P.solve_direct()
            sol, flux = P.recover(x)
            fields["Solution"][...] = sol
            fields["Flux"][...] = flux
            fields["Trace"][...] = x
            rk.stage(fields)
        rk.solution(fields)
    return fields


def device_steps(ctx, steps, n_stages, **solve):
    for _ in range(steps):
        ctx.rk_begin_step()
        for _s in range(n_stages):
            ctx.assemble()
            _, info = ctx.solve(**solve)
            assert info.status == 0
            ctx.recover()
            ctx.rk_compute_stage()
        ctx.rk_compute_solution()
    return ctx.get_state()


@pytest.mark.parametrize("name", ["FEuler", "SSPRK3", "RK4", "BEuler", "CrankNicolson", "KS2", "ALX2", "RK43"])
@pytest.mark.parametrize("dim,n,order,kappa", [(2, 4, 2, "cell"), (2, 3, 3, "tensor"), (3, 2, 2, "cell"),
                                               (3, 2, 3, "tensor")])
def test_rk_steps_match_oracle(hfx_lib, name, dim, n, order, kappa):
    from hyperfox_gb300 import capi
    P, ctx, (coords, cells) = build_pair(hfx_lib, dim, n, order, tau2=True, kappa=kappa)
    rng = np.random.default_rng(5)
    sol0 = rng.normal(size=(P.nCells, P.lenU))
    flux0 = rng.normal(size=(P.nCells, P.lenQ))
    trace0 = rng.normal(size=P.ndofs)
    dt = 0.02
    table = np.array(O.BUTCHER[name])
    fields = {"Solution": sol0.copy(), "Flux": flux0.copy(), "Trace": trace0.copy()}
    oracle_steps(P, table, dt, 2, fields)
    ctx.set_state(sol0, flux0)
    ctx.set_trace(trace0)
    ctx.rk_set(name, dt)
    sol, flux, trace = device_steps(ctx, 2, table.shape[0] - 1, rtol=1e-13)
    assert ctx.assembly_info() == (1 if kappa == "cell" else 0)
    assert relerr(trace, fields["Trace"]) < 1e-9
    assert relerr(sol, fields["Solution"]) < 1e-9
    assert relerr(flux, fields["Flux"]) < 1e-9


def test_rk_two_level_mixed_solve_and_fixed_point(hfx_lib):
    """The fast solver configuration inside the stages; the steady solution stays put."""
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 3, 3, 2, tau2=False, kappa="cell")
    ctx.assemble()
    x, _ = ctx.solve(rtol=1e-13)
    sol, flux = ctx.recover()
    ctx.rk_set("RK4", 1e-3)
    s2, f2, t2 = device_steps(ctx, 1, 4, rtol=1e-13, precond=capi.PC_TWOLEVEL, precision=capi.PREC_MIXED)
    assert relerr(t2, x) < 1e-9 and relerr(s2, sol) < 1e-9 and relerr(f2, flux) < 1e-9


def test_rk_errors(hfx_lib):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 2, 3, 2, tau2=False, kappa="cell")
    with pytest.raises(capi.HfxError) as ei:
        ctx.rk_begin_step()  # no scheme
    assert ei.value.code == capi.HFX_ERR_STATE
    # a user table with an implicit diagonal is refused like setButcherTable(EMatrix)
    with pytest.raises(capi.HfxError) as ei:
        ctx.rk_set(np.array(O.BUTCHER["BEuler"]), 0.1)
    assert ei.value.code == capi.HFX_ERR_ARG
    with pytest.raises(capi.HfxError):
        ctx.rk_set("RK4", 0.0)
    ctx.rk_set(np.array(O.BUTCHER["Heun"]), 0.1)  # explicit user table: accepted
    with pytest.raises(capi.HfxError) as ei:
        ctx.rk_compute_solution()  # stages missing
    assert ei.value.code == capi.HFX_ERR_STATE
    with pytest.raises(capi.HfxError) as ei:
        ctx.assemble(capi.PREC_MIXED)
    assert ei.value.code == capi.HFX_ERR_UNSUPPORTED
    ctx.rk_begin_step()
    for _ in range(2):
        ctx.assemble()
        ctx.solve(rtol=1e-12)
        ctx.recover()
        ctx.rk_compute_stage()
    with pytest.raises(capi.HfxError):
        ctx.rk_compute_stage()  # more stages than the method has
    ctx.rk_compute_solution()
    ctx.rk_set(None, 0.0)
    ctx.assemble()
