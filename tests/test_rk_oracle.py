"""Runge-Kutta on the oracle (CPU): the restated RungeKutta (tests/_oracle.py,
oracle/hdg_oracle.cpp) against what the reference's scheme must satisfy.

- the library's Butcher tables equal the restated RungeKutta::setUpDB tables;
- one BEuler stage is the reference's implicit Euler (Euler.cpp:18-34) exactly;
- the steady HDG solution is a fixed point of every scheme (all stage
  derivatives vanish), the consistency the stage algebra of apply() /
  computeStage() / computeSolution() has to keep.
"""
import numpy as np
import pytest

import _oracle as O
from hyperfox_gb300 import capi, meshgen


def small_problem(dim=2, n=3, order=2):
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    v = meshgen.jitter_vertices(v, n, 0.15, 2)
    re = capi.refel(dim, order)
    coords, cells = meshgen.high_order(v, s, re["nodes"])
    P = O.Problem(dim, order, coords, cells)
    g = np.prod(np.sin(np.pi * coords[P.faces]), axis=-1)
    return P, g, coords, cells


def test_butcher_tables_match_restatement():
    for i, name in enumerate(capi.RK_TYPES):
        assert np.array_equal(capi.rk_butcher(i), np.array(O.BUTCHER[name], float)), name
        assert np.array_equal(capi.rk_butcher(name), capi.rk_butcher(i))
    with pytest.raises(capi.HfxError):
        capi.rk_butcher(99)


def run_oracle(P, g, table, dt, steps, fields):
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


def test_beuler_stage_is_implicit_euler():
    P, g, coords, cells = small_problem()
    rng = np.random.default_rng(3)
    u_old = rng.normal(size=cells.shape)
    dt = 0.05
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=g.ravel(), dt=dt, u_old=u_old)
    P.assemble()
    x_e = P.solve_direct()
    sol_e, flux_e = P.recover(x_e)
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=g.ravel())
    fields = {"Solution": u_old.copy(), "Flux": rng.normal(size=(P.nCells, P.lenQ)), "Trace": rng.normal(size=P.ndofs)}
    run_oracle(P, g, O.BUTCHER["BEuler"], dt, 1, fields)
    assert np.allclose(fields["Solution"], sol_e, rtol=0, atol=1e-12 * np.abs(sol_e).max())
    assert np.allclose(fields["Trace"], x_e, rtol=0, atol=1e-12 * np.abs(x_e).max())


@pytest.mark.parametrize("name", ["FEuler", "Heun", "SSPRK3", "RK4", "BEuler", "CrankNicolson", "KS2", "ALX2", "RK43"])
def test_steady_solution_is_a_fixed_point(name):
    P, g, coords, cells = small_problem()
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=g.ravel())
    P.set_rk(0.0)
    P.assemble()
    x = P.solve_direct()
    sol, flux = P.recover(x)
    fields = {"Solution": sol.copy(), "Flux": flux.copy(), "Trace": x.copy()}
    run_oracle(P, g, O.BUTCHER[name], 1e-3, 2, fields)
    for k, ref in (("Solution", sol), ("Flux", flux), ("Trace", x)):
        assert np.abs(fields[k] - ref).max() < 1e-9 * np.abs(ref).max(), (name, k)
