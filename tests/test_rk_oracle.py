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


def _operators(n, seed):
    """A mass-like SPD M and a convection-like C (any matrices do: apply is linear algebra)."""
    rng = np.random.default_rng(seed)
    B = rng.normal(size=(n, n))
    return B @ B.T + n * np.eye(n), rng.normal(size=(n, n))


@pytest.mark.parametrize("n", [3, 6, 10])
def test_apply_matches_reference_unit_test(n):
    """tests/unittests/operator/TestRungeKutta.cpp: the stage matrices and right-hand sides
    of BEuler, FEuler and Crank-Nicolson (stages 0 and 1) for K = C, f = 1, OldSolution =
    RKStage_k = 0, 1, ..., n-1, dt = 0.1; computeStage gives (1 - 2)/dt for Solution 1 and
    OldSolution 2, and computeSolution the b-weighted update."""
    M, C = _operators(n, n)
    dt, f = 0.1, np.ones(n)
    old = np.arange(n, dtype=float)   # fm["OldSolution"], also every fm["RKStage_k"]
    zero = np.zeros(n)
    # BEuler (a_00 = 1): M + dt C, M old + dt f
    K, s = O.rk_apply(C, f, M, old, zero, dt, 1.0)
    assert np.abs(K - (M + dt * C)).max() < 1e-12 * np.abs(M).max()
    assert np.abs(s - (M @ old + dt * f)).max() < 1e-12 * np.abs(M @ old).max()
    # FEuler (a_00 = 0): M, (M - dt C) old + dt f
    K, s = O.rk_apply(C, f, M, old, zero, dt, 0.0)
    assert np.abs(K - M).max() == 0.0
    assert np.abs(s - ((M - dt * C) @ old + dt * f)).max() < 1e-12 * np.abs(M @ old).max()
    # Crank-Nicolson stage 0 (a_00 = 0): M, dt (-C old + f) + M old
    K, s = O.rk_apply(C, f, M, old, zero, dt, 0.0)
    assert np.abs(s - (dt * (-C @ old + f) + M @ old)).max() < 1e-12 * np.abs(M @ old).max()
    # stage 1 (a_10 = a_11 = 1/2, k_0 = RKStage_0 = 0..n-1): M + dt/2 C,
    # dt (-C (old + dt/2 k_0) + f) + (M + dt/2 C) old
    K, s = O.rk_apply(C, f, M, old, 0.5 * old, dt, 0.5)
    A1 = M + dt / 2 * C
    assert np.abs(K - A1).max() < 1e-12 * np.abs(M).max()
    ref = dt * (-C @ (old + dt / 2 * old) + f) + A1 @ old
    assert np.abs(s - ref).max() < 1e-12 * np.abs(ref).max()
    # computeStage / computeSolution on the Field values of the test: Solution 1, OldSolution 2
    for name in ("BEuler", "FEuler", "CrankNicolson"):
        rk = O.RungeKutta(O.BUTCHER[name], dt)
        fields = {"Solution": np.full(n, 2.0), "Flux": np.zeros(n), "Trace": np.zeros(n)}
        rk.begin_step(fields)
        fields["Solution"][...] = 1.0
        rk.stage(fields)
        assert np.all(rk.k["Solution"][0] == (1.0 - 2.0) / dt)
        if rk.S == 2:  # the second stage of Crank-Nicolson leaves Solution unchanged: k_1 = 0
            rk.stage(fields)
            assert np.all(rk.k["Solution"][1] == 0.0)
        rk.solution(fields)
        b = np.array(O.BUTCHER[name])[-1, 1:]
        expect = 2.0 + dt * sum(b[k] * rk.k["Solution"][k] for k in range(rk.S))
        assert np.abs(fields["Solution"] - expect).max() < 1e-12
