"""Oracle checks of the Burgers / Newton row (HDGUNabU, HDGBurgersModel,
NonLinearWrapper) against HyperFox's own tests:
tests/unittests/operator/TestHDGUNabU.cpp, tests/unittests/solver/TestNonLinearWrapper.cpp
and the stationary regression tests/regression/HDG/TestHDGBurgersStat.cpp."""
import numpy as np
import pytest

import _oracle as O
from hyperfox_gb300 import meshgen

TOL = 1e-12


def intx2n(dim, ord_):
    """TestUtils.h intx2n: integral of x^(2 ord) over the reference simplex."""
    return 2.0 / (2.0 * ord_ + 1) if dim < 3 else 1.0 / (2.0 * ord_ + 3.0) + 1.0 / (2.0 * ord_ + 1.0)


def _face_trace(re, sol):
    dim = re.dim
    tr = np.zeros((re.nFaces * re.nNodesFace, dim))
    for f in range(re.nFaces):
        for k in range(re.nNodesFace):
            tr[f * re.nNodesFace + k] = sol[re.faceNodes[f, k]]
    return tr


def _quad_form(re, op, sol, tr):
    u, t = sol.ravel(), tr.ravel()
    nU = u.size
    sL = nU * (re.dim + 1)
    return u @ op[:nU, :nU] @ u + u @ op[:nU, sL:] @ t


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("order", [3, 4, 5])
def test_unabu_polynomial_reference_element(dim, order):
    """TestHDGUNabU.cpp:29-105: u = (x, 0[, 0]) on the reference element, the
    quadratic form and the RHS integrate x^2 (n = 0, the only case the test's loop
    bounds run for these orders)."""
    if dim == 3 and order > 3:
        pytest.importorskip("numpy")  # 3D nodes exist for p <= 5 in the node database
    re = O.RefEl(dim, order)
    n = 0
    sol = np.zeros((re.nNodes, dim))
    sol[:, 0] = re.nodes[:, 0] ** (n + 1)
    tr = _face_trace(re, sol)
    op, rhs = O.unabu_refel(dim, order, sol, tr)
    ref = intx2n(dim, (3 * n + 2) // 2)
    assert abs(_quad_form(re, op, sol, tr) / (2.0 * (n + 1)) - ref) < TOL
    assert abs(rhs[: sol.size] @ sol.ravel() / (1.0 * (n + 1)) - ref) < TOL


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_unabu_constant_solution(dim, order):
    """TestHDGUNabU.cpp:107-166: a constant u = e_0 gives a vanishing quadratic form
    and RHS (here checked in absolute value, the reference checks the signed value)."""
    re = O.RefEl(dim, order)
    sol = np.zeros((re.nNodes, dim))
    sol[:, 0] = 1.0
    tr = _face_trace(re, sol)
    op, rhs = O.unabu_refel(dim, order, sol, tr)
    assert abs(_quad_form(re, op, sol, tr)) < TOL
    assert abs(rhs[: sol.size] @ sol.ravel()) < TOL


@pytest.mark.parametrize("dim,order", [(2, 1), (2, 3), (2, 5), (3, 2)])
def test_unabu_is_the_newton_linearisation(dim, order):
    """With the trace equal to the interior face values (the converged state), the
    operator of HDGUNabU about u0 is the derivative of its quadratic term
    N(u) = op(u) [u; t] / 2 (the RHS): op(u0) d = op(d) u0 on the U and L rows, so
    N(u0 + e d) - N(u0) - e op(u0) d = e^2 N(d) exactly. (The face flux is
    linearised with the trace in one term and the interior values in the other,
    HDGUNabU.cpp:126-145, so with an unrelated trace it is a Picard-Newton mix.)"""
    re = O.RefEl(dim, order)
    rng = np.random.default_rng(order)
    nU = re.nNodes * dim
    sL = nU * (dim + 1)
    u0, du = rng.standard_normal((2, re.nNodes, dim))
    t0, dt_ = _face_trace(re, u0), _face_trace(re, du)
    op0, r0 = O.unabu_refel(dim, order, u0, t0)
    opd, rd = O.unabu_refel(dim, order, du, dt_)
    rows = np.r_[0:nU, sL:op0.shape[0]]
    v0 = np.zeros(op0.shape[0])
    vd = np.zeros(op0.shape[0])
    v0[:nU], v0[sL:] = u0.ravel(), t0.ravel()
    vd[:nU], vd[sL:] = du.ravel(), dt_.ravel()
    a = (op0 @ vd)[rows]
    b = (opd @ v0)[rows]
    assert np.abs(a - b).max() < 1e-12 * np.abs(a).max()
    eps = 1e-3
    _, re_ = O.unabu_refel(dim, order, u0 + eps * du, t0 + eps * dt_)
    lhs = re_[rows] - r0[rows] - eps * a
    assert np.abs(lhs - eps ** 2 * rd[rows]).max() < 1e-12 * np.abs(r0).max()


def _wrapper(linearized, current, previous, res_tol=1e-6, max_iters=20, dampening=0.0):
    """NonLinearWrapper::solve (NonLinearWrapper.cpp:41-79) with a user linearised
    solver and the vanilla residual computer (NonLinearWrapper.cpp:14-34)."""
    res = None
    for _ in range(max_iters):
        linearized()
        diff = float(np.sum((current - previous) ** 2))
        ref = float(np.sum(previous ** 2))
        res = np.sqrt(diff / ref) if ref != 0 else np.sqrt(diff)
        if res < res_tol:
            break
        val = (1.0 - dampening) * current + dampening * previous
        current[...] = val
        previous[...] = val
    return res


@pytest.mark.parametrize("start", [1.0, 2.0, -1.0, 0.25, 42.0, 1e-8])
def test_nonlinear_wrapper_quadratic(start):
    """TestNonLinearWrapper.cpp:10-47: x <- x - x^2 / (2x) drives x to 0; the
    residual test stops the loop once ||x_new - x|| / ||x|| < 1e-6 cannot be met and
    the maximum iteration count (20) ends it, with |x| < 1e-4."""
    cur = np.zeros(9)
    prev = np.full(9, start)

    def lin():
        cur[...] = prev - prev ** 2 / (2.0 * prev)

    res = _wrapper(lin, cur, prev)
    # x halves every step: the relative change stays 1/2, the loop runs to max_iters
    assert res == pytest.approx(0.5)
    assert np.abs(prev).max() < 1e-4 * max(1.0, abs(start)) * 50


# ------------------------------------------------------------------ stationary Burgers
def cole_hopf(x, D=1.0, A=0.5, x0=(1.0, 0.0)):
    """TestHDGBurgersStat.cpp:26-104: u = -2 D grad(phi) / phi (Cole-Hopf) with
    phi = 0.001 A e^{(1+x0) A} (1+x) + (e^{A(x-x0)} + e^{-A(x-x0)}) cos(A (y-y0))."""
    X, Y = x[..., 0], x[..., 1]
    ep, em = np.exp(A * (X - x0[0])), np.exp(-A * (X - x0[0]))
    c, s = np.cos(A * (Y - x0[1])), np.sin(A * (Y - x0[1]))
    phi = 0.001 * A * np.exp((1 + x0[0]) * A) * (1 + X) + (ep + em) * c
    gx = 0.001 * A * np.exp((1 + x0[0]) * A) + A * (ep - em) * c
    gy = -A * (ep + em) * s
    return np.stack([-2 * D * gx / phi, -2 * D * gy / phi], -1)


def burgers_stationary(n, p, D=1.0):
    re = O.RefEl(2, p)
    v, s = meshgen.square_simplices(n)
    coords, cells = meshgen.high_order(v, s, re.nodes)
    P = O.BurgersProblem(2, p, coords, cells)
    h = 1.0 / n
    nd = 2
    tau = np.zeros((P.nFaces, re.nNodesFace, 2, nd * nd))
    tau[..., 0] = tau[..., 3] = 2.0 * D / h          # (D / carLen) * 2 * I on both sides
    g = cole_hopf(coords[P.faces], D)                 # Dirichlet at the face nodes
    nu = np.full((P.nCells, re.nNodes, 1), D)
    P.set_fields(tau=tau, tau_sides=2, nu=nu, dirichlet=g)
    return P, coords, cells


def l2_err_vec(P, coords, cells, sol, exact):
    re = P.re
    X = coords[cells]
    xq = np.einsum("qn,end->eqd", re.phi, X)
    uh = np.einsum("qn,enc->eqc", re.phi, sol.reshape(P.nCells, re.nNodes, 2))
    J = np.einsum("qnr,ens->eqrs", re.dphi, X)
    det = np.linalg.det(J)
    return np.sqrt(np.sum(np.sum((uh - exact(xq)) ** 2, -1) * det * re.ipW[None, :]))


@pytest.mark.parametrize("p", [1, 2, 3])
def test_burgers_stationary_cole_hopf(p):
    """TestHDGBurgersStat.cpp:107-399 on a structured unit-square mesh (the
    regression meshes stand for the same domain): Newton from Solution = 0 with
    the Set Dirichlet of the analytical solution converges (residual < 1e-6 within
    10 iterations, superlinearly: 4 iterations here), l2 error < 1 (the reference's bound) and it
    falls at least like h^p between two meshes."""
    errs = []
    for n in (4, 8):
        P, coords, cells = burgers_stationary(n, p)
        sol, flux, its, hist = P.newton(res_tol=1e-6, max_iters=10)
        assert hist[-1] < 1e-6 and its < 10, hist
        assert hist[-1] < 1e-2 * hist[-2] or hist[-1] < 1e-12  # superlinear tail
        errs.append(l2_err_vec(P, coords, cells, sol, cole_hopf))
    assert errs[-1] < 1.0
    assert errs[0] / errs[1] > 2.0 ** p, errs


def test_burgers_time_step_reduces_to_mass_solve_when_frozen():
    """With dt -> tiny the implicit Euler system is the mass matrix: one Newton step
    from u_old returns u_old (Euler.cpp:18-34 on the U rows of every operator)."""
    p, n = 2, 4
    re = O.RefEl(2, p)
    v, s = meshgen.square_simplices(n)
    coords, cells = meshgen.high_order(v, s, re.nodes)
    P = O.BurgersProblem(2, p, coords, cells)
    u_old = cole_hopf(coords[cells]).reshape(P.nCells, -1)
    g = cole_hopf(coords[P.faces])
    P.set_fields(nu=np.full((P.nCells, re.nNodes, 1), 1e-2), dirichlet=g, dt=1e-12, old=u_old)
    P.set_state(buf=u_old, trace=g.ravel() * 0 + 0.0)
    sol, _ = P.linearized_solve()
    assert np.abs(sol - u_old).max() < 1e-8


@pytest.mark.parametrize("p,dt", [(1, 0.0), (2, 0.0), (3, 1e-2)])
def test_zero_velocity_is_two_scalar_diffusion_problems(p, dt):
    """With BufferSolution = 0 and Trace = 0 the HDGUNabU terms vanish, and with
    tau = tau_s I the Burgers system is nd uncoupled copies of the scalar HDG
    diffusion-source problem (HDGBase/HDGDiffusion with nd unknowns, Euler with M (x) I):
    every block equals the scalar oracle's, component by component (data of component 1
    = 2 x component 0's)."""
    rng = np.random.default_rng(p)
    re = O.RefEl(2, p)
    v, s = meshgen.square_simplices(3)
    v = meshgen.jitter_vertices(v, 3, 0.15, p)
    coords, cells = meshgen.high_order(v, s, re.nodes)
    P1 = O.Problem(2, p, coords, cells)
    PB = O.BurgersProblem(2, p, coords, cells)
    Nf, N, nI = re.nNodesFace, re.nNodes, re.nIP
    tau = rng.uniform(0.5, 2.0, size=(P1.nFaces, Nf))
    kap = rng.uniform(0.2, 1.0, size=(P1.nCells, N, 1))
    f = rng.normal(size=(P1.nCells, nI))
    g = rng.normal(size=(P1.nFaces, Nf))
    u_old = rng.normal(size=(P1.nCells, N))
    P1.set_fields(tau.ravel(), kappa=kap.ravel(), src_mode=1, src=f, dirichlet=g.ravel(), dt=dt,
                  u_old=u_old if dt > 0 else None)
    tauB = np.zeros((P1.nFaces, Nf, 1, 4))
    tauB[..., 0, 0] = tauB[..., 0, 3] = tau
    fB = np.stack([f, 2 * f], -1)
    gB = np.stack([g, 2 * g], -1)
    oldB = np.stack([u_old, 2 * u_old], -1).reshape(P1.nCells, -1)
    PB.set_fields(tau=tauB, tau_sides=1, nu=kap, src=fB, dirichlet=gB, dt=dt, old=oldB if dt > 0 else None)
    PB.set_state(np.zeros((P1.nCells, PB.lenU)), np.zeros(PB.ndofs))
    P1.assemble()
    PB.assemble()
    a, b = P1.condensed(), PB.condensed()
    E, F = P1.nCells, re.nFaces
    LL, LU, LQ = F * Nf, N, 2 * N
    S1 = a["S"].reshape(E, LL, LL).transpose(0, 2, 1)              # [e][row][col]
    SB = b["S"].reshape(E, 2 * LL, 2 * LL).transpose(0, 2, 1)      # [e][row][col]
    scale = np.abs(S1).max()
    for c in range(2):
        for c2 in range(2):
            blk = SB[:, c::2, c2::2]
            ref = S1 if c == c2 else np.zeros_like(S1)
            assert np.abs(blk - ref).max() < 1e-12 * scale, (c, c2)
    # right-hand sides: component c carries (1 + c) x the scalar data (the Dirichlet rows too)
    S01, S0B = a["S0"], b["S0"].reshape(E, LL, 2)
    for c in range(2):
        assert np.abs(S0B[..., c] - (1 + c) * S01).max() < 1e-12 * np.abs(S01).max()
    # U, U0: rows (i, c), columns (f, a, c')
    U1 = a["U"].reshape(E, LL, LU).transpose(0, 2, 1)
    UB = b["U"].reshape(E, 2 * LL, 2 * LU).transpose(0, 2, 1)
    for c in range(2):
        assert np.abs(UB[:, c::2, c::2] - U1).max() < 1e-12 * np.abs(U1).max()
        assert np.abs(UB[:, c::2, (1 - c)::2]).max() < 1e-12 * np.abs(U1).max()
    U01, U0B = a["U0"], b["U0"].reshape(E, LU, 2)
    for c in range(2):
        assert np.abs(U0B[..., c] - (1 + c) * U01).max() < 1e-12 * np.abs(U01).max()
    # Q: scalar rows (i, k), Burgers rows ((i, k), c)
    Q1 = a["Q"].reshape(E, LL, LQ).transpose(0, 2, 1)
    QB = b["Q"].reshape(E, 2 * LL, 2 * LQ).transpose(0, 2, 1)
    for c in range(2):
        assert np.abs(QB[:, c::2, c::2] - Q1).max() < 1e-12 * np.abs(Q1).max()
