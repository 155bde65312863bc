"""Vector Burgers / Newton row on the GPU (hfx_burgers_*) vs the oracle.

HDGBurgersModel (HDGBase + HDGUNabU + HDGDiffusion with nd = dim unknowns, one
Source per component, implicit Euler), the nd-valued trace system, GMRES,
recovery and NonLinearWrapper's loop. Element blocks 1e-12 relative to the
oracle, CSR pattern bit-exact and values 1e-12, solves 1e-8 relative against a
direct FP64 solve of the oracle's system, Newton iterates 1e-8.
"""
import numpy as np
import pytest

import _oracle as O
from helpers import mesh
from test_burgers_oracle import cole_hopf, l2_err_vec
from test_gpu_parity import relerr

pytestmark = pytest.mark.gpu


def random_fields(P, re, rng, tau_sides=2, kappa="scalar", src=True, dt=0.0):
    nd = 2
    Nf, N = re["nNodesFace"], re["nNodes"]
    A = rng.uniform(-0.3, 0.3, size=(P.nFaces, Nf, tau_sides, nd, nd))
    A += np.eye(nd) * rng.uniform(0.8, 2.0, size=(P.nFaces, Nf, tau_sides, 1, 1))
    tau = np.ascontiguousarray(np.swapaxes(A, -1, -2)).reshape(P.nFaces, Nf, tau_sides, nd * nd)
    if kappa == "scalar":
        nu = rng.uniform(0.05, 0.5, size=(P.nCells, N, 1))
    elif kappa == "tensor":
        B = rng.normal(size=(P.nCells, N, 2, 2)) * 0.1
        nu = (np.einsum("enij,enkj->enik", B, B) + 0.2 * np.eye(2)).reshape(P.nCells, N, 4)
    else:
        nu = None
    f = rng.normal(size=(P.nCells, re["nIP"], nd)) if src else None
    g = rng.normal(size=(P.nFaces, Nf, nd))
    old = rng.normal(size=(P.nCells, N * nd)) if dt > 0 else None
    return tau, nu, f, g, old


def build(hfx_lib, n, order, seed=3, tau_sides=2, kappa="scalar", src=True, dt=0.0, jitter=0.15, scale=0.3,
          coords_noise=0.0, gpu=True):
    """A random linearisation state of size `scale` (BufferSolution and Trace) on a
    jittered mesh; coords_noise perturbs the oracle's copy of the coordinates;
    gpu=False builds the oracle problem only."""
    if gpu:
        from hyperfox_gb300 import capi
    rng = np.random.default_rng(seed)
    re, coords, cells = mesh(2, n, order, jitter=jitter, seed=seed)
    P = O.BurgersProblem(2, order, coords, cells)
    tau, nu, f, g, old = random_fields(P, re, rng, tau_sides, kappa, src, dt)
    buf = scale * rng.normal(size=(P.nCells, P.lenU))
    trace = scale * rng.normal(size=P.ndofs)
    if coords_noise:
        c2 = coords * (1 + coords_noise * np.random.default_rng(99).standard_normal(coords.shape))
        P = O.BurgersProblem(2, order, c2, cells)
    P.set_fields(tau=tau, tau_sides=tau_sides, nu=nu, src=f, dirichlet=g, dt=dt, old=old)
    P.set_state(buf, trace)
    if not gpu:
        return P, None, None, (coords, cells)
    ctx = capi.Context(0)
    ctx.upload_mesh(2, order, coords, cells)
    B = capi.Burgers(ctx)
    B.set_tau(tau, tau_sides)
    B.set_diffusion(nu, layout=1)
    B.set_source(f)
    B.set_dirichlet(g)
    B.set_time_step(dt)
    B.set_state(buffer=buf, trace=trace, old=old)
    return P, ctx, B, (coords, cells)


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("kappa,dt", [("scalar", 0.0), ("tensor", 1e-2), ("none", 1e-3)])
def test_element_blocks_match_oracle(hfx_lib, order, kappa, dt):
    P, ctx, B, _ = build(hfx_lib, 3, order, kappa=kappa, dt=dt)
    P.assemble()
    B.assemble()
    o, g = P.condensed(), B.condensed()
    for k in ("S", "S0", "U", "Q", "U0", "Q0"):
        assert relerr(g[k], o[k]) < 1e-12, k


def oracle_sensitivity(n, order, kappa, dt, scale, eps=1e-15):
    """How far the oracle's own blocks move when its coordinates change in the
    last digits (relative eps): the round-off floor of a parity comparison."""
    P0, _, _, _ = build(None, n, order, kappa=kappa, dt=dt, scale=scale, gpu=False)
    P1, _, _, _ = build(None, n, order, kappa=kappa, dt=dt, scale=scale, gpu=False, coords_noise=eps)
    P0.assemble()
    P1.assemble()
    a, b = P0.condensed(), P1.condensed()
    return {k: relerr(b[k], a[k]) for k in a}


def test_element_blocks_ill_conditioned_state(hfx_lib):
    """A unit-size random linearisation state with no mass term at p = 3 makes
    some element Schur blocks nearly singular: the oracle itself moves by about
    1.5e-12 under 1e-15 input perturbations. There the GPU must stay within ten
    times that floor (plus 1e-13)."""
    floor = oracle_sensitivity(3, 3, "scalar", 0.0, 1.0)
    P, ctx, B, _ = build(hfx_lib, 3, 3, kappa="scalar", dt=0.0, scale=1.0)
    P.assemble()
    B.assemble()
    o, g = P.condensed(), B.condensed()
    for k in ("S", "S0", "U", "Q", "U0", "Q0"):
        assert relerr(g[k], o[k]) < 10 * floor[k] + 1e-13, (k, relerr(g[k], o[k]), floor[k])


@pytest.mark.parametrize("order", [1, 3])
def test_trace_system_matches_oracle(hfx_lib, order):
    """CSR pattern and DOF numbering (face*Nf + node)*nd + k bit-exact, values and
    right-hand side 1e-12 (HDGSolver.cpp:531-675 with nd values per node)."""
    P, ctx, B, _ = build(hfx_lib, 4, order, tau_sides=1, dt=1e-2)
    P.assemble()
    B.assemble()
    rp_o, col_o, val_o, rhs_o = P.csr()
    rp_g, col_g, val_g, rhs_g = B.csr()
    assert np.array_equal(rp_g, rp_o.astype(np.int64))
    assert np.array_equal(col_g, col_o)
    assert relerr(val_g, val_o) < 1e-12
    assert relerr(rhs_g, rhs_o) < 1e-12


@pytest.mark.parametrize("order", [2, 3, 5])
def test_solve_and_recover_match_direct_solve(hfx_lib, order):
    P, ctx, B, _ = build(hfx_lib, 4, order, dt=1e-2)
    P.assemble()
    x = P.solve_direct()
    sol_o, flux_o = P.recover(x)
    B.assemble()
    info = B.solve(rtol=1e-13)
    assert info.status == 0 and info.iterations > 0
    sol, flux, trace, _ = B.get_state()
    assert relerr(trace, x) < 1e-8
    assert relerr(sol, sol_o) < 1e-8
    assert relerr(flux, flux_o) < 1e-8


def stationary_pair(hfx_lib, n, p, D=1.0):
    from hyperfox_gb300 import capi
    re, coords, cells = mesh(2, n, p)
    P = O.BurgersProblem(2, p, coords, cells)
    h = 1.0 / n
    tau = np.zeros((P.nFaces, re["nNodesFace"], 2, 4))
    tau[..., 0] = tau[..., 3] = 2.0 * D / h
    g = cole_hopf(coords[P.faces], D)
    nu = np.full((P.nCells, re["nNodes"], 1), D)
    P.set_fields(tau=tau, tau_sides=2, nu=nu, dirichlet=g)
    ctx = capi.Context(0)
    ctx.upload_mesh(2, p, coords, cells)
    B = capi.Burgers(ctx)
    B.set_tau(tau, 2)
    B.set_diffusion(nu, layout=1)
    B.set_dirichlet(g)
    return P, ctx, B, coords, cells


@pytest.mark.parametrize("p", [1, 2, 3])
def test_newton_cole_hopf_matches_oracle(hfx_lib, p):
    """TestHDGBurgersStat.cpp on the GPU: the device Newton loop takes the same
    iterations as the oracle's NonLinearWrapper restatement and lands on the same
    solution (1e-8), with the same error against the analytical solution."""
    P, ctx, B, coords, cells = stationary_pair(hfx_lib, 6, p)
    sol_o, flux_o, its_o, hist = P.newton(res_tol=1e-6, max_iters=10)
    info = B.newton(res_tol=1e-6, max_iters=10, lin_rtol=1e-13)
    assert info.status == 0
    assert info.iterations == its_o
    assert abs(info.residual - hist[-1]) <= 1e-3 * hist[-1] + 1e-10
    sol, flux, _, _ = B.get_state()
    assert relerr(sol, sol_o) < 1e-8
    assert relerr(flux, flux_o) < 1e-8
    e_g = l2_err_vec(P, coords, cells, sol, cole_hopf)
    e_o = l2_err_vec(P, coords, cells, sol_o, cole_hopf)
    assert abs(e_g - e_o) < 1e-8 * max(e_o, 1e-12) + 1e-13


def test_newton_damped_and_capped_matches_oracle(hfx_lib):
    """dampening 0.5 and a maximum of 3 iterations: the loop updates both fields
    with the damped value on every unconverged iteration (NonLinearWrapper.cpp:64-70)."""
    P, ctx, B, coords, cells = stationary_pair(hfx_lib, 4, 2)
    sol_o, _, its_o, hist = P.newton(res_tol=1e-6, max_iters=3, dampening=0.5)
    info = B.newton(res_tol=1e-6, max_iters=3, dampening=0.5, lin_rtol=1e-13)
    assert its_o == 3 and info.iterations == 3
    assert abs(info.residual - hist[-1]) <= 1e-6 * hist[-1]
    sol, _, _, buf = B.get_state()
    assert relerr(sol, P.buf) < 1e-8
    assert relerr(buf, P.buf) < 1e-8


@pytest.mark.parametrize("mixed", [False, True])
def test_time_steps_match_oracle(hfx_lib, mixed):
    """Implicit Euler Burgers, nu = 1e-2, dt = 1e-3, tau = I (TestHDGBurgers.cpp:290-297),
    u0 = sin(2 pi x) sin(2 pi y) + seeded noise on both components, Dirichlet 0:
    three steps, Newton to 1e-10 each, GPU vs oracle 1e-8 per step; the linear solves in
    FP64 GMRES, or (mixed) in FP32 GMRES inside FP64 residual refinement."""
    from hyperfox_gb300 import capi
    p, n = 3, 6
    re, coords, cells = mesh(2, n, p)
    P = O.BurgersProblem(2, p, coords, cells)
    rng = np.random.default_rng(7)
    x = coords[cells]
    u0 = np.sin(2 * np.pi * x[..., 0]) * np.sin(2 * np.pi * x[..., 1])
    u = np.stack([u0, u0], -1) + rng.normal(0, 0.01, size=x.shape)
    u = u.reshape(P.nCells, -1)
    tau = np.zeros((P.nFaces, re["nNodesFace"], 2, 4))
    tau[..., 0] = tau[..., 3] = 1.0
    nu = np.full((P.nCells, re["nNodes"], 1), 1e-2)
    zero = np.zeros((P.nFaces, re["nNodesFace"], 2))
    ctx = capi.Context(0)
    ctx.upload_mesh(2, p, coords, cells)
    B = capi.Burgers(ctx)
    B.set_tau(tau, 2)
    B.set_diffusion(nu, layout=1)
    B.set_dirichlet(zero)
    B.set_time_step(1e-3)
    B.set_state(solution=u)
    trace = np.zeros(P.ndofs)
    for step in range(3):
        P.set_fields(tau=tau, tau_sides=2, nu=nu, dirichlet=zero, dt=1e-3, old=u)
        P.buf, P.trace = u.copy(), trace
        u_next, _, its_o, _ = P.newton(res_tol=1e-10, max_iters=10)
        trace = P.trace
        B.begin_step()
        info = B.newton(res_tol=1e-10, max_iters=10, lin_rtol=1e-13,
                        lin_precision=capi.PREC_MIXED if mixed else capi.PREC_FP64)
        assert info.status == 0 and info.iterations == its_o
        sol, _, tr_g, _ = B.get_state()
        assert relerr(sol, u_next) < 1e-8, step
        assert relerr(tr_g, trace) < 1e-8, step
        u = u_next


def test_errors(hfx_lib):
    from hyperfox_gb300 import capi
    re, coords, cells = mesh(2, 2, 2)
    ctx = capi.Context(0)
    ctx.upload_mesh(2, 2, coords, cells)
    with pytest.raises(capi.HfxError) as e:
        ctx._chk(ctx.L.hfx_burgers_assemble(ctx.h), "burgers_assemble")
    assert e.value.code == 2  # HFX_ERR_STATE: setup first
    B = capi.Burgers(ctx)
    with pytest.raises(capi.HfxError) as e:
        B.solve()
    assert e.value.code == 2  # assemble first
    B.assemble()
    with pytest.raises(capi.HfxError) as e:
        B.solve(method=capi.KSP_CG)
    assert e.value.code == 1  # not symmetric
    re3, c3, s3 = mesh(3, 1, 1)
    ctx3 = capi.Context(0)
    ctx3.upload_mesh(3, 1, c3, s3)
    with pytest.raises(capi.HfxError) as e:
        capi.Burgers(ctx3)
    assert e.value.code == 9  # 2D cells only


def test_state_independent_cache(hfx_lib):
    """Later linearisations load the element blocks that depend only on geometry, tau
    and the diffusion field; a new tau or diffusion field recomputes them: every
    assembly still matches the oracle at 1e-12, and a repeated one is bit-identical."""
    P, ctx, B, _ = build(hfx_lib, 3, 3, kappa="scalar", dt=1e-2)
    B.assemble()
    first = B.condensed()
    B.assemble()  # from the cache
    again = B.condensed()
    for k in first:
        assert np.array_equal(first[k], again[k]), k
    rng = np.random.default_rng(21)
    re = ctx.re
    state = 0.3 * rng.normal(size=(P.nCells, P.lenU)), 0.3 * rng.normal(size=P.ndofs)
    tau2, nu2, f2, g2, old2 = random_fields(P, re, rng, 2, "tensor", True, 1e-3)
    steps = [dict(buf=state[0], trace=state[1]), dict(tau=tau2), dict(nu=nu2), dict(dt=1e-3, old=old2)]
    cur = dict(tau=None, nu=None, dt=1e-2, old=None)
    for change in steps:
        if "buf" in change:
            P.set_state(change["buf"], change["trace"])
            B.set_state(buffer=change["buf"], trace=change["trace"])
        if "tau" in change:
            B.set_tau(change["tau"], 2)
        if "nu" in change:
            B.set_diffusion(change["nu"], layout=1)
        if "dt" in change:
            B.set_time_step(change["dt"])
            B.set_state(old=change["old"])
        cur.update({k: v for k, v in change.items() if k in cur})
        P.set_fields(tau=cur["tau"], tau_sides=2, nu=cur["nu"] if cur["nu"] is not None else P._keep[1],
                     src=P._keep[2], dirichlet=P._keep[3], dt=cur["dt"],
                     old=cur["old"] if cur["old"] is not None else P._keep[4])
        P.assemble()
        B.assemble()
        o, g = P.condensed(), B.condensed()
        for k in ("S", "S0", "U", "Q", "U0", "Q0"):
            assert relerr(g[k], o[k]) < 1e-12, (list(change), k)


def test_krylov_history_guess(hfx_lib):
    """Krylov starts from the least-squares fit of the last trace solutions (history 6):
    four implicit Euler steps land on the oracle's solution (1e-8) like the warm start,
    with no more Krylov iterations than the warm start (the fitted span holds the
    previous solution, so the start's residual is never larger)."""
    from hyperfox_gb300 import capi
    p, n = 3, 6
    re, coords, cells = mesh(2, n, p)
    P = O.BurgersProblem(2, p, coords, cells)
    rng = np.random.default_rng(7)
    x = coords[cells]
    u0 = np.sin(2 * np.pi * x[..., 0]) * np.sin(2 * np.pi * x[..., 1])
    u0 = (np.stack([u0, u0], -1) + rng.normal(0, 0.01, size=x.shape)).reshape(P.nCells, -1)
    tau = np.zeros((P.nFaces, re["nNodesFace"], 2, 4))
    tau[..., 0] = tau[..., 3] = 1.0
    nu = np.full((P.nCells, re["nNodes"], 1), 1e-2)
    zero = np.zeros((P.nFaces, re["nNodesFace"], 2))
    # oracle trajectory
    u, trace, ref = u0.copy(), np.zeros(P.ndofs), []
    for step in range(4):
        P.set_fields(tau=tau, tau_sides=2, nu=nu, dirichlet=zero, dt=1e-3, old=u)
        P.buf, P.trace = u.copy(), trace
        u, _, _, _ = P.newton(res_tol=1e-10, max_iters=10)
        trace = P.trace
        ref.append(u)
    kry = {}
    for mode, (warm, hist) in {"warm": (1, 0), "history": (1, 6)}.items():
        ctx = capi.Context(0)
        ctx.upload_mesh(2, p, coords, cells)
        B = capi.Burgers(ctx)
        B.set_tau(tau, 2)
        B.set_diffusion(nu, layout=1)
        B.set_dirichlet(zero)
        B.set_time_step(1e-3)
        B.set_state(solution=u0)
        kry[mode] = 0
        for step in range(4):
            B.begin_step()
            info = B.newton(res_tol=1e-10, max_iters=10, lin_rtol=1e-13, warm_start=warm, history=hist)
            assert info.status == 0
            kry[mode] += info.krylov_iterations
            sol, _, _, _ = B.get_state()
            assert relerr(sol, ref[step]) < 1e-8, (mode, step)
        ctx.close()
    assert kry["history"] <= kry["warm"], kry
