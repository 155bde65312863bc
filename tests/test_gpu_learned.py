"""Learned coarse polynomial of the two-level preconditioner (needs a GPU).

The GPU forward/backward kernels are checked against the FP64 numpy oracle
(oracle/learned_coarse.py) on the coarse operator the library assembles; FP32
kernels with FP64 sums, so the bar is 1e-4 relative. Training must beat the
Chebyshev polynomial it starts from, keep the coarse solve positive
semidefinite, and the learned two-level solve must match the direct solve and
beat the method without it (block-Jacobi CG).
"""
import os
import sys

import numpy as np
import pytest
import scipy.sparse as sp

from test_gpu_parity import build_pair

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import learned_coarse as LC  # noqa: E402

pytestmark = pytest.mark.gpu


def coarse_matrix(ctx):
    rowptr, col, val, vn = ctx.coarse_operator()
    n = len(vn)
    return sp.csr_matrix((val.astype(np.float64), col, rowptr), shape=(n, n))


@pytest.mark.parametrize("dim,n,order", [(2, 6, 2), (3, 3, 2)])
def test_gpu_loss_and_gradient_match_oracle(hfx_lib, dim, n, order):
    P, ctx, _ = build_pair(hfx_lib, dim, n, order, tau2=False, kappa="cell")
    ctx.assemble()
    A = coarse_matrix(ctx)
    rng = np.random.default_rng(5)
    S = rng.normal(size=(6, A.shape[0])).astype(np.float32)
    Di = LC.dinv_of(A)
    S[:, Di == 0] = 0.0
    theta = LC.chebyshev_theta(0.05, 1.8, 4) * 0.9
    L, g = ctx.coarse_loss_grad(theta, S)
    Lo, go = LC.loss_grad(A, S, theta)
    assert abs(L - Lo) <= 1e-4 * abs(Lo), (L, Lo)
    assert np.abs(g - go).max() <= 1e-4 * np.abs(go).max(), (g, go)


def test_training_beats_chebyshev_and_keeps_cg_valid(hfx_lib):
    P, ctx, _ = build_pair(hfx_lib, 3, 6, 2, tau2=False, kappa="none", jitter=0.0)
    ctx.assemble()
    info = ctx.coarse_train(degree=4, samples=16, steps=200)
    diag = (info.accepted, info.loss_chebyshev, info.loss_learned, info.max_poly, info.samples, info.steps,
            info.loss_first_step, info.lower_steps, info.rejected_steps)
    assert info.accepted == 1, "train " + " ".join(str(x) for x in diag)
    assert info.loss_learned < info.loss_chebyshev
    assert info.max_poly <= 1.0 + 1e-9


def test_learned_twolevel_solve_matches_direct_and_beats_block_jacobi(hfx_lib):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 3, 6, 2, tau2=True, kappa="cell")
    P.assemble()
    ctx.assemble()
    x_ref = P.solve_direct()
    info = ctx.coarse_train(degree=4, samples=16, steps=200)
    assert info.accepted == 1
    for prec in (0, 1):
        trace, tl = ctx.solve(precision=prec, rtol=1e-13, precond=capi.PC_TWOLEVEL,
                              coarse_mode=capi.COARSE_LEARNED)
        assert tl.status == 0 and tl.fallback == 0 and tl.coarse_learned == 1 and tl.coarse_degree == 4
        assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
        _, bj = ctx.solve(precision=prec, rtol=1e-13, precond=capi.PC_BLOCK_JACOBI)
        assert tl.iterations < 0.7 * bj.iterations, (tl.iterations, bj.iterations)
        # what the training gains: Chebyshev of the same degree needs more outer iterations
        _, same = ctx.solve(precision=prec, rtol=1e-13, precond=capi.PC_TWOLEVEL, coarse_degree=4)
        assert same.coarse_degree == 4 and same.coarse_learned == 0
        assert tl.iterations < same.iterations, (tl.iterations, same.iterations)
        # and the adaptive Chebyshev coarse solve takes a higher degree
        _, ch = ctx.solve(precision=prec, rtol=1e-13, precond=capi.PC_TWOLEVEL)
        assert ch.coarse_degree > tl.coarse_degree


def test_learned_mode_without_training_uses_chebyshev(hfx_lib):
    from hyperfox_gb300 import capi
    P, ctx, _ = build_pair(hfx_lib, 2, 6, 2, tau2=False, kappa="cell")
    ctx.assemble()
    _, info = ctx.solve(precond=capi.PC_TWOLEVEL, coarse_mode=capi.COARSE_LEARNED)
    assert info.status == 0 and info.coarse_learned == 0
