"""CPU checks of the learned-coarse-polynomial oracle (no GPU)."""
import os
import sys

import numpy as np
import scipy.sparse as sp

sys.path.insert(0, os.path.join(os.path.dirname(__file__), "..", "oracle"))
import learned_coarse as LC  # noqa: E402


def laplacian(n):
    T = sp.diags([-1.0, 2.0, -1.0], [-1, 0, 1], shape=(n, n))
    I = sp.identity(n)
    return (sp.kron(T, I) + sp.kron(I, T)).tocsr()


def test_oracle_gradient_matches_finite_differences():
    A = laplacian(12)
    rng = np.random.default_rng(0)
    S = rng.normal(size=(5, A.shape[0]))
    theta = np.array([0.3, 0.6, 0.9, 0.45])
    L, g = LC.loss_grad(A, S, theta)
    for k in range(len(theta)):
        e = np.zeros_like(theta)
        e[k] = 1e-6
        fd = (LC.loss_grad(A, S, theta + e)[0] - LC.loss_grad(A, S, theta - e)[0]) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])


def test_chebyshev_weights_give_chebyshev_residual_polynomial():
    lmin, lmax, K = 0.05, 2.0, 5
    th = LC.chebyshev_theta(lmin, lmax, K)
    lam = np.linspace(lmin, lmax, 400)
    q = np.prod([1 - t * lam for t in th], axis=0)
    x = (lmax + lmin - 2 * lam) / (lmax - lmin)
    sig = (lmax + lmin) / (lmax - lmin)
    ref = np.cos(K * np.arccos(np.clip(x, -1, 1))) / np.cosh(K * np.arccosh(sig))
    assert np.allclose(q, ref, atol=1e-12)
