"""Learned coarse polynomial: CPU restatement, TEST INFRASTRUCTURE ONLY.

FP64 numpy restatement of the model, loss and gradient that the CUDA library
trains for the coarse solve of its two-level trace preconditioner (no
counterpart in HyperFox, whose trace solve is PETSc GMRES + Jacobi,
src/resolution/PetscInterface.cpp:222-247). Only the tests load it, as the
checker of the GPU forward/backward kernels.

Model: U_{k+1} = U_k - theta_k D^{-1} A U_k for k = 0..K-1 (Richardson steps
propagating coarse errors U, A the coarse operator, D its diagonal), loss
L = sum_s w_s U_K[s]^T A U_K[s] with w_s = 1 / (S U_0[s]^T A U_0[s]) (the energy
of the error left by the coarse solve). Gradient by reverse mode:
G_K = 2 w A U_K, dL/dtheta_k = -G_{k+1} . D^{-1} A U_k,
G_k = G_{k+1} - theta_k A D^{-1} G_{k+1}.
"""
import numpy as np


def dinv_of(A):
    d = np.asarray(A.diagonal(), dtype=np.float64)
    return np.where(d > 0, 1.0 / np.where(d > 0, d, 1.0), 0.0)


def loss_grad(A, samples, theta):
    """A: scipy sparse (nV x nV); error samples [S][nV]; theta [K] -> (loss, grad[K])."""
    A = A.astype(np.float64).tocsr()
    Di = dinv_of(A)
    U = np.asarray(samples, dtype=np.float64).T.copy()  # [nV][S]
    S = U.shape[1]
    w = 1.0 / (S * np.einsum("vs,vs->s", U, A @ U))
    Us, Ys = [U], []
    for t in theta:
        Y = Di[:, None] * (A @ Us[-1])
        Ys.append(Y)
        Us.append(Us[-1] - t * Y)
    AU = A @ Us[-1]
    L = float(np.einsum("s,vs,vs->", w, Us[-1], AU))
    G = 2.0 * w[None, :] * AU
    grad = np.zeros(len(theta))
    for k in range(len(theta) - 1, -1, -1):
        grad[k] = -np.sum(G * Ys[k])
        G = G - theta[k] * (A @ (Di[:, None] * G))
    return L, grad


def chebyshev_theta(lmin, lmax, K):
    """Richardson weights whose residual polynomial is Chebyshev of degree K on [lmin, lmax]."""
    j = np.arange(K)
    lam = 0.5 * (lmax + lmin) + 0.5 * (lmax - lmin) * np.cos(np.pi * (2 * j + 1) / (2.0 * K))
    return 1.0 / lam
