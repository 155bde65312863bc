"""HDG operator blocks on the reference element (identity Jacobians), as
HyperFox's TestHDGBase.cpp:59-133 and TestHDGDiffusion.cpp:38-102 check them,
computed by the oracle's full local-matrix path on a one-element mesh."""
import numpy as np
import pytest

import _oracle as O

REF_NORMALS = {  # tests/TestUtils.h.in:251-264
    2: [[0, -1], [1 / np.sqrt(2), 1 / np.sqrt(2)], [-1, 0]],
    3: [[0, -1, 0], [1 / np.sqrt(3)] * 3, [-1, 0, 0], [0, 0, -1]],
}
CASES = [(d, p) for d in (2, 3) for p in range(1, 6 if d == 2 else 4)]


def reference_element_problem(dim, p, kappa=None):
    re = O.RefEl(dim, p)
    cells = np.arange(re.nNodes, dtype=np.int32)[None, :]
    P = O.Problem(dim, p, re.nodes, cells)
    P.set_fields(np.ones(P.ndofs), kappa=kappa)
    A, r, f2c = P.local_matrix(0)
    return re, P, A


def face_mass(re, dim, p):
    """Mass matrix of the face element (Mass.cpp:5-38) with reference weights."""
    fre = O.RefEl(dim - 1, p)
    return fre.phi.T @ (fre.ipW[:, None] * fre.phi)


@pytest.mark.parametrize("dim,p", CASES)
def test_base_blocks_on_reference_element(dim, p):
    re, P, A = reference_element_problem(dim, p)
    N, F, Nf = re.nNodes, re.nFaces, re.nNodesFace
    lenU, lenQ = N, dim * N
    sL = lenU + lenQ
    # Sqq = Mass with dim DOFs per node (TestHDGBase.cpp:83-86)
    M = re.phi.T @ (re.ipW[:, None] * re.phi)
    Sqq = np.kron(M, np.eye(dim))
    assert np.abs(A[lenU:sL, lenU:sL] - Sqq).sum() < 1e-12
    # Squ = convection with unit velocities (TestHDGBase.cpp:87-100)
    Squ = np.zeros((lenQ, N))
    for k in range(dim):
        C = np.einsum("q,qj,ql->jl", re.ipW, re.phi, re.dphi[:, :, k])  # Conv(j, l)
        for l in range(N):
            Squ[l * dim + k, :] = C[:, l]
    assert np.abs(A[lenU:sL, :lenU] - Squ).sum() < 1e-12
    # face blocks, with the face measure of each face (dS = w * |face| / |ref face|)
    measures = {2: [1.0, np.sqrt(2.0), 1.0], 3: [1.0, np.sqrt(3.0), 1.0, 1.0]}[dim]
    Mf = face_mass(re, dim, p)
    Slu = np.zeros((F * Nf, N))
    for f in range(F):
        fm = Mf * measures[f]
        blk = A[sL + f * Nf:sL + (f + 1) * Nf, sL + f * Nf:sL + (f + 1) * Nf]
        assert np.abs(blk + fm).sum() < 1e-12  # Sll = -faceMass
        for k in range(Nf):
            Slu[f * Nf:(f + 1) * Nf, re.faceNodes[f][k]] += fm[:, k]
    assert np.abs(A[sL:, :lenU] - Slu).sum() < 1e-12
    assert np.abs(A[:lenU, sL:] + Slu.T).sum() < 1e-12
    Suu = np.zeros((N, N))
    for f in range(F):
        for k in range(Nf):
            Suu[re.faceNodes[f][k], :] += Slu[f * Nf + k, :]
    assert np.abs(A[:lenU, :lenU] - Suu).sum() < 1e-12
    # Sql = -faceMass * n (TestHDGBase.cpp:117-128)
    Slq = np.zeros((F * Nf, lenQ))
    for f in range(F):
        fm = Mf * measures[f]
        for k in range(Nf):
            for d in range(dim):
                Slq[f * Nf:(f + 1) * Nf, re.faceNodes[f][k] * dim + d] = fm[:, k] * REF_NORMALS[dim][f][d]
    assert np.abs(A[lenU:sL, sL:] + Slq.T).sum() < 1e-12


@pytest.mark.parametrize("dim,p", CASES)
@pytest.mark.parametrize("kap", [1.0, 3.0])
def test_diffusion_blocks_on_reference_element(dim, p, kap):
    """TestHDGDiffusion.cpp:66-101: Suq, Slq for kappa = 1 and kappa = 3."""
    N = O.RefEl(dim, p).nNodes
    kappa = None if kap == 1.0 else np.full(N, kap)
    re, P, A = reference_element_problem(dim, p, kappa=kappa)
    F, Nf = re.nFaces, re.nNodesFace
    lenU, lenQ = N, dim * N
    sL = lenU + lenQ
    measures = {2: [1.0, np.sqrt(2.0), 1.0], 3: [1.0, np.sqrt(3.0), 1.0, 1.0]}[dim]
    Mf = face_mass(re, dim, p)
    Suq = np.zeros((N, lenQ))
    for k in range(dim):
        C = np.einsum("q,qj,ql->jl", re.ipW, re.phi, re.dphi[:, :, k])
        for l in range(N):
            Suq[:, l * dim + k] += C[l, :]
    Slq = np.zeros((F * Nf, lenQ))
    for f in range(F):
        fm = Mf * measures[f]
        for k in range(Nf):
            for l in range(Nf):
                for d in range(dim):
                    Suq[re.faceNodes[f][k], re.faceNodes[f][l] * dim + d] -= fm[k, l] * REF_NORMALS[dim][f][d]
                    Slq[f * Nf + k, re.faceNodes[f][l] * dim + d] -= fm[k, l] * REF_NORMALS[dim][f][d]
    assert np.abs(A[:lenU, lenU:sL] - kap * Suq).max() < 1e-12
    assert np.abs(A[sL:, lenU:sL] - kap * Slq).max() < 1e-12


@pytest.mark.parametrize("dim,n,order", [(2, 3, 2), (2, 2, 4), (3, 2, 2), (3, 1, 3)])
def test_cg_operators_identities(dim, n, order):
    """Mass, Diffusion and Convection (Mass.cpp:5-38, Diffusion.cpp:5-43, Convection.cpp:21-46) on
    jittered meshes: the mass equals HDGBase's Sqq block, the stiffness is symmetric, kills
    constants and maps x to the row integrals of d phi_i / dx (HDGBase's C_0 times 1), and the
    convection with v = e_0 kills constants and maps x to the mass row sums."""
    from helpers import mesh
    re, coords, cells = mesh(dim, n, order, jitter=0.1, seed=3)
    P = O.Problem(dim, order, coords, cells)
    P.set_fields(np.ones(P.ndofs), src_mode=0, dirichlet=np.zeros(P.ndofs))
    N = P.lenU
    vel = np.zeros((P.nCells, N, dim))
    vel[..., 0] = 1.0
    ops = P.cg_operators(7, vel)
    x = coords[cells][..., 0]
    for e in range(P.nCells):
        M = ops[e, 0].reshape(N, N).T  # column-major
        Dm = ops[e, 1].reshape(N, N).T
        C = ops[e, 2].reshape(N, N).T
        A, _, _ = P.local_matrix(e)
        q0 = N
        Sqq = A[q0::dim, q0::dim][:N, :N]
        assert np.abs(M - Sqq).max() < 1e-14 * max(1.0, np.abs(Sqq).max())
        scale = np.abs(Dm).max()
        assert np.abs(Dm - Dm.T).max() < 1e-12 * scale
        assert np.abs(Dm @ np.ones(N)).max() < 1e-12 * scale
        C0 = A[q0::dim, :N][:N]  # Squ rows (i, 0): integral of d phi_i/dx phi_j
        assert np.abs(Dm @ x[e] - C0 @ np.ones(N)).max() < 1e-12 * scale
        assert np.abs(C @ np.ones(N)).max() < 1e-12 * np.abs(C).max()
        assert np.abs(C @ x[e] - M @ np.ones(N)).max() < 1e-12 * np.abs(M).max()
