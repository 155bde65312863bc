"""IntegratedDirichletModel vs DirichletModel on the oracle: the same trace solution.

IntegratedDirichletModel (src/model/IntegratedDirichletModel.cpp:36-56) is a CG-type
boundary model with assembly Set: on a Dirichlet face its local matrix is the face mass
matrix M_f (Mass on the face element, face node order) and its local RHS is M_f g.
HDGSolver::applyBoundaryConditions (src/solver/HDGSolver.cpp:490-502) zeroes the
face's rows of the cell's S and S0 and adds both into them, indexed as they are. The
cell-local face node j is global trace node perm[j], so the global row block of the
face becomes B_f = Pi M_f Pi^T (Pi[perm[j], j] = 1) with right-hand side Pi M_f g. With
DirichletModel's identity rows the same block is I with right-hand side Pi g. The
integrated rows are therefore B_f times the nodal rows, and B_f is invertible, so both
systems have the trace solution Pi g on the face and the same solution everywhere else.
The GPU path implements DirichletModel's Set; these tests restate the integrated rows on
the oracle's trace system and show that the two solutions agree to round-off, for the
scalar diffusion system and the vector Burgers system (nd = 2, B_f (x) I).
"""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import _oracle as O
from helpers import fields, mesh


def face_mass(P, f, dim, order):
    """Mass on the face element (HyperFox Mass.cpp:5-38 on a (dim-1)-simplex): face
    node order, measure |face| / |reference face| (the reference face has measure 2 in
    1D and 2D); the face's first dim nodes are its vertices."""
    fe = O.RefEl(dim - 1, order)
    v = P.coords[P.faces[f][:dim]]
    if dim == 2:
        meas = np.linalg.norm(v[1] - v[0])
    else:
        meas = 0.5 * np.linalg.norm(np.cross(v[1] - v[0], v[2] - v[0]))
    return (fe.phi.T * (fe.ipW * meas / 2.0)) @ fe.phi


def face_perm(P, f):
    """perm[j]: the global face-node index of the boundary cell's local face node j."""
    c = P.face2cell[f, 0]
    loc = list(P.cell2face[c]).index(f)
    local_nodes = P.cells[c][P.re.faceNodes[loc]]
    glob = list(P.faces[f])
    return np.array([glob.index(n) for n in local_nodes])


def integrated_system(P, dim, order, nd):
    rowptr, col, val, rhs = P.csr()
    n = rhs.size
    A = sp.csr_matrix((val, col, rowptr), shape=(n, n)).tolil()
    Nf = P.re.nNodesFace
    lenT = Nf * nd
    A_int = A.copy()
    rhs_int = rhs.copy()
    for f in P.boundary:
        rows = np.arange(f * lenT, (f + 1) * lenT)
        # premise: DirichletModel's Set left identity rows on the face's own block
        blk = A[rows, :].toarray()
        eye = np.zeros_like(blk)
        eye[:, rows] = np.eye(lenT)
        assert np.array_equal(blk, eye)
        perm = face_perm(P, f)
        Pi = np.zeros((Nf, Nf))
        Pi[perm, np.arange(Nf)] = 1.0
        B = np.kron(Pi @ face_mass(P, f, dim, order) @ Pi.T, np.eye(nd))
        A_int[rows, :] = 0.0
        for a in range(lenT):
            for b in range(lenT):
                A_int[rows[a], rows[b]] = B[a, b]
        rhs_int[rows] = B @ rhs[rows]
    return A.tocsr(), rhs, A_int.tocsr(), rhs_int


@pytest.mark.parametrize("dim,n,order", [(2, 4, 1), (2, 3, 3), (3, 2, 2)])
def test_integrated_dirichlet_gives_the_nodal_set_solution(dim, n, order):
    rng = np.random.default_rng(order)
    re, coords, cells = mesh(dim, n, order, jitter=0.15, seed=order)
    P = O.Problem(dim, order, coords, cells)
    tau, kap, g = fields(dim, order, coords, cells, P.faces, P.nFaces, rng, kappa="scalar")
    g = g + rng.normal(size=g.shape) * 0.1  # values that vary along every face
    P.set_fields(tau.ravel(), kappa=kap.ravel(), src_mode=2, dirichlet=g.ravel())
    P.assemble()
    A, b, Ai, bi = integrated_system(P, dim, order, 1)
    x = spla.spsolve(A.tocsc(), b)
    xi = spla.spsolve(Ai.tocsc(), bi)
    assert np.linalg.norm(xi - x) <= 1e-12 * np.linalg.norm(x)
    # on a Dirichlet face the solution is Pi g: the face's values in the cell-local order
    f = P.boundary[0]
    Nf = P.re.nNodesFace
    perm = face_perm(P, f)
    assert np.allclose(xi[f * Nf + perm], g[f], rtol=0, atol=1e-12)


def test_integrated_dirichlet_burgers_system():
    """nd = 2: the same for the linearised vector Burgers trace system (B_f (x) I)."""
    p = 2
    rng = np.random.default_rng(3)
    re, coords, cells = mesh(2, 3, p, jitter=0.15, seed=3)
    PB = O.BurgersProblem(2, p, coords, cells)
    Nf = PB.re.nNodesFace
    tau = np.zeros((PB.nFaces, Nf, 1, 4))
    tau[..., 0, 0] = tau[..., 0, 3] = 1.0
    nu = np.full((PB.nCells, PB.re.nNodes, 1), 0.05)
    g = rng.normal(size=(PB.nFaces, Nf, 2))
    PB.set_fields(tau=tau, tau_sides=1, nu=nu, dirichlet=g, dt=1e-2, old=rng.normal(size=(PB.nCells, PB.lenU)))
    PB.set_state(rng.normal(size=(PB.nCells, PB.lenU)) * 0.3, rng.normal(size=PB.ndofs) * 0.3)
    PB.assemble()
    A, b, Ai, bi = integrated_system(PB, 2, p, 2)
    x = spla.spsolve(A.tocsc(), b)
    xi = spla.spsolve(Ai.tocsc(), bi)
    assert np.linalg.norm(xi - x) <= 1e-12 * np.linalg.norm(x)
