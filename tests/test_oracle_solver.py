"""Solver-level checks of the oracle against HyperFox's regression tests
(TestHDGSolver.cpp:88-100, TestHDGLaplace.cpp:110-150) and the trace-system
sizes the workloads are quoted on."""
import numpy as np
import pytest

import _oracle as O
from hyperfox_gb300 import meshgen


def oracle_mesh(dim, n, p, jitter=0.0, seed=0):
    re = O.RefEl(dim, p)
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    if jitter:
        v = meshgen.jitter_vertices(v, n, jitter, seed)
    return meshgen.high_order(v, s, re.nodes)


def test_constant_dirichlet_gives_constant_solution():
    """TestHDGSolver.cpp:88-100 (lightTri2.h5 replaced by a jittered 2D p=2 mesh)."""
    coords, cells = oracle_mesh(2, 6, 2, jitter=0.2, seed=5)
    P = O.Problem(2, 2, coords, cells)
    P.set_fields(np.ones(P.ndofs), dirichlet=np.full(P.ndofs, 3.0))
    P.assemble()
    x = P.solve_direct()
    sol, flux = P.recover(x)
    assert np.abs(x - 3).max() < 1e-12
    assert np.abs(sol - 3).max() < 1e-12
    assert np.abs(flux).max() < 1e-11


def l2_error(P, coords, cells, sol, exact):
    """TestUtils l2 error of a cell field against an analytical function."""
    re = P.re
    err = 0.0
    X = coords[cells]                       # E x N x d
    xq = np.einsum("qn,end->eqd", re.phi, X)
    uh = np.einsum("qn,en->eq", re.phi, sol)
    J = np.einsum("qnr,ens->eqrs", re.dphi, X)
    det = np.linalg.det(J)
    err = np.sum((uh - exact(xq)) ** 2 * det * re.ipW[None, :])
    return np.sqrt(err)


@pytest.mark.parametrize("dim,n,p", [(2, 3, 1), (2, 5, 2), (2, 10, 3), (2, 10, 1), (3, 5, 1), (3, 5, 2)])
def test_laplace_sin_exp_regression(dim, n, p):
    """TestHDGLaplace.cpp:20-28,139: u = sin(x) e^y (harmonic), l2Err < 1e-2."""
    coords, cells = oracle_mesh(dim, n, p)
    P = O.Problem(dim, p, coords, cells)
    exact = lambda x: np.sin(x[..., 0]) * np.exp(x[..., 1])
    g = exact(coords[P.faces])
    P.set_fields(np.ones(P.ndofs), dirichlet=g.ravel())
    P.assemble()
    x = P.solve_direct()
    sol, _ = P.recover(x)
    assert l2_error(P, coords, cells, sol, exact) < 1e-2


def test_manufactured_rates():
    errs = []
    for n in (4, 8, 16):
        coords, cells = oracle_mesh(2, n, 2)
        P = O.Problem(2, 2, coords, cells)
        g = np.prod(np.sin(np.pi * coords[P.faces]), axis=-1)
        P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=g.ravel())
        P.assemble()
        sol, _ = P.recover(P.solve_direct())
        exact = lambda x: np.sin(np.pi * x[..., 0]) * np.sin(np.pi * x[..., 1])
        errs.append(l2_error(P, coords, cells, sol, exact))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert rates.min() > 2.7, (errs, rates)  # p+1 = 3


def test_cfg1_trace_system_sizes():
    """2D, 32x32x2 triangles, p=2: 3136 faces (128 boundary), 9408 DOFs, 138,816 nnz."""
    coords, cells = oracle_mesh(2, 32, 2)
    P = O.Problem(2, 2, coords, cells)
    P.set_fields(np.ones(P.ndofs))
    P.assemble()
    rowptr, col, val, rhs = P.csr()
    assert (P.nFaces, P.nBoundary, P.ndofs, len(col)) == (3136, 128, 9408, 138816)
    for r in range(0, P.ndofs, 97):
        c = col[rowptr[r]:rowptr[r + 1]]
        assert np.all(np.diff(c) > 0)


def _interior_block(P):
    import scipy.sparse as sp
    rowptr, col, val, rhs = P.csr()
    A = sp.csr_matrix((val, col, rowptr)).toarray()
    Nf = P.re.nNodesFace
    bnd = np.zeros(P.ndofs, bool)
    for f in P.boundary:
        bnd[f * Nf:(f + 1) * Nf] = True
    return A[~bnd][:, ~bnd]


def test_interior_block_symmetric_when_kappa_is_cellwise_constant():
    """With tau varying per face node and kappa constant per cell, the interior
    trace block is symmetric negative definite: CG on the negated system is valid."""
    coords, cells = oracle_mesh(3, 2, 2, jitter=0.1, seed=2)
    P = O.Problem(3, 2, coords, cells)
    rng = np.random.default_rng(0)
    kap = np.repeat(rng.uniform(0.5, 2, P.nCells), P.re.nNodes)
    P.set_fields(rng.uniform(0.5, 2, P.ndofs), kappa=kap)
    P.assemble()
    Aii = _interior_block(P)
    assert np.abs(Aii - Aii.T).max() < 1e-12 * np.abs(Aii).max()
    assert np.linalg.eigvalsh(-Aii).min() > 0


def test_interior_block_nonsymmetric_when_kappa_varies_in_cells():
    """HyperFox weights only Suq/Slq by kappa (HDGDiffusion.cpp:74-145) while Sqq
    stays the plain mass, so a kappa that varies inside a cell makes the
    condensed system non-symmetric (GMRES territory), with a positive real spectrum."""
    coords, cells = oracle_mesh(3, 2, 2, jitter=0.1, seed=2)
    P = O.Problem(3, 2, coords, cells)
    rng = np.random.default_rng(0)
    P.set_fields(np.ones(P.ndofs), kappa=rng.uniform(0.5, 2, P.nCells * P.re.nNodes))
    P.assemble()
    Aii = _interior_block(P)
    assert np.abs(Aii - Aii.T).max() > 1e-4 * np.abs(Aii).max()
    assert np.linalg.eigvals(-Aii).real.min() > 0


def test_gmres_matches_direct():
    coords, cells = oracle_mesh(2, 6, 3, jitter=0.1, seed=1)
    P = O.Problem(2, 3, coords, cells)
    g = np.prod(np.sin(np.pi * coords[P.faces]), axis=-1)
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=g.ravel())
    P.assemble()
    x, it = P.solve_gmres(1e-13, 20000)
    assert it > 0
    xd = P.solve_direct()
    assert np.linalg.norm(x - xd) / np.linalg.norm(xd) < 1e-9


@pytest.mark.parametrize("dim,n,order", [(2, 4, 2), (3, 2, 3)])
def test_sampled_blocks_and_face_rows_equal_full_assembly(dim, n, order):
    """The oracle's element sample and face rows (parity on meshes too large to
    condense whole) equal the full assembly's blocks and CSR rows."""
    from helpers import manufactured, mesh
    re, coords, cells = mesh(dim, n, order, jitter=0.1, seed=1)
    P = O.Problem(dim, order, coords, cells)
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=manufactured(coords, P.faces).ravel())
    P.assemble()
    full = P.condensed()
    ids = np.array([0, 3, 5, P.nCells - 1])
    smp = P.sample(ids)
    for k in smp:
        assert np.array_equal(smp[k], full[k][ids]), k
    rowptr, col, val, rhs = P.csr()
    faces = np.unique([0, 7, P.nFaces - 1, int(P.boundary[0]), int(P.boundary[-1])])
    rl, c2, v2, r2 = P.face_rows(faces)
    Nf, pos = P.re.nNodesFace, 0
    for k, f in enumerate(faces):
        for a in range(Nf):
            r, m = f * Nf + a, rl[k * Nf + a]
            assert m == rowptr[r + 1] - rowptr[r]
            assert np.array_equal(c2[pos:pos + m], col[rowptr[r]:rowptr[r + 1]])
            assert np.array_equal(v2[pos:pos + m], val[rowptr[r]:rowptr[r + 1]])
            assert r2[k * Nf + a] == rhs[r]
            pos += m
    with pytest.raises(RuntimeError):
        P.face_rows(np.array([faces[0], faces[0]]))
