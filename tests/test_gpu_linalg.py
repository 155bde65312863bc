"""LinAlgebraInterface drop-in on the device (TestLinAlgebraInterfaces.cpp:70-...)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture()
def la(hfx_lib):
    from hyperfox_gb300 import capi
    ctx = capi.Context(0)
    return ctx, capi.LinearSystem(ctx)


def test_identity(la):
    ctx, L = la
    for k in (1, 7, 50, 100):
        L.allocate(k)
        for i in range(k):
            L.values([i], [i], [1.0], insert=True)
            L.rhs([i], [float(i)], insert=True)
        L.assemble()
        x, info = L.solve(rtol=1e-16, maxits=1000)
        assert np.abs(x - np.arange(k)).max() < 1e-12


def test_triangular(la):
    ctx, L = la
    for k in (1, 10, 60):
        L.allocate(k)
        for i in range(k):
            L.values([i], list(range(i + 1)), np.ones(i + 1), insert=True)
            L.rhs([i], [1.0], insert=True)
        L.assemble()
        x, info = L.solve(rtol=1e-16, maxits=2000)
        ana = np.zeros(k)
        ana[0] = 1.0
        assert np.abs(x - ana).max() < 1e-12


def test_hinge(la):
    ctx, L = la
    k = 40
    L.allocate(k)
    for i in range(k):
        L.values([i], [i], [1.0], insert=True)
        if i:
            L.values([i], [i - 1], [1.0], insert=True)
        L.rhs([i], [1.0], insert=True)
    L.assemble()
    x, info = L.solve(rtol=1e-16, maxits=2000)
    ana = np.array([1.0 if i % 2 == 0 else 0.0 for i in range(k)])
    assert np.abs(x - ana).max() < 1e-12


def test_add_block_and_trace_system(la, hfx_lib):
    """Scatter the oracle's element blocks through the generic interface and solve."""
    import _oracle as O
    from helpers import manufactured, mesh
    ctx, L = la
    re, coords, cells = mesh(2, 4, 2)
    P = O.Problem(2, 2, coords, cells)
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=manufactured(coords, P.faces).ravel())
    P.assemble()
    rowptr, col, val, rhs = P.csr()
    L.allocate(P.ndofs)
    for r in range(P.ndofs):
        cols = col[rowptr[r]:rowptr[r + 1]]
        L.values([r], cols, val[rowptr[r]:rowptr[r + 1]])
    L.rhs(np.arange(P.ndofs), rhs)
    L.assemble()
    x, info = L.solve(rtol=1e-13, maxits=20000, restart=50)
    x_ref = P.solve_direct()
    assert np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref) < 1e-9
