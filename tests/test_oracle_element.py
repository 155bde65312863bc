"""Reference element and cubature: the oracle and the library's host tables
against HyperFox's own known-answer tests (TestCubature.cpp,
TestReferenceElement.cpp) and against the reference's compiled Cubature.cpp."""
import itertools
import json
import math
import os
from fractions import Fraction

import numpy as np
import pytest

import _oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
# TestCubature.cpp:43-44, simplex point counts for orders 0..10
NIP = {2: [1, 1, 3, 6, 6, 7, 12, 15, 16, 19, 25], 3: [1, 1, 4, 8, 14, 14, 24, 35, 46, 59, 81]}
VOLUME = {1: 2.0, 2: 2.0, 3: 4.0 / 3.0}


def simplex_monomial(a):
    """Exact integral of prod x_k^a_k over the reference simplex (vertices -1, e_k)."""
    d = len(a)
    # x = 2 lam - 1 on the unit simplex {lam >= 0, sum <= 1}: Dirichlet integrals
    total = Fraction(0)
    for ks in itertools.product(*[range(ak + 1) for ak in a]):
        coef = Fraction(1)
        for ak, k in zip(a, ks):
            coef *= math.comb(ak, k) * Fraction(2) ** k * (-1) ** (ak - k)
        num = 1
        for k in ks:
            num *= math.factorial(k)
        total += coef * Fraction(num, math.factorial(sum(ks) + d))
    return float(total * 2 ** d)


@pytest.mark.parametrize("dim", [2, 3])
def test_cubature_counts_and_volumes(dim):
    for order in range(1, 11):
        X, W = O.cubature(dim, order)
        assert len(W) == NIP[dim][order]
        assert abs(W.sum() - VOLUME[dim]) < 1e-13


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_cubature_exactness(dim):
    for order in range(1, 11):
        X, W = O.cubature(dim, order)
        for a in itertools.product(range(order + 1), repeat=dim):
            if sum(a) > order:
                continue
            q = np.sum(W * np.prod(X ** np.array(a), axis=1))
            assert abs(q - simplex_monomial(a)) < 1e-13, (dim, order, a)


def test_cubature_x10_known_answers():
    """TestCubature.cpp:120-121: int x^10 = 2/11 (triangle), 24/143 (tet)."""
    for dim, ans in ((2, 2.0 / 11.0), (3, 24.0 / 143.0)):
        X, W = O.cubature(dim, 10)
        assert abs(np.sum(W * X[:, 0] ** 10) - ans) < 1e-14


def test_cubature_matches_reference_golden():
    """Points and weights equal the reference's own Cubature.cpp (golden file made
    by tests/golden/make_cubature_golden.py from oracle/_ref)."""
    with open(os.path.join(HERE, "golden", "cubature_ref.json")) as fh:
        gold = json.load(fh)
    for key, rule in gold.items():
        dim, order = (int(v) for v in key.split("_"))
        X, W = O.cubature(dim, order)
        Xr = np.array(rule["points"]).reshape(-1, dim)
        Wr = np.array(rule["weights"])
        if dim >= 2:  # tabulated data: bit-exact
            assert np.array_equal(X, Xr) and np.array_equal(W, Wr), key
        else:  # Gauss-Legendre computed here, listed in the reference's order
            assert np.abs(X - Xr).max() < 1e-15 and np.abs(W - Wr).max() < 1e-15, key


def test_cubature_matches_reference_build():
    """Same check against the reference library itself when it was built here."""
    import ctypes
    path = os.path.join(O.ROOT, "oracle", "_ref", "libref_cubature.so")
    if not os.path.exists(path):
        pytest.skip("oracle/_ref not built (needs the HyperFox tree)")
    lib = ctypes.CDLL(path)
    f = lib.ref_cubature
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    for dim in (2, 3):
        for order in range(1, 11):
            Xr = np.zeros(400)
            Wr = np.zeros(200)
            n = f(dim, order, 0, Xr.ctypes.data, Wr.ctypes.data, 200)
            X, W = O.cubature(dim, order)
            assert n == len(W)
            assert np.array_equal(X.ravel(), Xr[:n * dim]) and np.array_equal(W, Wr[:n])


CASES = [(d, p) for d in (2, 3) for p in range(1, (6 if d == 2 else 4))]


@pytest.mark.parametrize("dim,p", CASES)
def test_lagrange_property(dim, p):
    """TestReferenceElement.cpp:117-145 (margin 1e-10)."""
    re = O.RefEl(dim, p)
    assert re.nNodes == math.comb(p + dim, dim)
    phi, _ = re.eval(re.nodes)
    assert np.abs(phi - np.eye(re.nNodes)).max() < 1e-10


@pytest.mark.parametrize("dim,p", CASES)
def test_monomial_interpolation(dim, p):
    """TestReferenceElement.cpp:146-236: x^p + y^p (+ z^p) and its gradient at (-0.5, ...)."""
    re = O.RefEl(dim, p)
    pt = np.full((1, dim), -0.5)
    phi, dphi = re.eval(pt)
    vals = np.sum(re.nodes ** p, axis=1)
    assert abs(phi[0] @ vals - np.sum(pt ** p)) < 1e-12
    grad = dphi[0].T @ vals
    assert np.abs(grad - p * pt[0] ** (p - 1)).max() < 1e-11


@pytest.mark.parametrize("dim,p", CASES)
def test_face_nodes_lie_on_faces(dim, p):
    re = O.RefEl(dim, p)
    verts = {2: [[0, 1], [1, 2], [2, 0]], 3: [[3, 1, 0], [2, 1, 3], [2, 3, 0], [0, 1, 2]]}[dim]
    for f, fv in enumerate(verts):
        V = re.nodes[fv]
        for n in re.faceNodes[f]:
            # barycentric coordinates w.r.t. the face vertices reproduce the node
            A = np.vstack([V.T, np.ones(dim)])
            lam = np.linalg.lstsq(A, np.append(re.nodes[n], 1.0), rcond=None)[0]
            assert np.abs(A @ lam - np.append(re.nodes[n], 1.0)).max() < 1e-12
            assert lam.min() > -1e-12
