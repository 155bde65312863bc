"""gmsh reading and high-order node construction (host only, no GPU).

Restates tools/convertGmsh2H5HO.cpp without MOAB. The high-order nodes must be the
affine images of the reference nodes in every cell and coincide with the
synthetic-mesh generator's; the shipped gmsh meshes of the reference are read
when the reference tree is present.
"""
import os

import numpy as np
import pytest

from gmsh_util import write_gmsh22
from helpers import reference_meshes
from hyperfox_gb300 import capi, meshgen

REF = reference_meshes() or ""


@pytest.mark.parametrize("dim,n", [(2, 4), (3, 2)])
def test_gmsh_roundtrip(tmp_path, dim, n):
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    v = meshgen.jitter_vertices(v, n, 0.15, 3)
    path = tmp_path / "m.msh"
    write_gmsh22(path, v, s)
    c, e = capi.gmsh_read(path, dim)
    assert c.shape == v.shape and e.shape == s.shape
    assert np.array_equal(c, v) and np.array_equal(e, s)


@pytest.mark.parametrize("dim,n,order", [(2, 3, 1), (2, 3, 3), (2, 2, 5), (3, 2, 2), (3, 2, 3)])
def test_high_order_matches_generator(dim, n, order):
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    v = meshgen.jitter_vertices(v, n, 0.15, 1)
    re = capi.refel(dim, order)
    c_ref, e_ref = meshgen.high_order(v, s, re["nodes"])
    c, e = capi.mesh_high_order(dim, order, v, s)
    assert c.shape == c_ref.shape and e.shape == e_ref.shape
    assert np.abs(c[e] - c_ref[e_ref]).max() < 1e-14
    assert np.array_equal(e, e_ref)
    # every node is the affine image of its reference node
    lam = (re["nodes"] + 1.0) / 2.0
    x0 = v[s[:, 0]]
    aff = x0[:, None, :] + np.einsum("nk,ekd->end", lam, np.stack([v[s[:, k + 1]] - x0 for k in range(dim)], 1))
    assert np.abs(c[e] - aff).max() < 1e-13


def test_gmsh_errors(tmp_path):
    p = tmp_path / "bad.msh"
    p.write_text("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
    with pytest.raises(capi.HfxError):
        capi.gmsh_read(p, 2)
    with pytest.raises(capi.HfxError):
        capi.gmsh_read(tmp_path / "missing.msh", 2)


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference meshes not present")
@pytest.mark.parametrize("name,nodes", [("regression/regression_dim-2_h-1e-1.msh", 142),
                                        ("lightSquareOrd1.msh", None), ("lightSquareOrd2.msh", None)])
def test_reference_gmsh_meshes(name, nodes):
    c, e = capi.gmsh_read(os.path.join(REF, name), 2)
    assert c.shape[1] == 2 and e.shape[1] == 3
    assert e.min() == 0 and e.max() == c.shape[0] - 1
    if nodes is not None:
        assert c.shape[0] == nodes
    # positively or negatively oriented, never degenerate
    u, w = c[e[:, 1]] - c[e[:, 0]], c[e[:, 2]] - c[e[:, 0]]
    a = u[:, 0] * w[:, 1] - u[:, 1] * w[:, 0]
    assert np.abs(a).min() > 0
    for order in (2, 3):
        hc, he = capi.mesh_high_order(2, order, c, e)
        assert he.shape == (e.shape[0], capi.refel(2, order)["nNodes"])
        assert np.array_equal(hc[he[:, :3]], c[e])


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference meshes not present")
def test_reference_regression_mesh_feeds_the_oracle():
    """The shipped regression mesh, raised to p=2, solves the manufactured problem."""
    import _oracle as O
    c, e = capi.gmsh_read(os.path.join(REF, "regression/regression_dim-2_h-1e-1.msh"), 2)
    hc, he = capi.mesh_high_order(2, 2, c, e)
    P = O.Problem(2, 2, hc, he)
    g = np.prod(np.sin(np.pi * hc[P.faces]), axis=-1)
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=g.ravel())
    P.assemble()
    x = P.solve_direct()
    sol, _ = P.recover(x)
    exact = np.prod(np.sin(np.pi * hc[he]), axis=-1)
    assert np.abs(sol - exact).max() < 5e-3


def test_high_order_merges_nodes_across_rounding_boundaries():
    """Two problems of the 1024-problem batch (seed 3: problem 247, 47x47x2 triangles at p = 2,
    and problem 68, 92x92x2 at p = 3, jittered vertices) have a shared edge node whose two
    computations, from the two cells of the edge, round to neighbouring merge keys; the node
    construction finds the node within one quantum there, so every cell's face nodes are the
    face's nodes (the topology the element kernels need)."""
    from hyperfox_gb300 import batch
    for prob in batch.uneven_batch(count=1024, seed=3, select=[247, 68]):
        c2f, _, faces, _ = prob.topology
        fn = np.asarray(capi.refel(2, prob.order)["faceNodes"]).reshape(3, -1)
        for i in range(3):
            assert np.array_equal(np.sort(prob.cells[:, fn[i]], axis=1), np.sort(faces[c2f[:, i]], axis=1))
        # merged means no two nodes closer than a small fraction of the mesh spacing
        assert prob.coords.shape[0] == len(np.unique(np.round(prob.coords, 8), axis=0))
