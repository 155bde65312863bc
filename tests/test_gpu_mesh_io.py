"""A gmsh-fed mesh through the whole CUDA path (read, high-order nodes, upload, solve)."""
import numpy as np
import pytest

import _oracle as O
from gmsh_util import write_gmsh22
from hyperfox_gb300 import capi, meshgen

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dim,n,order", [(2, 6, 3), (3, 3, 2)])
def test_gmsh_mesh_solves_like_the_oracle(hfx_lib, tmp_path, dim, n, order):
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    v = meshgen.jitter_vertices(v, n, 0.15, 7)
    path = tmp_path / "mesh.msh"
    write_gmsh22(path, v, s)
    lc, le = capi.gmsh_read(path, dim)
    coords, cells = capi.mesh_high_order(dim, order, lc, le)
    P = O.Problem(dim, order, coords, cells)
    g = np.prod(np.sin(np.pi * coords[P.faces]), axis=-1)
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=g.ravel())
    P.assemble()
    x_ref = P.solve_direct()
    ctx = capi.Context(0)
    ctx.upload_mesh(dim, order, coords, cells)
    ctx.set_tau(np.ones((P.nFaces, P.re.nNodesFace)))
    ctx.set_source(capi.SRC_SINPROD, param=dim * np.pi ** 2)
    ctx.set_dirichlet(g)
    ctx.assemble()
    trace, info = ctx.solve(rtol=1e-13, precond=capi.PC_TWOLEVEL, precision=capi.PREC_MIXED)
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
