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


@pytest.mark.parametrize("dim,n,order", [(2, 5, 2), (3, 2, 3)])
def test_hdf5_mesh_and_fields_through_the_cuda_path(hfx_lib, tmp_path, dim, n, order):
    """Mesh written to and read back from HDF5 (/Mesh), solved on the device, and the
    Solution / Flux / Trace fields stored in /FieldData and read back bit for bit."""
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    v = meshgen.jitter_vertices(v, n, 0.15, 11)
    hc, he = capi.mesh_high_order(dim, order, v, s)
    path = tmp_path / "mesh.h5"
    capi.h5_write(path, hc, he)
    coords, cells = capi.h5_read_mesh(path)
    assert np.array_equal(coords, hc) and np.array_equal(cells, he)
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
    trace, info = ctx.solve(rtol=1e-13)
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
    sol, flux = ctx.recover()
    out = tmp_path / "result.h5"
    N, Nf = cells.shape[1], P.re.nNodesFace
    fields = {"Solution": (capi.FIELD_CELL, sol.reshape(-1, N, 1)),
              "Flux": (capi.FIELD_CELL, flux.reshape(-1, N, dim)),
              "Trace": (capi.FIELD_FACE, trace.reshape(-1, Nf, 1))}
    capi.h5_write(out, coords, cells, fields)
    for name, (ft, vals) in fields.items():
        rft, rv = capi.h5_read_field(out, name)
        assert rft == ft and np.array_equal(rv, vals)
