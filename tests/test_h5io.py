"""HDF5 mesh and field files without the HDF5 library (host only, no GPU).

The reader is pinned on the reference's own fixtures and the values its HDF5Io
unit test expects (tests/unittests/io/TestHDF5Io.cpp: lightTri/lightQuad order 1
and 2, fieldTest NodeField = 0..8, CellField = (i, -i)), and on the converted
regression meshes (ressources/meshes/regression/*_ord-*.h5), which must equal
the gmsh reader + high-order construction of the same .msh cell by cell. The
writer is checked by round trips (the reference's write tests do the same).
"""
import os

import numpy as np
import pytest

from helpers import reference_meshes
from hyperfox_gb300 import capi, meshgen

REF = reference_meshes() or ""
have_ref = pytest.mark.skipif(not os.path.isdir(REF), reason="reference meshes not present")

# TestHDF5Io.cpp: nodes of the 3x3 square, connectivities of the light meshes
NODES = [[0, 0], [1, 0], [1, 1], [0, 1], [0.5, 0.5], [0.5, 0], [1, 0.5], [0.5, 1], [0, 0.5]]
TRI1 = [[0, 5, 4], [5, 1, 4], [1, 6, 4], [6, 2, 4], [2, 7, 4], [7, 3, 4], [3, 8, 4], [8, 0, 4]]
QUAD1 = [[0, 5, 4, 8], [5, 1, 6, 4], [4, 6, 2, 7], [8, 4, 7, 3]]
TRI2 = [[0, 1, 3, 5, 4, 8], [3, 1, 2, 4, 6, 7]]
QUAD2 = [[0, 1, 2, 3, 5, 6, 7, 8, 4]]


@have_ref
@pytest.mark.parametrize("name,cells", [("lightTri.h5", TRI1), ("lightQuad.h5", QUAD1),
                                        ("lightTri2.h5", TRI2), ("lightQuad2.h5", QUAD2)])
def test_reference_light_meshes(name, cells):
    c, e = capi.h5_read_mesh(os.path.join(REF, name))
    assert np.array_equal(c, np.array(NODES, float))
    assert np.array_equal(e, np.array(cells))


@have_ref
def test_reference_field_file():
    path = os.path.join(REF, "fieldTest.h5")
    assert capi.h5_field_names(path) == ["CellField", "NodeField"]
    ft, v = capi.h5_read_field(path, "NodeField")
    assert ft == capi.FIELD_NODE and v.shape == (9, 1, 1)
    assert np.array_equal(v.ravel(), np.arange(9.0))
    ft, v = capi.h5_read_field(path, "CellField")
    assert ft == capi.FIELD_CELL and v.shape == (8, 2, 1)
    i = np.arange(8.0)
    assert np.array_equal(v[:, :, 0], np.stack([i, -i], 1))
    with pytest.raises(capi.HfxError, match="not found in FieldData"):
        capi.h5_read_field(path, "Solution")
    with pytest.raises(capi.HfxError, match="Nodes"):
        capi.h5_read_mesh(path)  # a field-only file has no mesh


@have_ref
@pytest.mark.parametrize("dim,h,order", [(2, "3e-1", 1), (2, "3e-1", 5), (2, "1e-1", 2), (2, "1e-1", 4),
                                         (3, "3e-1", 2), (3, "3e-1", 3), (3, "2e-1", 1)])
def test_regression_meshes_equal_gmsh_high_order(dim, h, order):
    """tools/convertGmsh2H5HO output == gmsh reader + our high-order nodes, cell by cell."""
    reg = os.path.join(REF, "regression")
    c5, e5 = capi.h5_read_mesh(os.path.join(reg, f"regression_dim-{dim}_h-{h}_ord-{order}.h5"))
    v, s = capi.gmsh_read(os.path.join(reg, f"regression_dim-{dim}_h-{h}.msh"), dim)
    c, e = capi.mesh_high_order(dim, order, v, s)
    assert c.shape == c5.shape and e.shape == e5.shape
    # same cells in the same order with the same local node order
    assert np.abs(c[e] - c5[e5]).max() < 1e-12
    if dim == 2:  # 2-D node ids coincide too (3-D edge/face nodes follow MOAB's adjacency order)
        assert np.array_equal(e, e5)


def test_write_read_roundtrip(tmp_path):
    v, s = meshgen.cube_simplices(2)
    v = meshgen.jitter_vertices(v, 2, 0.1, 5)
    coords, cells = capi.mesh_high_order(3, 2, v, s)
    rng = np.random.default_rng(0)
    fields = {
        "Solution": (capi.FIELD_CELL, rng.standard_normal((cells.shape[0], cells.shape[1], 1))),
        "Flux": (capi.FIELD_CELL, rng.standard_normal((cells.shape[0], cells.shape[1], 3))),
        "Trace": (capi.FIELD_FACE, rng.standard_normal((17, 6))),
        "Tau": (capi.FIELD_FACE, np.full((17, 6, 2), 0.5)),
    }
    path = tmp_path / "out.h5"
    capi.h5_write(path, coords, cells, fields)
    c, e = capi.h5_read_mesh(path)
    assert np.array_equal(c, coords) and np.array_equal(e, cells)
    assert capi.h5_field_names(path) == sorted(fields)
    for name, (ft, vals) in fields.items():
        rft, rv = capi.h5_read_field(path, name)
        assert rft == ft
        assert np.array_equal(rv, vals if vals.ndim == 3 else vals[:, :, None])


def test_write_many_fields_and_field_only_files(tmp_path):
    """More names than one symbol node holds (8): the group B-tree gets several children."""
    fields = {f"f{i:02d}": (i % 4 - 1, np.full((3, 2), float(i))) for i in range(37)}
    path = tmp_path / "many.h5"
    capi.h5_write(path, fields=fields)
    assert capi.h5_field_names(path) == sorted(fields)
    for name, (ft, vals) in fields.items():
        rft, rv = capi.h5_read_field(path, name)
        assert rft == ft and np.array_equal(rv[:, :, 0], vals)
    with pytest.raises(capi.HfxError):
        capi.h5_read_mesh(path)


def test_h5_errors(tmp_path):
    with pytest.raises(capi.HfxError, match="cannot open"):
        capi.h5_read_mesh(tmp_path / "missing.h5")
    p = tmp_path / "text.h5"
    p.write_text("not an hdf5 file\n")
    with pytest.raises(capi.HfxError, match="not an HDF5 file"):
        capi.h5_read_mesh(p)
    with pytest.raises(capi.HfxError, match="nothing to write"):
        capi.h5_write(tmp_path / "empty.h5")
    # a truncated file fails cleanly
    v, s = meshgen.square_simplices(2)
    full = tmp_path / "full.h5"
    capi.h5_write(full, v, s)
    data = full.read_bytes()
    cut = tmp_path / "cut.h5"
    cut.write_bytes(data[: len(data) // 2])
    with pytest.raises(capi.HfxError):
        capi.h5_read_mesh(cut)


@have_ref
def test_every_shipped_h5_file_reads():
    """All HDF5 files the reference ships (meshes and field files) open, and their
    meshes are consistent (cells index existing nodes)."""
    import glob
    files = sorted(glob.glob(os.path.join(os.path.dirname(REF), "**", "*.h5"), recursive=True))
    assert len(files) >= 60
    meshes = 0
    for f in files:
        for name in capi.h5_field_names(f):
            capi.h5_read_field(f, name)
        try:
            c, e = capi.h5_read_mesh(f)
        except capi.HfxError:
            continue  # field-only files
        meshes += 1
        assert e.min() >= 0 and e.max() < c.shape[0] and c.shape[1] in (1, 2, 3)
    assert meshes >= 50
