"""The C ABI library on the host: it loads, exports every symbol the header
declares, and its host-side tables and topology equal the oracle's (no GPU
compute calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

import _oracle as O
from hyperfox_gb300 import capi, meshgen

HEADER = os.path.join(O.ROOT, "include", "hfx_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(hfx_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(hfx_lib):
    names = declared_symbols()
    assert len(names) >= 30
    for n in names:
        assert hasattr(hfx_lib, n), n
    assert set(names) <= set(capi.EXPORTED)


def test_version_and_bad_arguments(hfx_lib):
    assert hfx_lib.hfx_version() >= 100
    info = capi.RefElInfo()
    assert hfx_lib.hfx_refel_query(3, 9, ctypes.byref(info)) == capi.HFX_ERR_ARG
    assert hfx_lib.hfx_refel_query(1, 2, ctypes.byref(info)) == capi.HFX_ERR_ARG
    bad = np.array([[0, 1, 1]], np.int32)  # degenerate cell: a face shared thrice is impossible
    nf, nb = ctypes.c_int(), ctypes.c_int()
    cells = np.array([[0, 1, 2], [0, 1, 3], [0, 1, 4]], np.int32)
    rc = hfx_lib.hfx_mesh_compute_topology(2, 1, 3, cells.ctypes.data, ctypes.byref(nf), ctypes.byref(nb),
                                           None, None, None, None)
    assert rc == capi.HFX_ERR_ARG  # edge (0,1) shared by three triangles
    assert bad.size == 3


@pytest.mark.parametrize("dim,p", [(2, 1), (2, 2), (2, 3), (2, 4), (2, 5), (3, 1), (3, 2), (3, 3)])
def test_refel_tables_match_oracle(hfx_lib, dim, p):
    t = capi.refel(dim, p)
    o = O.RefEl(dim, p)
    assert np.abs(t["nodes"] - o.nodes).max() < 1e-14
    assert np.array_equal(t["faceNodes"], o.faceNodes)
    assert np.array_equal(t["ipX"], o.ipX) and np.array_equal(t["ipW"], o.ipW)
    assert np.abs(t["phi"] - o.phi).max() < 1e-12
    assert np.abs(t["dphi"] - o.dphi).max() < 1e-12
    fo = O.RefEl(dim - 1, p)
    assert np.abs(t["fPhi"] - fo.phi).max() < 1e-12
    assert np.abs(t["fIpW"] - fo.ipW).max() < 1e-15


@pytest.mark.parametrize("dim,n,p,jit,shuffle", [(2, 5, 2, 0.0, False), (2, 4, 3, 0.2, True),
                                                  (3, 2, 2, 0.1, False), (3, 3, 1, 0.0, True)])
def test_topology_matches_oracle(hfx_lib, dim, n, p, jit, shuffle):
    re = capi.refel(dim, p)
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    if jit:
        v = meshgen.jitter_vertices(v, n, jit, 3)
    if shuffle:
        s = s[np.random.default_rng(0).permutation(len(s))]
    coords, cells = meshgen.high_order(v, s, re["nodes"])
    c2f, f2c, faces, bnd = capi.mesh_topology(dim, p, cells)
    P = O.Problem(dim, p, coords, cells)
    assert np.array_equal(c2f, P.cell2face)
    assert np.array_equal(f2c, P.face2cell)
    assert np.array_equal(faces, P.faces)
    assert np.array_equal(bnd, P.boundary)


def test_cfg2_topology_counts(hfx_lib):
    """3D 40^3 x 6 tets, p=3: 777,600 faces, 19,200 on the boundary."""
    v, s = meshgen.cube_simplices(40)
    c2f, f2c, faces, bnd = capi.mesh_topology(3, 1, s.astype(np.int32))
    assert (f2c.shape[0], bnd.size) == (777600, 19200)
