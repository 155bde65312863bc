"""Synthetic simplex meshes for the HDG workloads (host side, numpy).

HyperFox loads its meshes from HDF5 files (``src/io/HDF5Io.cpp:111-152``) whose
high-order nodes come from ``tools/convertGmsh2H5HO.cpp``. Neither the files
nor an HDF5 reader are available, so the workloads use seeded synthetic meshes
with the same element types:

* unit square, ``n x n`` squares each cut into two right triangles along a
  fixed diagonal;
* unit cube, ``n^3`` cubes each cut into six tetrahedra (Kuhn/Freudenthal
  split along the main diagonal, conforming between cubes);
* optional seeded vertex jitter (interior vertices only).

High-order nodes are the reference element's nodes mapped by each cell's
affine map, merged across cells by position, so shared nodes carry one global
id. Every cell has positive orientation (``det J > 0``).
"""
import itertools

import numpy as np


def _square_vertices(n):
    h = 1.0 / n
    ij = np.stack(np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij"), -1).reshape(-1, 2)
    return ij * h, lambda i, j: i * (n + 1) + j


def square_simplices(n):
    """Vertices and linear triangles of the unit square split into 2*n*n triangles."""
    verts, vid = _square_vertices(n)
    # square (i, j) in row-major order, its two triangles (v00, v10, v01) and (v11, v01, v10)
    i, j = (a.ravel() for a in np.meshgrid(np.arange(n), np.arange(n), indexing="ij"))
    v00, v10, v01, v11 = vid(i, j), vid(i + 1, j), vid(i, j + 1), vid(i + 1, j + 1)
    tris = np.stack([np.stack([v00, v10, v01], -1), np.stack([v11, v01, v10], -1)], 1).reshape(-1, 3)
    return verts, tris.astype(np.int64)


def cube_simplices(n):
    """Vertices and linear tets of the unit cube split into 6*n^3 Kuhn tetrahedra."""
    h = 1.0 / n
    ijk = np.stack(np.meshgrid(np.arange(n + 1), np.arange(n + 1), np.arange(n + 1), indexing="ij"),
                   -1).reshape(-1, 3)
    verts = ijk * h

    def vid(i, j, k):
        return (i * (n + 1) + j) * (n + 1) + k

    perms = list(itertools.permutations(range(3)))
    base = np.stack(np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij"), -1).reshape(-1, 3)
    tets = []
    for perm in perms:
        steps = [np.zeros(3, dtype=np.int64)]
        cur = np.zeros(3, dtype=np.int64)
        for ax in perm:
            cur = cur.copy()
            cur[ax] += 1
            steps.append(cur)
        ids = [vid(base[:, 0] + s[0], base[:, 1] + s[1], base[:, 2] + s[2]) for s in steps]
        # orientation: det of [e_perm0, e_perm0+e_perm1, 1] = sign(perm)
        sign = np.linalg.det(np.eye(3)[list(perm)])
        if sign < 0:
            ids[1], ids[2] = ids[2], ids[1]
        tets.append(np.stack(ids, -1))
    # order cells cube by cube
    tets = np.stack(tets, 1).reshape(-1, 4)
    return verts, tets.astype(np.int64)


def jitter_vertices(verts, n, amount, seed):
    """Move interior vertices by U(-amount*h, amount*h) per coordinate (seeded)."""
    h = 1.0 / n
    rng = np.random.default_rng(seed)
    out = verts.copy()
    interior = np.all((verts > 1e-12) & (verts < 1 - 1e-12), axis=1)
    out[interior] += rng.uniform(-amount * h, amount * h, size=(interior.sum(), verts.shape[1]))
    return out


def high_order(verts, simplices, ref_nodes, quantum=1e-10):
    """Map reference nodes into every cell and merge coincident nodes.

    ``ref_nodes`` is the reference element's node table (N x d, reference
    simplex with vertices (-1,..), e_k), whose first d+1 entries are the
    vertices. Returns (coords [nNodes x d], cells [nCells x N] int32).
    """
    dim = verts.shape[1]
    ref = np.asarray(ref_nodes, dtype=np.float64).reshape(-1, dim)
    v0 = verts[simplices[:, 0]]                                   # E x d
    edges = np.stack([verts[simplices[:, k + 1]] - v0 for k in range(dim)], 1)  # E x d(k) x d
    lam = (ref + 1.0) * 0.5                                       # N x d(k)
    pts = v0[:, None, :] + np.einsum("nk,ekd->end", lam, edges)  # E x N x d
    # vertices reproduce exactly
    pts[:, :dim + 1, :] = verts[simplices[:, :dim + 1]]
    flat = pts.reshape(-1, dim)
    key = np.round(flat / quantum).astype(np.int64)
    _, first, inv = np.unique(key, axis=0, return_index=True, return_inverse=True)
    # number merged nodes in order of first appearance (cell by cell)
    order = np.argsort(first, kind="stable")
    rank = np.empty_like(order)
    rank[order] = np.arange(order.size)
    gid = rank[inv.reshape(-1)]
    coords = flat[first[order]]
    cells = gid.reshape(simplices.shape[0], -1).astype(np.int32)
    return np.ascontiguousarray(coords), np.ascontiguousarray(cells)
