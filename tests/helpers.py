"""Shared problem builders for the parity tests (seeded, small)."""
import os

import numpy as np

from hyperfox_gb300 import capi, meshgen


def mesh(dim, n, order, jitter=0.0, seed=0):
    re = capi.refel(dim, order)
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    if jitter:
        v = meshgen.jitter_vertices(v, n, jitter, seed)
    coords, cells = meshgen.high_order(v, s, re["nodes"])
    return re, coords, cells


def manufactured(coords, faces):
    """u = prod sin(pi x) at the face nodes (Dirichlet values, face order)."""
    return np.prod(np.sin(np.pi * coords[faces]), axis=-1)


def fields(dim, order, coords, cells, faces, nfaces, rng, tau2=False, kappa="none"):
    """Random but valid fields: tau > 0 (optionally double valued), kappa SPD per cell node."""
    Nf = faces.shape[1]
    N = cells.shape[1]
    if tau2:
        tau = rng.uniform(0.5, 2.0, size=(nfaces, Nf, 2))
    else:
        tau = rng.uniform(0.5, 2.0, size=(nfaces, Nf, 1))
    if kappa == "scalar":
        kap = rng.uniform(0.5, 3.0, size=(cells.shape[0], N, 1))
    elif kappa == "cell":  # constant inside each cell: symmetric trace system
        kap = np.repeat(rng.uniform(0.5, 3.0, size=(cells.shape[0], 1, 1)), N, axis=1)
    elif kappa == "tensor":
        A = rng.normal(size=(cells.shape[0], N, dim, dim)) * 0.3
        kap = np.einsum("enij,enkj->enik", A, A) + np.eye(dim)
        kap = np.ascontiguousarray(np.swapaxes(kap, -1, -2)).reshape(cells.shape[0], N, dim * dim)  # column-major
    else:
        kap = None
    g = manufactured(coords, faces)
    return tau, kap, g


def reference_meshes():
    """The HyperFox source tree's mesh fixtures, or None when no tree is known here.

    The tree is HYPERFOX_REFERENCE, else the one oracle/build_ref.sh was built from
    (recorded in oracle/_ref/REFERENCE_ROOT). Tests that read its fixtures skip
    without it."""
    root = os.environ.get("HYPERFOX_REFERENCE")
    if not root:
        marker = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle", "_ref",
                              "REFERENCE_ROOT")
        if os.path.exists(marker):
            root = open(marker).read().strip()
    path = os.path.join(root, "ressources", "meshes") if root else None
    return path if path and os.path.isdir(path) else None
