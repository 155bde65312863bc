"""Generates tests/golden/subcube12_p3_trace.npz: the oracle's direct FP64 solve of
the 12^3 x 6 tet sub-cube of the 3D p=3 diffusion-source workload (unit cube, Kuhn
split, tau = 1, kappa = 1, f = 3 pi^2 prod sin(pi x), Dirichlet u = prod sin(pi x)
at the face nodes): 10,368 elements, 216,000 trace DOFs.

The sparse LU of that system takes minutes, too long to repeat inside a GPU test;
the trace is stored once (with the mesh description, the solve's relative residual
and a checksum of the right-hand side, so that a changed oracle or mesh is noticed).
Run from the repository root: python tests/golden/make_subcube_trace.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

N, ORDER = 12, 3


def problem():
    import _oracle as O
    from hyperfox_gb300 import capi, meshgen
    v, s = meshgen.cube_simplices(N)
    coords, cells = meshgen.high_order(v, s, capi.refel(3, ORDER)["nodes"])
    P = O.Problem(3, ORDER, coords, cells)
    g = np.prod(np.sin(np.pi * coords[P.faces]), axis=-1)
    P.set_fields(np.ones(P.ndofs), src_mode=2, dirichlet=g.ravel())
    return P, coords, cells, g


def main():
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    P, coords, cells, g = problem()
    P.assemble(nthreads=os.cpu_count() or 1)
    rowptr, col, val, rhs = P.csr()
    A = sp.csr_matrix((val, col, rowptr), shape=(P.ndofs, P.ndofs)).tocsc()
    x = spla.splu(A, permc_spec="MMD_AT_PLUS_A").solve(rhs)
    res = np.linalg.norm(A @ x - rhs) / np.linalg.norm(rhs)
    np.savez_compressed(os.path.join(HERE, "subcube12_p3_trace.npz"), trace=x, n=N, order=ORDER,
                        rel_residual=res, rhs_sum=rhs.sum(), rhs_norm=np.linalg.norm(rhs), nnz=len(col))
    print("trace of %d DOFs, relative residual %.2e" % (P.ndofs, res))


if __name__ == "__main__":
    main()
