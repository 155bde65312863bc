"""CG element operators through the C ABI vs the oracle (needs a GPU).

Mass, Diffusion and Convection (Mass.cpp:5-38, Diffusion.cpp:5-43, Convection.cpp:21-46),
one DOF per node, with a nodal diffusion field (none, scalar, tensor) and a nodal velocity,
on jittered meshes with one bent cell: the FP64 kernel within 1e-12 of the oracle's
restatement of the reference loops, the tensor-core contraction (TF32 hi/lo split, FP32
accumulation) within 2e-5 of each operator's largest entry.
"""
import numpy as np
import pytest

import _oracle as O
from helpers import fields, mesh

pytestmark = pytest.mark.gpu

CASES = [(2, 3, 1), (2, 3, 2), (2, 2, 4), (2, 2, 5), (3, 2, 1), (3, 2, 2), (3, 1, 3)]


def build(dim, n, order, kappa, seed=4):
    from hyperfox_gb300 import capi
    rng = np.random.default_rng(seed)
    re, coords, cells = mesh(dim, n, order, jitter=0.15, seed=seed)
    coords = coords.copy()
    coords[cells[0, -1]] += 0.01
    P = O.Problem(dim, order, coords, cells)
    tau, kap, g = fields(dim, order, coords, cells, P.faces, P.nFaces, rng, kappa=kappa)
    P.set_fields(tau.ravel(), kappa=None if kap is None else kap.ravel(), src_mode=0, dirichlet=g.ravel())
    ctx = capi.Context(0)
    ctx.upload_mesh(dim, order, coords, cells)
    if kap is not None:
        ctx.set_kappa(kap, layout=1)
    vel = rng.normal(size=(cells.shape[0], cells.shape[1], dim))
    return P, ctx, vel


def relerr_per_op(a, b):
    return [np.abs(a[:, k] - b[:, k]).max() / np.abs(b[:, k]).max() for k in range(3)]


@pytest.mark.parametrize("kappa", ["none", "scalar", "tensor"])
@pytest.mark.parametrize("dim,n,order", CASES)
def test_cg_operators_match_oracle(hfx_lib, dim, n, order, kappa):
    from hyperfox_gb300 import capi
    P, ctx, vel = build(dim, n, order, kappa)
    ref = P.cg_operators(7, vel)
    f64 = ctx.cg_operators(7, capi.PREC_FP64, vel)
    assert max(relerr_per_op(f64, ref)) < 1e-12, relerr_per_op(f64, ref)
    tc = ctx.cg_operators(7, capi.PREC_MIXED, vel)
    assert max(relerr_per_op(tc, ref)) < 2e-5, relerr_per_op(tc, ref)
    # a subset leaves the other operators alone and gives the same values
    only = ctx.cg_operators(capi.OP_DIFFUSION, capi.PREC_FP64)
    assert np.array_equal(only[:, 1], f64[:, 1])
