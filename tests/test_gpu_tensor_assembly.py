"""Element contractions on the tensor cores (tcgen05) vs the FP64 oracle (needs a GPU).

The mixed assembly contracts HyperFox's element operators on the tensor cores
(TF32 hi/lo split, FP32 accumulation): the volume blocks C_d (Squ), K_d (volume
part of Suq), M (Sqq per dimension) and the face blocks T (tau face mass), E_d
(n phi phi) and H_d (kappa n phi phi), and the source load f_u
(HDGBase.cpp:67-158, HDGDiffusion.cpp:74-145, Mass.cpp:5-38, Source.cpp:24-48).
Each block is compared with the same block of the oracle's FP64 local matrix
(local_system, the reference's index layout [U | Q node-major | Lambda
face-major]) on meshes with jittered vertices, one bent (curved) cell and a
nodal diffusion tensor that varies inside the cells. Stated bound: 2e-5 of the
largest entry of each block type. The solve that starts from these blocks (FP32
condensation inside FP64 refinement of the full HDG system) must still meet the
FP64 direct solution to 1e-8.
"""
import numpy as np
import pytest

import _oracle as O
from helpers import fields, mesh

pytestmark = pytest.mark.gpu

TC_BOUND = 2e-5
CASES = [(2, 3, 1), (2, 3, 2), (2, 2, 3), (2, 2, 5), (3, 2, 1), (3, 2, 2), (3, 1, 3)]


def build(dim, n, order, seed=2):
    from hyperfox_gb300 import capi
    rng = np.random.default_rng(seed)
    re, coords, cells = mesh(dim, n, order, jitter=0.15, seed=seed)
    coords = coords.copy()
    coords[cells[0, -1]] += 0.01  # bend one cell
    P = O.Problem(dim, order, coords, cells)
    tau, kap, g = fields(dim, order, coords, cells, P.faces, P.nFaces, rng, tau2=True, kappa="tensor")
    P.set_fields(tau.ravel(), kappa=kap.ravel(), src_mode=2, dirichlet=g.ravel())
    ctx = capi.Context(0)
    ctx.upload_mesh(dim, order, coords, cells)
    ctx.set_tau(tau)
    ctx.set_kappa(kap, layout=1)
    ctx.set_source(capi.SRC_SINPROD, param=dim * np.pi ** 2)
    ctx.set_dirichlet(g)
    return P, ctx


def oracle_blocks(P, e):
    """The tensor-core block set of element e, read off the oracle's FP64 local matrix."""
    d, N, F, NF = P.dim, P.lenU, P.re.nFaces, P.re.nNodesFace
    A, r, _ = P.local_matrix(e)
    q0, l0 = N, N + d * N
    fn = P.re.faceNodes
    C = np.array([[[A[q0 + i * d + k, j] for j in range(N)] for i in range(N)] for k in range(d)])
    M = np.array([[A[q0 + i * d, q0 + j * d] for j in range(N)] for i in range(N)])
    T = np.array([[[-A[l0 + f * NF + a, l0 + f * NF + b] for b in range(NF)] for a in range(NF)] for f in range(F)])
    E = np.array([[[[-A[q0 + fn[f][a] * d + k, l0 + f * NF + b] for b in range(NF)] for a in range(NF)]
                   for k in range(d)] for f in range(F)])
    H = np.array([[[[-A[l0 + f * NF + a, q0 + fn[f][b] * d + k] for b in range(NF)] for a in range(NF)]
                   for k in range(d)] for f in range(F)])
    Suq = np.array([[[A[i, q0 + j * d + k] for j in range(N)] for i in range(N)] for k in range(d)])
    return dict(C=C, M=M, T=T, E=E, H=H, Suq=Suq, fu=r[:N])


def split_tc(row, dim, N, F, NF):
    d = dim
    vol = row[:(2 * d * N + N) * N].reshape(2 * d * N + N, N)
    C = vol[:d * N].reshape(d, N, N)
    K = vol[d * N:2 * d * N].reshape(d, N, N)
    M = vol[2 * d * N:]
    fo = (2 * d * N + N) * N
    face = row[fo:fo + F * NF * (1 + 2 * d) * NF].reshape(F * NF * (1 + 2 * d), NF)
    T = face[:F * NF].reshape(F, NF, NF)
    E = face[F * NF:F * NF + F * d * NF].reshape(F, d, NF, NF)
    H = face[F * NF + F * d * NF:].reshape(F, d, NF, NF)
    fu = row[fo + F * NF * (1 + 2 * d) * NF:fo + F * NF * (1 + 2 * d) * NF + N]
    return dict(C=C, K=K, M=M, T=T, E=E, H=H, fu=fu)


@pytest.mark.parametrize("dim,n,order", CASES)
def test_tensor_core_blocks_match_oracle(hfx_lib, dim, n, order):
    from hyperfox_gb300 import capi
    P, ctx = build(dim, n, order)
    ctx.assemble(precision=capi.PREC_MIXED)
    assert ctx.mixed_assembly_info() == 1
    cells = np.arange(P.nCells)
    tc = ctx.tc_blocks(cells)
    N, F, NF = P.lenU, P.re.nFaces, P.re.nNodesFace
    fn = P.re.faceNodes
    errs = {k: 0.0 for k in ("C", "M", "T", "E", "H", "Suq", "fu")}
    scale = dict(errs)
    for e in cells:
        o = oracle_blocks(P, e)
        g = split_tc(tc[e].astype(np.float64), dim, N, F, NF)
        # Suq = K_d minus the face terms H_d placed at the face nodes (HDGDiffusion.cpp:110-145)
        suq = g["K"].copy()
        for f in range(F):
            for k in range(dim):
                suq[k][np.ix_(fn[f], fn[f])] -= g["H"][f, k]
        g["Suq"] = suq
        for k in errs:
            errs[k] = max(errs[k], np.abs(g[k] - o[k]).max())
            scale[k] = max(scale[k], np.abs(o[k]).max())
    rel = {k: errs[k] / scale[k] for k in errs}
    assert all(v < TC_BOUND for v in rel.values()), rel


@pytest.mark.parametrize("dim,n,order", [(2, 3, 2), (2, 2, 5), (3, 2, 2), (3, 1, 3)])
def test_tensor_core_mixed_solve_matches_direct(hfx_lib, dim, n, order):
    from hyperfox_gb300 import capi
    P, ctx = build(dim, n, order, seed=3)
    P.assemble()
    x_ref = P.solve_direct()
    osol, oflux = P.recover(x_ref)
    ctx.assemble(precision=capi.PREC_MIXED)
    assert ctx.mixed_assembly_info() == 1
    trace, info = ctx.solve(rtol=1e-12, inner_rtol=1e-5, restart=40)
    assert info.status == 0 and info.rel_residual < 1e-12
    sol, flux = ctx.recover()
    assert np.linalg.norm(trace - x_ref) / np.linalg.norm(x_ref) < 1e-8
    assert np.linalg.norm(sol - osol) / np.linalg.norm(osol) < 1e-8
    assert np.linalg.norm(flux - oflux) / np.linalg.norm(oflux) < 1e-8
    # the CUDA-core quadrature of the same mixed path gives the same refined solution
    ctx.L.hfx_set_assembly_path(ctx.h, 1)
    ctx.assemble(precision=capi.PREC_MIXED)
    assert ctx.mixed_assembly_info() == 0
    trace2, _ = ctx.solve(rtol=1e-12, inner_rtol=1e-5, restart=40)
    assert np.linalg.norm(trace2 - x_ref) / np.linalg.norm(x_ref) < 1e-8
