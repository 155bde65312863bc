"""Batched independent problems (hyperfox_gb300.batch), host side and on the oracle.

The batch uploads the problems of one order as the disjoint union of their meshes.
Checked here without a GPU: the union's shifted topology is the library's own
topology of the union mesh; on the oracle, the union's trace system decouples into
the problems' own systems (per-problem slices of the union's direct solution equal
every problem solved alone); the group tolerance bounds every problem's relative
residual; the workload builder's sizes, orders and fields.
"""
import numpy as np
import pytest

import _oracle as O
from hyperfox_gb300 import batch, capi


def small_batch(count=9, seed=2, orders=(1, 2, 3, 4, 5)):
    return batch.uneven_batch(count=count, seed=seed, min_elements=8, max_elements=120, orders=orders)


def oracle_problem(p):
    P = O.Problem(p.dim, p.order, p.coords, p.cells)
    P.set_fields(p.tau.ravel(), kappa=p.kappa.ravel(), src_mode=2, dirichlet=p.dirichlet.ravel())
    return P


def test_union_topology_is_the_library_topology():
    probs = small_batch(count=12, seed=4)
    for q in sorted({p.order for p in probs}):
        same = [p for p in probs if p.order == q]
        coords, cells, topo, (n0, c0, f0) = batch.union(same)
        ref = capi.mesh_topology(2, q, cells)
        for a, b in zip(topo, ref):
            assert np.array_equal(a, b)
        assert n0[-1] == coords.shape[0] and c0[-1] == cells.shape[0] and f0[-1] == topo[2].shape[0]
        # every boundary face keeps face2cell[., 1] = -1; interior faces join cells of one problem
        f2c = topo[1]
        prob_of_cell = np.repeat(np.arange(len(same)), np.diff(c0))
        inner = f2c[:, 1] >= 0
        assert np.array_equal(prob_of_cell[f2c[inner, 0]], prob_of_cell[f2c[inner, 1]])
        assert np.array_equal(np.flatnonzero(~inner), topo[3])


@pytest.mark.parametrize("order", [1, 3, 5])
def test_union_decouples_on_the_oracle(order):
    """The oracle's direct solve of the union system, sliced per problem, equals every
    problem's own direct solve (trace, Solution, Flux)."""
    probs = [p for p in batch.uneven_batch(count=20, seed=order, min_elements=8, max_elements=60,
                                           orders=(order,))][:4]
    coords, cells, topo, (_, c0, f0) = batch.union(probs)
    U = O.Problem(2, order, coords, cells)
    tau = np.concatenate([p.tau.ravel() for p in probs])
    kap = np.concatenate([p.kappa.ravel() for p in probs])
    g = np.concatenate([p.dirichlet.ravel() for p in probs])
    U.set_fields(tau, kappa=kap, src_mode=2, dirichlet=g)
    U.assemble()
    xu = U.solve_direct()
    su, qu = U.recover(xu)
    nf = U.re.nNodesFace
    for k, p in enumerate(probs):
        P = oracle_problem(p)
        P.assemble()
        x = P.solve_direct()
        s, q = P.recover(x)
        xs = xu[f0[k] * nf:f0[k + 1] * nf]
        assert np.linalg.norm(xs - x) <= 1e-10 * np.linalg.norm(x)
        assert np.abs(su[c0[k]:c0[k + 1]] - s).max() <= 1e-10 * np.abs(s).max()
        assert np.abs(qu[c0[k]:c0[k + 1]] - q).max() <= 1e-10 * np.abs(q).max()


def test_group_tolerance_bounds_every_problem():
    rng = np.random.default_rng(0)
    nf = 3
    faces = np.array([0, 5, 6, 40, 41, 200])
    rhs = rng.normal(size=faces[-1] * nf) * np.repeat(rng.uniform(0.01, 10, size=5), np.diff(faces) * nf)
    rtol = 1e-8
    tol = batch.group_tolerance(rtol, rhs, faces, nf)
    bk = np.array([np.linalg.norm(rhs[a * nf:b * nf]) for a, b in zip(faces[:-1], faces[1:])])
    assert tol == pytest.approx(rtol * bk.min() / np.linalg.norm(rhs), rel=1e-12)
    # the worst case: the whole admissible residual on one problem's rows
    for k in range(5):
        r = np.zeros_like(rhs)
        r[faces[k] * nf] = tol * np.linalg.norm(rhs)
        assert np.linalg.norm(r[faces[k] * nf:faces[k + 1] * nf]) <= rtol * bk[k] * (1 + 1e-12)
    # a problem with no data does not tighten the tolerance; no data at all keeps rtol
    rhs[faces[1] * nf:faces[2] * nf] = 0.0
    bk[1] = 0.0
    assert batch.group_tolerance(rtol, rhs, faces, nf) == pytest.approx(
        rtol * bk[bk > 0].min() / np.linalg.norm(rhs), rel=1e-12)
    assert batch.group_tolerance(rtol, np.zeros_like(rhs), faces, nf) == rtol


def test_lognormal_field_lattice_is_the_feature_sum():
    rng = np.random.default_rng(7)
    w = rng.normal(0.0, 1.0 / 0.1, size=(2, 256))
    ph = rng.uniform(0.0, 2 * np.pi, size=256)
    t = np.linspace(0, 1, 129)
    P = np.stack(np.meshgrid(t, t, indexing="ij"), -1)
    direct = np.exp(np.sqrt(2 / 256) * np.cos(P.reshape(-1, 2) @ w + ph).sum(1)).reshape(129, 129)
    lat = batch.lognormal_field(P, 1.0, 0.1, 7)
    assert np.abs(lat / direct - 1).max() < 1e-12
    assert 0.7 < np.log(lat).std() < 1.3


def test_uneven_batch_workload():
    a = batch.uneven_batch(count=64, seed=11, min_elements=200, max_elements=20000)
    b = batch.uneven_batch(count=64, seed=11, min_elements=200, max_elements=20000)
    for p, q in zip(a, b):
        assert p.order == q.order and np.array_equal(p.cells, q.cells) and np.array_equal(p.kappa, q.kappa)
    counts = np.array([p.nCells for p in a])
    # 2 n^2 elements with n = round(sqrt(c / 2)), c in [200, 20000]
    assert counts.min() >= 2 * 10 ** 2 and counts.max() <= 2 * 100 ** 2
    assert set(p.order for p in a) == {1, 2, 3, 4, 5}
    nodal = batch.uneven_batch(count=64, seed=11, min_elements=200, max_elements=20000, kappa_at="nodes")
    for p, q in zip(a[:4], nodal):
        # centroid sampling: one value per cell; node sampling varies inside cells
        assert np.array_equal(p.kappa, np.broadcast_to(p.kappa[:, :1], p.kappa.shape))
        assert q.kappa.shape == p.kappa.shape and np.ptp(q.kappa, axis=1).max() > 0
    for p in a[:8]:
        assert p.kappa.shape == (p.nCells, p.cells.shape[1], 1) and (p.kappa > 0).all()
        assert np.allclose(p.dirichlet, np.prod(np.sin(np.pi * p.coords[p.faces]), axis=-1))
        # the jitter moved interior vertices, and only those
        n = int(round(np.sqrt(p.nCells / 2)))
        v = p.coords[p.cells[:, :3]].reshape(-1, 2)
        on_bnd = (np.abs(v) < 1e-12) | (np.abs(v - 1) < 1e-12)
        assert np.any(np.abs(v * n - np.rint(v * n)) > 1e-6)
        assert on_bnd.any()


def test_batch_rejects_bad_input():
    """Inconsistent inputs are refused before any device work (no GPU needed)."""
    with pytest.raises(ValueError):
        batch.Batch([])
    a, b = small_batch(count=40, seed=6, orders=(2,))[:2]
    b.tau = np.ones((b.nFaces, b.faces.shape[1], 2))  # double valued next to single valued
    with pytest.raises(ValueError, match="tau"):
        batch.Batch([a, b])
    a, b = small_batch(count=40, seed=6, orders=(2,))[:2]
    b.kappa = None
    with pytest.raises(ValueError, match="kappa"):
        batch.Batch([a, b])
    a, b = small_batch(count=40, seed=6, orders=(2,))[:2]
    b.kappa = np.ones((b.nCells, b.cells.shape[1], 3))
    with pytest.raises(ValueError, match="kappa"):
        batch.Batch([a, b])
    a, b = small_batch(count=40, seed=6, orders=(2,))[:2]
    with pytest.raises(ValueError, match="source"):
        batch.Batch([a, b], src_mode=capi.SRC_VALUES)
    c = small_batch(count=40, seed=6, orders=(3,))[0]
    c.dim = 3
    with pytest.raises(ValueError, match="dimension"):
        batch.Batch([a, c])


def test_shard_partitions_and_balances():
    plan = batch.uneven_plan()
    costs = [batch.problem_cost(n, q) for n, q, _ in plan]
    for world in (1, 2, 4, 8):
        parts = batch.shard(costs, world)
        flat = sorted(i for part in parts for i in part)
        assert flat == list(range(len(plan)))
        loads = [sum(costs[i] for i in part) for part in parts]
        # greedy LPT: no rank exceeds the mean by more than the largest single problem
        assert max(loads) - sum(loads) / world <= max(costs)
        assert batch.shard(costs, world) == parts


def test_select_builds_the_same_problems():
    full = batch.uneven_batch(count=12, seed=4, min_elements=8, max_elements=120)
    some = batch.uneven_batch(count=12, seed=4, min_elements=8, max_elements=120, select=[3, 7, 11])
    for k, p in zip([3, 7, 11], some):
        assert p.order == full[k].order and np.array_equal(p.cells, full[k].cells)
        assert np.array_equal(p.kappa, full[k].kappa) and np.array_equal(p.coords, full[k].coords)


def _shard_worker(rank, world, port, q):
    import os
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch
    import torch.distributed as dist
    from hyperfox_gb300 import batch as hb
    dist.init_process_group("gloo")
    plan = hb.uneven_plan(count=64, seed=3)
    mine = hb.shard([hb.problem_cost(n, p) for n, p, _ in plan], world)[rank]
    probs = hb.uneven_batch(count=64, seed=3, select=mine[:2])  # each rank builds only its own problems
    lens = [None] * world
    dist.all_gather_object(lens, (rank, mine, [p.nCells for p in probs]))
    q.put(lens)
    dist.destroy_process_group()


def test_two_gloo_ranks_split_the_batch_without_exchange():
    """World size 2 on CPU: every rank computes the split alone; gathered afterwards, the
    ranks' problem sets are disjoint and cover the batch."""
    import multiprocessing as mp
    import os
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    ps = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    outs = [q.get(timeout=180) for _ in ps]
    for p in ps:
        p.join(timeout=60)
    assert outs[0] == outs[1]
    (r0, s0, e0), (r1, s1, e1) = sorted(outs[0])
    assert (r0, r1) == (0, 1) and not set(s0) & set(s1) and sorted(s0 + s1) == list(range(64))
    plan = batch.uneven_plan(count=64, seed=3)
    assert e0 == [2 * plan[i][0] ** 2 for i in s0[:2]] and e1 == [2 * plan[i][0] ** 2 for i in s1[:2]]
