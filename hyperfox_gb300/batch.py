"""Batches of independent HDG problems: one set of device launches per order.

HyperFox solves one problem per Mesh, and a Mesh carries one ReferenceElement
(src/mesh/Mesh.cpp:24-29): the order is uniform inside a problem, and a batch of
mixed order is a set of such problems. Here the problems of each order are uploaded
to one context as ONE mesh, the disjoint union of their meshes: the nodes, cells and
faces of problem k follow those of problems 0..k-1, and each problem keeps its own
face numbering (hfx_mesh_compute_topology, the MOAB creation-order rule) shifted by
its face offset. No face or vertex is shared between problems, so the union's trace
system and its block-Jacobi and two-level preconditioners are block diagonal: every
element computes exactly what it computes in its own problem, and one assembly
launch, one Krylov solve and one recovery launch serve the whole group. Trace,
Solution and Flux of a problem are contiguous slices of its group's arrays, in the
problem's own numbering.

The Krylov solve stops on the group's relative residual |r| <= tol |b| (b the group's
trace right-hand side, r the true residual). With tol = rtol min_k |b_k| / |b| over
the problems whose part b_k of b is non-zero, every problem's own relative residual is
at most rtol: |r_k| <= |r| <= rtol min_j |b_j| <= rtol |b_k|. A problem with b_k = 0
keeps an exactly zero trace, since every Krylov vector stays zero on its rows.

The groups are independent: ``run(concurrent=True)`` drives each group from its own
host thread on its own context (and stream), so their launches, reductions and host
checks overlap on the GPU.
"""
import ctypes
import threading

import numpy as np

from . import capi, meshgen


class Problem:
    """One independent HDG diffusion-source problem of one order.

    Fields are given in the problem's own numbering: tau [nFaces][Nf][1 or 2],
    kappa [nCells][N][kc] (cell-node layout, kc 1 or dim*dim; None = identity),
    dirichlet [nFaces][Nf] in face order (``faces`` gives the face nodes), source
    values [nCells][nIP] when the batch's source mode is values."""

    def __init__(self, dim, order, coords, cells, tau=None, kappa=None, dirichlet=None, source=None):
        self.dim, self.order = dim, order
        self.coords = np.ascontiguousarray(coords, np.float64)
        self.cells = np.ascontiguousarray(cells, np.int32)
        self.topology = capi.mesh_topology(dim, order, self.cells)
        self.faces = self.topology[2]
        self.nCells, self.nFaces = self.cells.shape[0], self.faces.shape[0]
        Nf = self.faces.shape[1]
        self.tau = np.ones((self.nFaces, Nf, 1)) if tau is None else np.asarray(tau, np.float64)
        self.kappa = None if kappa is None else np.asarray(kappa, np.float64)
        self.dirichlet = np.zeros((self.nFaces, Nf)) if dirichlet is None else np.asarray(dirichlet, np.float64)
        self.source = None if source is None else np.asarray(source, np.float64)


def union(problems):
    """Disjoint union of same-order problems: coords, cells, the shifted topology
    (cell2face, face2cell with -1 kept for boundary faces, faces, boundary) and the
    node, cell and face offsets [len(problems) + 1]."""
    nodes = np.cumsum([0] + [p.coords.shape[0] for p in problems])
    cellsOff = np.cumsum([0] + [p.nCells for p in problems])
    facesOff = np.cumsum([0] + [p.nFaces for p in problems])
    if nodes[-1] >= 2 ** 31 or facesOff[-1] >= 2 ** 31 or cellsOff[-1] >= 2 ** 31:
        raise ValueError("batch union: more than 2^31 - 1 nodes, cells or faces in one order group")
    coords = np.concatenate([p.coords for p in problems])
    cells = np.concatenate([p.cells + nodes[k] for k, p in enumerate(problems)]).astype(np.int32)
    c2f = np.concatenate([p.topology[0] + facesOff[k] for k, p in enumerate(problems)])
    f2c = np.concatenate([np.where(p.topology[1] >= 0, p.topology[1] + cellsOff[k], -1)
                          for k, p in enumerate(problems)])
    faces = np.concatenate([p.topology[2] + nodes[k] for k, p in enumerate(problems)])
    bnd = np.concatenate([p.topology[3] + facesOff[k] for k, p in enumerate(problems)])
    topo = tuple(np.ascontiguousarray(a, np.int32) for a in (c2f, f2c, faces, bnd))
    return coords, cells, topo, (nodes, cellsOff, facesOff)


def group_tolerance(rtol, rhs, face_offsets, nf):
    """Group tolerance that bounds every problem's own relative residual by rtol
    (module docstring); rhs is the group's trace right-hand side."""
    sq = np.array([float(np.dot(rhs[a * nf:b * nf], rhs[a * nf:b * nf]))
                   for a, b in zip(face_offsets[:-1], face_offsets[1:])])
    total = float(sq.sum())
    live = sq[sq > 0]
    if total == 0.0 or live.size == 0:
        return rtol
    return rtol * float(np.sqrt(live.min() / total))


class _Group:
    def __init__(self, device, problems, src_mode, src_param):
        self.problems = problems
        dim, order = problems[0].dim, problems[0].order
        coords, cells, topo, self.offsets = union(problems)
        N = cells.shape[1]
        self.nf = topo[2].shape[1]
        # the fields of the union, checked before any device work
        for p in problems:
            if p.tau.size % (p.nFaces * self.nf) or p.dirichlet.size != p.nFaces * self.nf:
                raise ValueError("batch: tau [nFaces][Nf][1|2] and dirichlet [nFaces][Nf] of every problem")
        widths = {p.tau.size // (p.nFaces * self.nf) for p in problems}
        if len(widths) != 1 or widths.pop() not in (1, 2):
            raise ValueError("batch: within one order every problem's tau has 1, or every one 2, values per node")
        self.tau = np.ascontiguousarray(np.concatenate([p.tau.reshape(p.nFaces, self.nf, -1) for p in problems]))
        self.dirichlet = np.ascontiguousarray(np.concatenate([p.dirichlet.reshape(p.nFaces, self.nf)
                                                              for p in problems]))
        kaps = [p.kappa for p in problems]
        if any(k is None for k in kaps) and not all(k is None for k in kaps):
            raise ValueError("batch: within one order every problem gives kappa, or none does")
        self.kappa = None
        if kaps[0] is not None:
            kcs = {k.size // (p.nCells * N) if k.size % (p.nCells * N) == 0 else -1 for k, p in zip(kaps, problems)}
            if len(kcs) != 1 or kcs.pop() not in (1, dim * dim):
                raise ValueError("batch: kappa [nCells][N][1 or dim*dim], the same width within one order")
            self.kappa = np.ascontiguousarray(np.concatenate(
                [k.reshape(p.nCells, N, -1) for k, p in zip(kaps, problems)]))
        self.src_mode, self.src_param = src_mode, src_param
        self.source = None
        if src_mode == capi.SRC_VALUES:
            if any(p.source is None for p in problems):
                raise ValueError("batch: source values [nCells][nIP] for every problem")
            self.source = np.ascontiguousarray(np.concatenate([p.source.reshape(p.nCells, -1) for p in problems]))
        self.tol = self.rtol = None
        self.ctx = capi.Context(device)
        self.ctx.upload_mesh(dim, order, coords, cells, topology=topo)
        self.upload()

    def upload(self):
        c = self.ctx
        c.set_tau(self.tau)
        c.set_dirichlet(self.dirichlet)
        if self.kappa is not None:
            c.set_kappa(self.kappa, layout=1)
        c.set_source(self.src_mode, self.source, self.src_param)


class Batch:
    """Independent HDG diffusion-source problems of orders 1..5 on one GPU.

    One context (one stream) per order present. Per step either the phases over all
    groups (``assemble()``, ``solve(rtol)``, ``recover()``, then ``results()`` for every
    problem's Trace, Solution and Flux) or ``run()``, which takes the groups one after
    another, or all at once from one host thread each, and times each on its own stream."""

    def __init__(self, problems, device=0, src_mode=capi.SRC_NONE, src_param=0.0):
        if not problems:
            raise ValueError("batch: no problems")
        dims = {p.dim for p in problems}
        if len(dims) != 1:
            raise ValueError("batch: all problems have one dimension")
        self.problems = list(problems)
        self.orders = sorted({p.order for p in problems})
        # (order, index inside the order's group) of every problem, in the batch's order
        self.where = []
        members = {q: [] for q in self.orders}
        for p in self.problems:
            self.where.append((p.order, len(members[p.order])))
            members[p.order].append(p)
        self.groups = {q: _Group(device, members[q], src_mode, src_param) for q in self.orders}
        self.nCells = sum(p.nCells for p in self.problems)
        self.infos = {}

    def upload(self):
        """Upload every group's fields again (host buffers to the device)."""
        for g in self.groups.values():
            g.upload()

    def assemble(self):
        for g in self.groups.values():
            g.ctx.assemble()

    def _tolerance(self, g, rtol):
        if g.tol is None or g.rtol != rtol:
            rhs = np.zeros(g.ctx.ndofs)
            g.ctx._chk(g.ctx.L.hfx_get_csr(g.ctx.h, None, None, None, capi._p(rhs)), "get_csr")
            g.tol, g.rtol = group_tolerance(rtol, rhs, g.offsets[2], g.nf), rtol
        return g.tol

    def group_tolerances(self, rtol):
        """Per-order Krylov tolerances from the assembled right-hand sides (module
        docstring). They are kept for later solves at the same rtol: call this again
        after new field values."""
        for g in self.groups.values():
            g.tol = None
        return {q: self._tolerance(g, rtol) for q, g in self.groups.items()}

    def _solve(self, q, g, rtol, trace, opts, group_rtol=None):
        tol = self._tolerance(g, rtol) if group_rtol is None else group_rtol
        o = capi.solve_opts(**dict(opts, rtol=tol))
        info = capi.SolveInfo()
        g.ctx._chk(g.ctx.L.hfx_solve(g.ctx.h, ctypes.byref(o), capi._p(trace), ctypes.byref(info)), "solve")
        self.infos[q] = info

    def solve(self, rtol=1e-8, traces=None, group_rtol=None, **opts):
        """Krylov solve of every group at its group tolerance (computed on the first
        solve at this rtol), or at group_rtol relative to the whole group's right-hand side
        when that is given. traces: {order: host buffer [ndofs]} to download the group
        traces into, or None to keep them on the device. Returns {order: SolveInfo}."""
        for q, g in self.groups.items():
            self._solve(q, g, rtol, None if traces is None else traces[q], opts, group_rtol)
        return self.infos

    def recover(self, solutions=None, fluxes=None):
        for q, g in self.groups.items():
            sol = None if solutions is None else solutions[q]
            flux = None if fluxes is None else fluxes[q]
            g.ctx._chk(g.ctx.L.hfx_recover(g.ctx.h, capi._p(sol), capi._p(flux)), "recover")

    def host_buffers(self, alloc=np.zeros):
        """{order: (trace [ndofs], solution [nCells][N], flux [nCells][N*dim])} host arrays."""
        return {q: (alloc(g.ctx.ndofs), alloc((g.ctx.nCells, g.ctx.lenU)), alloc((g.ctx.nCells, g.ctx.lenQ)))
                for q, g in self.groups.items()}

    def _run_group(self, q, g, rtol, bufs, opts):
        L = capi.load()
        c = g.ctx
        c._chk(L.hfx_mark(c.h, 0), "mark")
        if bufs is not None:
            g.upload()
        c.assemble()
        b = (None, None, None) if bufs is None else bufs[q]
        self._solve(q, g, rtol, b[0], opts)
        c._chk(L.hfx_recover(c.h, capi._p(b[1]), capi._p(b[2])), "recover")
        c._chk(L.hfx_mark(c.h, 1), "mark")
        c._chk(L.hfx_synchronize(c.h), "synchronize")

    def run(self, rtol, bufs=None, concurrent=False, **opts):
        """One pass over the batch: assembly, Krylov solve and recovery of every group;
        with host buffers (``host_buffers()``) also the field uploads and the downloads of
        Trace, Solution and Flux. Group after group, or with concurrent=True every group
        from its own host thread at once. Returns {order: device ms}, from events on the
        group's stream around its work; ``span_ms`` is then the device time from the first
        group's start to the last group's end."""
        L = capi.load()
        if concurrent and len(self.groups) > 1:
            errors = []

            def work(q, g):
                try:
                    self._run_group(q, g, rtol, bufs, opts)
                except Exception as e:  # reported by the calling thread
                    errors.append(e)

            threads = [threading.Thread(target=work, args=(q, g)) for q, g in self.groups.items()]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
            if errors:
                raise errors[0]
        else:
            for q, g in self.groups.items():
                self._run_group(q, g, rtol, bufs, opts)
        ms = {}
        for q, g in self.groups.items():
            t = ctypes.c_double()
            g.ctx._chk(L.hfx_elapsed_ms(g.ctx.h, 0, 1, ctypes.byref(t)), "elapsed")
            ms[q] = t.value
        # span: earliest start to latest end, measured from the first group's start
        first = next(iter(self.groups.values())).ctx
        starts, ends = [], []
        for g in self.groups.values():
            for slot, out in ((0, starts), (1, ends)):
                t = ctypes.c_double()
                first._chk(L.hfx_elapsed_between(first.h, 0, g.ctx.h, slot, ctypes.byref(t)), "elapsed_between")
                out.append(t.value)
        self.span_ms = max(ends) - min(starts)
        return ms

    def step(self, rtol, bufs, concurrent=False, **opts):
        """``run()`` through host buffers."""
        return self.run(rtol, bufs, concurrent=concurrent, **opts)

    def results(self):
        """Per problem (in the batch's order): Trace [nFaces*Nf], Solution [nCells][N],
        Flux [nCells][N*dim], in the problem's own numbering."""
        state = {q: g.ctx.get_state() for q, g in self.groups.items()}
        out = []
        for q, k in self.where:
            g = self.groups[q]
            sol, flux, trace = state[q]
            c0, c1 = g.offsets[1][k], g.offsets[1][k + 1]
            f0, f1 = g.offsets[2][k], g.offsets[2][k + 1]
            out.append((trace[f0 * g.nf:f1 * g.nf], sol[c0:c1], flux[c0:c1]))
        return out

    def close(self):
        for g in self.groups.values():
            g.ctx.close()


def lognormal_field(points, sigma, corr, seed, modes=256, grid=129):
    """exp(g(points)) for points in the unit square, g a Gaussian random field of standard
    deviation sigma and squared-exponential correlation length corr: the random Fourier
    features sum sigma sqrt(2/M) sum_m cos(w_m . x + phi_m) (seeded w_m ~ N(0, I/corr^2),
    phi_m ~ U(0, 2 pi)) evaluated on a grid x grid lattice, where it separates into
    two matrix products, and interpolated bilinearly at the points."""
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, 1.0 / corr, size=(2, modes))
    phase = rng.uniform(0.0, 2.0 * np.pi, size=modes)
    t = np.linspace(0.0, 1.0, grid)
    ax = t[:, None] * w[0] + phase
    ay = t[:, None] * w[1]
    lat = sigma * np.sqrt(2.0 / modes) * (np.cos(ax) @ np.cos(ay).T - np.sin(ax) @ np.sin(ay).T)  # [x][y]
    flat = np.clip(points.reshape(-1, 2), 0.0, 1.0) * (grid - 1)
    i = np.minimum(flat[:, 0].astype(np.int64), grid - 2)
    j = np.minimum(flat[:, 1].astype(np.int64), grid - 2)
    fx, fy = flat[:, 0] - i, flat[:, 1] - j
    g = ((1 - fx) * (1 - fy) * lat[i, j] + fx * (1 - fy) * lat[i + 1, j] + (1 - fx) * fy * lat[i, j + 1]
         + fx * fy * lat[i + 1, j + 1])
    return np.exp(g).reshape(points.shape[:-1])


def _uneven_problem(args):
    n, p, fseed, jitter, sigma, corr, kappa_at = args
    v, s = meshgen.square_simplices(n)
    if jitter:
        v = meshgen.jitter_vertices(v, n, jitter, fseed + 1)
    coords, cells = capi.mesh_high_order(2, p, v, s)
    if kappa_at == "nodes":
        kap = lognormal_field(coords[cells], sigma, corr, fseed)[..., None]
    else:
        cent = coords[cells[:, :3]].mean(axis=1)
        kap = np.repeat(lognormal_field(cent, sigma, corr, fseed)[:, None, None], cells.shape[1], axis=1)
    prob = Problem(2, p, coords, cells, kappa=kap)
    prob.dirichlet = np.prod(np.sin(np.pi * coords[prob.faces]), axis=-1)
    return prob


def uneven_plan(count=1024, seed=3, min_elements=200, max_elements=20000, orders=(1, 2, 3, 4, 5)):
    """The seeded draws of ``uneven_batch``: per problem (n, order, field seed), the mesh
    n x n x 2 triangles with n = round(sqrt(c / 2)), c log-uniform in
    [min_elements, max_elements], the order uniform in ``orders``."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(np.log(min_elements), np.log(max_elements), size=count))
    ns = np.maximum(1, np.rint(np.sqrt(counts / 2.0))).astype(int)
    ps = rng.choice(np.asarray(orders), size=count)
    fseeds = rng.integers(0, 2 ** 31, size=count)
    return [(int(ns[k]), int(ps[k]), int(fseeds[k])) for k in range(count)]


def problem_cost(n, order):
    """Work estimate of one 2D problem: elements x (trace values per element)^2."""
    return 2 * n * n * (3 * (order + 1)) ** 2


def shard(costs, world):
    """Problem indices per rank, balanced by cost (longest-processing-time greedy: the
    most expensive problem first, each to the least loaded rank; ties to the lower rank).
    Deterministic, so every rank computes the same split without communication."""
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += costs[i]
    return [sorted(o) for o in out]


def uneven_batch(count=1024, seed=3, min_elements=200, max_elements=20000, orders=(1, 2, 3, 4, 5),
                 jitter=0.2, sigma=1.0, corr=0.1, kappa_at="cells", select=None):
    """Seeded batch of 2D unit-square problems of uneven size and order.

    Problem k (draws of ``uneven_plan``): mesh n x n x 2 triangles, interior vertices
    jittered by U(-jitter h, jitter h), kappa = exp(g) with g a Gaussian random field
    (sigma, corr, its own seed) sampled at the cell centroids (kappa_at "cells": constant
    inside every cell, so the trace system is symmetric and CG with the two-level
    preconditioner applies) or at the cell nodes ("nodes": GMRES), tau = 1, Dirichlet
    u = sin(pi x) sin(pi y) at the face nodes. The source is the batch's (the workload uses
    f = 2 pi^2 sin(pi x) sin(pi y)). select: the problem indices to build (default all),
    e.g. one rank's ``shard``."""
    if kappa_at not in ("cells", "nodes"):
        raise ValueError("uneven_batch: kappa_at is 'cells' or 'nodes'")
    plan = uneven_plan(count, seed, min_elements, max_elements, orders)
    idx = range(count) if select is None else select
    return [_uneven_problem(plan[k] + (jitter, sigma, corr, kappa_at)) for k in idx]
