"""Benchmark: HDG diffusion-source time-to-solve on GB300.

Workload (default, one GPU): 3D HDG diffusion-source on the unit cube, 40^3
cubes x 6 tetrahedra = 384,000 tets, p = 3, manufactured u = prod sin(pi x),
tau = 1, kappa = 1, Dirichlet from u. One step = the whole hot path with the
mesh and fields resident on the device: element assembly + static
condensation + Dirichlet + scatter into the trace system, the Krylov solve to
the stated tolerance, and local recovery of Solution and Flux.

value = elements per second of that step (elements / time-to-solve), device
time from CUDA events on the library's stream. e2e = the same through the C
ABI with host buffers: the field uploads (Tau, Dirichlet) and the downloads of
Trace, Solution and Flux are inside the timed region.

Inputs are far larger than L2 (element blocks ~15 GB, trace matrix ~4 GB), so
no L2 flush is needed between steps.

Other workloads (--config): cfg4 viscous Burgers with Newton every time step, cfg5
anisotropic lognormal diffusion, cfg3 a batch of 1024 independent problems of orders
1-5 (hyperfox_gb300.batch: one disjoint-union mesh per order).

--impl reference times the CPU oracle (C++ restatement of HyperFox's path:
per-element dense assembly + LU condensation, CSR scatter, GMRES(30)+Jacobi,
recovery) on the host cores with all threads, on a bounded sample of the same
workload (a sub-cube of the same element type and order).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "time-to-solve @1e-8 rel err, learned+mixed vs plain FP64 GPU; elements/s"
# DRAM bytes per unit from the committed ncu captures (profiles/): the FP32 trace
# SpMV over the symmetric half storage moves 2.60 bytes per non-zero of the full
# operator (175.1 MB at 67.44M non-zeros), the FP64 one (full storage) 8.75; the
# affine element kernel reads and writes 19.7 KB per p=3 tetrahedron.
TRAFFIC_PER_NNZ = {"spmv32": 175.1e6 / 67.44e6, "spmv64": 590.2e6 / 67.44e6}
TRAFFIC_PER_ELEMENT_LOCAL = (54.0e6 + 890.3e6) / 48000
FP64_NOMINAL_TFLOPS = 1.25

CONFIGS = {
    # name: dim, n (cubes per side), order
    "cfg2": dict(dim=3, n=40, order=3, desc="3D HDG diffusion-source, unit cube 40^3x6 tets (384k), p=3"),
    "cfg1": dict(dim=2, n=32, order=2, desc="2D HDG diffusion-source, unit square 32x32x2 tris (2048), p=2"),
    "small3d": dict(dim=3, n=12, order=3, desc="3D HDG diffusion-source, 12^3x6 tets, p=3"),
    "mid3d": dict(dim=3, n=20, order=3, desc="3D HDG diffusion-source, 20^3x6 tets (48k), p=3"),
    "cfg5mesh": dict(dim=3, n=60, order=2, desc="3D HDG diffusion-source, 60^3x6 tets (1.296M), p=2"),
    # anisotropic lognormal diffusion: kappa = exp(g) (I + 99 a a^T), g a Gaussian random field
    # (sigma 1.5, correlation length 0.05) sampled at the cell centroids, a a seeded random axis
    "cfg5": dict(dim=3, n=60, order=2, aniso=dict(sigma=1.5, corr=0.05, ratio=100.0, seed=5), cpu_n=8,
                 desc="3D anisotropic diffusion, unit cube 60^3x6 tets (1.296M), p=2, kappa = exp(g) x "
                      "(I + 99 a a^T), g Gaussian random field (sigma 1.5, corr 0.05) per cell, seeded axis a"),
    # the cfg2 mesh with a diffusion coefficient that varies inside the cells (HyperFox's nodal
    # DiffusionTensor field): the general element path (per-element quadrature), GMRES
    "cfg2-nodal": dict(dim=3, n=40, order=3, nodal_kappa=True,
                       desc="3D HDG diffusion-source, unit cube 40^3x6 tets (384k), p=3, nodal kappa = "
                            "exp(0.5 sin(2 pi x) sin(2 pi y) sin(2 pi z))"),
    "mid3d-nodal": dict(dim=3, n=20, order=3, nodal_kappa=True,
                        desc="3D HDG diffusion-source, 20^3x6 tets (48k), p=3, nodal kappa = "
                             "exp(0.5 sin(2 pi x) sin(2 pi y) sin(2 pi z))"),
    "cfg5-small": dict(dim=3, n=20, order=2, aniso=dict(sigma=1.5, corr=0.05, ratio=100.0, seed=5), cpu_n=8,
                       desc="3D anisotropic diffusion, 20^3x6 tets (48k), p=2, the cfg5 coefficient field"),
    # independent problems of uneven size and order, one order per problem (a Mesh has one
    # ReferenceElement), each order's problems solved as one disjoint-union mesh
    "cfg3": dict(dim=2, batch=dict(count=1024, seed=3, min_elements=200, max_elements=20000), cpu_budget=12000,
                 desc="1024 independent 2D HDG diffusion-source problems: unit-square meshes of 2n^2 triangles, "
                      "n = round(sqrt(c/2)), c log-uniform in [200, 20000]; interior vertices jittered "
                      "U(+-0.2h); p uniform in 1..5 per problem; kappa = exp(g) at the cell centroids (constant per "
                      "cell), g Gaussian "
                      "random field (sigma 1, corr 0.1); tau = 1; f = 2 pi^2 sin(pi x) sin(pi y), "
                      "Dirichlet u = sin(pi x) sin(pi y)"),
    "cfg3-small": dict(dim=2, batch=dict(count=64, seed=3, min_elements=200, max_elements=20000), cpu_budget=1500,
                       desc="64 independent 2D HDG diffusion-source problems, the cfg3 distribution"),
    # viscous Burgers (HDGBurgersModel + HDGUNabU, nd = 2), implicit Euler, Newton every step
    "cfg4": dict(dim=2, n=180, order=3, burgers=True, nu=1e-2, dt=1e-3, time_steps=200,
                 desc="2D viscous Burgers HDG, unit square 180x180x2 tris (64,800), p=3, nu=1e-2, "
                      "implicit Euler dt=1e-3, Newton to 1e-6 every step"),
    "burgers-mid": dict(dim=2, n=96, order=3, burgers=True, nu=1e-2, dt=1e-3, time_steps=20,
                        desc="2D viscous Burgers HDG, 96x96x2 tris (18,432), p=3, nu=1e-2, dt=1e-3"),
    "burgers-small": dict(dim=2, n=48, order=3, burgers=True, nu=1e-2, dt=1e-3, time_steps=20,
                          desc="2D viscous Burgers HDG, 48x48x2 tris (4,608), p=3, nu=1e-2, dt=1e-3"),
}
BURGERS_METRIC = ("Burgers implicit-Euler steps, Newton to 1e-6 (GMRES 1e-10): elements x Newton iterations / s "
                  "(assemble + condense + scatter + Krylov + recover per iteration)")


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def aniso_kappa(coords, cells, dim, sigma, corr, ratio, seed, modes=256):
    """Cell-constant anisotropic lognormal diffusion tensor [nCells][N][dim*dim] (column-major,
    exactly symmetric): exp(g(centroid)) (I + (ratio - 1) a a^T), with g a Gaussian random field
    of standard deviation sigma and squared-exponential correlation length corr (random Fourier
    features, seeded) and a a seeded random unit axis."""
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, 1.0 / corr, size=(dim, modes))
    phase = rng.uniform(0.0, 2.0 * np.pi, size=modes)
    axis = rng.normal(size=dim)
    axis /= np.linalg.norm(axis)
    A = np.eye(dim) + (ratio - 1.0) * np.outer(axis, axis)
    A = 0.5 * (A + A.T)
    nC, N = cells.shape
    cent = coords[cells[:, :dim + 1]].mean(axis=1)
    g = np.empty(nC)
    for a in range(0, nC, 65536):
        g[a:a + 65536] = sigma * np.sqrt(2.0 / modes) * np.cos(cent[a:a + 65536] @ w + phase).sum(axis=1)
    kap = np.exp(g)[:, None, None] * A.T.reshape(1, 1, dim * dim)
    return np.ascontiguousarray(np.broadcast_to(kap, (nC, N, dim * dim)))


def nodal_kappa(coords, cells):
    """Scalar diffusion coefficient at the cell nodes [nCells][N][1], varying inside every cell:
    exp(0.5 sin(2 pi x) sin(2 pi y) sin(2 pi z))."""
    x = coords[cells]
    return np.exp(0.5 * np.prod(np.sin(2 * np.pi * x), axis=-1))[..., None]


def make_problem(cfg):
    from hyperfox_gb300 import capi, meshgen
    dim, n, p = cfg["dim"], cfg["n"], cfg["order"]
    re = capi.refel(dim, p)
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    coords, cells = meshgen.high_order(v, s, re["nodes"])
    return coords, cells


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("HFX_BENCH_GLOO") is None else "gloo")
    return world, rank, local


def barrier_max(world, value):
    """Max of value over the ranks (the slowest replica sets the time)."""
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cpu" if dist.get_backend() == "gloo" else "cuda"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_ours(args, world, rank, local):
    import torch
    from hyperfox_gb300 import capi
    torch.cuda.set_device(local)
    cfg = CONFIGS[args.config]
    dim, p = cfg["dim"], cfg["order"]
    t0 = time.time()
    coords, cells = make_problem(cfg)
    t_mesh = time.time() - t0
    ctx = capi.Context(local)
    t1 = time.time()
    ctx.upload_mesh(dim, p, coords, cells)
    t_upload = time.time() - t1
    t_setup = time.time() - t0
    _, _, faces, _ = ctx.topology()
    Nf = ctx.re["nNodesFace"]
    # pinned host buffers for the per-step inputs and results (e2e)
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    tau_h = pin((ctx.nFaces, Nf))
    tau_h[:] = 1.0
    dir_h = pin((ctx.nFaces, Nf))
    dir_h[:] = np.prod(np.sin(np.pi * coords[faces]), axis=-1)
    trace_h = pin(ctx.ndofs)
    sol_h = pin((ctx.nCells, ctx.lenU))
    flux_h = pin((ctx.nCells, ctx.lenQ))
    ctx.set_tau(tau_h)
    ctx.set_dirichlet(dir_h)
    ctx.set_source(capi.SRC_SINPROD, param=dim * np.pi ** 2)
    if cfg.get("aniso"):
        ctx.set_kappa(aniso_kappa(coords, cells, dim, **cfg["aniso"]), layout=1)
    if cfg.get("nodal_kappa"):
        ctx.set_kappa(nodal_kappa(coords, cells), layout=1)
    L = ctx.L
    if args.assembly_path:
        ctx._chk(L.hfx_set_assembly_path(ctx.h, args.assembly_path), "assembly_path")
    if args.spmv_kernel >= 0:
        ctx._chk(L.hfx_set_tuning(ctx.h, args.spmv_kernel), "set_tuning")
    prec = capi.PREC_FP64 if args.precision == "fp64" else capi.PREC_MIXED
    pc = capi.PC_TWOLEVEL if args.precond == "twolevel" else capi.PC_BLOCK_JACOBI
    opts = capi.solve_opts(precision=prec, rtol=args.rtol, precond=pc, maxits=200000,
                           inner_rtol=args.inner_rtol, coarse_guess=int(args.coarse_guess),
                           coarse_rtol=args.coarse_rtol,
                           coarse_mode=capi.COARSE_LEARNED if args.coarse == "learned" else capi.COARSE_CHEBYSHEV)
    info = capi.SolveInfo()

    asm_prec = capi.PREC_MIXED if args.precision == "mixed-full" else capi.PREC_FP64

    def step_device():
        ctx._chk(L.hfx_assemble_ex(ctx.h, asm_prec), "assemble")
        ctx._chk(L.hfx_solve(ctx.h, capi.ctypes.byref(opts), None, capi.ctypes.byref(info)), "solve")
        ctx._chk(L.hfx_recover(ctx.h, None, None), "recover")

    def step_e2e():
        ctx.set_tau(tau_h)
        ctx.set_dirichlet(dir_h)
        ctx._chk(L.hfx_assemble_ex(ctx.h, asm_prec), "assemble")
        ctx._chk(L.hfx_solve(ctx.h, capi.ctypes.byref(opts), capi._p(trace_h), capi.ctypes.byref(info)), "solve")
        ctx._chk(L.hfx_recover(ctx.h, capi._p(sol_h), capi._p(flux_h)), "recover")

    if args.assembly_only:
        return run_assembly_only(args, world, ctx, asm_prec, cfg), ctx
    # accuracy reference: plain FP64 CG to 1e-13 (untimed)
    ctx.assemble()
    # (a diffusion coefficient varying inside the cells makes the system non-symmetric: GMRES(100) to 1e-11)
    ref_opts = capi.solve_opts(precision=capi.PREC_FP64, rtol=1e-11 if cfg.get("nodal_kappa") else 1e-13,
                               precond=capi.PC_BLOCK_JACOBI, maxits=500000, restart=100)
    ref_info = capi.SolveInfo()
    x_ref = np.zeros(ctx.ndofs)
    ctx._chk(L.hfx_solve(ctx.h, capi.ctypes.byref(ref_opts), capi._p(x_ref), capi.ctypes.byref(ref_info)), "ref solve")
    # learned coarse polynomial: trained once on this system's own coarse residuals (setup, untimed)
    learned = None
    if args.precond == "twolevel" and args.coarse == "learned" and args.precision != "mixed-full":
        ti = ctx.coarse_train(degree=args.coarse_degree, samples=16, steps=300)
        learned = dict(degree=ti.degree, samples=ti.samples, steps=ti.steps, accepted=bool(ti.accepted),
                       loss_chebyshev_same_degree=ti.loss_chebyshev, loss_learned=ti.loss_learned,
                       max_residual_polynomial=ti.max_poly, train_s=ti.train_ms / 1e3,
                       loss_first_step=ti.loss_first_step, lower_steps=ti.lower_steps,
                       rejected_steps=ti.rejected_steps)
    for _ in range(args.warmup):
        step_device()
    # device-resident timed region
    barrier(world)
    ctx._chk(L.hfx_synchronize(ctx.h), "sync")
    clocks = ClockSampler(local)
    clocks.start()
    ctx._chk(L.hfx_mark(ctx.h, 0), "mark")
    for _ in range(args.steps):
        step_device()
    ctx._chk(L.hfx_mark(ctx.h, 1), "mark")
    ms = capi.ctypes.c_double()
    ctx._chk(L.hfx_elapsed_ms(ctx.h, 0, 1, capi.ctypes.byref(ms)), "elapsed")
    clk = clocks.stop()
    dev_ms = barrier_max(world, ms.value)
    # per-kernel device times from a second pass of the same steps with the event timer on
    # (its events would otherwise add host work to the timed region)
    ctx._chk(L.hfx_profile_enable(ctx.h, 1), "profile")
    for _ in range(args.steps):
        step_device()
    ctx._chk(L.hfx_synchronize(ctx.h), "sync")
    kt = {}
    for name, kid in (("local", 0), ("scatter", 1), ("spmv64", 2), ("spmv32", 3), ("update", 4), ("recover", 5),
                      ("other", 6), ("residual", 7), ("coarse", 8), ("tensor", 9)):
        n_l, t_l = capi.ctypes.c_int(), capi.ctypes.c_double()
        L.hfx_kernel_time(ctx.h, kid, capi.ctypes.byref(n_l), capi.ctypes.byref(t_l))
        kt[name] = (n_l.value, t_l.value)
    ctx._chk(L.hfx_profile_enable(ctx.h, 0), "profile")
    iters, refinements = info.iterations, info.refinements
    # accuracy of the last solve vs the FP64 reference
    x = np.zeros(ctx.ndofs)
    ctx._chk(L.hfx_assemble_ex(ctx.h, asm_prec), "assemble")
    ctx._chk(L.hfx_solve(ctx.h, capi.ctypes.byref(opts), capi._p(x), capi.ctypes.byref(info)), "solve")
    rel_err = float(np.linalg.norm(x - x_ref) / np.linalg.norm(x_ref))
    # e2e timed region (host buffers, copies inside), after untimed warm-up steps of the same
    # calls (the first copies from a pinned buffer carry one-off costs)
    for _ in range(max(1, min(args.warmup, 3))):
        step_e2e()
    barrier(world)
    ctx._chk(L.hfx_synchronize(ctx.h), "sync")
    e2e_clocks = ClockSampler(local)
    e2e_clocks.start()
    t0 = time.perf_counter()
    ctx._chk(L.hfx_mark(ctx.h, 6), "mark")
    for _ in range(args.steps):
        step_e2e()
    ctx._chk(L.hfx_mark(ctx.h, 7), "mark")
    ctx._chk(L.hfx_synchronize(ctx.h), "sync")
    e2e_s = barrier_max(world, time.perf_counter() - t0)
    e2e_clk = e2e_clocks.stop()
    # the same region on the device clock (events on the library's stream): the copies
    # and the step's kernels, without the host time before the first and after the last
    e2e_dev = capi.ctypes.c_double()
    ctx._chk(L.hfx_elapsed_ms(ctx.h, 6, 7, capi.ctypes.byref(e2e_dev)), "elapsed")
    h2d = tau_h.nbytes + dir_h.nbytes
    d2h = trace_h.nbytes + sol_h.nbytes + flux_h.nbytes
    # plain FP64 GPU time-to-solve (same tolerance), for the learned+mixed vs plain comparison
    plain = None
    if args.precision != "fp64" and not args.no_plain:
        fp_opts = capi.solve_opts(precision=capi.PREC_FP64, rtol=args.rtol, precond=capi.PC_BLOCK_JACOBI, maxits=500000)
        fp_info = capi.SolveInfo()
        ctx._chk(L.hfx_mark(ctx.h, 2), "mark")
        for _ in range(max(1, args.plain_steps)):
            ctx._chk(L.hfx_assemble(ctx.h), "assemble")
            ctx._chk(L.hfx_solve(ctx.h, capi.ctypes.byref(fp_opts), None, capi.ctypes.byref(fp_info)), "solve")
            ctx._chk(L.hfx_recover(ctx.h, None, None), "recover")
        ctx._chk(L.hfx_mark(ctx.h, 3), "mark")
        pms = capi.ctypes.c_double()
        ctx._chk(L.hfx_elapsed_ms(ctx.h, 2, 3, capi.ctypes.byref(pms)), "elapsed")
        plain = dict(time_to_solve_s=pms.value / 1e3 / max(1, args.plain_steps), iterations=fp_info.iterations)
    # the learned coarse solve on its own: the same two-level mixed solve with Chebyshev of the
    # learned polynomial's degree and with Chebyshev at its adaptive degree, and the first solve
    # of a new system including the training (wall clock: training + one step)
    coarse_arms = None
    if learned is not None and not args.no_plain:
        coarse_arms = {}
        for name, kw in (("chebyshev_same_degree", dict(coarse_mode=capi.COARSE_CHEBYSHEV,
                                                        coarse_degree=args.coarse_degree)),
                         ("chebyshev_adaptive", dict(coarse_mode=capi.COARSE_CHEBYSHEV, coarse_degree=0)),
                         ("learned", dict(coarse_mode=capi.COARSE_LEARNED, coarse_degree=0)),
                         # the trained coarse network also gives the initial guess: x0 = P q(A_c) P^T b'
                         ("learned_initial_guess", dict(coarse_mode=capi.COARSE_LEARNED, coarse_degree=0,
                                                        coarse_guess=1))):
            kw.setdefault("coarse_guess", int(args.coarse_guess))
            o2 = capi.solve_opts(precision=prec, rtol=args.rtol, precond=pc, maxits=200000,
                                 inner_rtol=args.inner_rtol, coarse_rtol=args.coarse_rtol, **kw)
            i2 = capi.SolveInfo()
            x2 = np.zeros(ctx.ndofs)
            ctx._chk(L.hfx_mark(ctx.h, 4), "mark")
            for _ in range(max(1, args.plain_steps)):
                ctx._chk(L.hfx_assemble_ex(ctx.h, asm_prec), "assemble")
                ctx._chk(L.hfx_solve(ctx.h, capi.ctypes.byref(o2), None, capi.ctypes.byref(i2)), "solve")
                ctx._chk(L.hfx_recover(ctx.h, None, None), "recover")
            ctx._chk(L.hfx_mark(ctx.h, 5), "mark")
            ams = capi.ctypes.c_double()
            ctx._chk(L.hfx_elapsed_ms(ctx.h, 4, 5, capi.ctypes.byref(ams)), "elapsed")
            ctx._chk(L.hfx_solve(ctx.h, capi.ctypes.byref(o2), capi._p(x2), capi.ctypes.byref(i2)), "solve")
            coarse_arms[name] = dict(time_to_solve_s=ams.value / 1e3 / max(1, args.plain_steps),
                                     iterations=i2.iterations, coarse_degree=i2.coarse_degree,
                                     coarse_learned=bool(i2.coarse_learned),
                                     rel_err_vs_fp64=float(np.linalg.norm(x2 - x_ref) / np.linalg.norm(x_ref)))
        ctx._chk(L.hfx_synchronize(ctx.h), "sync")
        t0 = time.perf_counter()
        ti = ctx.coarse_train(degree=args.coarse_degree, samples=16, steps=300)
        step_device()
        ctx._chk(L.hfx_synchronize(ctx.h), "sync")
        coarse_arms["time_to_first_solve_s"] = time.perf_counter() - t0
        coarse_arms["time_to_first_solve_accepted"] = bool(ti.accepted)
    # error against the oracle's direct FP64 solve of the 12^3 x 6 sub-cube of this workload
    # (stored fixture), with the same solver options
    oracle_check = None
    gold_path = os.path.join(ROOT, "tests", "golden", "subcube12_p3_trace.npz")
    if (dim, p) == (3, 3) and not cfg.get("aniso") and not cfg.get("nodal_kappa") and os.path.exists(gold_path):
        from hyperfox_gb300 import meshgen
        gold = np.load(gold_path)
        vs, ss = meshgen.cube_simplices(int(gold["n"]))
        sc, scl = meshgen.high_order(vs, ss, capi.refel(3, 3)["nodes"])
        sub = capi.Context(local)
        sub.upload_mesh(3, 3, sc, scl)
        _, _, sfaces, _ = sub.topology()
        sub.set_source(capi.SRC_SINPROD, param=3 * np.pi ** 2)
        sub.set_dirichlet(np.prod(np.sin(np.pi * sc[sfaces]), axis=-1))
        if args.assembly_path:
            sub._chk(sub.L.hfx_set_assembly_path(sub.h, args.assembly_path), "assembly_path")
        sub._chk(sub.L.hfx_assemble_ex(sub.h, asm_prec), "assemble")
        if learned is not None:
            sub.coarse_train(degree=args.coarse_degree, samples=16, steps=300)
        si = capi.SolveInfo()
        xs = np.zeros(sub.ndofs)
        sub._chk(sub.L.hfx_solve(sub.h, capi.ctypes.byref(opts), capi._p(xs), capi.ctypes.byref(si)), "solve")
        oracle_check = dict(rel_err=float(np.linalg.norm(xs - gold["trace"]) / np.linalg.norm(gold["trace"])),
                            sample="12^3x6 sub-cube (10,368 elements, 216,000 trace DOFs) of this workload, same "
                                   "solver options; oracle = FP64 assembly + sparse LU (tests/golden)",
                            iterations=si.iterations)
        sub.close()
    E = ctx.nCells
    step_s = dev_ms / 1e3 / args.steps
    # roofline of the dominant kernel, and of the dominant HBM-bound kernel
    hbm, peak_kind = peaks()
    nnz, n = ctx.nnz, ctx.ndofs
    nblocks = nnz // (Nf * Nf)

    def spmv_roof(key):
        sv = 4 if key == "spmv32" else 8
        # values once, block columns + row pointers once, z and p_old gathered once, p_new and q written;
        # the FP32 operator of a symmetric problem is stored as its upper block triangle
        # (diagonal blocks + half the off-diagonal ones) plus one int per block locating it
        if key == "spmv32":
            # rows as fixed-width (block column, block location) slots: 8 bytes per slot
            n_half = (nblocks - ctx.nFaces) // 2 + ctx.nFaces
            width = 7 if dim == 3 else 5
            alg = n_half * Nf * Nf * sv + ctx.nFaces * width * 8 + 4 * n * sv
        else:
            alg = nnz * sv + nblocks * 4 + (ctx.nFaces + 1) * 8 + 4 * n * sv
        # launches that did work: one per Krylov iteration (launches queued after
        # convergence return at entry and are not counted)
        launches = min(kt[key][0], iters * args.steps) if iters else kt[key][0]
        avg_ms = kt[key][1] / max(1, launches)
        achieved = alg / (avg_ms / 1e3) / 1e9
        kname = {1: "cg_spmv_half_tma<float>", 2: "cg_spmv_half_ell<float, paired>",
                 3: "cg_spmv_half_ell<float, paired, float4 x>"}.get(
            ctx.tuning_info()[0], "cg_spmv_half_ell<float>") if sv == 4 else "cg_spmv<double>"
        return dict(bound="hbm", kernel=kname,
                    achieved=round(achieved, 1), peak=hbm, unit="GB/s", frac=round(achieved / hbm, 4),
                    traffic=(TRAFFIC_PER_NNZ[key] * nnz) if (dim, p) == (3, 3) else None, bytes_per_launch=int(alg),
                    avg_launch_ms=round(avg_ms, 4), peak_source=peak_kind)

    def local_roof():
        # FP64 FMAs the affine element kernel executes per element (reference-operator algorithm)
        N, NF_, F_ = ctx.re["nNodes"], Nf, ctx.re["nFaces"]
        LL, NI = F_ * NF_, ctx.re["nIP"]
        fma = (F_ * NF_ ** 3 + N * N * (dim * dim + 1) + N * LL * dim + NI * N * dim + N * NI + N ** 3 / 6
               + 2 * (LL + 1) * N * (N - 1) / 2 + LL * (LL + 1) / 2 * N + LL * N)
        # the symmetric W^T W product runs as double-float pairs on the FP32 pipe: not FP64-pipe work
        df_fma = LL * (LL + 1) / 2 * N
        fma64 = fma - df_fma
        avg_ms = kt["local"][1] / max(1, kt["local"][0])
        tf = 2 * fma64 * E / (avg_ms / 1e3) / 1e12
        # the reference's own algorithm per element (dense quadrature assembly plus the dense
        # LU-equivalent condensation of HDGSolver.cpp:331-348): the same elements per second
        # expressed in its FLOP count
        lenU, lenQ, lenL, NIF = N, dim * N, LL, ctx.re["nIPFace"]
        ref_asm = 2 * NI * N * N * (1 + 2 * dim) + F_ * 2 * NIF * NF_ ** 2 * (1 + 2 * dim) + 2 * NI * N
        ref_cond = (2 / 3 * lenQ ** 3 + 2 * lenQ ** 2 * (lenU + lenL) + 2 * lenU * lenQ * lenU + 2 * lenU * lenQ * lenL
                    + 2 / 3 * lenU ** 3 + 2 * lenU ** 2 * lenL + 2 * lenQ * lenU * lenL + 2 * lenL * lenU * lenL
                    + 2 * lenL * lenQ * lenL)
        return dict(bound="fp64", kernel="local_affine (FP64 element assembly + condensation)",
                    achieved=round(tf, 3), peak=FP64_NOMINAL_TFLOPS, unit="TFLOP/s",
                    frac=round(tf / FP64_NOMINAL_TFLOPS, 4),
                    traffic=TRAFFIC_PER_ELEMENT_LOCAL * E if (dim, p) == (3, 3) else None,
                    flops_per_element=int(2 * fma64), avg_launch_ms=round(avg_ms, 4),
                    count="FP64-pipe FLOPs of the executed algorithm (reference operators, Cholesky Schur); "
                          "the W^T W product's %d double-float multiply-adds per element run on the FP32 pipe "
                          "and are not counted" % int(df_fma),
                    double_float_fma_per_element=int(df_fma),
                    flops_per_element_reference_algorithm=int(ref_asm + ref_cond),
                    reference_algorithm_equivalent_tflops=round((ref_asm + ref_cond) * E / (avg_ms / 1e3) / 1e12, 2),
                    peak_source="nominal GB300 FP64 (no measured FP64 peak); ncu: FP64 pipe 86% active")

    dom = max(("local", "spmv64", "spmv32", "update", "scatter", "recover", "residual"), key=lambda k: kt[k][1])
    roof = None
    if dom in ("spmv32", "spmv64"):
        roof = spmv_roof(dom)
    elif dom == "local":
        roof = local_roof()
    hbm_key = max(("spmv32", "spmv64"), key=lambda k: kt[k][1])
    roof_hbm = spmv_roof(hbm_key) if kt[hbm_key][0] else None
    if args.traffic and roof is not None:
        roof["traffic"] = args.traffic
    res = {
        "metric": METRIC,
        "value": E / step_s,
        "unit": "elements/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": step_s * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64+f32" if prec else "f64",
        "data": "synthetic (seedless structured mesh, manufactured solution)",
        "config": {"workload": cfg["desc"], "elements": E, "order": p, "trace_dofs": n, "csr_nnz": nnz,
                   "precision": args.precision, "preconditioner": ("two-level: per-face block Jacobi + vertex coarse space (%s coarse polynomial, degree %d)"
                                      % ("learned" if info.coarse_learned else "Chebyshev", info.coarse_degree))
                                     if args.precond == "twolevel" else "block-Jacobi (per face)",
                   "rtol": args.rtol, "l2_flush": "inputs > L2 (no flush needed)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "time_to_solve_s": step_s,
        "assembly_elements_per_s": E / (kt["local"][1] / 1e3 / max(1, kt["local"][0])) if kt["local"][0] else None,
        "krylov_iterations": iters,
        "refinements": refinements,
        "rel_err_vs_fp64": rel_err,
        "rel_err_vs_fp64_reference": "the same library's FP64 block-Jacobi CG of the same system to relative "
                                     "residual 1e-13 (GPU)",
        "rel_err_vs_oracle": oracle_check,
        "meets_1e-8_rel_err": bool(rel_err <= 1e-8),
        "coarse_solve_comparison": coarse_arms,
        "spmv_tuner": dict(zip(("kernel", "ms_per_launch"), ctx.tuning_info())),
        "fp64_reference_iterations": ref_info.iterations,
        "plain_fp64": plain,
        "learned_coarse": learned,
        "kernel_ms": {k: dict(launches=v[0], total_ms=round(v[1], 3)) for k, v in kt.items()},
        "roofline": roof,
        "roofline_hbm": roof_hbm,
        "clocks": clk,
        "e2e_clocks": e2e_clk,
        "e2e_device_ms_per_step": e2e_dev.value / args.steps,
        "e2e": {"value": E * args.steps / e2e_s, "unit": "elements/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(sum(v[0] for v in kt.values())),
        "setup_s": t_setup,
        # host-side setup: the synthetic mesh (numpy) and hfx_mesh_upload (faces by the MOAB
        # rule, face permutations, the trace system's block pattern, in C++; device uploads)
        "setup_split_s": {"mesh_generation": round(t_mesh, 3), "mesh_upload_topology_pattern": round(t_upload, 3)},
    }
    if plain:
        res["speedup_vs_plain_fp64"] = plain["time_to_solve_s"] / step_s
    return res, ctx


def run_assembly_only(args, world, ctx, asm_prec, cfg):
    """Element assembly + condensation + scatter alone (hfx_assemble_ex), K timed calls:
    elements/s of the assembly and the per-kernel device times."""
    from hyperfox_gb300 import capi
    L = ctx.L
    for _ in range(args.warmup):
        ctx._chk(L.hfx_assemble_ex(ctx.h, asm_prec), "assemble")
    barrier(world)
    ctx._chk(L.hfx_synchronize(ctx.h), "sync")
    ctx._chk(L.hfx_profile_enable(ctx.h, 1), "profile")
    ctx._chk(L.hfx_mark(ctx.h, 0), "mark")
    for _ in range(args.steps):
        ctx._chk(L.hfx_assemble_ex(ctx.h, asm_prec), "assemble")
    ctx._chk(L.hfx_mark(ctx.h, 1), "mark")
    ms = capi.ctypes.c_double()
    ctx._chk(L.hfx_elapsed_ms(ctx.h, 0, 1, capi.ctypes.byref(ms)), "elapsed")
    dev_ms = barrier_max(world, ms.value)
    kt = {}
    for name, kid in (("local", 0), ("scatter", 1), ("residual", 7), ("tensor", 9)):
        n_l, t_l = capi.ctypes.c_int(), capi.ctypes.c_double()
        L.hfx_kernel_time(ctx.h, kid, capi.ctypes.byref(n_l), capi.ctypes.byref(t_l))
        kt[name] = dict(launches=n_l.value, total_ms=round(t_l.value, 3))
    ctx._chk(L.hfx_profile_enable(ctx.h, 0), "profile")
    step_s = dev_ms / 1e3 / args.steps
    return {"metric": "element assembly + condensation + scatter; elements/s", "value": ctx.nCells / step_s,
            "unit": "elements/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if asm_prec == capi.PREC_FP64 else "tf32x3+f32+f64",
            "data": "synthetic", "config": {"workload": cfg["desc"], "elements": ctx.nCells,
                                            "precision": args.precision, "assembly_path": args.assembly_path},
            "tensor_cores": ctx.mixed_assembly_info() if asm_prec != capi.PREC_FP64 else 0, "kernel_ms": kt}


def burgers_initial(coords, cells, seed=0):
    """u0 = sin(2 pi x) sin(2 pi y) + N(0, 0.01) (seeded), the same field on both components."""
    x = coords[cells]
    u0 = np.sin(2 * np.pi * x[..., 0]) * np.sin(2 * np.pi * x[..., 1])
    u = np.stack([u0, u0], -1) + np.random.default_rng(seed).normal(0.0, 0.01, size=x.shape)
    return u.reshape(cells.shape[0], -1)


def burgers_flops_per_element(N, NF, F, NI, NIF, D=2, cached=False):
    """FP64 operations the Burgers element kernel executes per element (its loops);
    cached: a linearisation that loads the state-independent blocks (M, M^-1 C, M^-1 E,
    tau masses, H, the Schur products) instead of computing them."""
    ND, NT = D, D * D
    NU, NQ, NLF = N * ND, D * N * ND, NF * ND
    NL = F * NLF
    W = NU + NL + 1
    ops = 2 * NI * D * D * N + 2 * NI * N * D * D                     # G; (Ds at the IPs)
    ops += 2 * NI * N * D * D                                            # Ds G
    face_state = F * NIF * (4 * ND * NF + 4 * D)                         # u, t at the face IPs, t.n
    face_static = F * NIF * (2 * NT * NF + 2 * D * D * NF)               # tau, Ds n at the face IPs
    ops += face_state + face_static
    ops += 2 * NI * N * ND + 2 * NI * N * D + NI * N * (2 * D + 3 + 2 * ND)  # u, div u, AQ, BQ
    t1 = N * N * NI * 2
    scalar_static = N * N * NI * (2 + 4 * D)                             # M, C_k, K'_k
    ehT = F * NF * NF * NIF * (4 * D + 2 * NT)                           # E, H, tau masses
    ops += t1 + scalar_static + ehT
    ops += F * NLF * NLF * NIF * 6 + NU * NU * (2 * NI + 2)             # convection blocks
    minv = sum(2 * (N - 1) * (2 * N - k - 1) + (2 * N - k - 1) for k in range(N))  # M^-1 (Gauss-Jordan)
    mcme = 2 * D * N * N * N + 2 * D * N * F * NF * NF                  # M^-1 C, M^-1 E
    kmke = 2 * D * N * (N * N + N * F * NF)                             # sum_k K' M^-1 C, K' M^-1 E
    ops += minv + mcme + kmke
    ops += NU * NU * 6 + NU * NL * 6 + NU * (2 * NU + 2 * NL + 2 * NI + 2 * N)  # [A | -B | Fu]
    ops += sum(2 * (NU - 1) * (W - k - 1) + (W - k - 1) for k in range(NU))  # Gauss-Jordan
    hmce = 2 * NF * D * (F * NF * N + F * NF * F * NF)                  # H M^-1 C, H M^-1 E
    ops += hmce
    ops += NL * (NL + 1) * (2 * NF * ND + 2 * N)                         # S (Q is not formed)
    if cached:
        ops -= (2 * NI * D * D * N + 2 * NI * N * D * D + face_static + scalar_static + ehT + minv + mcme + kmke
                + hmce)
    return ops


def run_burgers(args, world, rank, local):
    import torch
    from hyperfox_gb300 import capi
    torch.cuda.set_device(local)
    cfg = CONFIGS[args.config]
    p = cfg["order"]
    t0 = time.time()
    coords, cells = make_problem(cfg)
    ctx = capi.Context(local)
    ctx.upload_mesh(2, p, coords, cells)
    B = capi.Burgers(ctx)
    Nf = ctx.re["nNodesFace"]
    tau = np.zeros((ctx.nFaces, Nf, 2, 4))
    tau[..., 0] = tau[..., 3] = 1.0                  # tau = I on both sides (TestHDGBurgers.cpp:290-297)
    B.set_tau(tau, 2)
    B.set_diffusion(np.full((coords.shape[0], 1), cfg["nu"]), layout=0)
    B.set_dirichlet(np.zeros((ctx.nFaces, Nf, 2)))  # u0 vanishes on the boundary
    B.set_time_step(cfg["dt"])
    u0 = burgers_initial(coords, cells)
    t_setup = time.time() - t0
    L = ctx.L
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    sol_h = pin(u0.shape)
    sol_h[:] = u0

    starts = {"zero": (0, 0), "warm": (1, 0), "history": (1, 6)}  # (warm_start, history)

    def newton(mode):
        ws, hist = starts[mode]
        o = capi.newton_opts(res_tol=1e-6, max_iters=20, warm_start=ws, history=hist, lin_rtol=1e-10,
                             lin_precond=capi.PC_BLOCK_JACOBI, lin_maxits=20000)
        info = capi.NewtonInfo()
        ctx._chk(L.hfx_burgers_newton(ctx.h, capi.ctypes.byref(o), capi.ctypes.byref(info)), "burgers_newton")
        return info

    steps = args.steps if args.steps_given else cfg["time_steps"] - args.warmup
    warm = args.krylov_start
    B.set_state(solution=u0, trace=np.zeros(B.ndofs))
    for _ in range(args.warmup):
        ctx._chk(L.hfx_burgers_begin_step(ctx.h), "begin_step")
        newton(warm)
    barrier(world)
    ctx._chk(L.hfx_synchronize(ctx.h), "sync")
    clocks = ClockSampler(local)
    clocks.start()
    ctx._chk(L.hfx_profile_enable(ctx.h, 1), "profile")
    ctx._chk(L.hfx_mark(ctx.h, 0), "mark")
    its, kits = [], []
    for _ in range(steps):
        ctx._chk(L.hfx_burgers_begin_step(ctx.h), "begin_step")
        info = newton(warm)
        its.append(info.iterations)
        kits.append(info.krylov_iterations)
    ctx._chk(L.hfx_mark(ctx.h, 1), "mark")
    ms = capi.ctypes.c_double()
    ctx._chk(L.hfx_elapsed_ms(ctx.h, 0, 1, capi.ctypes.byref(ms)), "elapsed")
    clk = clocks.stop()
    dev_ms = barrier_max(world, ms.value)
    kt = {}
    for name, kid in (("local", 0), ("scatter", 1), ("spmv64", 2), ("update", 4), ("recover", 5), ("other", 6)):
        n_l, t_l = capi.ctypes.c_int(), capi.ctypes.c_double()
        L.hfx_kernel_time(ctx.h, kid, capi.ctypes.byref(n_l), capi.ctypes.byref(t_l))
        kt[name] = (n_l.value, t_l.value)
    ctx._chk(L.hfx_profile_enable(ctx.h, 0), "profile")
    # the Krylov starts compared: five steps from the same state with each other choice
    sol_keep, _, trace_keep, _ = B.get_state()
    alt = {}
    for mode in starts:
        if mode == warm:
            continue
        B.set_state(solution=sol_keep, trace=trace_keep)
        infos = []
        for _ in range(5):
            ctx._chk(L.hfx_burgers_begin_step(ctx.h), "begin_step")
            infos.append(newton(mode))
        alt[mode] = infos
    B.set_state(solution=sol_keep, trace=trace_keep)
    # e2e: the step's Solution uploaded from pinned host memory and downloaded after the Newton loop
    barrier(world)
    ctx._chk(L.hfx_synchronize(ctx.h), "sync")
    e2e_steps = min(steps, 20)
    e2e_its = 0
    t1 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx._chk(L.hfx_burgers_set_state(ctx.h, capi._p(sol_h), None, None, None), "set_state")
        ctx._chk(L.hfx_burgers_begin_step(ctx.h), "begin_step")
        e2e_its += newton(warm).iterations
        ctx._chk(L.hfx_burgers_get_state(ctx.h, capi._p(sol_h), None, None, None), "get_state")
    e2e_s = barrier_max(world, time.perf_counter() - t1)
    E = ctx.nCells
    step_s = dev_ms / 1e3 / steps
    re = ctx.re
    # the timed linearisations load the state-independent blocks (stored by the first one)
    flops = burgers_flops_per_element(re["nNodes"], Nf, re["nFaces"], re["nIP"], re["nIPFace"], cached=True)
    avg_ms = kt["local"][1] / max(1, kt["local"][0])
    tf = flops * E / (avg_ms / 1e3) / 1e12
    roof = dict(bound="fp64", kernel="burgers_local<2,3> (FP64 assembly + condensation, vector Burgers, "
                                     "state-independent blocks from the per-element cache)",
                achieved=round(tf, 3), peak=FP64_NOMINAL_TFLOPS, unit="TFLOP/s", frac=round(tf / FP64_NOMINAL_TFLOPS, 4),
                traffic=args.traffic,  # no ncu capture of the current kernel (the committed one still formed Q)
                flops_per_element=int(flops), avg_launch_ms=round(avg_ms, 4),
                peak_source="nominal GB300 FP64 (no measured FP64 peak)")
    nl = sum(its)
    res = {
        "metric": BURGERS_METRIC,
        "value": E * sum(its) / (dev_ms / 1e3),
        "unit": "elements*newton_iterations/s",
        "elements_steps_per_s": E * steps / (dev_ms / 1e3),
        "n_gpus": world, "steps": steps, "warmup": args.warmup,
        "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (structured mesh, seeded initial noise N(0, 0.01) on both components)",
        "config": {"workload": cfg["desc"], "elements": E, "order": p, "trace_dofs": B.ndofs, "csr_nnz": B.nnz,
                   "krylov": "GMRES(30) + per-face block Jacobi, FP64, rtol 1e-10",
                   "krylov_start": {"zero": "zero (PETSc default)", "warm": "previous trace (warm)",
                                    "history": "least-squares fit of the last 6 trace solutions"}[warm],
                   "l2_flush": "none: inputs (element blocks 1.1 GB) exceed L2", "parallelism": "single GPU"},
        "newton_iterations_per_step": nl / steps,
        "krylov_iterations_per_newton": sum(kits) / max(1, nl),
        "other_krylov_starts": {mode: {"newton_iterations_per_step": sum(a.iterations for a in v) / len(v),
                                       "krylov_iterations_per_newton": sum(a.krylov_iterations for a in v) /
                                       max(1, sum(a.iterations for a in v)),
                                       "assemble_plus_solve_ms_per_step": sum(a.assemble_ms + a.solve_ms for a in v) / len(v)}
                                for mode, v in alt.items()},
        "element_kernel_elements_per_s": E / (avg_ms / 1e3),
        "kernel_ms": {k: dict(launches=v[0], total_ms=round(v[1], 3)) for k, v in kt.items()},
        "roofline": roof,
        "clocks": clk,
        "e2e": {"value": E * e2e_its / e2e_s, "unit": "elements*newton_iterations/s",
                "h2d_bytes_per_step": int(sol_h.nbytes), "d2h_bytes_per_step": int(sol_h.nbytes)},
        "gpu_launches": int(sum(v[0] for v in kt.values())),
        "setup_s": t_setup,
    }
    return res, ctx


def run_batch(args, world, rank, local):
    """configs with batch=...: the uneven batch through hyperfox_gb300.batch, one context per
    order; a step = every group's assembly, Krylov solve (CG, every problem's own relative
    residual <= rtol) and recovery; the order groups run at once, each from its own host thread
    on its own context and stream (--batch-serial: one after another)."""
    import torch
    from hyperfox_gb300 import batch as hb, capi
    torch.cuda.set_device(local)
    cfg = CONFIGS[args.config]
    t0 = time.time()
    # N > 1: the problems are split across the ranks by cost (every rank computes the same
    # split), no data-path collective; the job is the whole batch at any N
    bcfg = cfg["batch"]
    plan = hb.uneven_plan(**{k: bcfg[k] for k in ("count", "seed", "min_elements", "max_elements", "orders")
                             if k in bcfg})
    mine = hb.shard([hb.problem_cost(n, q) for n, q, _ in plan], world)[rank] if world > 1 else None
    E_all = sum(2 * n * n for n, _, _ in plan)
    probs = hb.uneven_batch(**bcfg, select=mine)
    B = hb.Batch(probs, local, capi.SRC_SINPROD, 2 * np.pi ** 2)
    t_setup = time.time() - t0
    L = capi.load()
    # kappa constant per cell: symmetric trace systems, CG; precision and preconditioner as
    # for the single-problem workloads (the coarse solve Chebyshev: no per-group training)
    prec = capi.PREC_FP64 if args.precision == "fp64" else capi.PREC_MIXED
    pc = capi.PC_TWOLEVEL if args.precond == "twolevel" else capi.PC_BLOCK_JACOBI
    # fixed Chebyshev degree (--coarse-degree, default 32; 0: the degree coarse_rtol asks for on the
    # union's spectrum: about as fast, but with fewer, costlier iterations)
    opts = dict(precision=prec, precond=pc, maxits=200000, inner_rtol=args.inner_rtol, coarse_rtol=args.coarse_rtol,
                coarse_mode=capi.COARSE_CHEBYSHEV, coarse_degree=args.coarse_degree)
    pin = lambda shape: torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    bufs = B.host_buffers(alloc=pin)
    for g in B.groups.values():  # pinned copies of the per-step inputs
        g.tau, g.dirichlet = _pinned(pin, g.tau), _pinned(pin, g.dirichlet)
        if g.kappa is not None:
            g.kappa = _pinned(pin, g.kappa)
    conc = not args.batch_serial
    for _ in range(args.warmup):
        B.run(args.rtol, concurrent=conc, **opts)
    barrier(world)
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    step_ms = []
    for _ in range(args.steps):
        ms = B.run(args.rtol, concurrent=conc, **opts)
        # concurrent: first group's start to last group's end; serial: the groups' own times
        step_ms.append(B.span_ms if conc else sum(ms.values()))
    clk = clocks.stop()
    torch.cuda.synchronize()
    dev_ms = barrier_max(world, sum(step_ms))
    # per-kernel times from a second pass of the same steps, groups in sequence, with the
    # event timer on (its events would otherwise add host work to the timed region, and
    # kernels of overlapping groups would share their event intervals)
    for g in B.groups.values():
        g.ctx._chk(L.hfx_profile_enable(g.ctx.h, 1), "profile")
    prof_ms = 0.0
    for _ in range(args.steps):
        prof_ms += sum(B.run(args.rtol, **opts).values())
    kt = {}
    names = (("local", 0), ("scatter", 1), ("spmv64", 2), ("spmv32", 3), ("update", 4), ("recover", 5),
             ("other", 6), ("residual", 7), ("coarse", 8))
    # algorithmic bytes of the trace SpMV launches that did work (one per Krylov iteration;
    # launches queued after convergence return at entry), summed over the groups
    spmv_alg = {"spmv64": 0.0, "spmv32": 0.0}
    spmv_n = {"spmv64": 0, "spmv32": 0}
    for q, g in B.groups.items():
        c = g.ctx
        its = B.infos[q].iterations
        for name, kid in names:
            n_l, t_l = capi.ctypes.c_int(), capi.ctypes.c_double()
            L.hfx_kernel_time(c.h, kid, capi.ctypes.byref(n_l), capi.ctypes.byref(t_l))
            a = kt.setdefault(name, [0, 0.0])
            a[0] += n_l.value
            a[1] += t_l.value
            if name in spmv_alg and n_l.value:
                Nf = g.nf
                nblocks = c.nnz // (Nf * Nf)
                if name == "spmv32":  # upper block triangle in fixed-width rows of (column, location) slots
                    alg = ((nblocks - c.nFaces) // 2 + c.nFaces) * Nf * Nf * 4 + c.nFaces * 5 * 8 + 4 * c.ndofs * 4
                else:  # values, block columns, row pointers once; z, p_old gathered, p_new, q written
                    alg = c.nnz * 8 + nblocks * 4 + (c.nFaces + 1) * 8 + 4 * c.ndofs * 8
                launches = min(n_l.value, its * args.steps) if its else n_l.value
                spmv_alg[name] += launches * alg
                spmv_n[name] += launches
        c._chk(L.hfx_profile_enable(c.h, 0), "profile")
    infos = {q: dict(iterations=i.iterations, rel_residual=i.rel_residual) for q, i in B.infos.items()}
    # e2e: field uploads from pinned host buffers, downloads of Trace, Solution, Flux
    B.step(args.rtol, bufs, concurrent=conc, **opts)  # untimed warm-up of the host-buffer path
    barrier(world)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        B.step(args.rtol, bufs, concurrent=conc, **opts)
    torch.cuda.synchronize()
    e2e_s = barrier_max(world, time.perf_counter() - t1)
    h2d = sum(g.tau.nbytes + g.dirichlet.nbytes + (g.kappa.nbytes if g.kappa is not None else 0)
              for g in B.groups.values())
    d2h = sum(a.nbytes for b in bufs.values() for a in b)
    # accuracy: every problem's trace against an FP64 solve of its group to 1e-12 of the
    # group's right-hand side (untimed)
    tr = [t.copy() for t, _, _ in B.results()]
    worst = None
    try:
        B.solve(group_rtol=1e-12, **dict(opts, precision=capi.PREC_FP64))
        worst = max(float(np.linalg.norm(a - b[0]) / max(np.linalg.norm(b[0]), 1e-300))
                    for a, b in zip(tr, B.results()))
    except capi.HfxError as e:  # reported, not required
        worst = "reference solve: %s" % e
    E = E_all
    step_s = dev_ms / 1e3 / args.steps
    hbm, peak_kind = peaks()
    key = max(("spmv32", "spmv64"), key=lambda k: kt[k][1])
    roof = None
    if spmv_n[key]:
        ach = spmv_alg[key] / (kt[key][1] / 1e3) / 1e9
        roof = dict(bound="hbm", kernel=("cg_spmv_half_ell<float>" if key == "spmv32" else "cg_spmv<double>")
                    + " (all order groups)", achieved=round(ach, 1), peak=hbm, unit="GB/s",
                    frac=round(ach / hbm, 4), traffic=None, bytes_per_launch=int(spmv_alg[key] / spmv_n[key]),
                    avg_launch_ms=round(kt[key][1] / spmv_n[key], 4),
                    share_of_step=round(kt[key][1] / max(prof_ms, 1e-9), 3), peak_source=peak_kind)
    from collections import Counter
    per_order = Counter()
    for n, q, _ in plan:
        per_order[q] += 2 * n * n
    res = {
        "metric": METRIC, "value": E / step_s, "unit": "elements/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "strong",
        "vs_baseline": None, "dtype": "f64+f32" if prec else "f64",
        "data": "synthetic (seeded meshes, fields and orders)",
        "config": {"workload": cfg["desc"], "problems": len(plan), "elements": E,
                   "rank0_problems": len(probs), "rank0_elements": B.nCells,
                   "elements_per_order": {str(k): v for k, v in sorted(per_order.items())},
                   "trace_dofs": int(sum(g.ctx.ndofs for g in B.groups.values())),
                   "precision": args.precision,
                   "preconditioner": (("two-level: per-face block Jacobi + vertex coarse space (Chebyshev, %s)"
                                       % ("degree %d" % args.coarse_degree if args.coarse_degree > 0
                                          else "adaptive degree"))
                                      if pc == capi.PC_TWOLEVEL else "block-Jacobi (per face)"),
                   "krylov": "CG (symmetric trace systems)",
                   "rtol": args.rtol, "rtol_per_problem": True,
                   "group_tolerances": {str(q): g.tol for q, g in B.groups.items()},
                   "l2_flush": "inputs > L2 (no flush needed)",
                   "parallelism": ("problems split across %d ranks by cost, no collective" % world)
                                  if world > 1 else "single GPU",
                   "timing": ("CUDA events on every order group's stream around its work; the groups run at "
                              "once from one host thread each, a step is the first start to the last end"
                              if conc else "CUDA events on every order group's stream around its work, groups "
                              "in sequence")},
        "time_to_solve_s": step_s,
        "group_ms_alone": {str(q): round(v, 3) for q, v in B.run(args.rtol, **opts).items()},
        "krylov": {str(q): v for q, v in infos.items()},
        "max_rel_err_vs_fp64": worst,
        "kernel_ms": {k: dict(launches=v[0], total_ms=round(v[1], 3)) for k, v in kt.items()},
        "roofline": roof, "clocks": clk,
        "e2e": {"value": E * args.steps / e2e_s, "unit": "elements/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h)},
        "gpu_launches": int(sum(v[0] for v in kt.values())),
        "setup_s": t_setup,
    }
    return res, B


def _pinned(pin, a):
    out = pin(a.shape)
    np.copyto(out, a)
    return out


def batch_cpu_sample(cfg_name, nthreads, rtol):
    """The oracle on a bounded sample of the batch: its problems in order until the
    config's cpu_budget elements, each solved alone (as the reference runs one problem per Mesh) with
    GMRES(30)+Jacobi to rtol; assemble + condense + scatter + solve + recover."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    from hyperfox_gb300 import batch as hb
    cfg = CONFIGS[cfg_name]
    budget = cfg["cpu_budget"]
    probs = hb.uneven_batch(**dict(cfg["batch"], count=min(cfg["batch"]["count"], 64)))
    take, tot = [], 0
    for p in probs:
        if tot + p.nCells > budget and take:
            continue
        take.append(p)
        tot += p.nCells
        if tot >= budget:
            break
    dt, its = 0.0, 0
    for p in take:
        P = O.Problem(2, p.order, p.coords, p.cells)
        P.set_fields(p.tau.ravel(), kappa=p.kappa.ravel(), src_mode=2, dirichlet=p.dirichlet.ravel())
        t0 = time.perf_counter()
        P.assemble(nthreads)
        x, it = P.solve_gmres(rtol, 200000, nthreads)
        P.recover(x)
        dt += time.perf_counter() - t0
        its += abs(it)
    return dict(value=tot / dt, unit="elements/s", cores=nthreads, kind="port",
                sample="%d of the batch's problems (%d elements, orders %s), each alone: oracle assemble+condense"
                       "+scatter, GMRES(30)+Jacobi to %g (%d its in all), recovery"
                       % (len(take), tot, sorted({p.order for p in take}), rtol, its), seconds=dt)


def burgers_cpu_sample(cfg_name, nthreads, n=64):
    """The oracle (HDGBurgersModel restatement, dense LU condensation, GMRES(30)+Jacobi)
    on a bounded sample: the second implicit Euler step of the same physics on an
    n x n x 2 mesh (the first, untimed, gives the timed one a trace to start from, as
    the GPU arm's timed steps have)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    from hyperfox_gb300 import meshgen
    cfg = CONFIGS[cfg_name]
    p = cfg["order"]
    re = O.RefEl(2, p)
    v, s = meshgen.square_simplices(n)
    coords, cells = meshgen.high_order(v, s, re.nodes)
    P = O.BurgersProblem(2, p, coords, cells)
    tau = np.zeros((P.nFaces, re.nNodesFace, 2, 4))
    tau[..., 0] = tau[..., 3] = 1.0
    nu = np.full((P.nCells, re.nNodes, 1), cfg["nu"])
    zero = np.zeros((P.nFaces, re.nNodesFace, 2))
    u = burgers_initial(coords, cells)
    P.trace = np.zeros(P.ndofs)
    for step in range(2):
        P.set_fields(tau=tau, tau_sides=2, nu=nu, dirichlet=zero, dt=cfg["dt"], old=u)
        P.buf = u.copy()
        t0 = time.perf_counter()
        its = kits = 0
        for _ in range(20):
            P.set_state(P.buf, P.trace)
            P.assemble(nthreads)
            x, k = P.solve_gmres(1e-10, 200000, nthreads)
            sol, _ = P.recover(x)
            P.trace = x
            its += 1
            kits += abs(k)
            diff, ref = float(np.sum((sol - P.buf) ** 2)), float(np.sum(P.buf ** 2))
            if np.sqrt(diff / ref) < 1e-6:
                break
            P.buf = sol
        dt = time.perf_counter() - t0
        u = sol
    return dict(value=P.nCells * its / dt, unit="elements*newton_iterations/s", cores=nthreads, kind="port",
                sample="the second implicit Euler step (Newton %d iterations, %d GMRES(30)+Jacobi iterations, "
                       "Krylov from zero) on %dx%dx2 tris (%d elements, %d trace DOFs): oracle assemble + LU "
                       "condense + scatter + solve + recover" % (its, kits, n, n, P.nCells, P.ndofs), seconds=dt)


def cpu_sample(cfg_name, nthreads, rtol, budget_elems=None):
    """Time the CPU oracle on a bounded sample: a sub-cube of the same workload, solved to
    the same relative residual as the GPU arm."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import _oracle as O
    from hyperfox_gb300 import meshgen
    cfg = CONFIGS[cfg_name]
    dim, p = cfg["dim"], cfg["order"]
    n = cfg.get("cpu_n", {3: 12, 2: 32}[dim]) if budget_elems is None else budget_elems
    n = min(n, cfg["n"])
    re = O.RefEl(dim, p)
    v, s = meshgen.square_simplices(n) if dim == 2 else meshgen.cube_simplices(n)
    coords, cells = meshgen.high_order(v, s, re.nodes)
    P = O.Problem(dim, p, coords, cells)
    g = np.prod(np.sin(np.pi * coords[P.faces]), axis=-1)
    kap = aniso_kappa(coords, cells, dim, **cfg["aniso"]).ravel() if cfg.get("aniso") else None
    if cfg.get("nodal_kappa"):
        kap = nodal_kappa(coords, cells).ravel()
    P.set_fields(np.ones(P.ndofs), kappa=kap, src_mode=2, dirichlet=g.ravel())
    t0 = time.perf_counter()
    P.assemble(nthreads)
    x, it = P.solve_gmres(rtol, 200000, nthreads)
    P.recover(x)
    dt = time.perf_counter() - t0
    return dict(value=P.nCells / dt, unit="elements/s", cores=nthreads, kind="port",
                sample="%s sub-mesh n=%d (%d elements, %d trace DOFs): oracle assemble+condense+scatter, "
                       "GMRES(30)+Jacobi to %g (%d its), recovery" % (cfg_name, n, P.nCells, P.ndofs, rtol, it),
                seconds=dt)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="cfg2", choices=sorted(CONFIGS))
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "mixed-full"],
                    help="mixed: FP64 assembly, FP32 CG with FP64 reliable updates of the trace residual; "
                         "fp64: FP64 throughout; mixed-full: FP32 element condensation inside FP64 "
                         "refinement of the full HDG system")
    ap.add_argument("--rtol", type=float, default=1e-8,
                    help="relative FP64 residual of the trace system (mixed-full: of the full HDG system); "
                         "both arms stop there, and the error against the FP64 solution (rtol 1e-13) is "
                         "reported as rel_err_vs_fp64")
    ap.add_argument("--inner-rtol", type=float, default=1e-2,
                    help="FP32 reduction between FP64 residual replacements (mixed)")
    ap.add_argument("--precond", default="twolevel", choices=["twolevel", "bj"],
                    help="two-level (block Jacobi + vertex coarse space) or block Jacobi alone")
    ap.add_argument("--coarse-guess", action="store_true", help="start CG from the prolongated coarse solution")
    ap.add_argument("--coarse-rtol", type=float, default=0.3, help="Chebyshev coarse-solve reduction target")
    ap.add_argument("--coarse", default="learned", choices=["learned", "chebyshev"],
                    help="coarse solve of the two-level preconditioner: trained polynomial or Chebyshev")
    ap.add_argument("--coarse-degree", type=int, default=None,
                    help="degree of the learned coarse polynomial (default 8); the batch workload: of its "
                         "Chebyshev coarse solve (default 32; 0 = the degree --coarse-rtol asks for)")
    ap.add_argument("--assembly-path", type=int, default=0, choices=[0, 1],
                    help="element kernel choice (hfx_set_assembly_path): 0 automatic (affine kernel, or the "
                         "tensor-core contractions in the mixed assembly), 1 quadrature on the CUDA cores")
    ap.add_argument("--assembly-only", action="store_true",
                    help="time the element assembly (+ condensation + scatter) alone")
    ap.add_argument("--spmv-kernel", type=int, default=-1, choices=[-1, 0, 1, 2, 3],
                    help="FP32 trace operator kernel (hfx_set_tuning): -1 timed per system by the launch "
                         "tuner, else 0 row per lane, 1 blocks staged by bulk copies, 2 paired loads, "
                         "3 paired loads and float4 reads of the gathered x")
    ap.add_argument("--batch-serial", action="store_true",
                    help="batch workloads: the order groups one after another instead of at once")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--traffic", type=float, default=None, help="ncu DRAM bytes per launch of the top kernel")
    ap.add_argument("--krylov-start", default="history", choices=["zero", "warm", "history"],
                    help="Burgers: Krylov initial guess: zero (PETSc), the previous trace, or the least-squares "
                         "fit of the last 6 trace solutions")
    args = ap.parse_args()
    args.steps_given = args.steps is not None
    if args.steps is None:
        args.steps = 5
    world, rank, local = dist_init()
    burgers = CONFIGS[args.config].get("burgers", False)
    is_batch = "batch" in CONFIGS[args.config]
    if is_batch and not args.steps_given:
        args.steps = 3
    if args.coarse_degree is None:
        args.coarse_degree = 32 if is_batch else 8
    if is_batch and args.impl == "reference":
        if rank != 0:
            return
        nthreads = os.cpu_count() or 1
        vals = []
        for i in range(args.warmup + args.steps):
            r = batch_cpu_sample(args.config, nthreads, args.rtol)
            if i >= args.warmup:
                vals.append(r["value"])
        v = statistics.median(vals)
        out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "elements/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": {"workload": CONFIGS[args.config]["desc"]}, "cpu_baseline": dict(r, value=v),
               "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return
    if is_batch:
        res, B = run_batch(args, world, rank, local)
        if rank == 0:
            if not args.no_cpu:
                try:
                    res["cpu_baseline"] = batch_cpu_sample(args.config, os.cpu_count() or 1, args.rtol)
                except Exception as e:  # the baseline is reported, not required
                    res["cpu_baseline"] = {"error": str(e)}
            print(json.dumps(res))
        B.close()
        return
    if args.impl == "reference" and burgers:
        if rank != 0:
            return
        nthreads = os.cpu_count() or 1
        vals = []
        for i in range(args.warmup + args.steps):
            r = burgers_cpu_sample(args.config, nthreads)
            if i >= args.warmup:
                vals.append(r["value"])
        v = statistics.median(vals)
        out = {"impl": "reference", "metric": BURGERS_METRIC, "value": v, "unit": "elements*newton_iterations/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": {"workload": CONFIGS[args.config]["desc"]}, "cpu_baseline": dict(r, value=v),
               "e2e": {"value": v, "unit": "elements*newton_iterations/s", "h2d_bytes_per_step": 0,
                       "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return
    if burgers:
        res, ctx = run_burgers(args, world, rank, local)
        if rank == 0:
            if not args.no_cpu:
                try:
                    res["cpu_baseline"] = burgers_cpu_sample(args.config, os.cpu_count() or 1)
                except Exception as e:  # the baseline is reported, not required
                    res["cpu_baseline"] = {"error": str(e)}
            print(json.dumps(res))
        ctx.close()
        return
    if args.impl == "reference":
        if rank != 0:
            return
        nthreads = os.cpu_count() or 1
        vals = []
        for i in range(args.warmup + args.steps):
            r = cpu_sample(args.config, nthreads, args.rtol)
            if i >= args.warmup:
                vals.append(r["value"])
        v = statistics.median(vals)
        out = {"impl": "reference", "metric": METRIC, "value": v, "unit": "elements/s", "n_gpus": world,
               "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic",
               "config": {"workload": CONFIGS[args.config]["desc"]},
               "cpu_baseline": dict(r, value=v),
               "e2e": {"value": v, "unit": "elements/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return
    res, ctx = run_ours(args, world, rank, local)
    if rank == 0:
        if not args.no_cpu:
            try:
                res["cpu_baseline"] = cpu_sample(args.config, os.cpu_count() or 1, args.rtol)
                # one thread, as the reference runs per MPI rank (no threading in its element loop)
                res["cpu_baseline_1t"] = cpu_sample(args.config, 1, args.rtol,
                                                    budget_elems=8 if CONFIGS[args.config]["dim"] == 3 else None)
            except Exception as e:  # the baseline is reported, not required
                res["cpu_baseline"] = {"error": str(e)}
        print(json.dumps(res))
    ctx.close()


if __name__ == "__main__":
    main()
