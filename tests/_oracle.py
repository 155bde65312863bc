"""ctypes bindings of the CPU oracle (oracle/hdg_oracle.cpp).

Test infrastructure only: the oracle is what the CUDA path is compared with,
never the thing measured or shipped.
"""
import ctypes
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(ROOT, "oracle", "_build", "libhdg_oracle.so")
SRC_PATH = os.path.join(ROOT, "oracle", "hdg_oracle.cpp")

_lib = None


def build():
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if (not os.path.exists(LIB_PATH)) or os.path.getmtime(LIB_PATH) < os.path.getmtime(SRC_PATH):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-pthread",
                               SRC_PATH, "-o", LIB_PATH])
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        L.orc_last_error.restype = ctypes.c_char_p
        L.orc_refel_sizes.argtypes = [ip, ip, vp]
        L.orc_refel_tables.argtypes = [ip, ip] + [vp] * 6
        L.orc_refel_eval.argtypes = [ip, ip, ip, vp, vp, vp]
        L.orc_cubature.argtypes = [ip, ip, vp, vp, ip]
        L.orc_problem_create.restype = vp
        L.orc_problem_create.argtypes = [ip, ip, ip, vp, ip, vp]
        L.orc_problem_destroy.argtypes = [vp]
        L.orc_problem_face_counts.argtypes = [vp, vp]
        L.orc_problem_faces.argtypes = [vp] * 5
        L.orc_problem_set_fields.argtypes = [vp, vp, ip, vp, ip, ip, vp, vp, dp, vp]
        L.orc_problem_ip_coords.argtypes = [vp, vp]
        L.orc_problem_local.argtypes = [vp, ip, ip, ip]
        L.orc_problem_assemble.argtypes = [vp, ip]
        L.orc_problem_local_matrix.argtypes = [vp, ip, vp, vp, vp]
        L.orc_problem_condensed.argtypes = [vp] * 7
        L.orc_problem_sample.argtypes = [vp, ip, ip, vp] + [vp] * 6
        L.orc_problem_cg_operators.argtypes = [vp, ip, vp, vp]
        L.orc_problem_face_rows.restype = ctypes.c_long
        L.orc_problem_face_rows.argtypes = [vp, ip, ip, vp, vp, vp, vp, vp, ctypes.c_long]
        L.orc_problem_nnz.restype = ctypes.c_long
        L.orc_problem_nnz.argtypes = [vp]
        L.orc_problem_csr.argtypes = [vp] * 5
        L.orc_problem_solve.argtypes = [vp, dp, ip, ip, vp]
        L.orc_problem_recover.argtypes = [vp] * 4
        L.orc_problem_timings.argtypes = [vp, vp]
        L.orc_problem_set_solver.argtypes = [vp, ip, vp, vp]
        L.orc_problem_solve_faces.argtypes = [vp, vp]
        L.orc_problem_set_rk.argtypes = [vp, dp, dp] + [vp] * 6
        L.orc_rk_apply.argtypes = [ip, ip, vp, vp, vp, vp, vp, dp, dp]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle: " + lib().orc_last_error().decode())


def cubature(dim, order):
    X = np.zeros((200, dim))
    W = np.zeros(200)
    n = lib().orc_cubature(dim, order, _ptr(X), _ptr(W), 200)
    if n < 0:
        raise RuntimeError("oracle cubature(%d, %d) failed" % (dim, order))
    return X[:n].copy(), W[:n].copy()


class RefEl:
    def __init__(self, dim, order):
        L = lib()
        s = np.zeros(5, dtype=np.int32)
        _check(L.orc_refel_sizes(dim, order, _ptr(s)))
        self.dim, self.order = dim, order
        self.nNodes, self.nFaces, self.nNodesFace, self.nIP, self.nIPFace = (int(v) for v in s)
        N, F, Nf, nI = self.nNodes, self.nFaces, self.nNodesFace, self.nIP
        self.nodes = np.zeros((N, dim))
        self.faceNodes = np.zeros((F, Nf), dtype=np.int32)
        self.ipX = np.zeros((nI, dim))
        self.ipW = np.zeros(nI)
        self.phi = np.zeros((nI, N))
        self.dphi = np.zeros((nI, N, dim))
        _check(L.orc_refel_tables(dim, order, _ptr(self.nodes), _ptr(self.faceNodes), _ptr(self.ipX),
                                  _ptr(self.ipW), _ptr(self.phi), _ptr(self.dphi)))

    def eval(self, pts):
        pts = np.ascontiguousarray(pts, dtype=np.float64).reshape(-1, self.dim)
        phi = np.zeros((pts.shape[0], self.nNodes))
        dphi = np.zeros((pts.shape[0], self.nNodes, self.dim))
        _check(lib().orc_refel_eval(self.dim, self.order, pts.shape[0], _ptr(pts), _ptr(phi), _ptr(dphi)))
        return phi, dphi


class Problem:
    """One HDG diffusion-source problem on the oracle."""

    def __init__(self, dim, order, coords, cells):
        L = lib()
        self.dim, self.order = dim, order
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.cells = np.ascontiguousarray(cells, dtype=np.int32)
        self.h = L.orc_problem_create(dim, order, self.coords.shape[0], _ptr(self.coords),
                                      self.cells.shape[0], _ptr(self.cells))
        if not self.h:
            raise RuntimeError("oracle: " + L.orc_last_error().decode())
        self.re = RefEl(dim, order)
        c = np.zeros(2, dtype=np.int32)
        L.orc_problem_face_counts(self.h, _ptr(c))
        self.nFaces, self.nBoundary = int(c[0]), int(c[1])
        F, Nf = self.re.nFaces, self.re.nNodesFace
        nC = self.cells.shape[0]
        self.cell2face = np.zeros((nC, F), dtype=np.int32)
        self.face2cell = np.zeros((self.nFaces, 2), dtype=np.int32)
        self.faces = np.zeros((self.nFaces, Nf), dtype=np.int32)
        self.boundary = np.zeros(self.nBoundary, dtype=np.int32)
        L.orc_problem_faces(self.h, _ptr(self.cell2face), _ptr(self.face2cell), _ptr(self.faces),
                            _ptr(self.boundary))
        self.nCells = nC
        self.lenU = self.re.nNodes
        self.lenQ = dim * self.re.nNodes
        self.lenL = F * Nf
        self.ndofs = self.nFaces * Nf

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_problem_destroy(self.h)
            self.h = None

    def ip_coords(self):
        out = np.zeros((self.nCells, self.re.nIP, self.dim))
        lib().orc_problem_ip_coords(self.h, _ptr(out))
        return out

    def set_fields(self, tau, kappa=None, src_mode=0, src=None, dirichlet=None, dt=0.0, u_old=None):
        tau = np.ascontiguousarray(tau, dtype=np.float64)
        tau_vals = tau.size // (self.nFaces * self.re.nNodesFace)
        kc = 0
        if kappa is not None:
            kappa = np.ascontiguousarray(kappa, dtype=np.float64)
            kc = kappa.size // (self.nCells * self.re.nNodes)
        src = None if src is None else np.ascontiguousarray(src, dtype=np.float64)
        dirichlet = None if dirichlet is None else np.ascontiguousarray(dirichlet, dtype=np.float64)
        u_old = None if u_old is None else np.ascontiguousarray(u_old, dtype=np.float64)
        self._keep = (tau, kappa, src, dirichlet, u_old)
        _check(lib().orc_problem_set_fields(self.h, _ptr(tau), tau_vals, _ptr(kappa), kc, src_mode,
                                            _ptr(src), _ptr(dirichlet), float(dt), _ptr(u_old)))

    def local(self, nthreads=1, first=0, count=0):
        _check(lib().orc_problem_local(self.h, nthreads, first, count))

    def assemble(self, nthreads=1):
        _check(lib().orc_problem_assemble(self.h, nthreads))

    def local_matrix(self, iel):
        n = self.lenU + self.lenQ + self.lenL
        A = np.zeros((n, n), order="F")
        r = np.zeros(n)
        f2c = np.zeros(self.lenL, dtype=np.int32)
        _check(lib().orc_problem_local_matrix(self.h, iel, A.ctypes.data, _ptr(r), _ptr(f2c)))
        return A, r, f2c

    def condensed(self):
        nC, U, Q, L_ = self.nCells, self.lenU, self.lenQ, self.lenL
        S = np.zeros((nC, L_ * L_))
        S0 = np.zeros((nC, L_))
        Um = np.zeros((nC, U * L_))
        Qm = np.zeros((nC, Q * L_))
        U0 = np.zeros((nC, U))
        Q0 = np.zeros((nC, Q))
        lib().orc_problem_condensed(self.h, _ptr(S), _ptr(S0), _ptr(Um), _ptr(Qm), _ptr(U0), _ptr(Q0))
        return dict(S=S, S0=S0, U=Um, Q=Qm, U0=U0, Q0=Q0)

    def sample(self, ids, nthreads=1):
        """Condensed blocks (Dirichlet Set applied) of the listed elements only."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        n, U, Q, L_ = len(ids), self.lenU, self.lenQ, self.lenL
        out = dict(S=np.zeros((n, L_ * L_)), S0=np.zeros((n, L_)), U=np.zeros((n, U * L_)),
                   Q=np.zeros((n, Q * L_)), U0=np.zeros((n, U)), Q0=np.zeros((n, Q)))
        _check(lib().orc_problem_sample(self.h, nthreads, n, _ptr(ids), *[_ptr(out[k]) for k in
                                                                           ("S", "S0", "U", "Q", "U0", "Q0")]))
        return out

    def cg_operators(self, which=7, velocity=None):
        """CG element operators [nCells][3][N*N] (column-major): Mass, Diffusion (the kappa field
        set with set_fields), Convection (nodal velocity [nCells][N][d])."""
        out = np.zeros((self.nCells, 3, self.lenU * self.lenU))
        v = None if velocity is None else np.ascontiguousarray(velocity, dtype=np.float64)
        _check(lib().orc_problem_cg_operators(self.h, which, _ptr(v), _ptr(out)))
        return out

    def face_rows(self, faces, nthreads=1):
        """The trace-system rows (all nodes) of the listed faces, from their cells only:
        (rowlen, col, val, rhs) with the rows back to back in face, node order."""
        faces = np.ascontiguousarray(faces, dtype=np.int32)
        Nf = self.re.nNodesFace
        nr = len(faces) * Nf
        cap = nr * (2 * self.re.nFaces) * Nf
        rowlen = np.zeros(nr, np.int32)
        col = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        rhs = np.zeros(nr)
        n = lib().orc_problem_face_rows(self.h, nthreads, len(faces), _ptr(faces), _ptr(rowlen), _ptr(col),
                                        _ptr(val), _ptr(rhs), cap)
        if n < 0:
            raise RuntimeError("oracle face_rows: %s" % lib().orc_last_error().decode())
        return rowlen, col[:n], val[:n], rhs

    def csr(self):
        nnz = lib().orc_problem_nnz(self.h)
        rowptr = np.zeros(self.ndofs + 1, dtype=np.int32)
        col = np.zeros(nnz, dtype=np.int32)
        val = np.zeros(nnz)
        rhs = np.zeros(self.ndofs)
        lib().orc_problem_csr(self.h, _ptr(rowptr), _ptr(col), _ptr(val), _ptr(rhs))
        return rowptr, col, val, rhs

    def solve_gmres(self, rtol=1e-12, maxit=20000, nthreads=1):
        x = np.zeros(self.ndofs)
        it = lib().orc_problem_solve(self.h, rtol, maxit, nthreads, _ptr(x))
        return x, it

    def solve_direct(self):
        import scipy.sparse as sp
        import scipy.sparse.linalg as spla
        rowptr, col, val, rhs = self.csr()
        A = sp.csr_matrix((val, col, rowptr), shape=(self.ndofs, self.ndofs))
        return spla.spsolve(A.tocsc(), rhs)

    def recover(self, trace):
        trace = np.ascontiguousarray(trace, dtype=np.float64)
        sol = np.zeros((self.nCells, self.lenU))
        flux = np.zeros((self.nCells, self.lenQ))
        _check(lib().orc_problem_recover(self.h, _ptr(trace), _ptr(sol), _ptr(flux)))
        return sol, flux

    def set_solver(self, type_, sol=None, flux=None):
        """HDGSolverType: 0 IMPLICIT, 1 WEXPLICIT, 2 SEXPLICIT (explicit modes read sol, flux)."""
        sol = None if sol is None else np.ascontiguousarray(sol, dtype=np.float64)
        flux = None if flux is None else np.ascontiguousarray(flux, dtype=np.float64)
        self._keep_state = (sol, flux)
        _check(lib().orc_problem_set_solver(self.h, type_, _ptr(sol), _ptr(flux)))

    def set_rk(self, dt, a_diag=0.0, old=None, comb=None):
        """Runge-Kutta stage on the U rows (RungeKutta::apply): old = (OldSolution,
        OldFlux, OldTrace), comb = sum_{i<s} a_si (RKStage_i, RKStage_Flux_i,
        RKStage_Trace_i); dt <= 0 switches it off."""
        if dt <= 0:
            _check(lib().orc_problem_set_rk(self.h, 0.0, 0.0, None, None, None, None, None, None))
            return
        arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (*old, *comb)]
        self._keep_rk = arrs
        _check(lib().orc_problem_set_rk(self.h, dt, a_diag, *[_ptr(a) for a in arrs]))

    def solve_faces(self):
        x = np.zeros(self.ndofs)
        _check(lib().orc_problem_solve_faces(self.h, _ptr(x)))
        return x

    def timings(self):
        t = np.zeros(5)
        lib().orc_problem_timings(self.h, _ptr(t))
        return dict(local=t[0], dirichlet=t[1], scatter=t[2], solve=t[3], recover=t[4])


def rk_apply(K, rhs, M, ut, comb, dt, a_diag):
    """RungeKutta::apply on a dense stiffness K [lenU x n] and rhs [lenU] (the oracle's code)."""
    K = np.asfortranarray(K, dtype=np.float64).copy(order="F")
    rhs = np.ascontiguousarray(rhs, dtype=np.float64).copy()
    M = np.asfortranarray(M, dtype=np.float64)
    ut = np.ascontiguousarray(ut, dtype=np.float64)
    comb = np.ascontiguousarray(comb, dtype=np.float64)
    _check(lib().orc_rk_apply(K.shape[0], K.shape[1], K.ctypes.data, rhs.ctypes.data, M.ctypes.data,
                              ut.ctypes.data, comb.ctypes.data, dt, a_diag))
    return K, rhs


# Butcher tables of RungeKutta::setUpDB (RungeKutta.cpp:215-286): rows [c_i | a_i.], last row [0 | b]
_G = 1.0 - np.sqrt(2.0) / 2.0
BUTCHER = {
    "FEuler": [[0, 0], [0, 1]],
    "EMidpoint": [[0, 0, 0], [0.5, 0.5, 0], [0, 0, 1]],
    "Heun": [[0, 0, 0], [1, 1, 0], [0, 0.5, 0.5]],
    "Kutta3": [[0, 0, 0, 0], [0.5, 0.5, 0, 0], [1, -1, 2, 0], [0, 1 / 6, 2 / 3, 1 / 6]],
    "Heun3": [[0, 0, 0, 0], [1 / 3, 1 / 3, 0, 0], [2 / 3, 0, 2 / 3, 0], [0, 1 / 4, 0, 3 / 4]],
    "SSPRK3": [[0, 0, 0, 0], [1, 1, 0, 0], [0.5, 0.25, 0.25, 0], [0, 1 / 6, 1 / 6, 2 / 3]],
    "RK4": [[0, 0, 0, 0, 0], [0.5, 0.5, 0, 0, 0], [0.5, 0, 0.5, 0, 0], [1, 0, 0, 1, 0],
            [0, 1 / 6, 1 / 3, 1 / 3, 1 / 6]],
    "BEuler": [[1, 1], [0, 1]],
    "IMidpoint": [[0.5, 0.5], [0, 1]],
    "CrankNicolson": [[0, 0, 0], [1, 0.5, 0.5], [0, 0.5, 0.5]],
    "KS2": [[0.5, 0.5, 0], [1.5, -0.5, 2], [0, -0.5, 1.5]],
    "QZ2": [[0.25, 0.25, 0], [0.75, 0.5, 0.25], [0, 0.5, 0.5]],
    "ALX2": [[_G, _G, 0], [1, 1 - _G, _G], [0, 1 - _G, _G]],
    "RK43": [[0.5, 0.5, 0, 0, 0], [2 / 3, 1 / 6, 0.5, 0, 0], [0.5, -0.5, 0.5, 0.5, 0], [1, 1.5, -1.5, 0.5, 0.5],
             [0, 1.5, -1.5, 0.5, 0.5]],
}


class RungeKutta:
    """RungeKutta.cpp restated on host arrays: fields is a dict of the current
    Solution / Flux / Trace arrays (updated in place), stage() and solution()
    follow computeStage (:131-170) and computeSolution (:172-213); apply() sets the
    oracle problem's U-row modification for the current stage (:90-129)."""

    NAMES = ("Solution", "Flux", "Trace")

    def __init__(self, table, dt):
        self.b = np.array(table, dtype=np.float64)
        self.S = self.b.shape[0] - 1
        self.dt = dt
        self.stage_counter = 0
        self.old = None
        self.k = {n: [] for n in self.NAMES}

    def begin_step(self, fields):
        self.old = {n: fields[n].copy() for n in self.NAMES}
        self.k = {n: [None] * self.S for n in self.NAMES}

    def apply(self, problem):
        s = self.stage_counter
        a = self.b[s, 1:]
        comb = [sum((a[i] * self.k[n][i] for i in range(s)), np.zeros_like(self.old[n])) for n in self.NAMES]
        problem.set_rk(self.dt, a[s], [self.old[n] for n in self.NAMES], comb)

    def stage(self, fields):
        s = self.stage_counter
        a = self.b[s, 1:]
        for n in self.NAMES:
            self.k[n][s] = (fields[n] - self.old[n]) / self.dt
            fields[n][...] = self.old[n] + self.dt * sum(a[j] * self.k[n][j] for j in range(s + 1))
        self.stage_counter += 1

    def solution(self, fields):
        bs = self.b[self.S, 1:]
        for n in self.NAMES:
            fields[n][...] = self.old[n] + sum(bs[k] * self.dt * self.k[n][k] for k in range(self.S))
        self.stage_counter = 0


def _burgers_sigs(L):
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    if getattr(L, "_burgers_sigs", False):
        return
    L.orc_burgers_create.restype = vp
    L.orc_burgers_create.argtypes = [ip, ip, ip, vp, ip, vp]
    L.orc_burgers_destroy.argtypes = [vp]
    L.orc_burgers_set_fields.argtypes = [vp, vp, ip, vp, ip, vp, vp, dp, vp]
    L.orc_burgers_set_state.argtypes = [vp, vp, vp]
    L.orc_burgers_local_matrix.argtypes = [vp, ip, vp, vp]
    L.orc_burgers_assemble.argtypes = [vp, ip]
    L.orc_burgers_recover.argtypes = [vp] * 4
    L.orc_unabu_refel.argtypes = [ip, ip, vp, vp, vp, vp]
    L._burgers_sigs = True


def unabu_refel(dim, order, sol, trace):
    """HDGUNabU on the reference element as TestHDGUNabU.cpp sets it up; returns (op, rhs)."""
    L = lib()
    _burgers_sigs(L)
    re = RefEl(dim, order)
    N, F, Nf = re.nNodes, re.nFaces, re.nNodesFace
    n = N * dim * (dim + 1) + F * Nf * dim
    sol = np.ascontiguousarray(sol, dtype=np.float64).reshape(N * dim)
    trace = np.ascontiguousarray(trace, dtype=np.float64).reshape(F * Nf * dim)
    op = np.zeros((n, n), order="F")
    rhs = np.zeros(n)
    _check(L.orc_unabu_refel(dim, order, _ptr(sol), _ptr(trace), op.ctypes.data, _ptr(rhs)))
    return op, rhs


class BurgersProblem(Problem):
    """HDGBurgersModel on the oracle: nd = dim unknowns per node (vector Burgers,
    HDGBurgersModel.cpp:35-60), the HDGSolver assembly / recovery of the nd-valued
    trace system, and NonLinearWrapper's loop (newton)."""

    def __init__(self, dim, order, coords, cells):
        L = lib()
        _burgers_sigs(L)
        self.dim, self.order = dim, order
        self.coords = np.ascontiguousarray(coords, dtype=np.float64)
        self.cells = np.ascontiguousarray(cells, dtype=np.int32)
        self.h = L.orc_burgers_create(dim, order, self.coords.shape[0], _ptr(self.coords),
                                      self.cells.shape[0], _ptr(self.cells))
        if not self.h:
            raise RuntimeError("oracle: " + L.orc_last_error().decode())
        self.re = RefEl(dim, order)
        c = np.zeros(2, dtype=np.int32)
        L.orc_problem_face_counts(self.h, _ptr(c))
        self.nFaces, self.nBoundary = int(c[0]), int(c[1])
        F, Nf, N = self.re.nFaces, self.re.nNodesFace, self.re.nNodes
        nC = self.cells.shape[0]
        self.cell2face = np.zeros((nC, F), dtype=np.int32)
        self.face2cell = np.zeros((self.nFaces, 2), dtype=np.int32)
        self.faces = np.zeros((self.nFaces, Nf), dtype=np.int32)
        self.boundary = np.zeros(self.nBoundary, dtype=np.int32)
        L.orc_problem_faces(self.h, _ptr(self.cell2face), _ptr(self.face2cell), _ptr(self.faces),
                            _ptr(self.boundary))
        self.nCells = nC
        self.nd = dim
        self.lenU = N * dim
        self.lenQ = dim * N * dim
        self.lenL = F * Nf * dim
        self.ndofs = self.nFaces * Nf * dim
        self.buf = np.zeros((nC, self.lenU))
        self.trace = np.zeros(self.ndofs)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_burgers_destroy(self.h)
            self.h = None

    def set_fields(self, tau=None, tau_sides=1, nu=None, src=None, dirichlet=None, dt=0.0, old=None):
        """tau [nFaces][Nf][sides][nd*nd]; nu [nCells][N][kc] with kc 1 or d*d (None: no
        diffusion operator); src [nCells][nI][nd]; dirichlet [nFaces][Nf][nd]; dt > 0:
        implicit Euler about old [nCells][N*nd]."""
        arr = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
        tau, nu, src, dirichlet, old = arr(tau), arr(nu), arr(src), arr(dirichlet), arr(old)
        kc = 0 if nu is None else nu.size // (self.nCells * self.re.nNodes)
        self._keep = (tau, nu, src, dirichlet, old)
        _check(lib().orc_burgers_set_fields(self.h, _ptr(tau), tau_sides, _ptr(nu), kc, _ptr(src),
                                            _ptr(dirichlet), float(dt), _ptr(old)))

    def set_state(self, buf=None, trace=None):
        if buf is not None:
            self.buf = np.ascontiguousarray(buf, dtype=np.float64).reshape(self.nCells, self.lenU).copy()
        if trace is not None:
            self.trace = np.ascontiguousarray(trace, dtype=np.float64).reshape(self.ndofs).copy()
        _check(lib().orc_burgers_set_state(self.h, _ptr(self.buf), _ptr(self.trace)))

    def assemble(self, nthreads=1):
        _check(lib().orc_burgers_assemble(self.h, nthreads))

    def local_matrix(self, iel):
        n = self.lenU + self.lenQ + self.lenL
        A = np.zeros((n, n), order="F")
        r = np.zeros(n)
        _check(lib().orc_burgers_local_matrix(self.h, iel, A.ctypes.data, _ptr(r)))
        return A, r

    def recover(self, trace):
        trace = np.ascontiguousarray(trace, dtype=np.float64)
        sol = np.zeros((self.nCells, self.lenU))
        flux = np.zeros((self.nCells, self.lenQ))
        _check(lib().orc_burgers_recover(self.h, _ptr(trace), _ptr(sol), _ptr(flux)))
        return sol, flux

    def linearized_solve(self):
        """NonLinearWrapper::vanillaLinearizedSolver (NonLinearWrapper.cpp:36-39):
        assemble about (buf, trace), solve the trace system (direct FP64), recover."""
        self.set_state(self.buf, self.trace)
        self.assemble()
        x = self.solve_direct()
        sol, flux = self.recover(x)
        self.trace = x
        return sol, flux

    def newton(self, res_tol=1e-6, max_iters=20, dampening=0.0):
        """NonLinearWrapper::solve (NonLinearWrapper.cpp:41-79) on host arrays: the
        residual is ||sol - buf|| / ||buf|| (||sol - buf|| when buf = 0); while it
        is above res_tol, both become (1 - d) sol + d buf. Returns (sol, flux,
        iterations, residual history)."""
        hist = []
        sol = flux = None
        for it in range(max_iters):
            sol, flux = self.linearized_solve()
            diff = float(np.sum((sol - self.buf) ** 2))
            ref = float(np.sum(self.buf ** 2))
            res = np.sqrt(diff / ref) if ref != 0 else np.sqrt(diff)
            hist.append(res)
            if res < res_tol:
                return sol, flux, it + 1, hist
            self.buf = (1.0 - dampening) * sol + dampening * self.buf
            sol = self.buf.copy()
        return sol, flux, max_iters, hist
