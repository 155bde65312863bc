"""ctypes binding of the C ABI (include/hfx_gb300.h) and a small host-side
mirror of HyperFox's HDGSolver for Python callers, tests and the bench.

The library is the in-tree ``_lib/libhfx_gb300.so``; loading fails loudly if
it has not been built (there is no CPU fallback).
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "libhfx_gb300.so")

HFX_OK = 0
HFX_ERR_ARG = 1
HFX_ERR_STATE = 2
HFX_ERR_CUDA = 3
HFX_ERR_ALLOC = 4
HFX_ERR_NOT_CONVERGED = 5
HFX_ERR_BREAKDOWN = 6
HFX_ERR_NAN = 7
HFX_ERR_SINGULAR = 8
HFX_ERR_UNSUPPORTED = 9

KSP_CG, KSP_GMRES, KSP_AUTO = 0, 1, 2
PC_NONE, PC_JACOBI, PC_BLOCK_JACOBI, PC_TWOLEVEL = 0, 1, 2, 3
COARSE_CHEBYSHEV, COARSE_LEARNED = 0, 1
IMPLICIT, WEXPLICIT, SEXPLICIT = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
OP_MASS, OP_DIFFUSION, OP_CONVECTION = 1, 2, 4
SRC_NONE, SRC_VALUES, SRC_SINPROD = 0, 1, 2

# Every symbol include/hfx_gb300.h declares.
EXPORTED = [
    "hfx_ctx_create", "hfx_ctx_destroy", "hfx_last_error", "hfx_version",
    "hfx_refel_query", "hfx_refel_tables",
    "hfx_mesh_upload", "hfx_mesh_sizes", "hfx_mesh_topology", "hfx_mesh_compute_topology",
    "hfx_gmsh_read", "hfx_mesh_high_order", "hfx_mesh_io_error",
    "hfx_h5_read_mesh", "hfx_h5_field_names", "hfx_h5_read_field", "hfx_h5_write",
    "hfx_rk_butcher", "hfx_rk_set", "hfx_rk_set_type", "hfx_rk_begin_step", "hfx_rk_compute_stage",
    "hfx_rk_compute_solution", "hfx_set_trace", "hfx_get_state",
    "hfx_set_tau", "hfx_set_kappa", "hfx_set_source", "hfx_set_dirichlet", "hfx_set_time_scheme",
    "hfx_ip_coords", "hfx_assemble", "hfx_assemble_ex", "hfx_set_solver_type", "hfx_set_state", "hfx_set_assembly_path", "hfx_assembly_info", "hfx_get_condensed", "hfx_get_csr", "hfx_get_condensed_sample", "hfx_get_csr_rows", "hfx_mixed_assembly_info", "hfx_get_tc_blocks", "hfx_test_coarse_barrier", "hfx_cg_operators", "hfx_tuning_info", "hfx_set_tuning",
    "hfx_solve_opts_default", "hfx_solve", "hfx_recover", "hfx_coarse_operator", "hfx_coarse_bounds",
    "hfx_coarse_train",
    "hfx_coarse_loss_grad",
    "hfx_la_create", "hfx_la_destroy", "hfx_la_allocate", "hfx_la_set_values", "hfx_la_set_rhs",
    "hfx_la_zero_rows", "hfx_la_assemble", "hfx_la_clear", "hfx_la_solve", "hfx_la_nnz",
    "hfx_profile_enable", "hfx_kernel_time", "hfx_mark", "hfx_elapsed_ms", "hfx_elapsed_between", "hfx_synchronize",
    "hfx_burgers_setup", "hfx_burgers_set_tau", "hfx_burgers_set_diffusion", "hfx_burgers_set_source",
    "hfx_burgers_set_dirichlet", "hfx_burgers_set_time_step", "hfx_burgers_set_state", "hfx_burgers_get_state",
    "hfx_burgers_begin_step", "hfx_burgers_assemble", "hfx_burgers_solve", "hfx_newton_opts_default",
    "hfx_burgers_newton", "hfx_burgers_get_condensed", "hfx_burgers_nnz", "hfx_burgers_get_csr",
    "hfx_trace_solve_noalloc",
]
NOALLOC_MAX_DOFS = 65536
NOALLOC_MAX_NF = 10


class HfxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("hfx error %d: %s" % (code, msg))
        self.code = code


class RefElInfo(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("dim", "order", "nNodes", "nFaces", "nNodesFace", "nIP", "nIPFace")]


class SolveOpts(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int), ("precond", ctypes.c_int), ("precision", ctypes.c_int),
                ("rtol", ctypes.c_double), ("maxits", ctypes.c_int), ("restart", ctypes.c_int),
                ("inner_rtol", ctypes.c_double), ("use_initial_guess", ctypes.c_int),
                ("coarse_guess", ctypes.c_int), ("coarse_rtol", ctypes.c_double), ("coarse_mode", ctypes.c_int),
                ("coarse_degree", ctypes.c_int)]


class SolveInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int), ("refinements", ctypes.c_int),
                ("rel_residual", ctypes.c_double), ("solve_ms", ctypes.c_double),
                ("fallback", ctypes.c_int), ("coarse_degree", ctypes.c_int), ("coarse_learned", ctypes.c_int)]


class TrainInfo(ctypes.Structure):
    _fields_ = [("degree", ctypes.c_int), ("samples", ctypes.c_int), ("steps", ctypes.c_int),
                ("accepted", ctypes.c_int), ("loss_chebyshev", ctypes.c_double), ("loss_learned", ctypes.c_double),
                ("max_poly", ctypes.c_double), ("train_ms", ctypes.c_double), ("loss_first_step", ctypes.c_double),
                ("lower_steps", ctypes.c_int), ("rejected_steps", ctypes.c_int)]


class NewtonOpts(ctypes.Structure):
    _fields_ = [("res_tol", ctypes.c_double), ("max_iters", ctypes.c_int), ("dampening", ctypes.c_double),
                ("lin", SolveOpts), ("warm_start", ctypes.c_int), ("history", ctypes.c_int)]


class NewtonInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("iterations", ctypes.c_int), ("residual", ctypes.c_double),
                ("krylov_iterations", ctypes.c_int), ("assemble_ms", ctypes.c_double),
                ("solve_ms", ctypes.c_double), ("recover_ms", ctypes.c_double)]


_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it is missing: no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError("libhfx_gb300.so is not built (run __graft_entry__.build()): %s" % path)
    L = ctypes.CDLL(path)
    vp, ip, dp = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    sig = {
        "hfx_ctx_create": ([ip, ctypes.POINTER(vp)], ip),
        "hfx_ctx_destroy": ([vp], ip),
        "hfx_last_error": ([vp], ctypes.c_char_p),
        "hfx_version": ([], ip),
        "hfx_refel_query": ([ip, ip, ctypes.POINTER(RefElInfo)], ip),
        "hfx_refel_tables": ([ip, ip] + [vp] * 10, ip),
        "hfx_mesh_upload": ([vp, ip, ip, ip, vp, ip, vp, ip, vp, vp, vp, ip, vp], ip),
        "hfx_mesh_sizes": ([vp, vp, vp, vp], ip),
        "hfx_mesh_topology": ([vp] * 5, ip),
        "hfx_mesh_compute_topology": ([ip, ip, ip, vp, vp, vp, vp, vp, vp, vp], ip),
        "hfx_set_tau": ([vp, vp, ip], ip),
        "hfx_set_kappa": ([vp, vp, ip, ip], ip),
        "hfx_set_source": ([vp, ip, vp, dp], ip),
        "hfx_set_dirichlet": ([vp, vp], ip),
        "hfx_set_time_scheme": ([vp, dp, vp], ip),
        "hfx_ip_coords": ([vp, vp], ip),
        "hfx_assemble": ([vp], ip),
        "hfx_assemble_ex": ([vp, ip], ip),
        "hfx_get_condensed": ([vp] * 7, ip),
        "hfx_get_csr": ([vp] * 5, ip),
        "hfx_get_condensed_sample": ([vp, ip, vp] + [vp] * 6, ip),
        "hfx_mixed_assembly_info": ([vp, vp], ip),
        "hfx_test_coarse_barrier": ([vp], ip),
        "hfx_cg_operators": ([vp, ip, ip, vp, ip, vp], ip),
        "hfx_tuning_info": ([vp, vp, vp], ip),
        "hfx_set_tuning": ([vp, ip], ip),
        "hfx_get_tc_blocks": ([vp, ip, vp, vp, vp], ip),
        "hfx_get_csr_rows": ([vp, ip, vp, vp, vp, vp, vp, ctypes.c_int64], ip),
        "hfx_solve_opts_default": ([ctypes.POINTER(SolveOpts)], None),
        "hfx_solve": ([vp, ctypes.POINTER(SolveOpts), vp, ctypes.POINTER(SolveInfo)], ip),
        "hfx_recover": ([vp, vp, vp], ip),
        "hfx_coarse_operator": ([vp, vp, vp, vp, vp, vp, vp], ip),
        "hfx_coarse_bounds": ([vp, vp], ip),
        "hfx_coarse_train": ([vp, ip, ip, ip, ctypes.POINTER(TrainInfo)], ip),
        "hfx_coarse_loss_grad": ([vp, ip, vp, ip, vp, vp, vp], ip),
        "hfx_set_assembly_path": ([vp, ip], ip),
        "hfx_set_solver_type": ([vp, ip], ip),
        "hfx_set_state": ([vp, vp, vp], ip),
        "hfx_gmsh_read": ([ctypes.c_char_p, ip, vp, vp, vp, vp], ip),
        "hfx_mesh_high_order": ([ip, ip, ip, vp, ip, vp, vp, vp, vp], ip),
        "hfx_mesh_io_error": ([], ctypes.c_char_p),
        "hfx_h5_read_mesh": ([ctypes.c_char_p, vp, vp, vp, vp, vp, vp], ip),
        "hfx_h5_field_names": ([ctypes.c_char_p, ctypes.c_char_p, ip, vp, vp], ip),
        "hfx_h5_read_field": ([ctypes.c_char_p, ctypes.c_char_p, vp, vp, vp], ip),
        "hfx_h5_write": ([ctypes.c_char_p, ip, ip, vp, ip, ip, vp, ip, vp, vp, vp, vp], ip),
        "hfx_rk_butcher": ([ip, vp, vp], ip),
        "hfx_rk_set": ([vp, ip, vp, ctypes.c_double], ip),
        "hfx_rk_set_type": ([vp, ip, ctypes.c_double], ip),
        "hfx_rk_begin_step": ([vp], ip),
        "hfx_rk_compute_stage": ([vp], ip),
        "hfx_rk_compute_solution": ([vp], ip),
        "hfx_set_trace": ([vp, vp], ip),
        "hfx_get_state": ([vp, vp, vp, vp], ip),
        "hfx_assembly_info": ([vp, vp], ip),
        "hfx_la_create": ([vp, ctypes.POINTER(vp)], ip),
        "hfx_la_destroy": ([vp], ip),
        "hfx_la_allocate": ([vp, ip], ip),
        "hfx_la_set_values": ([vp, ip, vp, ip, vp, vp, ip], ip),
        "hfx_la_set_rhs": ([vp, ip, vp, vp, ip], ip),
        "hfx_la_zero_rows": ([vp, ip, vp], ip),
        "hfx_la_assemble": ([vp], ip),
        "hfx_la_clear": ([vp], ip),
        "hfx_la_solve": ([vp, ctypes.POINTER(SolveOpts), vp, ctypes.POINTER(SolveInfo)], ip),
        "hfx_la_nnz": ([vp, vp], ip),
        "hfx_profile_enable": ([vp, ip], ip),
        "hfx_kernel_time": ([vp, ip, vp, vp], ip),
        "hfx_mark": ([vp, ip], ip),
        "hfx_elapsed_ms": ([vp, ip, ip, vp], ip),
        "hfx_elapsed_between": ([vp, ip, vp, ip, vp], ip),
        "hfx_synchronize": ([vp], ip),
        "hfx_burgers_setup": ([vp], ip),
        "hfx_burgers_set_tau": ([vp, vp, ip], ip),
        "hfx_burgers_set_diffusion": ([vp, vp, ip, ip], ip),
        "hfx_burgers_set_source": ([vp, vp], ip),
        "hfx_burgers_set_dirichlet": ([vp, vp], ip),
        "hfx_burgers_set_time_step": ([vp, dp], ip),
        "hfx_burgers_set_state": ([vp, vp, vp, vp, vp], ip),
        "hfx_burgers_get_state": ([vp, vp, vp, vp, vp], ip),
        "hfx_burgers_begin_step": ([vp], ip),
        "hfx_burgers_assemble": ([vp], ip),
        "hfx_burgers_solve": ([vp, ctypes.POINTER(SolveOpts), ctypes.POINTER(SolveInfo)], ip),
        "hfx_newton_opts_default": ([ctypes.POINTER(NewtonOpts)], None),
        "hfx_burgers_newton": ([vp, ctypes.POINTER(NewtonOpts), ctypes.POINTER(NewtonInfo)], ip),
        "hfx_burgers_get_condensed": ([vp] * 7, ip),
        "hfx_burgers_nnz": ([vp, vp], ip),
        "hfx_burgers_get_csr": ([vp] * 5, ip),
        "hfx_trace_solve_noalloc": ([ip, ip, ip, vp, vp, vp, vp, vp, vp, dp, ip, vp, ctypes.POINTER(SolveInfo)], ip),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data


def refel(dim, order):
    """Reference-element tables from the library (host only, no GPU)."""
    L = load()
    info = RefElInfo()
    rc = L.hfx_refel_query(dim, order, ctypes.byref(info))
    if rc:
        raise HfxError(rc, "refel_query(%d, %d)" % (dim, order))
    N, F, Nf, nI, nIf = info.nNodes, info.nFaces, info.nNodesFace, info.nIP, info.nIPFace
    t = dict(nodes=np.zeros((N, dim)), faceNodes=np.zeros((F, Nf), np.int32), ipX=np.zeros((nI, dim)),
             ipW=np.zeros(nI), phi=np.zeros((nI, N)), dphi=np.zeros((nI, N, dim)),
             fIpX=np.zeros((nIf, dim - 1)), fIpW=np.zeros(nIf), fPhi=np.zeros((nIf, Nf)),
             fDphi=np.zeros((nIf, Nf, dim - 1)))
    rc = L.hfx_refel_tables(dim, order, *[_p(t[k]) for k in ("nodes", "faceNodes", "ipX", "ipW", "phi", "dphi",
                                                              "fIpX", "fIpW", "fPhi", "fDphi")])
    if rc:
        raise HfxError(rc, "refel_tables")
    t.update(dim=dim, order=order, nNodes=N, nFaces=F, nNodesFace=Nf, nIP=nI, nIPFace=nIf)
    return t


def mesh_topology(dim, order, cells):
    """Face topology by the MOAB creation-order rule (host only, no GPU)."""
    L = load()
    cells = np.ascontiguousarray(cells, np.int32)
    nf, nb = ctypes.c_int(), ctypes.c_int()
    rc = L.hfx_mesh_compute_topology(dim, order, cells.shape[0], _p(cells), ctypes.byref(nf), ctypes.byref(nb),
                                     None, None, None, None)
    if rc:
        raise HfxError(rc, "mesh_compute_topology")
    F = dim + 1
    Nf = refel(dim, order)["nNodesFace"]
    c2f = np.zeros((cells.shape[0], F), np.int32)
    f2c = np.zeros((nf.value, 2), np.int32)
    faces = np.zeros((nf.value, Nf), np.int32)
    bnd = np.zeros(nb.value, np.int32)
    rc = L.hfx_mesh_compute_topology(dim, order, cells.shape[0], _p(cells), ctypes.byref(nf), ctypes.byref(nb),
                                     _p(c2f), _p(f2c), _p(faces), _p(bnd))
    if rc:
        raise HfxError(rc, "mesh_compute_topology")
    return c2f, f2c, faces, bnd


def gmsh_read(path, dim):
    """Linear simplex mesh of dimension dim from a gmsh 2.2 ASCII file (host only)."""
    L = load()
    nn, nc = ctypes.c_int(), ctypes.c_int()
    rc = L.hfx_gmsh_read(str(path).encode(), dim, ctypes.byref(nn), ctypes.byref(nc), None, None)
    if rc:
        raise HfxError(rc, "gmsh_read: " + L.hfx_mesh_io_error().decode())
    coords = np.zeros((nn.value, dim))
    cells = np.zeros((nc.value, dim + 1), np.int32)
    rc = L.hfx_gmsh_read(str(path).encode(), dim, ctypes.byref(nn), ctypes.byref(nc), _p(coords), _p(cells))
    if rc:
        raise HfxError(rc, "gmsh_read: " + L.hfx_mesh_io_error().decode())
    return coords, cells


def mesh_high_order(dim, order, coords, cells):
    """High-order nodes of a linear simplex mesh (host only): (coords [n][dim], cells [nCells][N])."""
    L = load()
    coords = np.ascontiguousarray(coords, np.float64)
    cells = np.ascontiguousarray(cells, np.int32)
    nn = ctypes.c_int()
    args = (dim, order, coords.shape[0], _p(coords), cells.shape[0], _p(cells), ctypes.byref(nn))
    rc = L.hfx_mesh_high_order(*args, None, None)
    if rc:
        raise HfxError(rc, "mesh_high_order: " + L.hfx_mesh_io_error().decode())
    N = refel(dim, order)["nNodes"]
    out_c = np.zeros((nn.value, dim))
    out_e = np.zeros((cells.shape[0], N), np.int32)
    rc = L.hfx_mesh_high_order(*args, _p(out_c), _p(out_e))
    if rc:
        raise HfxError(rc, "mesh_high_order: " + L.hfx_mesh_io_error().decode())
    return out_c, out_e


FIELD_NONE, FIELD_NODE, FIELD_EDGE, FIELD_FACE, FIELD_CELL = -1, 0, 1, 2, 3

# RKType (RKType.h): explicit FEuler..RK4, implicit BEuler..RK43
RK_TYPES = ["FEuler", "EMidpoint", "Heun", "Kutta3", "Heun3", "SSPRK3", "RK4",
            "BEuler", "IMidpoint", "CrankNicolson", "KS2", "QZ2", "ALX2", "RK43"]


def rk_butcher(rk_type):
    """Butcher table [(S+1) x (S+1)] of a named scheme (index or name in RK_TYPES)."""
    L = load()
    t = RK_TYPES.index(rk_type) if isinstance(rk_type, str) else int(rk_type)
    S = ctypes.c_int()
    rc = L.hfx_rk_butcher(t, ctypes.byref(S), None)
    if rc:
        raise HfxError(rc, "rk_butcher: unknown type")
    tab = np.zeros((S.value + 1, S.value + 1))
    L.hfx_rk_butcher(t, ctypes.byref(S), _p(tab))
    return tab


def h5_read_mesh(path):
    """(coords [nNodes][nodeDim], cells [nCells][nodesPerCell]) from /Mesh of an HDF5 file (host only)."""
    L = load()
    nd, nn, nc, npc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    refs = (ctypes.byref(nd), ctypes.byref(nn), ctypes.byref(nc), ctypes.byref(npc))
    rc = L.hfx_h5_read_mesh(str(path).encode(), *refs, None, None)
    if rc:
        raise HfxError(rc, "h5_read_mesh: " + L.hfx_mesh_io_error().decode())
    coords = np.zeros((nn.value, nd.value))
    cells = np.zeros((nc.value, npc.value), np.int32)
    rc = L.hfx_h5_read_mesh(str(path).encode(), *refs, _p(coords), _p(cells))
    if rc:
        raise HfxError(rc, "h5_read_mesh: " + L.hfx_mesh_io_error().decode())
    return coords, cells


def h5_field_names(path):
    """Names of the datasets under /FieldData (sorted)."""
    L = load()
    n, need = ctypes.c_int(), ctypes.c_int()
    rc = L.hfx_h5_field_names(str(path).encode(), None, 0, ctypes.byref(n), ctypes.byref(need))
    if rc:
        raise HfxError(rc, "h5_field_names: " + L.hfx_mesh_io_error().decode())
    buf = ctypes.create_string_buffer(need.value)
    rc = L.hfx_h5_field_names(str(path).encode(), buf, need.value, ctypes.byref(n), ctypes.byref(need))
    if rc:
        raise HfxError(rc, "h5_field_names: " + L.hfx_mesh_io_error().decode())
    return [x for x in buf.value.decode().split("\n") if x]


def h5_read_field(path, name):
    """(ftype, values [entities][objs][vals]) of /FieldData/<name>."""
    L = load()
    ft = ctypes.c_int()
    shape = np.zeros(3, np.int64)
    rc = L.hfx_h5_read_field(str(path).encode(), name.encode(), ctypes.byref(ft), _p(shape), None)
    if rc:
        raise HfxError(rc, "h5_read_field: " + L.hfx_mesh_io_error().decode())
    vals = np.zeros(tuple(int(x) for x in shape))
    rc = L.hfx_h5_read_field(str(path).encode(), name.encode(), ctypes.byref(ft), _p(shape), _p(vals))
    if rc:
        raise HfxError(rc, "h5_read_field: " + L.hfx_mesh_io_error().decode())
    return ft.value, vals


def h5_write(path, coords=None, cells=None, fields=None):
    """Write /Mesh (when coords and cells are given) and /FieldData (fields: {name: (ftype, values)},
    values reshaped to [entities][objs][vals] when 3-D, [entities][objs][1] when 2-D)."""
    L = load()
    nd = nn = nc = npc = 0
    pc = pe = None
    if coords is not None:
        coords = np.ascontiguousarray(coords, np.float64)
        cells = np.ascontiguousarray(cells, np.int32)
        nn, nd = coords.shape
        nc, npc = cells.shape
        pc, pe = _p(coords), _p(cells)
    fields = fields or {}
    names = (ctypes.c_char_p * max(1, len(fields)))()
    ftypes = np.zeros(max(1, len(fields)), np.int32)
    shapes = np.zeros(3 * max(1, len(fields)), np.int64)
    vptrs = (ctypes.c_void_p * max(1, len(fields)))()
    keep = []
    for i, (name, (ft, vals)) in enumerate(fields.items()):
        v = np.ascontiguousarray(vals, np.float64)
        if v.ndim == 2:
            v = v[:, :, None]
        if v.ndim != 3:
            raise ValueError("field values must be 2-D or 3-D")
        keep.append(v)
        names[i] = name.encode()
        ftypes[i] = ft
        shapes[3 * i:3 * i + 3] = v.shape
        vptrs[i] = v.ctypes.data
    rc = L.hfx_h5_write(str(path).encode(), nd, nn, pc, nc, npc, pe, len(fields), ctypes.cast(names, ctypes.c_void_p),
                        _p(ftypes), _p(shapes), ctypes.cast(vptrs, ctypes.c_void_p))
    if rc:
        raise HfxError(rc, "h5_write: " + L.hfx_mesh_io_error().decode())


def solve_opts(**kw):
    o = SolveOpts()
    load().hfx_solve_opts_default(ctypes.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


class Context:
    """One device context (one stream) holding one HDG problem."""

    def __init__(self, device=0):
        L = load()
        h = ctypes.c_void_p()
        rc = L.hfx_ctx_create(device, ctypes.byref(h))
        if rc:
            raise HfxError(rc, "ctx_create(device=%d)" % device)
        self.h = h
        self.L = L

    def close(self):
        if getattr(self, "h", None):
            self.L.hfx_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _chk(self, rc, what):
        if rc:
            raise HfxError(rc, "%s: %s" % (what, self.L.hfx_last_error(self.h).decode()))

    # ---- mesh and fields
    def upload_mesh(self, dim, order, coords, cells, topology=None):
        coords = np.ascontiguousarray(coords, np.float64)
        cells = np.ascontiguousarray(cells, np.int32)
        self._keep = (coords, cells)
        if topology is None:
            rc = self.L.hfx_mesh_upload(self.h, dim, order, coords.shape[0], _p(coords), cells.shape[0], _p(cells),
                                        0, None, None, None, 0, None)
        else:
            c2f, f2c, faces, bnd = [np.ascontiguousarray(a, np.int32) for a in topology]
            rc = self.L.hfx_mesh_upload(self.h, dim, order, coords.shape[0], _p(coords), cells.shape[0], _p(cells),
                                        faces.shape[0], _p(c2f), _p(f2c), _p(faces), bnd.size, _p(bnd))
        self._chk(rc, "mesh_upload")
        self.dim, self.order = dim, order
        self.re = refel(dim, order)
        self.nCells = cells.shape[0]
        nf, nb, nnz = ctypes.c_int(), ctypes.c_int(), ctypes.c_int64()
        self._chk(self.L.hfx_mesh_sizes(self.h, ctypes.byref(nf), ctypes.byref(nb), ctypes.byref(nnz)), "mesh_sizes")
        self.nFaces, self.nBoundary, self.nnz = nf.value, nb.value, nnz.value
        self.ndofs = self.nFaces * self.re["nNodesFace"]
        self.lenU = self.re["nNodes"]
        self.lenQ = dim * self.re["nNodes"]
        self.lenL = self.re["nFaces"] * self.re["nNodesFace"]

    def topology(self):
        F, Nf = self.re["nFaces"], self.re["nNodesFace"]
        c2f = np.zeros((self.nCells, F), np.int32)
        f2c = np.zeros((self.nFaces, 2), np.int32)
        faces = np.zeros((self.nFaces, Nf), np.int32)
        bnd = np.zeros(self.nBoundary, np.int32)
        self._chk(self.L.hfx_mesh_topology(self.h, _p(c2f), _p(f2c), _p(faces), _p(bnd)), "mesh_topology")
        return c2f, f2c, faces, bnd

    def set_tau(self, tau):
        tau = np.ascontiguousarray(tau, np.float64)
        nvals = tau.size // self.ndofs
        self._chk(self.L.hfx_set_tau(self.h, _p(tau), nvals), "set_tau")

    def set_kappa(self, kappa, layout=1):
        if kappa is None:
            self._chk(self.L.hfx_set_kappa(self.h, None, 0, 0), "set_kappa")
            return
        kappa = np.ascontiguousarray(kappa, np.float64)
        rows = self.nCells * self.re["nNodes"] if layout == 1 else None
        comps = kappa.size // rows if rows else kappa.shape[-1]
        self._chk(self.L.hfx_set_kappa(self.h, _p(kappa), comps, layout), "set_kappa")

    def set_source(self, mode, values=None, param=0.0):
        v = None if values is None else np.ascontiguousarray(values, np.float64)
        self._chk(self.L.hfx_set_source(self.h, mode, _p(v), float(param)), "set_source")

    def set_dirichlet(self, values):
        v = np.ascontiguousarray(values, np.float64)
        self._chk(self.L.hfx_set_dirichlet(self.h, _p(v)), "set_dirichlet")

    def set_time_scheme(self, dt, u_old=None):
        v = None if u_old is None else np.ascontiguousarray(u_old, np.float64)
        self._chk(self.L.hfx_set_time_scheme(self.h, float(dt), _p(v)), "set_time_scheme")

    def ip_coords(self):
        out = np.zeros((self.nCells, self.re["nIP"], self.dim))
        self._chk(self.L.hfx_ip_coords(self.h, _p(out)), "ip_coords")
        return out

    # ---- hot path
    def assemble(self, precision=PREC_FP64):
        self._chk(self.L.hfx_assemble_ex(self.h, precision), "assemble")

    def condensed(self):
        E, U, Q, Ll = self.nCells, self.lenU, self.lenQ, self.lenL
        out = dict(S=np.zeros((E, Ll * Ll)), S0=np.zeros((E, Ll)), U=np.zeros((E, U * Ll)), Q=np.zeros((E, Q * Ll)),
                   U0=np.zeros((E, U)), Q0=np.zeros((E, Q)))
        self._chk(self.L.hfx_get_condensed(self.h, *[_p(out[k]) for k in ("S", "S0", "U", "Q", "U0", "Q0")]),
                  "get_condensed")
        return out

    def cg_operators(self, which=7, precision=0, velocity=None, vel_layout=1):
        """CG element operators [nCells][3][N*N] (column-major per element): Mass, Diffusion
        (this context's diffusion field), Convection (nodal velocity)."""
        N = self.re["nNodes"]
        out = np.zeros((self.nCells, 3, N * N))
        v = None if velocity is None else np.ascontiguousarray(velocity, np.float64)
        self._chk(self.L.hfx_cg_operators(self.h, which, precision, _p(v), vel_layout, _p(out)), "cg_operators")
        return out

    def tuning_info(self):
        """(kernel chosen for the FP32 trace operator or -1, [ms per launch of kernels 0..3])."""
        k = ctypes.c_int()
        t = (ctypes.c_float * 4)()
        self._chk(self.L.hfx_tuning_info(self.h, ctypes.byref(k), t), "tuning_info")
        return k.value, [t[0], t[1], t[2], t[3]]

    def mixed_assembly_info(self):
        """1 when the last mixed assembly contracted the element blocks on the tensor cores."""
        v = ctypes.c_int()
        self._chk(self.L.hfx_mixed_assembly_info(self.h, ctypes.byref(v)), "mixed_assembly_info")
        return v.value

    def tc_blocks(self, cells):
        """FP32 element blocks of the tensor-core mixed assembly, [len(cells)][stride]."""
        cells = np.ascontiguousarray(cells, np.int32)
        st = ctypes.c_int64()
        self.L.hfx_get_tc_blocks(self.h, 0, None, None, ctypes.byref(st))
        out = np.zeros((len(cells), st.value), np.float32)
        self._chk(self.L.hfx_get_tc_blocks(self.h, len(cells), _p(cells), _p(out), ctypes.byref(st)), "get_tc_blocks")
        return out

    def condensed_sample(self, cells):
        cells = np.ascontiguousarray(cells, np.int32)
        n, U, Q, Ll = len(cells), self.lenU, self.lenQ, self.lenL
        out = dict(S=np.zeros((n, Ll * Ll)), S0=np.zeros((n, Ll)), U=np.zeros((n, U * Ll)), Q=np.zeros((n, Q * Ll)),
                   U0=np.zeros((n, U)), Q0=np.zeros((n, Q)))
        self._chk(self.L.hfx_get_condensed_sample(self.h, n, _p(cells),
                                                  *[_p(out[k]) for k in ("S", "S0", "U", "Q", "U0", "Q0")]),
                  "get_condensed_sample")
        return out

    def csr_rows(self, faces):
        """AIJ rows of the listed faces: (rowlen, col, val, rhs), rows back to back."""
        faces = np.ascontiguousarray(faces, np.int32)
        Nf = self.re["nNodesFace"]
        nr = len(faces) * Nf
        cap = nr * 2 * self.re["nFaces"] * Nf
        rowlen = np.zeros(nr, np.int32)
        col = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        rhs = np.zeros(nr)
        self._chk(self.L.hfx_get_csr_rows(self.h, len(faces), _p(faces), _p(rowlen), _p(col), _p(val), _p(rhs), cap),
                  "get_csr_rows")
        n = int(rowlen.sum())
        return rowlen, col[:n], val[:n], rhs

    def csr(self):
        rowptr = np.zeros(self.ndofs + 1, np.int64)
        col = np.zeros(self.nnz, np.int32)
        val = np.zeros(self.nnz)
        rhs = np.zeros(self.ndofs)
        self._chk(self.L.hfx_get_csr(self.h, _p(rowptr), _p(col), _p(val), _p(rhs)), "get_csr")
        return rowptr, col, val, rhs

    def solve(self, want_trace=True, **opts):
        o = solve_opts(**opts)
        info = SolveInfo()
        trace = np.zeros(self.ndofs) if want_trace else None
        rc = self.L.hfx_solve(self.h, ctypes.byref(o), _p(trace), ctypes.byref(info))
        self._chk(rc, "solve")
        return trace, info

    def coarse_operator(self):
        """Two-level coarse operator: (rowptr, col, val FP32, vertexNode)."""
        nV = ctypes.c_int()
        nnz = ctypes.c_int64()
        self._chk(self.L.hfx_coarse_operator(self.h, ctypes.byref(nV), ctypes.byref(nnz), None, None, None, None),
                  "coarse_operator")
        rowptr = np.zeros(nV.value + 1, np.int32)
        col = np.zeros(nnz.value, np.int32)
        val = np.zeros(nnz.value, np.float32)
        vn = np.zeros(nV.value, np.int32)
        self._chk(self.L.hfx_coarse_operator(self.h, ctypes.byref(nV), ctypes.byref(nnz), _p(rowptr), _p(col),
                                             _p(val), _p(vn)), "coarse_operator")
        return rowptr, col, val, vn

    def coarse_bounds(self):
        """Spectral bounds of D^-1 A_c: dict lmin, lmax (Chebyshev interval), ritz_min, ritz_max
        (Lanczos), row_bound (infinity norm of D^-1/2 A_c D^-1/2)."""
        out = (ctypes.c_double * 5)()
        self._chk(self.L.hfx_coarse_bounds(self.h, out), "coarse_bounds")
        return dict(zip(("lmin", "lmax", "ritz_min", "ritz_max", "row_bound"), list(out)))

    def assembly_info(self):
        """1 when the last FP64 assembly ran the affine element kernel, else 0."""
        v = ctypes.c_int()
        self._chk(self.L.hfx_assembly_info(self.h, ctypes.byref(v)), "assembly_info")
        return v.value

    def set_solver_type(self, t):
        self._chk(self.L.hfx_set_solver_type(self.h, t), "set_solver_type")

    def set_state(self, sol, flux):
        sol = np.ascontiguousarray(sol, np.float64)
        flux = np.ascontiguousarray(flux, np.float64)
        self._chk(self.L.hfx_set_state(self.h, _p(sol), _p(flux)), "set_state")

    def set_trace(self, trace):
        trace = np.ascontiguousarray(trace, np.float64)
        self._chk(self.L.hfx_set_trace(self.h, _p(trace)), "set_trace")

    def get_state(self):
        """(Solution [nCells][N], Flux [nCells][N*dim], Trace [ndofs]) as held on the device."""
        sol = np.zeros((self.nCells, self.lenU))
        flux = np.zeros((self.nCells, self.lenQ))
        trace = np.zeros(self.ndofs)
        self._chk(self.L.hfx_get_state(self.h, _p(sol), _p(flux), _p(trace)), "get_state")
        return sol, flux, trace

    def rk_set(self, scheme, dt):
        """Runge-Kutta scheme: a name / RKType index (table taken as is) or a user
        table (checked like RungeKutta::setButcherTable); None switches it off."""
        if scheme is None:
            self._chk(self.L.hfx_rk_set(self.h, 0, None, 0.0), "rk_set")
        elif isinstance(scheme, (str, int)):
            t = RK_TYPES.index(scheme) if isinstance(scheme, str) else scheme
            self._chk(self.L.hfx_rk_set_type(self.h, t, dt), "rk_set_type")
        else:
            tab = np.ascontiguousarray(scheme, np.float64)
            self._chk(self.L.hfx_rk_set(self.h, tab.shape[0] - 1, _p(tab), dt), "rk_set")

    def rk_begin_step(self):
        self._chk(self.L.hfx_rk_begin_step(self.h), "rk_begin_step")

    def rk_compute_stage(self):
        self._chk(self.L.hfx_rk_compute_stage(self.h), "rk_compute_stage")

    def rk_compute_solution(self):
        self._chk(self.L.hfx_rk_compute_solution(self.h), "rk_compute_solution")

    def coarse_train(self, degree=4, samples=16, steps=300):
        info = TrainInfo()
        self._chk(self.L.hfx_coarse_train(self.h, degree, samples, steps, ctypes.byref(info)), "coarse_train")
        return info

    def coarse_loss_grad(self, theta, samples):
        theta = np.ascontiguousarray(theta, np.float64)
        samples = np.ascontiguousarray(samples, np.float32)
        loss = ctypes.c_double()
        grad = np.zeros(len(theta))
        self._chk(self.L.hfx_coarse_loss_grad(self.h, len(theta), _p(theta), samples.shape[0], _p(samples),
                                              ctypes.byref(loss), _p(grad)), "coarse_loss_grad")
        return loss.value, grad

    def recover(self):
        sol = np.zeros((self.nCells, self.lenU))
        flux = np.zeros((self.nCells, self.lenQ))
        self._chk(self.L.hfx_recover(self.h, _p(sol), _p(flux)), "recover")
        return sol, flux


class LinearSystem:
    """hfx_la_* handle (LinAlgebraInterface drop-in on the device)."""

    def __init__(self, ctx):
        self.ctx = ctx
        h = ctypes.c_void_p()
        ctx._chk(ctx.L.hfx_la_create(ctx.h, ctypes.byref(h)), "la_create")
        self.h = h

    def __del__(self):
        if getattr(self, "h", None):
            self.ctx.L.hfx_la_destroy(self.h)
            self.h = None

    def allocate(self, n):
        self.n = n
        self.ctx._chk(self.ctx.L.hfx_la_allocate(self.h, n), "la_allocate")

    def values(self, rows, cols, vals, insert=False):
        r = np.ascontiguousarray(rows, np.int32)
        c = np.ascontiguousarray(cols, np.int32)
        v = np.ascontiguousarray(vals, np.float64)
        self.ctx._chk(self.ctx.L.hfx_la_set_values(self.h, r.size, _p(r), c.size, _p(c), _p(v), int(insert)),
                      "la_set_values")

    def rhs(self, idx, vals, insert=False):
        i = np.ascontiguousarray(idx, np.int32)
        v = np.ascontiguousarray(vals, np.float64)
        self.ctx._chk(self.ctx.L.hfx_la_set_rhs(self.h, i.size, _p(i), _p(v), int(insert)), "la_set_rhs")

    def zero_rows(self, rows):
        r = np.ascontiguousarray(rows, np.int32)
        self.ctx._chk(self.ctx.L.hfx_la_zero_rows(self.h, r.size, _p(r)), "la_zero_rows")

    def assemble(self):
        self.ctx._chk(self.ctx.L.hfx_la_assemble(self.h), "la_assemble")

    def clear(self):
        self.ctx._chk(self.ctx.L.hfx_la_clear(self.h), "la_clear")

    def solve(self, **opts):
        kw = dict(method=KSP_GMRES, precond=PC_JACOBI)
        kw.update(opts)
        o = solve_opts(**kw)
        info = SolveInfo()
        x = np.zeros(self.n)
        self.ctx._chk(self.ctx.L.hfx_la_solve(self.h, ctypes.byref(o), _p(x), ctypes.byref(info)), "la_solve")
        return x, info


def newton_opts(**kw):
    """hfx_newton_opts with the library defaults; lin_* keys set the linear solve's options."""
    o = NewtonOpts()
    load().hfx_newton_opts_default(ctypes.byref(o))
    for k, v in kw.items():
        if k.startswith("lin_"):
            setattr(o.lin, k[4:], v)
        else:
            setattr(o, k, v)
    return o


class Burgers:
    """Vector Burgers (HDGBurgersModel + NonLinearWrapper) on a context's mesh:
    nd = dim unknowns per node, fields and outputs of its own."""

    def __init__(self, ctx):
        self.c = ctx
        ctx._chk(ctx.L.hfx_burgers_setup(ctx.h), "burgers_setup")
        re = ctx.re
        self.nd = ctx.dim
        self.NLF = re["nNodesFace"] * self.nd
        self.lenU = re["nNodes"] * self.nd
        self.lenQ = ctx.dim * re["nNodes"] * self.nd
        self.lenL = re["nFaces"] * self.NLF
        self.ndofs = ctx.nFaces * self.NLF
        nnz = ctypes.c_int64()
        ctx._chk(ctx.L.hfx_burgers_nnz(ctx.h, ctypes.byref(nnz)), "burgers_nnz")
        self.nnz = nnz.value
        self._keep = {}

    def _arr(self, name, a):
        a = None if a is None else np.ascontiguousarray(a, np.float64)
        self._keep[name] = a
        return a

    def set_tau(self, tau, sides=1):
        t = self._arr("tau", tau)
        self.c._chk(self.c.L.hfx_burgers_set_tau(self.c.h, _p(t), sides), "burgers_set_tau")

    def set_diffusion(self, nu, layout=1):
        if nu is None:
            self.c._chk(self.c.L.hfx_burgers_set_diffusion(self.c.h, None, 0, 0), "burgers_set_diffusion")
            return
        v = self._arr("nu", nu)
        rows = self.c.nCells * self.c.re["nNodes"] if layout == 1 else v.shape[0]
        self.c._chk(self.c.L.hfx_burgers_set_diffusion(self.c.h, _p(v), v.size // rows, layout),
                    "burgers_set_diffusion")

    def set_source(self, values):
        v = self._arr("src", values)
        self.c._chk(self.c.L.hfx_burgers_set_source(self.c.h, _p(v)), "burgers_set_source")

    def set_dirichlet(self, values):
        v = self._arr("dir", values)
        self.c._chk(self.c.L.hfx_burgers_set_dirichlet(self.c.h, _p(v)), "burgers_set_dirichlet")

    def set_time_step(self, dt):
        self.c._chk(self.c.L.hfx_burgers_set_time_step(self.c.h, float(dt)), "burgers_set_time_step")

    def set_state(self, solution=None, buffer=None, trace=None, old=None):
        a = [None if x is None else np.ascontiguousarray(x, np.float64) for x in (solution, buffer, trace, old)]
        self.c._chk(self.c.L.hfx_burgers_set_state(self.c.h, *[_p(x) for x in a]), "burgers_set_state")

    def get_state(self):
        E = self.c.nCells
        sol, flux = np.zeros((E, self.lenU)), np.zeros((E, self.lenQ))
        trace, buf = np.zeros(self.ndofs), np.zeros((E, self.lenU))
        self.c._chk(self.c.L.hfx_burgers_get_state(self.c.h, _p(sol), _p(flux), _p(trace), _p(buf)),
                    "burgers_get_state")
        return sol, flux, trace, buf

    def begin_step(self):
        self.c._chk(self.c.L.hfx_burgers_begin_step(self.c.h), "burgers_begin_step")

    def assemble(self):
        self.c._chk(self.c.L.hfx_burgers_assemble(self.c.h), "burgers_assemble")

    def solve(self, **opts):
        o = solve_opts(**dict({"method": KSP_GMRES}, **opts))
        info = SolveInfo()
        self.c._chk(self.c.L.hfx_burgers_solve(self.c.h, ctypes.byref(o), ctypes.byref(info)), "burgers_solve")
        return info

    def newton(self, **kw):
        o = newton_opts(**kw)
        info = NewtonInfo()
        self.c._chk(self.c.L.hfx_burgers_newton(self.c.h, ctypes.byref(o), ctypes.byref(info)), "burgers_newton")
        return info

    def condensed(self):
        E, U, Q, Ll = self.c.nCells, self.lenU, self.lenQ, self.lenL
        out = dict(S=np.zeros((E, Ll * Ll)), S0=np.zeros((E, Ll)), U=np.zeros((E, U * Ll)), Q=np.zeros((E, Q * Ll)),
                   U0=np.zeros((E, U)), Q0=np.zeros((E, Q)))
        self.c._chk(self.c.L.hfx_burgers_get_condensed(self.c.h, *[_p(out[k]) for k in ("S", "S0", "U", "Q", "U0", "Q0")]),
                    "burgers_get_condensed")
        return out

    def cg_operators(self, which=7, precision=0, velocity=None, vel_layout=1):
        """CG element operators [nCells][3][N*N] (column-major per element): Mass, Diffusion
        (this context's diffusion field), Convection (nodal velocity)."""
        N = self.re["nNodes"]
        out = np.zeros((self.nCells, 3, N * N))
        v = None if velocity is None else np.ascontiguousarray(velocity, np.float64)
        self._chk(self.L.hfx_cg_operators(self.h, which, precision, _p(v), vel_layout, _p(out)), "cg_operators")
        return out

    def tuning_info(self):
        """(kernel chosen for the FP32 trace operator or -1, [ms per launch of kernels 0..3])."""
        k = ctypes.c_int()
        t = (ctypes.c_float * 4)()
        self._chk(self.L.hfx_tuning_info(self.h, ctypes.byref(k), t), "tuning_info")
        return k.value, [t[0], t[1], t[2], t[3]]

    def mixed_assembly_info(self):
        """1 when the last mixed assembly contracted the element blocks on the tensor cores."""
        v = ctypes.c_int()
        self._chk(self.L.hfx_mixed_assembly_info(self.h, ctypes.byref(v)), "mixed_assembly_info")
        return v.value

    def tc_blocks(self, cells):
        """FP32 element blocks of the tensor-core mixed assembly, [len(cells)][stride]."""
        cells = np.ascontiguousarray(cells, np.int32)
        st = ctypes.c_int64()
        self.L.hfx_get_tc_blocks(self.h, 0, None, None, ctypes.byref(st))
        out = np.zeros((len(cells), st.value), np.float32)
        self._chk(self.L.hfx_get_tc_blocks(self.h, len(cells), _p(cells), _p(out), ctypes.byref(st)), "get_tc_blocks")
        return out

    def condensed_sample(self, cells):
        cells = np.ascontiguousarray(cells, np.int32)
        n, U, Q, Ll = len(cells), self.lenU, self.lenQ, self.lenL
        out = dict(S=np.zeros((n, Ll * Ll)), S0=np.zeros((n, Ll)), U=np.zeros((n, U * Ll)), Q=np.zeros((n, Q * Ll)),
                   U0=np.zeros((n, U)), Q0=np.zeros((n, Q)))
        self._chk(self.L.hfx_get_condensed_sample(self.h, n, _p(cells),
                                                  *[_p(out[k]) for k in ("S", "S0", "U", "Q", "U0", "Q0")]),
                  "get_condensed_sample")
        return out

    def csr_rows(self, faces):
        """AIJ rows of the listed faces: (rowlen, col, val, rhs), rows back to back."""
        faces = np.ascontiguousarray(faces, np.int32)
        Nf = self.re["nNodesFace"]
        nr = len(faces) * Nf
        cap = nr * 2 * self.re["nFaces"] * Nf
        rowlen = np.zeros(nr, np.int32)
        col = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        rhs = np.zeros(nr)
        self._chk(self.L.hfx_get_csr_rows(self.h, len(faces), _p(faces), _p(rowlen), _p(col), _p(val), _p(rhs), cap),
                  "get_csr_rows")
        n = int(rowlen.sum())
        return rowlen, col[:n], val[:n], rhs

    def csr(self):
        rowptr = np.zeros(self.ndofs + 1, np.int64)
        col = np.zeros(self.nnz, np.int32)
        val = np.zeros(self.nnz)
        rhs = np.zeros(self.ndofs)
        self.c._chk(self.c.L.hfx_burgers_get_csr(self.c.h, _p(rowptr), _p(col), _p(val), _p(rhs)), "burgers_get_csr")
        return rowptr, col, val, rhs
