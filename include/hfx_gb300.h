/*
 * hfx_gb300.h -- C ABI of the GB300 (sm_103a) HDG hot path.
 *
 * Drop-in for HyperFox's HDG element-local path and the trace solve behind it:
 * every entry point below replaces one reference interface, cited as
 * file:line of the HyperFox source tree. Plain pointers and sizes only; every
 * function returns an int status (HFX_OK == 0) and never throws or aborts.
 * The message of the last failure on a context is hfx_last_error(ctx).
 *
 * Host arrays are copied; device state is owned by the context. A context is
 * used from one host thread at a time and runs its work on its own stream.
 *
 * Layouts (all follow HyperFox):
 *   coords      [nNodes][dim]                        (Mesh nodes, Mesh.cpp:31-46)
 *   cells       [nCells][nNodesPerCell]   int32      (vertices first)
 *   cell2face   [nCells][nFacesPerCell]              (Mesh.cpp:404-425)
 *   face2cell   [nFaces][2], -1 on the boundary      (Mesh.cpp:377-402)
 *   faces       [nFaces][nNodesPerFace]              (Mesh.cpp:517-537)
 *   Tau         [nFaces][nNodesPerFace][1 or 2]      (Face field, HDGSolver.cpp:276-304)
 *   Dirichlet   [nFaces][nNodesPerFace]              (Face field, TestHDGLaplace.cpp:37-46)
 *   Trace       [nFaces][nNodesPerFace]              (global DOF (face*Nf+node), HDGSolver.cpp:596)
 *   Solution    [nCells][nNodesPerCell]              (Cell field, HDGSolver.cpp:768)
 *   Flux        [nCells][nNodesPerCell][dim]         (Cell field, HDGSolver.cpp:769)
 *   S,S0,U,Q,U0,Q0 per element, column-major         (HDGSolver.cpp:93-104,331-348)
 */
#ifndef HFX_GB300_H
#define HFX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HFX_OK 0
#define HFX_ERR_ARG 1           /* bad argument (sizes, pointers, unsupported order) */
#define HFX_ERR_STATE 2         /* call out of order (HyperFox throws ErrorHandle) */
#define HFX_ERR_CUDA 3          /* CUDA runtime error */
#define HFX_ERR_ALLOC 4         /* device allocation failed */
#define HFX_ERR_NOT_CONVERGED 5 /* Krylov solve hit maxits */
#define HFX_ERR_BREAKDOWN 6     /* Krylov breakdown (zero curvature) */
#define HFX_ERR_NAN 7           /* NaN/Inf detected */
#define HFX_ERR_SINGULAR 8      /* singular element block in condensation */
#define HFX_ERR_UNSUPPORTED 9   /* feature not built */

/* Krylov method / preconditioner / precision (PetscOpts.h:8-29 analogue). */
#define HFX_KSP_CG 0        /* CG on the symmetric-eliminated trace system */
#define HFX_KSP_GMRES 1     /* restarted GMRES, any nonsingular system */
#define HFX_KSP_AUTO 2      /* CG when the trace system is symmetric (diffusion tensor constant
                               inside every cell), else GMRES (the default) */
#define HFX_PC_NONE 0
#define HFX_PC_JACOBI 1
#define HFX_PC_BLOCK_JACOBI 2 /* one dense block per face (HDG trace systems) */
#define HFX_PC_TWOLEVEL 3     /* block Jacobi + coarse correction on the mesh vertices (CG only;
                                 no counterpart in the reference, see hfx_solve) */
#define HFX_PREC_FP64 0
#define HFX_PREC_MIXED 1    /* FP32 inner Krylov inside FP64 iterative refinement */

/* Source modes for hfx_set_source (Source::calcSource, Source.cpp:5-22). */
#define HFX_SRC_NONE 0      /* no source (HDGLaplaceModel) */
#define HFX_SRC_VALUES 1    /* caller gives f at every volume IP: [nCells][nIP] */
#define HFX_SRC_SINPROD 2   /* f = param * prod_k sin(pi x_k)  (manufactured u = prod sin) */

typedef struct hfx_ctx hfx_ctx;

typedef struct {
  int dim, order, nNodes, nFaces, nNodesFace, nIP, nIPFace;
} hfx_refel_info;

typedef struct {
  int method;            /* HFX_KSP_* */
  int precond;           /* HFX_PC_* */
  int precision;         /* HFX_PREC_* */
  double rtol;           /* ||b - A x|| <= rtol ||b|| (PetscOpts::rtol) */
  int maxits;            /* total inner iterations allowed (PetscOpts::maxits) */
  int restart;           /* GMRES restart length (PETSc default 30) */
  double inner_rtol;     /* mixed precision: FP32 residual reduction between FP64 residual
                            replacements (CG) or per refinement step (default 1e-2) */
  int use_initial_guess; /* start from the trace already on the device */
  int coarse_guess;      /* HFX_PC_TWOLEVEL: start from the prolongated coarse solution */
  double coarse_rtol;    /* HFX_PC_TWOLEVEL: residual reduction the Chebyshev coarse solve targets */
  int coarse_mode;       /* HFX_PC_TWOLEVEL: HFX_COARSE_CHEBYSHEV or HFX_COARSE_LEARNED */
  int coarse_degree;     /* HFX_PC_TWOLEVEL Chebyshev: fixed degree (1-64); 0 = the degree
                            coarse_rtol asks for */
} hfx_solve_opts;

/* ---- CG element operators (Mass.cpp:5-38, Diffusion.cpp:5-43, Convection.cpp:21-46) ----
 * Per element, one DOF per node: Mass M(i,j) = sum dV phi_i phi_j; Diffusion D(i,j) = sum dV
 * (K grad phi_i)^T grad phi_j with K the context's diffusion field (hfx_set_kappa: nodal scalar
 * or d x d tensor interpolated to the IPs as Diffusion::setDiffTensor does; none: identity);
 * Convection C(k,l) = sum dV phi_k (v . grad phi_l) with the nodal velocity v (layout 0
 * [nNodes][dim], 1 [nCells][N][dim]; interpolated as Convection::setVelocity does). which: a
 * sum of HFX_OP_*. out (host): [nCells][3][N*N], entry (i, j) of operator k at k*N*N + j*N + i
 * (Eigen's column-major); operators not asked are left unspecified. precision HFX_PREC_FP64:
 * FP64 quadrature on the CUDA cores (agrees with the reference's FP64 assembly to round-off);
 * HFX_PREC_MIXED: the contractions on the tensor cores (TF32 hi/lo split, FP32 accumulation;
 * within 2e-5 of each operator's largest entry). */
#define HFX_OP_MASS 1
#define HFX_OP_DIFFUSION 2
#define HFX_OP_CONVECTION 4
int hfx_cg_operators(hfx_ctx* ctx, int which, int precision, const double* velocity, int velLayout, double* out);

/* Test hook of the failure path (no counterpart in the reference): the next two-level solve
 * runs the cooperative one-launch coarse solve (also where the coarse space is small enough
 * for the one-cluster solve), one block withholds its first grid-barrier arrival, so the
 * others' bounded wait (about a second) runs out; the solve must then report
 * info->fallback = 1 and finish with block-Jacobi CG. One shot. */
int hfx_test_coarse_barrier(hfx_ctx* ctx);

/* Coarse solve of HFX_PC_TWOLEVEL. LEARNED applies the polynomial trained by
 * hfx_coarse_train; until one has been accepted it applies Chebyshev of the trained degree
 * (of the reduction target's degree when no training has run). */
#define HFX_COARSE_CHEBYSHEV 0
#define HFX_COARSE_LEARNED 1

typedef struct {
  int status;              /* HFX_OK or an error code */
  int iterations;          /* Krylov iterations (inner, summed) */
  int refinements;         /* FP64 refinement steps (mixed precision) */
  double rel_residual;     /* final FP64 ||b-Ax||/||b|| of the reference system */
  double solve_ms;         /* device time of the solve */
  int fallback;            /* 1: the two-level solve failed and block Jacobi finished it */
  int coarse_degree;       /* HFX_PC_TWOLEVEL: degree of the coarse polynomial used */
  int coarse_learned;      /* 1: the learned coarse polynomial was applied */
} hfx_solve_info;

typedef struct {
  int degree, samples, steps, accepted;
  double loss_chebyshev;   /* loss of Chebyshev of the same degree (the starting point) */
  double loss_learned;     /* loss after training (accepted only if lower) */
  double max_poly;         /* max of the residual polynomial on [0, lmax]: <= 1 keeps CG valid */
  double train_ms;         /* sample collection + training, host wall time */
  double loss_first_step;  /* loss after the first optimiser step */
  int lower_steps;         /* optimiser steps that lowered the best loss */
  int rejected_steps;      /* lower-loss steps refused by the polynomial check */
} hfx_train_info;

/* ---- context ------------------------------------------------------------ */
int hfx_ctx_create(int device, hfx_ctx** out);
int hfx_ctx_destroy(hfx_ctx* ctx);
const char* hfx_last_error(const hfx_ctx* ctx);
int hfx_version(void);

/* ---- reference element (host, no GPU needed) -----------------------------
 * Replaces ReferenceElement(dim, ord, "simplex") (ReferenceElement.cpp:5-26):
 * nodes (ReferenceElement.cpp:614-1150), face nodes (:136-202), cubature of
 * order 2p (:102-106, Cubature.cpp:5-139), shape functions and derivatives at
 * the integration points (:447-480). Sizes from hfx_refel_query.
 *   nodes[N*dim] faceNodes[F*Nf] ipCoords[nIP*dim] ipWeights[nIP]
 *   phi[nIP*N] dphi[nIP*N*dim]; face element: fIpCoords[nIPf*(dim-1)],
 *   fIpWeights[nIPf], fPhi[nIPf*Nf], fDphi[nIPf*Nf*(dim-1)] (any may be NULL) */
int hfx_refel_query(int dim, int order, hfx_refel_info* info);
int hfx_refel_tables(int dim, int order, double* nodes, int* faceNodes, double* ipCoords,
                     double* ipWeights, double* phi, double* dphi, double* fIpCoords,
                     double* fIpWeights, double* fPhi, double* fDphi);

/* ---- mesh ------------------------------------------------------------------
 * Replaces Mesh::setMesh + Mesh::computeFaces (Mesh.cpp:31-46,183-537). When
 * cell2face is NULL the face topology is computed on the host with the MOAB
 * creation-order rule (cells in order, sides in MOAB canonical order); else
 * the caller's topology (cell2face, face2cell, faces, boundary) is used. */
int hfx_mesh_upload(hfx_ctx* ctx, int dim, int order, int nNodes, const double* coords, int nCells,
                    const int* cells, int nFaces, const int* cell2face, const int* face2cell,
                    const int* faces, int nBoundary, const int* boundary);
int hfx_mesh_sizes(hfx_ctx* ctx, int* nFaces, int* nBoundary, int64_t* nnz);
/* Host only, no context: the same MOAB-rule topology as hfx_mesh_upload
 * computes. Call with NULL arrays for nFaces/nBoundary, then with arrays
 * sized cell2face[nCells*F], face2cell[2*nFaces], faces[nFaces*Nf],
 * boundary[nBoundary]. */
int hfx_mesh_compute_topology(int dim, int order, int nCells, const int* cells, int* nFaces, int* nBoundary,
                              int* cell2face, int* face2cell, int* faces, int* boundary);
int hfx_mesh_topology(hfx_ctx* ctx, int* cell2face, int* face2cell, int* faces, int* boundary);

/* ---- mesh input (host, no GPU needed) ----------------------------------------
 * Replaces tools/convertGmsh2H5HO.cpp:117-257,367-398 (gmsh reading through
 * MOAB and high-order node construction) without MOAB. hfx_gmsh_read reads a
 * gmsh .msh file (format 2.2, ASCII) and returns the linear simplex mesh of
 * dimension dim: coords [nNodes][dim] (vertices used by the cells, in gmsh id
 * order) and cells [nCells][dim+1] (0-based); call with coords == NULL for the
 * sizes. hfx_mesh_high_order maps the reference nodes of order `order` into every
 * linear cell and merges coincident nodes: coords [nNodes][dim], cells
 * [nCells][N] in reference-node order, ready for hfx_mesh_upload (two-call
 * likewise). hfx_mesh_io_error returns the last message of these and of the HDF5 calls below. */
int hfx_gmsh_read(const char* path, int dim, int* nNodes, int* nCells, double* coords, int* cells);
int hfx_mesh_high_order(int dim, int order, int nLinNodes, const double* linCoords, int nCells, const int* linCells,
                        int* nNodes, double* coords, int* cells);
const char* hfx_mesh_io_error(void);

/* ---- HDF5 mesh and field files (host, no GPU, no HDF5 library) --------------
 * Replace HDF5Io::load / loadMesh / loadFields and HDF5Io::write / writeMesh /
 * writeFields (src/io/HDF5Io.cpp:13-62,111-191 and :64-109,193-393) for the
 * files they exchange: /Mesh/Nodes float64 [nNodes][nodeDim], /Mesh/Cells int32
 * [nCells][nodesPerCell], /FieldData/<name> float64 [entities][objs][vals] with
 * the int attribute "ftype" (FieldType: -1 None, 0 Node, 1 Edge, 2 Face, 3 Cell).
 * hfx_h5_read_mesh: call with coords == cells == NULL for the sizes.
 * hfx_h5_field_names: the names under /FieldData, each followed by '\n', into
 * buf (truncated to bufLen-1 and terminated); *needLen = the length it needs.
 * hfx_h5_read_field: shape[3] and *ftype always; values when not NULL. Missing
 * field or attribute -> HFX_ERR_ARG with the reference's message.
 * hfx_h5_write: mesh when nNodes > 0, then nFields fields (names[i], ftypes[i],
 * shapes[3*i..3*i+2], values[i]); at least one of the two. Errors in
 * hfx_mesh_io_error(). */
int hfx_h5_read_mesh(const char* path, int* nodeDim, int* nNodes, int* nCells, int* nodesPerCell, double* coords,
                     int* cells);
int hfx_h5_field_names(const char* path, char* buf, int bufLen, int* nFields, int* needLen);
int hfx_h5_read_field(const char* path, const char* name, int* ftype, int64_t* shape, double* values);
int hfx_h5_write(const char* path, int nodeDim, int nNodes, const double* coords, int nCells, int nodesPerCell,
                 const int* cells, int nFields, const char* const* names, const int* ftypes, const int64_t* shapes,
                 const double* const* values);

/* ---- fields (the HDGSolver field map) --------------------------------------
 * Tau: Face field, nVals 1 or 2 (double valued, side 0 = face2cell[0]).
 * Kappa (DiffusionTensor, HDGDiffusionSource.cpp:60-79): comps 0 (identity),
 * 1 (scalar) or dim*dim (column-major tensor); layout 0 = per mesh node
 * [nNodes][comps], 1 = per cell node [nCells][N][comps].
 * Dirichlet: Face field [nFaces][Nf] (only boundary faces are read).
 * Time scheme: implicit Euler (Euler.cpp:18-34) when dt > 0, with the previous
 * Solution [nCells][N]. */
int hfx_set_tau(hfx_ctx* ctx, const double* tau, int nVals);
int hfx_set_kappa(hfx_ctx* ctx, const double* kappa, int comps, int layout);
int hfx_set_source(hfx_ctx* ctx, int mode, const double* values, double param);
int hfx_set_dirichlet(hfx_ctx* ctx, const double* values);
int hfx_set_time_scheme(hfx_ctx* ctx, double dt, const double* uOld);
/* HDGSolverType (HDGSolverOpts.h:6-10). IMPLICIT (default) condenses as usual.
 * WEXPLICIT and SEXPLICIT (HDGSolver.cpp:349-354,709-729) build the trace system
 * from the current Solution and Flux: S = Sll, S0 = -Slu Solution - Slq Flux; WEXPLICIT
 * solves it with hfx_solve's Krylov method, SEXPLICIT face by face (S_f^{-1} S0_f).
 * The state is the last hfx_recover result, or what hfx_set_state uploads
 * (Solution [nCells][N], Flux [nCells][N*dim] node-major); it starts at 0. */
#define HFX_IMPLICIT 0
#define HFX_WEXPLICIT 1
#define HFX_SEXPLICIT 2
int hfx_set_solver_type(hfx_ctx* ctx, int type);
int hfx_set_state(hfx_ctx* ctx, const double* solution, const double* flux);
int hfx_ip_coords(hfx_ctx* ctx, double* out /* [nCells][nIP][dim] */);

/* ---- assembly ----------------------------------------------------------------
 * Replaces HDGSolver::assemble (HDGSolver.cpp:166-174): element Jacobians,
 * normals, HDGBase + HDGDiffusion + Source operators, static condensation
 * (:331-348), Dirichlet Set (:361-529) and the scatter into the trace CSR
 * (:531-675). All on the device, FP64. */
int hfx_assemble(hfx_ctx* ctx);
/* hfx_assemble_ex(ctx, HFX_PREC_FP64) == hfx_assemble. HFX_PREC_MIXED assembles
 * in FP32 for a mixed-precision solve: hfx_solve then refines the full HDG
 * system (u, q, lambda) with FP64 residuals (matrix free, the reference's
 * element operators) and FP32 condensed corrections until the FP64 residual
 * meets rtol; hfx_recover returns the refined FP64 Solution and Flux. The
 * element blocks and CSR stay FP32 (hfx_get_condensed / hfx_get_csr refuse). */
int hfx_assemble_ex(hfx_ctx* ctx, int precision);
/* Element kernel choice. 0 (default): straight-sided cells with a symmetric diffusion
 * tensor constant inside every cell use reference operators (same blocks, far fewer
 * FP64 operations; Q and Q0 are then formed on demand by hfx_get_condensed and by
 * the recovery); everything else uses per-element quadrature. 1: quadrature always.
 * hfx_assembly_info reports whether the last FP64 assembly took the affine path. */
int hfx_set_assembly_path(hfx_ctx* ctx, int path);
int hfx_assembly_info(hfx_ctx* ctx, int* affine);
/* The mixed assembly (HFX_PREC_MIXED) contracts the element operators of HDGBase, HDGDiffusion
 * and Mass (HDGBase.cpp:67-158, HDGDiffusion.cpp:74-145, Mass.cpp:5-38: the volume blocks C_d,
 * K_d, M and the face blocks T, E_d, H_d) on the tensor cores (tcgen05, TF32 hi/lo split,
 * FP32 accumulation; agreement with the FP64 quadrature within 2e-5 of each block's largest
 * entry) for orders 1-5 (2D) / 1-3 (3D) under path 0; path 1 integrates them on the CUDA
 * cores. *tensorCores = 1 when the last mixed assembly used the tensor cores. */
int hfx_mixed_assembly_info(hfx_ctx* ctx, int* tensorCores);
/* Launch tuner (no counterpart in the reference): the first mixed-precision CG solve on a mesh
 * times the kernels of the FP32 trace operator on the system's own values (0 row per lane,
 * 1 the blocks staged in shared memory by bulk copies (cp.async.bulk, for Nf even), 2 row
 * per lane with paired (float2) loads of the blocks read transposed, 3 the same with the
 * gathered x read back as float4s) and keeps the fastest for that mesh.
 * *spmvKernel: -1 not tuned yet, else the kernel chosen; spmvMs[4]: their measured times per
 * launch (ms; 0 for a kernel not tried). */
int hfx_tuning_info(hfx_ctx* ctx, int* spmvKernel, float* spmvMs);
/* Sets the choice instead: 0..3 fixes the kernel (1 only where Nf is even, elsewhere it runs
 * kernel 0), -1 tunes again at the next mixed solve. */
int hfx_set_tuning(hfx_ctx* ctx, int spmvKernel);
/* Those FP32 blocks for a list of cells, [count][*stride]: volume rows [C_0..C_{d-1} | K_0..
 * K_{d-1} | M] of N values (row (k, i) = block k, node i), face rows [T | E | H] of Nf values
 * (T row (f, a); E, H rows (f, k, a)), then the source load f_u (N). */
int hfx_get_tc_blocks(hfx_ctx* ctx, int count, const int* cells, float* out, int64_t* stride);

/* ---- Runge-Kutta time integration (RungeKutta.cpp:5-213, HDGModel.cpp:39-47) --
 * A scheme applies to the U rows of every element system at hfx_assemble:
 * K' = dt a_ss K + M, f' = dt f - dt K uj + K' ut (ut the Old fields, uj = ut +
 * dt sum_{i<s} a_si k_i over Solution, Flux and Trace, the reference's
 * auxiliary fields {"Flux", "Trace"}). The fields live on the device:
 * Solution/Flux are the last recovery (or hfx_set_state), Trace the last solve
 * (or hfx_set_trace). Per time step: hfx_rk_begin_step (Old* = current), then per
 * stage hfx_assemble, hfx_solve, hfx_recover, hfx_rk_compute_stage, and finally
 * hfx_rk_compute_solution. hfx_rk_set takes a user table ((S+1)^2 row-major, rows
 * [c_i | a_i.], last row [0 | b]) whose strictly upper part must be zero
 * (RungeKutta::setButcherTable(EMatrix)); hfx_rk_set_type takes a named table
 * as is; nStages 0 switches the scheme off. FP64 assembly only (the
 * mixed-precision assembly refuses a scheme). While a scheme is set it replaces
 * hfx_set_time_scheme's implicit Euler. */
#define HFX_RK_FEULER 0
#define HFX_RK_EMIDPOINT 1
#define HFX_RK_HEUN 2
#define HFX_RK_KUTTA3 3
#define HFX_RK_HEUN3 4
#define HFX_RK_SSPRK3 5
#define HFX_RK_RK4 6
#define HFX_RK_BEULER 7
#define HFX_RK_IMIDPOINT 8
#define HFX_RK_CRANKNICOLSON 9
#define HFX_RK_KS2 10
#define HFX_RK_QZ2 11
#define HFX_RK_ALX2 12
#define HFX_RK_RK43 13
int hfx_rk_butcher(int type, int* nStages, double* table);
int hfx_rk_set(hfx_ctx* ctx, int nStages, const double* table, double dt);
int hfx_rk_set_type(hfx_ctx* ctx, int type, double dt);
int hfx_rk_begin_step(hfx_ctx* ctx);
int hfx_rk_compute_stage(hfx_ctx* ctx);
int hfx_rk_compute_solution(hfx_ctx* ctx);
int hfx_set_trace(hfx_ctx* ctx, const double* trace);
int hfx_get_state(hfx_ctx* ctx, double* solution, double* flux, double* trace);
/* Condensed element blocks, column-major per element (any pointer may be NULL). */
int hfx_get_condensed(hfx_ctx* ctx, double* S, double* S0, double* U, double* Q, double* U0,
                      double* Q0);
/* Global trace system in PETSc AIJ form: sorted columns, explicit zeros kept. */
int hfx_get_csr(hfx_ctx* ctx, int64_t* rowptr, int* col, double* val, double* rhs);
/* The condensed blocks of a list of elements only, compact ([count][...], column-major per
 * element, any output may be NULL): element-block inspection of meshes too large to export
 * whole (HDGSolver's U, Q, S, U0, Q0, S0 fields of those cells). */
int hfx_get_condensed_sample(hfx_ctx* ctx, int count, const int* cells, double* S, double* S0, double* U,
                             double* Q, double* U0, double* Q0);
/* The AIJ rows of a list of distinct faces (every node of each face, in face then node
 * order), as hfx_get_csr would export them: rowlen[count*Nf], then the rows' col / val
 * back to back (cap entries at most; HFX_ERR_ARG if cap is too small), rhs[count*Nf]. */
int hfx_get_csr_rows(hfx_ctx* ctx, int count, const int* faces, int* rowlen, int* col, double* val, double* rhs,
                     int64_t cap);

/* ---- solve and recovery --------------------------------------------------------
 * hfx_solve replaces LinAlgebraInterface::solve / PetscInterface::solve
 * (PetscInterface.cpp:222-247) on the assembled trace system; trace may be NULL
 * (the result stays on the device). hfx_recover replaces the recovery loop of
 * HDGSolver::solve (HDGSolver.cpp:741-775); NULL outputs keep
 * Solution and Flux on the device. */
void hfx_solve_opts_default(hfx_solve_opts* opts);
int hfx_solve(hfx_ctx* ctx, const hfx_solve_opts* opts, double* trace, hfx_solve_info* info);
int hfx_recover(hfx_ctx* ctx, double* solution, double* flux);

/* Coarse operator of HFX_PC_TWOLEVEL (no counterpart in the reference): one
 * coarse DOF per mesh vertex (vertexNode[nV] = mesh node id), prolongation
 * P[f*Nf + a, v] = barycentric coordinate of face node a w.r.t. face vertex v
 * (rows of Dirichlet faces zero), A_c = P^T A' P with A' the sign-flipped
 * interior block of the trace system, in CSR (rowptr[nV+1], col/val[nnz],
 * FP32). Call with rowptr == NULL for the sizes. Needs an assembled system. */
int hfx_coarse_operator(hfx_ctx* ctx, int* nV, int64_t* nnz, int* rowptr, int* col, float* val, int* vertexNode);
/* Spectral bounds of D^{-1} A_c (D its diagonal) behind the Chebyshev coarse solve of
 * HFX_PC_TWOLEVEL (no counterpart in the reference), set up like hfx_coarse_operator:
 * out[5] = lmin, lmax (the Chebyshev interval), the smallest and largest Ritz values of
 * the Lanczos steps (inside the spectrum) and the infinity norm of D^{-1/2} A_c D^{-1/2}
 * (above the spectral radius); lmax = min(1.1 * largest Ritz value, that norm). */
int hfx_coarse_bounds(hfx_ctx* ctx, double* out);

/* Learned coarse correction (no counterpart in the reference). The coarse solve
 * of HFX_PC_TWOLEVEL becomes a degree-K polynomial in D^{-1} A_c, Richardson
 * steps y += theta_k D^{-1} (r - A_c y), whose weights are trained on the GPU
 * with this library's forward and backward kernels to minimise the energy
 * (A_c-norm) of the coarse error left after the solve, averaged over `samples`
 * coarse errors A_c^{-1} P^T r taken from the residuals r of a two-level CG run
 * on the current system (every second iteration). Training starts from
 * Chebyshev of degree K; the result is kept only if it beats it and keeps the
 * coarse solve positive semidefinite. hfx_solve(coarse_mode =
 * HFX_COARSE_LEARNED) then applies it; block-Jacobi CG stays the fallback of
 * the whole two-level solve. hfx_coarse_loss_grad evaluates the same loss and
 * its gradient for given theta on caller error samples [S][nV] (host, FP32)
 * with the same kernels. */
int hfx_coarse_train(hfx_ctx* ctx, int degree, int samples, int steps, hfx_train_info* info);
int hfx_coarse_loss_grad(hfx_ctx* ctx, int degree, const double* theta, int samples, const float* values,
                         double* loss, double* grad);

/* ---- timing on the context's stream (CUDA events; no profiler) ---------------
 * hfx_profile_enable(ctx, 1) resets and starts per-kernel event timing;
 * hfx_kernel_time reads launches and total device ms of one kernel class
 * (HFX_K_*). hfx_mark records an event in one of 8 slots; hfx_elapsed_ms
 * returns the device time between two marks. hfx_synchronize waits for the
 * context's stream. These replace the std::chrono stage timers of the
 * reference's tests (TestHDGDiffusionSource.cpp:238-251). */
#define HFX_K_LOCAL 0
#define HFX_K_SCATTER 1
#define HFX_K_SPMV64 2
#define HFX_K_SPMV32 3
#define HFX_K_UPDATE 4
#define HFX_K_RECOVER 5
#define HFX_K_OTHER 6
#define HFX_K_RESIDUAL 7
#define HFX_K_COARSE 8
#define HFX_K_TENSOR 9   /* element contractions on the tensor cores (mixed assembly) */
int hfx_profile_enable(hfx_ctx* ctx, int on);
int hfx_kernel_time(hfx_ctx* ctx, int kernel, int* launches, double* ms);
int hfx_mark(hfx_ctx* ctx, int slot);
int hfx_elapsed_ms(hfx_ctx* ctx, int slot0, int slot1, double* ms);
/* Device time from mark slot0 of ctx0 to mark slot1 of ctx1 (contexts on one device; negative
 * when the second event came first): the span of work that ran on several contexts' streams
 * at once. */
int hfx_elapsed_between(hfx_ctx* ctx0, int slot0, hfx_ctx* ctx1, int slot1, double* ms);
int hfx_synchronize(hfx_ctx* ctx);

/* ---- generic sparse system (LinAlgebraInterface, LinAlgebraInterface.h:23-162) ----
 * The state machine initialize -> configure -> allocate -> set/add -> assemble ->
 * solve is kept by the host C++ wrapper; these entry points take values in the
 * reference's row-major is.size() x js.size() block convention. */
typedef struct hfx_la hfx_la;
int hfx_la_create(hfx_ctx* ctx, hfx_la** out);
int hfx_la_destroy(hfx_la* la);
int hfx_la_allocate(hfx_la* la, int ndofs);
int hfx_la_set_values(hfx_la* la, int nr, const int* rows, int nc, const int* cols,
                      const double* vals, int insert);
int hfx_la_set_rhs(hfx_la* la, int n, const int* idx, const double* vals, int insert);
int hfx_la_zero_rows(hfx_la* la, int n, const int* rows);
int hfx_la_assemble(hfx_la* la);
int hfx_la_clear(hfx_la* la);
int hfx_la_solve(hfx_la* la, const hfx_solve_opts* opts, double* x, hfx_solve_info* info);
int hfx_la_nnz(hfx_la* la, int64_t* nnz);

/* ---- viscous Burgers, Newton (HDGBurgersModel, HDGUNabU, NonLinearWrapper) ----
 * Vector Burgers with nd = dim unknowns per node (HDGBurgersModel.cpp:35-60): local
 * matrix HDGBase + HDGUNabU (+ HDGDiffusion when a diffusion tensor is set), RHS the
 * HDGUNabU RHS + one Source per component, optional implicit Euler (Euler.cpp:18-34),
 * linearised about BufferSolution and Trace (HDGBurgersModel.cpp:5-33). Built for 2D
 * cells, p = 1..5; uses the mesh of hfx_mesh_upload and its own fields and outputs
 * (the scalar path's are untouched). Layouts, nd = dim:
 *   Tau          [nFaces][nNodesPerFace][sides][nd*nd]  nd x nd column-major, sides 1 or 2
 *   Dirichlet    [nFaces][nNodesPerFace][nd]            face order (added to the local rows as
 *                                                       they are, HDGSolver.cpp:493-497)
 *   Source       [nCells][nIP][nd]                      f_c at the volume IPs
 *   Solution, BufferSolution, OldSolution [nCells][nNodesPerCell][nd]
 *   Flux         [nCells][nNodesPerCell][dim][nd]       (local Q order)
 *   Trace        [nFaces][nNodesPerFace][nd]            global DOF (face*Nf + node)*nd + k
 *   S,S0,U,Q,U0,Q0 per element, column-major, lenU = N*nd, lenQ = dim*N*nd, lenL = F*Nf*nd */
typedef struct {
  double res_tol;          /* NonLinearWrapper::setResidualTolerance (default 1e-6) */
  int max_iters;           /* NonLinearWrapper::setMaxIterations (default 20) */
  double dampening;        /* NonLinearWrapper::setDampening (default 0) */
  hfx_solve_opts lin;      /* the linear solve of every iteration (GMRES, block Jacobi) */
  int warm_start;          /* 1: each Krylov solve starts from the current trace (PETSc starts
                              from zero, KSPSetInitialGuessNonzero is not called) */
  int history;             /* 1..8: each Krylov solve starts from the least-squares fit of the
                              last `history` trace solutions to the new system (min ||b' - A' x||
                              over their span, which holds the previous solution), 0: off.
                              No counterpart in the reference. */
} hfx_newton_opts;

typedef struct {
  int status;              /* HFX_OK, or the linear solve's / element kernel's error */
  int iterations;          /* Newton iterations run */
  double residual;         /* last ||Solution - BufferSolution|| / ||BufferSolution|| */
  int krylov_iterations;   /* summed over the iterations */
  double assemble_ms, solve_ms, recover_ms;  /* device times, summed */
} hfx_newton_info;

/* HDGSolver::allocate with HDGBurgersModel (HDGSolver.cpp:81-115, HDGBurgersModel.cpp:35-60):
 * device fields and outputs; defaults tau = I, no diffusion, no source, Dirichlet 0, stationary,
 * every state field 0. */
int hfx_burgers_setup(hfx_ctx* ctx);
/* Tau field (HDGBase::setTau, HDGBase.cpp:18-32; double valued when sides == 2). */
int hfx_burgers_set_tau(hfx_ctx* ctx, const double* tau, int sides);
/* DiffusionTensor (HDGBurgersModel::parseDiffusionVals, HDGBurgersModel.cpp:128-150): comps 1
 * (scalar) or dim*dim per node; layout 0 per mesh node [nNodes][comps], 1 per cell node
 * [nCells][N][comps]; nu == NULL or comps == 0: no diffusion operator. */
int hfx_burgers_set_diffusion(hfx_ctx* ctx, const double* nu, int comps, int layout);
/* One Source per component (HDGBurgersModel::setSourceFunction, HDGBurgersModel.cpp:80-89), given
 * at the volume IPs; NULL: none. */
int hfx_burgers_set_source(hfx_ctx* ctx, const double* values);
int hfx_burgers_set_dirichlet(hfx_ctx* ctx, const double* values);
/* Euler::setTimeStep (Euler.h): dt > 0 applies implicit Euler about OldSolution; 0 = stationary. */
int hfx_burgers_set_time_step(hfx_ctx* ctx, double dt);
/* Upload fields; a NULL pointer leaves that field as it is. */
int hfx_burgers_set_state(hfx_ctx* ctx, const double* solution, const double* buffer, const double* trace,
                          const double* oldSolution);
/* Download fields; a NULL pointer skips that field. */
int hfx_burgers_get_state(hfx_ctx* ctx, double* solution, double* flux, double* trace, double* buffer);
/* A time step's field copies on the device (TestHDGBurgers.cpp:362-365): BufferSolution and
 * OldSolution <- Solution. */
int hfx_burgers_begin_step(hfx_ctx* ctx);
/* HDGSolver::assemble with the Burgers model (HDGSolver.cpp:166-174): element kernel
 * (assembly + condensation + Dirichlet Set) and the scatter into the trace system. */
int hfx_burgers_assemble(hfx_ctx* ctx);
/* HDGSolver::solve (HDGSolver.cpp:677-779): GMRES on the trace system (PetscInterface::solve,
 * PetscInterface.cpp:222-247), Trace <- the solution, then the local recovery of Solution and Flux.
 * opts->precision HFX_PREC_MIXED: FP32 GMRES on an FP32 copy of the system inside FP64 residual
 * refinement (opts->inner_rtol per refinement, at least 1e-5), to the same FP64 rtol. */
int hfx_burgers_solve(hfx_ctx* ctx, const hfx_solve_opts* opts, hfx_solve_info* info);
/* NonLinearWrapper::solve (NonLinearWrapper.cpp:41-79) with the vanilla linearised solver and
 * residual (assemble + solve; ||Solution - BufferSolution|| / ||BufferSolution||), run on the
 * device: the host reads two numbers per iteration. opts/info may be NULL. Returns HFX_OK also
 * when max_iters ends the loop (as the reference); info->residual says where it stopped. */
void hfx_newton_opts_default(hfx_newton_opts* opts);
int hfx_burgers_newton(hfx_ctx* ctx, const hfx_newton_opts* opts, hfx_newton_info* info);
int hfx_burgers_get_condensed(hfx_ctx* ctx, double* S, double* S0, double* U, double* Q, double* U0,
                              double* Q0);
/* The assembled trace system in PETSc's AIJ layout (sorted columns, explicit zeros kept). */
int hfx_burgers_nnz(hfx_ctx* ctx, int64_t* nnz);
int hfx_burgers_get_csr(hfx_ctx* ctx, int64_t* rowptr, int* col, double* val, double* rhs);

/* ---- allocation-free trace solve -------------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device
 * memory: code under a framework whose caching allocator owns the device
 * memory (a raw cudaMalloc would fragment its pool or break its budget), and
 * real-time loops that cannot take an allocation's latency or failure in the
 * middle of a step. Same FP64 CG + per-face block-Jacobi solve as hfx_solve
 * (HFX_KSP_CG, HFX_PC_BLOCK_JACOBI) on a trace system the caller already holds
 * in device memory: browptr[nFaces+1] and bcol[nBlocks] (face-block pattern),
 * isBoundary[nFaces] (Dirichlet faces), val in the scalar-CSR order
 * hfx_get_csr exports, rhs and the output x [nFaces*nodesPerFace]; stream is a
 * cudaStream_t. The solver's working memory is one fixed __device__ array
 * (about 7.9 MB, held by every GPU that loads the library until exit), so
 * systems above HFX_NOALLOC_MAX_DOFS trace DOFs or HFX_NOALLOC_MAX_NF nodes per
 * face are refused with HFX_ERR_ARG. CG needs a symmetric interior block: a
 * system whose interior block is not symmetric (relative asymmetry above
 * 1e-10), or whose pattern has a row without its diagonal block or a block
 * without its transposed partner, is refused with HFX_ERR_ARG. The first call
 * on a device looks up the array's device address: make that first call
 * before any stream capture. Calls share the array; calls that overlap on the
 * GPU race and must be serialised by the caller. The host drives the
 * iterations and synchronises the stream; the call returns after the solve,
 * with HFX_ERR_NOT_CONVERGED when maxits ends it. info may be NULL. */
#define HFX_NOALLOC_MAX_DOFS 65536
#define HFX_NOALLOC_MAX_NF 10
int hfx_trace_solve_noalloc(int dim, int nodesPerFace, int nFaces, const int64_t* browptr, const int* bcol,
                            const unsigned char* isBoundary, const double* val, const double* rhs, double* x,
                            double rtol, int maxits, void* stream, hfx_solve_info* info);

#ifdef __cplusplus
}
#endif

#endif /* HFX_GB300_H */
