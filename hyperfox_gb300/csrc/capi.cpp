#include <chrono>
// C ABI of the GB300 HDG hot path (declared in include/hfx_gb300.h).
//
// The context owns every device buffer and one CUDA stream. Host arrays are
// copied in; results are copied out into caller buffers, as HyperFox writes
// into Field::getValues()->data().
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/hfx_gb300.h"
#include "hfx_device.h"
#include "hdg_mixed.h"
#include "hfx_host.h"
#include "cg_operators.h"
#include "krylov.h"
#include "la_gmres.h"
#include "tc_assembly.h"
#include "timer.h"

using namespace hfx;

namespace {

struct DevMem {
  std::vector<void*> ptrs;
  ~DevMem() { release(); }
  void release() {
    for (void* p : ptrs) cudaFree(p);
    ptrs.clear();
  }
};

// A field's device buffer, reallocated only when it must grow.
struct FieldBuf {
  double* p = nullptr;
  size_t cap = 0;
  ~FieldBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  cudaError_t set(const double* h, size_t n, cudaStream_t s) {
    if (n > cap) {
      cudaStreamSynchronize(s);
      release();
      cudaError_t e = cudaMalloc(&p, sizeof(double) * (n > 0 ? n : 1));
      if (e != cudaSuccess) {
        p = nullptr;
        return e;
      }
      cap = n;
    }
    return n ? cudaMemcpyAsync(p, h, sizeof(double) * n, cudaMemcpyHostToDevice, s) : cudaSuccess;
  }
};

// Vector Burgers problem on the context's mesh (hfx_burgers_*): nd = dim unknowns
// per node, its own fields, element outputs, trace system and Krylov workspace.
struct BurgersState {
  bool ready = false, assembled = false, solved = false;
  int nd = 0, NLF = 0, NU = 0, NQ = 0, NL = 0;
  int64_t nDofs = 0, nnz = 0;
  int tauSides = 1, kc = 0, nuLayout = 0;
  bool haveSrc = false;
  double dt = 0.0;
  FieldBuf tau, nu, src, dir;
  DevMem mem;
  double *buf = nullptr, *sol = nullptr, *old = nullptr, *flux = nullptr, *trace = nullptr;
  double *S = nullptr, *S0 = nullptr, *U = nullptr, *Q = nullptr, *U0 = nullptr, *Q0 = nullptr;
  double *val = nullptr, *rhs = nullptr, *partials = nullptr, *red = nullptr;
  uint8_t* permx = nullptr;  // face2CellMap at DOF level: [nCells][F][Nf*nd]
  double* cache = nullptr;   // state-independent element blocks, valid while cacheValid
  bool cacheValid = false;
  // the last trace solutions (ring, most recent at histHead - 1) and their images under A'
  double *hist = nullptr, *histY = nullptr;
  int histCap = 0, histCount = 0, histHead = 0;
  int* status = nullptr;
  unsigned* ticket = nullptr;
  DevMem wsMem;
  TraceWorkspace ws{};
  bool wsReady = false;
  int wsRestart = 0;
  bool wsMixed = false;     // FP32 copies for the mixed-precision GMRES allocated
  int wsRestart32 = 0;      // FP32 Krylov basis size
  void release() {
    wsMem.release();
    ws = TraceWorkspace{};
    wsReady = false;
    wsRestart = 0;
    wsMixed = false;
    wsRestart32 = 0;
    mem.release();
    tau.release();
    nu.release();
    src.release();
    dir.release();
    ready = assembled = solved = cacheValid = false;
    hist = histY = nullptr;
    histCap = histCount = histHead = 0;
  }
};

}  // namespace

struct hfx_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string err;
  // mesh and tables
  bool haveMesh = false;
  int dim = 0, order = 0, nNodes = 0, nCells = 0;
  RefEl re;
  Topology topo;
  BlockPattern bp;
  std::vector<uint8_t> perm;
  DevMem meshMem;
  double* d_tab = nullptr;
  float* d_tab32 = nullptr;
  int* d_itab = nullptr;
  double* d_phi = nullptr;
  double* d_coords = nullptr;
  int* d_cells = nullptr;
  int* d_cell2face = nullptr;
  uint8_t* d_perm = nullptr;
  int* d_face2cell = nullptr;
  uint8_t* d_isBnd = nullptr;
  int64_t* d_browptr = nullptr;
  int* d_bcol = nullptr;
  int* d_hidx = nullptr;     // symmetric half storage map of the face blocks
  int2* d_ell = nullptr;     // the rows as fixed-width (bcol, hidx) slots
  int ellWidth = 0;
  int64_t nHalf = 0;
  int* d_brow = nullptr;
  int *d_src0 = nullptr, *d_src1 = nullptr;
  uint8_t *d_loc0 = nullptr, *d_loc1 = nullptr;
  // fields
  FieldBuf tau, kappa, src, dir, uold;
  int tauVals = 1;
  int kc = 0, kLayout = 0;
  bool kappaCellConstant = true;  // symmetric trace system (CG applies)
  int srcMode = 0;
  double srcParam = 0.0;
  double dt = 0.0;
  // affine element path (hdg_affine.cu): straight-sided cells and a symmetric
  // diffusion tensor constant inside every cell
  bool affineMesh = false;
  bool kappaSymmetric = true;
  int assemblyPath = 0;        // 0 automatic, 1 quadrature kernel always
  int solverType = 0;          // HFX_IMPLICIT / HFX_WEXPLICIT / HFX_SEXPLICIT
  bool lastAffine = false;     // the last FP64 assembly used the affine kernel
  bool qValid = false;         // d_Q / d_Q0 hold the current Q, Q0
  double* d_atab = nullptr;    // affine reference operators
  double* d_geo = nullptr;     // [nCells][D*D + F*D]
  double* d_prep = nullptr;    // [nCells][affine_prep_doubles] per-element affine record
  // Runge-Kutta (RungeKutta.cpp): Butcher table (S+1)^2 row-major, stage counter,
  // Old*/RKStage_* fields and the stage vector w on the device
  int rkStages = 0, rkStage = 0;
  std::vector<double> rkTable;
  double rkDt = 0.0;
  DevMem rkMem;
  double *d_oldSol = nullptr, *d_oldFlux = nullptr, *d_oldTrace = nullptr;
  std::vector<double*> d_kSol, d_kFlux, d_kTrace;
  double *d_wU = nullptr, *d_wQ = nullptr, *d_wL = nullptr;
  // outputs
  DevMem outMem;
  double *d_S = nullptr, *d_S0 = nullptr, *d_U = nullptr, *d_Q = nullptr, *d_U0 = nullptr, *d_Q0 = nullptr;
  double *d_val = nullptr, *d_rhs = nullptr, *d_trace = nullptr, *d_sol = nullptr, *d_flux = nullptr;
  int* d_status = nullptr;
  bool assembled = false, solved = false;
  // solver workspace
  DevMem wsMem;
  TraceWorkspace ws{};
  bool wsReady = false, wsMixed = false;
  int wsRestart = 0;
  // mixed-precision state: FP32 element blocks, FP64 residual rows
  bool mixedMode = false;
  DevMem mixMem;
  float *d_S32 = nullptr, *d_S032 = nullptr, *d_U32 = nullptr, *d_Q32 = nullptr, *d_U032 = nullptr,
        *d_Q032 = nullptr, *d_dl32 = nullptr;
  double *d_ru = nullptr, *d_rq = nullptr, *d_rl = nullptr, *d_rtrace = nullptr, *d_part = nullptr;
  double mixedBB = 0.0, mixedRR = 0.0;
  // tensor-core element contractions of the mixed assembly (tc_assembly.cu): packed table
  // (per mesh order) and the per-element FP32 blocks; lastTensor: the last mixed assembly used them
  float* d_tctab = nullptr;
  float* d_tcb = nullptr;
  bool lastTensor = false;
  // CG element operators (hfx_cg_operators): their tensor-core table, output and velocity buffers
  DevMem cgMem;
  float* d_cgtab = nullptr;
  double *d_cgout = nullptr, *d_cgvel = nullptr;
  size_t cgVelCap = 0;
  // two-level preconditioner: vertex coarse space (built on first use)
  std::vector<int> cellVerts;  // [nCells][dim+1]
  CoarseHost coarseHost;
  CoarseSolver coarse;
  DevMem coarseMem;
  bool coarseBuilt = false;
  double coarseTarget = 0.0;
  // launch tuner of the FP32 trace operator (mixed CG): -1 until the first mixed solve times both
  int spmvChoice = -1;
  // degree of the last coarse training; a learned solve without an accepted polynomial runs
  // Chebyshev of that degree (0: no training yet, the reduction target decides)
  int learnDegree = 0;
  float spmvTimes[4] = {0.f, 0.f, 0.f, 0.f};
  int stretchHint = 0;  // first-stretch length of the last mixed CG solve
  int coarseMaxDeg = 64;      // degree cap of the Chebyshev coarse solve (a fixed degree when target ~ 0)
  // vector Burgers (hfx_burgers_*)
  BurgersState burgers;
  // timing
  KernelTimer timer;
  cudaEvent_t marks[8] = {};

  int64_t nnz() const { return bp.rowptr.empty() ? 0 : bp.rowptr.back() * re.nNodesFace * re.nNodesFace; }
  int64_t ndofs() const { return (int64_t)topo.nFaces * re.nNodesFace; }
};

struct hfx_la {
  hfx_ctx* ctx;
  LaSystem sys;
};

namespace {

int set_err(hfx_ctx* c, int code, const std::string& msg) {
  if (c) c->err = msg;
  return code;
}

int cuda_err(hfx_ctx* c, cudaError_t e, const char* where) {
  return set_err(c, e == cudaErrorMemoryAllocation ? HFX_ERR_ALLOC : HFX_ERR_CUDA,
                 std::string(where) + ": " + cudaGetErrorString(e));
}

template <typename T>
cudaError_t dalloc(DevMem& m, T** p, size_t count) {
  void* ptr = nullptr;
  cudaError_t e = cudaMalloc(&ptr, sizeof(T) * (count > 0 ? count : 1));
  if (e != cudaSuccess) return e;
  m.ptrs.push_back(ptr);
  *p = (T*)ptr;
  return cudaSuccess;
}

template <typename T>
cudaError_t upload(DevMem& m, T** p, const T* host, size_t count, cudaStream_t s) {
  cudaError_t e = dalloc(m, p, count);
  if (e != cudaSuccess || count == 0) return e;
  return cudaMemcpyAsync(*p, host, sizeof(T) * count, cudaMemcpyHostToDevice, s);
}

#define HFX_CUDA(c, call)                              \
  do {                                                 \
    cudaError_t e_ = (call);                           \
    if (e_ != cudaSuccess) return cuda_err(c, e_, #call); \
  } while (0)

void free_outputs(hfx_ctx* c) {
  cudaStreamSynchronize(c->stream);
  c->outMem.release();
  c->wsMem.release();
  c->d_S = c->d_S0 = c->d_U = c->d_Q = c->d_U0 = c->d_Q0 = c->d_val = c->d_rhs = c->d_trace = nullptr;
  c->d_sol = c->d_flux = c->d_geo = c->d_prep = nullptr;
  c->rkStages = c->rkStage = 0;  // Runge-Kutta fields follow the mesh
  c->rkMem.release();
  c->d_kSol.clear();
  c->d_kFlux.clear();
  c->d_kTrace.clear();
  c->d_oldSol = c->d_oldFlux = c->d_oldTrace = c->d_wU = c->d_wQ = c->d_wL = nullptr;
  c->qValid = c->lastAffine = false;
  c->mixMem.release();
  c->d_S32 = c->d_S032 = c->d_U32 = c->d_Q32 = c->d_U032 = c->d_Q032 = c->d_dl32 = nullptr;
  c->d_tctab = c->d_tcb = nullptr;
  c->lastTensor = false;
  c->spmvChoice = -1;
  c->learnDegree = 0;
  c->cgMem.release();
  c->d_cgtab = nullptr;
  c->d_cgout = c->d_cgvel = nullptr;
  c->cgVelCap = 0;
  c->d_ru = c->d_rq = c->d_rl = c->d_rtrace = c->d_part = nullptr;
  c->mixedMode = false;
  c->d_status = nullptr;
  c->wsReady = false;
  c->wsMixed = false;
  c->wsRestart = 0;
  c->ws = TraceWorkspace{};
  c->assembled = c->solved = false;
}

// True when every cell's nodes are the affine image of the reference nodes
// (straight-sided simplices): node i sits at sum_m lambda_m(ref node i) x_m,
// x_m the cell's vertices, within 1e-12 of the cell's size.
bool cells_affine(const RefEl& re, int nCells, const int* cells, const double* coords) {
  const int d = re.dim, N = re.nNodes;
  std::vector<double> lam((size_t)N * (d + 1));
  for (int i = 0; i < N; ++i) {
    // reference vertices are nodes 0..d: solve sum_m l_m V_m = x, sum_m l_m = 1
    double A[4][5];
    for (int r = 0; r <= d; ++r) {
      for (int m = 0; m <= d; ++m) A[r][m] = r < d ? re.nodes[m * d + r] : 1.0;
      A[r][d + 1] = r < d ? re.nodes[i * d + r] : 1.0;
    }
    for (int k = 0; k <= d; ++k) {
      int piv = k;
      for (int r = k + 1; r <= d; ++r)
        if (std::fabs(A[r][k]) > std::fabs(A[piv][k])) piv = r;
      for (int j = 0; j <= d + 1; ++j) std::swap(A[k][j], A[piv][j]);
      for (int r = 0; r <= d; ++r) {
        if (r == k) continue;
        double l = A[r][k] / A[k][k];
        for (int j = k; j <= d + 1; ++j) A[r][j] -= l * A[k][j];
      }
    }
    for (int m = 0; m <= d; ++m) lam[(size_t)i * (d + 1) + m] = A[m][d + 1] / A[m][m];
  }
  for (int64_t e = 0; e < nCells; ++e) {
    const int* cn = cells + e * N;
    double h = 0.0;
    for (int m = 1; m <= d; ++m)
      for (int k = 0; k < d; ++k) h = std::max(h, std::fabs(coords[(int64_t)cn[m] * d + k] - coords[(int64_t)cn[0] * d + k]));
    for (int i = d + 1; i < N; ++i)
      for (int k = 0; k < d; ++k) {
        double x = 0.0;
        for (int m = 0; m <= d; ++m) x += lam[(size_t)i * (d + 1) + m] * coords[(int64_t)cn[m] * d + k];
        if (std::fabs(x - coords[(int64_t)cn[i] * d + k]) > 1e-12 * h) return false;
      }
  }
  return true;
}

}  // namespace

extern "C" {

int hfx_version(void) { return 100; }

int hfx_ctx_create(int device, hfx_ctx** out) {
  if (!out) return HFX_ERR_ARG;
  *out = nullptr;
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0) return HFX_ERR_CUDA;
  if (device < 0 || device >= n) return HFX_ERR_ARG;
  if ((e = cudaSetDevice(device)) != cudaSuccess) return HFX_ERR_CUDA;
  std::unique_ptr<hfx_ctx> c(new hfx_ctx());
  c->device = device;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return HFX_ERR_CUDA;
  *out = c.release();
  return HFX_OK;
}

int hfx_ctx_destroy(hfx_ctx* c) {
  if (!c) return HFX_OK;
  cudaSetDevice(c->device);
  cudaStreamSynchronize(c->stream);
  c->burgers.release();
  c->wsMem.release();
  c->mixMem.release();
  c->cgMem.release();
  c->outMem.release();
  c->tau.release();
  c->kappa.release();
  c->src.release();
  c->dir.release();
  c->uold.release();
  c->meshMem.release();
  c->timer.reset();
  for (auto& e : c->marks)
    if (e) cudaEventDestroy(e);
  cudaStreamDestroy(c->stream);
  delete c;
  return HFX_OK;
}

const char* hfx_last_error(const hfx_ctx* c) { return c ? c->err.c_str() : "null context"; }

int hfx_refel_query(int dim, int order, hfx_refel_info* info) {
  if (!info) return HFX_ERR_ARG;
  RefEl r;
  std::string err;
  if (!build_refel(dim, order, &r, &err)) return HFX_ERR_ARG;
  *info = {r.dim, r.order, r.nNodes, r.nFaces, r.nNodesFace, r.nIP, r.nIPFace};
  return HFX_OK;
}

int hfx_refel_tables(int dim, int order, double* nodes, int* faceNodes, double* ipCoords, double* ipWeights,
                     double* phi, double* dphi, double* fIpCoords, double* fIpWeights, double* fPhi,
                     double* fDphi) {
  RefEl r;
  std::string err;
  if (!build_refel(dim, order, &r, &err)) return HFX_ERR_ARG;
  auto cp = [](double* dst, const std::vector<double>& v) {
    if (dst) std::copy(v.begin(), v.end(), dst);
  };
  cp(nodes, r.nodes);
  if (faceNodes) std::copy(r.faceNodes.begin(), r.faceNodes.end(), faceNodes);
  cp(ipCoords, r.ipX);
  cp(ipWeights, r.ipW);
  cp(phi, r.phi);
  cp(dphi, r.dphi);
  cp(fIpCoords, r.fIpX);
  cp(fIpWeights, r.fIpW);
  cp(fPhi, r.fPhi);
  cp(fDphi, r.fDphi);
  return HFX_OK;
}

int hfx_mesh_upload(hfx_ctx* c, int dim, int order, int nNodes, const double* coords, int nCells, const int* cells,
                    int nFaces, const int* cell2face, const int* face2cell, const int* faces, int nBoundary,
                    const int* boundary) {
  if (!c) return HFX_ERR_ARG;
  if (!coords || !cells || nNodes <= 0 || nCells <= 0) return set_err(c, HFX_ERR_ARG, "mesh_upload: empty mesh");
  cudaSetDevice(c->device);
  std::string err;
  RefEl re;
  if (!build_refel(dim, order, &re, &err)) return set_err(c, HFX_ERR_ARG, err);
  if (!local_condense_supported(dim, order))
    return set_err(c, HFX_ERR_ARG, "mesh_upload: element (dim, order) not built (2D p<=5, 3D p<=3)");
  const int N = re.nNodes, F = re.nFaces, Nf = re.nNodesFace;
  for (int64_t i = 0; i < (int64_t)nCells * N; ++i)
    if (cells[i] < 0 || cells[i] >= nNodes) return set_err(c, HFX_ERR_ARG, "mesh_upload: cell node index out of range");
  Topology topo;
  if (cell2face) {
    if (!face2cell || !faces || nFaces <= 0 || (nBoundary > 0 && !boundary))
      return set_err(c, HFX_ERR_ARG, "mesh_upload: incomplete topology");
    topo.nFaces = nFaces;
    topo.cell2face.assign(cell2face, cell2face + (int64_t)nCells * F);
    topo.face2cell.assign(face2cell, face2cell + 2 * (int64_t)nFaces);
    topo.faces.assign(faces, faces + (int64_t)nFaces * Nf);
    if (nBoundary > 0) topo.boundary.assign(boundary, boundary + nBoundary);
    for (int v : topo.cell2face)
      if (v < 0 || v >= nFaces) return set_err(c, HFX_ERR_ARG, "mesh_upload: cell2face out of range");
  } else if (!compute_topology(re, nCells, cells, &topo, &err)) {
    return set_err(c, HFX_ERR_ARG, err);
  }
  std::vector<uint8_t> perm;
  if (!compute_face_perm(re, nCells, cells, topo, &perm, &err)) return set_err(c, HFX_ERR_ARG, err);
  BlockPattern bp;
  if (!compute_block_pattern(re, nCells, topo, &bp, &err)) return set_err(c, HFX_ERR_ARG, err);
  // release previous state
  free_outputs(c);
  c->burgers.release();
  c->meshMem.release();
  c->re = std::move(re);
  c->topo = std::move(topo);
  c->bp = std::move(bp);
  c->perm = std::move(perm);
  c->dim = dim;
  c->order = order;
  c->nNodes = nNodes;
  c->nCells = nCells;
  c->cellVerts.resize((size_t)nCells * (dim + 1));
  for (int64_t e = 0; e < nCells; ++e)
    for (int m = 0; m <= dim; ++m) c->cellVerts[e * (dim + 1) + m] = cells[e * N + m];
  c->coarseMem.release();
  c->coarse = CoarseSolver{};
  c->coarseHost = CoarseHost{};
  c->coarseBuilt = false;
  cudaStream_t s = c->stream;
  DevMem& m = c->meshMem;
  // packed tables: phi, dphi, w, fphi, fdphi, fw
  std::vector<double> tab;
  tab.insert(tab.end(), c->re.phi.begin(), c->re.phi.end());
  tab.insert(tab.end(), c->re.dphi.begin(), c->re.dphi.end());
  tab.insert(tab.end(), c->re.ipW.begin(), c->re.ipW.end());
  tab.insert(tab.end(), c->re.fPhi.begin(), c->re.fPhi.end());
  tab.insert(tab.end(), c->re.fDphi.begin(), c->re.fDphi.end());
  tab.insert(tab.end(), c->re.fIpW.begin(), c->re.fIpW.end());
  std::vector<int> itab(c->re.faceNodes);
  itab.insert(itab.end(), c->re.faceOpposite.begin(), c->re.faceOpposite.end());
  std::vector<uint8_t> isBnd(c->topo.nFaces, 0);
  for (int f : c->topo.boundary) isBnd[f] = 1;
  // whole 16-byte units for the element kernel's bulk copy (FP64 and FP32 copies)
  tab.resize((tab.size() + 3) / 4 * 4, 0.0);
  std::vector<float> tab32(tab.begin(), tab.end());
  HFX_CUDA(c, upload(m, &c->d_tab, tab.data(), tab.size(), s));
  HFX_CUDA(c, upload(m, &c->d_tab32, tab32.data(), tab32.size(), s));
  HFX_CUDA(c, upload(m, &c->d_itab, itab.data(), itab.size(), s));
  HFX_CUDA(c, upload(m, &c->d_phi, c->re.phi.data(), c->re.phi.size(), s));
  HFX_CUDA(c, upload(m, &c->d_coords, coords, (size_t)nNodes * dim, s));
  HFX_CUDA(c, upload(m, &c->d_cells, cells, (size_t)nCells * N, s));
  HFX_CUDA(c, upload(m, &c->d_cell2face, c->topo.cell2face.data(), c->topo.cell2face.size(), s));
  HFX_CUDA(c, upload(m, &c->d_perm, c->perm.data(), c->perm.size(), s));
  HFX_CUDA(c, upload(m, &c->d_face2cell, c->topo.face2cell.data(), c->topo.face2cell.size(), s));
  HFX_CUDA(c, upload(m, &c->d_isBnd, isBnd.data(), isBnd.size(), s));
  HFX_CUDA(c, upload(m, &c->d_browptr, c->bp.rowptr.data(), c->bp.rowptr.size(), s));
  HFX_CUDA(c, upload(m, &c->d_bcol, c->bp.col.data(), c->bp.col.size(), s));
  HFX_CUDA(c, upload(m, &c->d_src0, c->bp.src0.data(), c->bp.src0.size(), s));
  HFX_CUDA(c, upload(m, &c->d_src1, c->bp.src1.data(), c->bp.src1.size(), s));
  HFX_CUDA(c, upload(m, &c->d_loc0, c->bp.loc0.data(), c->bp.loc0.size(), s));
  HFX_CUDA(c, upload(m, &c->d_loc1, c->bp.loc1.data(), c->bp.loc1.size(), s));
  HFX_CUDA(c, dalloc(m, &c->d_brow, c->bp.col.size()));
  {
    // half storage of symmetric trace operators: block (f, g >= f) stored, (g < f) mirrored
    const std::vector<int64_t>& rp = c->bp.rowptr;
    const std::vector<int>& cl = c->bp.col;
    std::vector<int> hidx(cl.size(), 0);
    int64_t nh = 0;
    bool ok = cl.size() < (size_t)2147483647;
    for (int f = 0; f < c->topo.nFaces && ok; ++f)
      for (int64_t k = rp[f]; k < rp[f + 1]; ++k) {
        const int g = cl[k];
        if (g >= f) {
          hidx[k] = (int)nh++;
        } else {
          auto it = std::lower_bound(cl.begin() + rp[g], cl.begin() + rp[g + 1], f);
          if (it == cl.begin() + rp[g + 1] || *it != f) {
            ok = false;  // pattern not structurally symmetric
            break;
          }
          hidx[k] = -(hidx[it - cl.begin()] + 1);
        }
      }
    c->nHalf = ok ? nh : 0;
    c->d_hidx = nullptr;
    c->d_ell = nullptr;
    c->ellWidth = 0;
    if (ok) {
      HFX_CUDA(c, upload(m, &c->d_hidx, hidx.data(), hidx.size(), s));
      // fixed-width rows (bcol, hidx) for the half-storage SpMV: no row pointers to chase
      const int W = dim == 2 ? 5 : 7;
      bool fits = true;
      for (int f = 0; f < c->topo.nFaces && fits; ++f) fits = rp[f + 1] - rp[f] <= W;
      if (fits) {
        std::vector<int2> ell((size_t)c->topo.nFaces * W, make_int2(0, INT32_MIN));
        for (int f = 0; f < c->topo.nFaces; ++f)
          for (int64_t k = rp[f]; k < rp[f + 1]; ++k) ell[(size_t)f * W + (k - rp[f])] = make_int2(cl[k], hidx[k]);
        HFX_CUDA(c, upload(m, &c->d_ell, ell.data(), ell.size(), s));
        c->ellWidth = W;
      }
    }
  }
  {
    std::vector<double> atab;
    c->d_atab = nullptr;
    if (affine_tables(c->re, &atab)) HFX_CUDA(c, upload(m, &c->d_atab, atab.data(), atab.size(), s));
    c->affineMesh = c->d_atab != nullptr && cells_affine(c->re, nCells, cells, coords);
  }
  HFX_CUDA(c, launch_block_rows(c->d_browptr, c->topo.nFaces, c->d_brow, s));
  // default fields: tau = 1, Dirichlet = 0, kappa = identity, no source
  std::vector<double> ones((size_t)c->topo.nFaces * Nf, 1.0), zeros((size_t)c->topo.nFaces * Nf, 0.0);
  c->tauVals = 1;
  HFX_CUDA(c, c->tau.set(ones.data(), ones.size(), s));
  HFX_CUDA(c, c->dir.set(zeros.data(), zeros.size(), s));
  c->kc = 0;
  c->srcMode = 0;
  c->dt = 0.0;
  HFX_CUDA(c, cudaStreamSynchronize(s));
  c->haveMesh = true;
  return HFX_OK;
}

int hfx_mesh_compute_topology(int dim, int order, int nCells, const int* cells, int* nFaces, int* nBoundary,
                              int* cell2face, int* face2cell, int* faces, int* boundary) {
  if (!cells || nCells <= 0 || !nFaces || !nBoundary) return HFX_ERR_ARG;
  RefEl re;
  std::string err;
  if (!build_refel(dim, order, &re, &err)) return HFX_ERR_ARG;
  Topology t;
  if (!compute_topology(re, nCells, cells, &t, &err)) return HFX_ERR_ARG;
  *nFaces = t.nFaces;
  *nBoundary = (int)t.boundary.size();
  if (cell2face) std::copy(t.cell2face.begin(), t.cell2face.end(), cell2face);
  if (face2cell) std::copy(t.face2cell.begin(), t.face2cell.end(), face2cell);
  if (faces) std::copy(t.faces.begin(), t.faces.end(), faces);
  if (boundary) std::copy(t.boundary.begin(), t.boundary.end(), boundary);
  return HFX_OK;
}

int hfx_mesh_sizes(hfx_ctx* c, int* nFaces, int* nBoundary, int64_t* nnz) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "mesh_sizes: no mesh");
  if (nFaces) *nFaces = c->topo.nFaces;
  if (nBoundary) *nBoundary = (int)c->topo.boundary.size();
  if (nnz) *nnz = c->nnz();
  return HFX_OK;
}

int hfx_mesh_topology(hfx_ctx* c, int* cell2face, int* face2cell, int* faces, int* boundary) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "mesh_topology: no mesh");
  if (cell2face) std::copy(c->topo.cell2face.begin(), c->topo.cell2face.end(), cell2face);
  if (face2cell) std::copy(c->topo.face2cell.begin(), c->topo.face2cell.end(), face2cell);
  if (faces) std::copy(c->topo.faces.begin(), c->topo.faces.end(), faces);
  if (boundary) std::copy(c->topo.boundary.begin(), c->topo.boundary.end(), boundary);
  return HFX_OK;
}

static int replace_field(hfx_ctx* c, FieldBuf* dst, const double* src, size_t n) {
  HFX_CUDA(c, dst->set(src, n, c->stream));
  c->assembled = false;
  return HFX_OK;
}

int hfx_set_tau(hfx_ctx* c, const double* tau, int nVals) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "set_tau: upload a mesh first");
  if (!tau || (nVals != 1 && nVals != 2)) return set_err(c, HFX_ERR_ARG, "set_tau: Tau needs 1 or 2 values per face node");
  c->tauVals = nVals;
  return replace_field(c, &c->tau, tau, (size_t)c->topo.nFaces * c->re.nNodesFace * nVals);
}

int hfx_set_kappa(hfx_ctx* c, const double* kappa, int comps, int layout) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "set_kappa: upload a mesh first");
  if (comps == 0) {
    c->kc = 0;
    c->kappaCellConstant = true;
    c->kappaSymmetric = true;
    c->assembled = false;
    return HFX_OK;
  }
  if (!kappa || (comps != 1 && comps != c->dim * c->dim) || (layout != 0 && layout != 1))
    return set_err(c, HFX_ERR_ARG, "set_kappa: the diffusion tensor must be scalar or dim x dim");
  c->kc = comps;
  c->kLayout = layout;
  // A tensor that varies inside a cell makes the trace system non-symmetric
  // (only Suq/Slq carry it, HDGDiffusion.cpp:74-145): record it for the solver.
  {
    const int N = c->re.nNodes;
    const int* cells = nullptr;
    std::vector<int> hcells;
    if (layout == 0) {
      hcells.resize((size_t)c->nCells * N);
      cudaMemcpy(hcells.data(), c->d_cells, sizeof(int) * hcells.size(), cudaMemcpyDeviceToHost);
      cells = hcells.data();
    }
    bool cst = true;
    for (int64_t e = 0; e < c->nCells && cst; ++e)
      for (int i = 1; i < N && cst; ++i)
        for (int k = 0; k < comps && cst; ++k) {
          double a = layout == 0 ? kappa[(int64_t)cells[e * N] * comps + k] : kappa[(e * N) * comps + k];
          double b = layout == 0 ? kappa[(int64_t)cells[e * N + i] * comps + k] : kappa[(e * N + i) * comps + k];
          if (a != b) cst = false;
        }
    bool sym = true;  // a dim x dim tensor must be symmetric for the affine kernel and for CG
    if (comps == c->dim * c->dim) {
      const int d = c->dim;
      const int64_t nv = layout == 0 ? (int64_t)c->nNodes : (int64_t)c->nCells * N;
      for (int64_t v = 0; v < nv && sym; ++v)
        for (int a = 0; a < d && sym; ++a)
          for (int b = a + 1; b < d && sym; ++b) {
            double x = kappa[v * comps + a + b * d], y = kappa[v * comps + b + a * d];
            if (std::fabs(x - y) > 1e-14 * (std::fabs(x) + std::fabs(y))) sym = false;
          }
    }
    c->kappaSymmetric = sym;
    c->kappaCellConstant = cst && sym;  // the trace system is symmetric only then
  }
  size_t n = (layout == 0 ? (size_t)c->nNodes : (size_t)c->nCells * c->re.nNodes) * comps;
  return replace_field(c, &c->kappa, kappa, n);
}

int hfx_set_source(hfx_ctx* c, int mode, const double* values, double param) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "set_source: upload a mesh first");
  if (mode < HFX_SRC_NONE || mode > HFX_SRC_SINPROD) return set_err(c, HFX_ERR_ARG, "set_source: unknown mode");
  c->srcMode = mode;
  c->srcParam = param;
  c->assembled = false;
  if (mode == HFX_SRC_VALUES) {
    if (!values) return set_err(c, HFX_ERR_ARG, "set_source: values required");
    return replace_field(c, &c->src, values, (size_t)c->nCells * c->re.nIP);
  }
  return HFX_OK;
}

int hfx_set_dirichlet(hfx_ctx* c, const double* values) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "set_dirichlet: upload a mesh first");
  if (!values) return set_err(c, HFX_ERR_ARG, "set_dirichlet: values required");
  return replace_field(c, &c->dir, values, (size_t)c->topo.nFaces * c->re.nNodesFace);
}

int hfx_set_time_scheme(hfx_ctx* c, double dt, const double* uOld) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "set_time_scheme: upload a mesh first");
  if (dt < 0.0 || (dt > 0.0 && !uOld)) return set_err(c, HFX_ERR_ARG, "set_time_scheme: dt >= 0 and the old Solution");
  c->dt = dt;
  c->assembled = false;
  if (dt > 0.0) return replace_field(c, &c->uold, uOld, (size_t)c->nCells * c->re.nNodes);
  return HFX_OK;
}

int hfx_ip_coords(hfx_ctx* c, double* out) {
  if (!c || !out) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "ip_coords: upload a mesh first");
  size_t n = (size_t)c->nCells * c->re.nIP * c->dim;
  double* d = nullptr;
  DevMem tmp;
  HFX_CUDA(c, dalloc(tmp, &d, n));
  IpCoordParams p{c->nCells, c->re.nNodes, c->re.nIP, c->dim, c->d_coords, c->d_cells, c->d_phi, d};
  HFX_CUDA(c, launch_ip_coords(p, c->stream));
  HFX_CUDA(c, cudaMemcpyAsync(out, d, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

static int ensure_outputs(hfx_ctx* c) {
  if (c->d_S) return HFX_OK;
  const int64_t E = c->nCells;
  const int LU = c->re.nNodes, LQ = c->dim * c->re.nNodes, LL = c->re.nFaces * c->re.nNodesFace;
  DevMem& m = c->outMem;
  HFX_CUDA(c, dalloc(m, &c->d_S, (size_t)E * LL * LL));
  HFX_CUDA(c, dalloc(m, &c->d_S0, (size_t)E * LL));
  HFX_CUDA(c, dalloc(m, &c->d_U, (size_t)E * LU * LL));
  HFX_CUDA(c, dalloc(m, &c->d_Q, (size_t)E * LQ * LL));
  HFX_CUDA(c, dalloc(m, &c->d_U0, (size_t)E * LU));
  HFX_CUDA(c, dalloc(m, &c->d_Q0, (size_t)E * LQ));
  HFX_CUDA(c, dalloc(m, &c->d_val, (size_t)c->nnz()));
  HFX_CUDA(c, dalloc(m, &c->d_rhs, (size_t)c->ndofs()));
  HFX_CUDA(c, dalloc(m, &c->d_trace, (size_t)c->ndofs()));
  HFX_CUDA(c, dalloc(m, &c->d_status, 1));
  HFX_CUDA(c, dalloc(m, &c->d_sol, (size_t)E * LU));
  HFX_CUDA(c, dalloc(m, &c->d_flux, (size_t)E * LQ));
  HFX_CUDA(c, dalloc(m, &c->d_geo, (size_t)E * (c->dim * c->dim + c->re.nFaces * c->dim)));
  if (c->d_atab) HFX_CUDA(c, dalloc(m, &c->d_prep, (size_t)E * affine_prep_doubles(c->dim, c->order)));
  // Solution and Flux start at 0 (the state the explicit modes read before a first recovery)
  HFX_CUDA(c, cudaMemsetAsync(c->d_sol, 0, sizeof(double) * E * LU, c->stream));
  HFX_CUDA(c, cudaMemsetAsync(c->d_flux, 0, sizeof(double) * E * LQ, c->stream));
  HFX_CUDA(c, cudaMemsetAsync(c->d_trace, 0, sizeof(double) * c->ndofs(), c->stream));
  return HFX_OK;
}

static int assemble_fp64(hfx_ctx* c) {
  int rc = ensure_outputs(c);
  if (rc) return rc;
  cudaStream_t s = c->stream;
  HFX_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
  LocalParams p{};
  p.nCells = c->nCells;
  p.coords = c->d_coords;
  p.cells = c->d_cells;
  p.cell2face = c->d_cell2face;
  p.perm = c->d_perm;
  p.face2cell = c->d_face2cell;
  p.isBoundary = c->d_isBnd;
  p.tau = c->tau.p;
  p.tauVals = c->tauVals;
  p.kappa = c->kappa.p;
  p.kc = c->kc;
  p.kappaLayout = c->kLayout;
  p.srcMode = c->srcMode;
  p.src = c->src.p;
  p.srcParam = c->srcParam;
  p.dirichlet = c->dir.p;
  p.dt = c->dt;
  p.uOld = c->uold.p;
  p.tab = c->d_tab;
  p.tab32 = c->d_tab32;
  p.itab = c->d_itab;
  p.S = c->d_S;
  p.S0 = c->d_S0;
  p.U = c->d_U;
  p.Q = c->d_Q;
  p.U0 = c->d_U0;
  p.Q0 = c->d_Q0;
  p.status = c->d_status;
  p.fp32 = 0;
  p.rhsU = p.rhsQ = nullptr;
  p.writeOps = 1;
  p.explicitMode = c->solverType;
  p.solState = c->d_sol;
  p.fluxState = c->d_flux;
  if (c->rkStages > 0) {
    // RungeKutta::apply (RungeKutta.cpp:90-129) for stage s: w = (dt - c) ut + dt^2 sum_{i<s} a_si k_i
    const int S = c->rkStages, st = c->rkStage;
    const double dt = c->rkDt, cst = dt * c->rkTable[(size_t)st * (S + 1) + 1 + st];
    const int64_t E = c->nCells, LU = c->re.nNodes, LQ = (int64_t)c->dim * c->re.nNodes;
    double* outs[3] = {c->d_wU, c->d_wQ, c->d_wL};
    const double* olds[3] = {c->d_oldSol, c->d_oldFlux, c->d_oldTrace};
    const std::vector<double*>* ks[3] = {&c->d_kSol, &c->d_kFlux, &c->d_kTrace};
    const int64_t len[3] = {E * LU, E * LQ, c->ndofs()};
    for (int f = 0; f < 3; ++f) {
      RkTerms tr{};
      for (int i = 0; i < st; ++i) {
        tr.coef[tr.n] = dt * dt * c->rkTable[(size_t)st * (S + 1) + 1 + i];
        tr.ptr[tr.n++] = (*ks[f])[i];
      }
      HFX_CUDA(c, launch_rk_lincomb(len[f], outs[f], dt - cst, olds[f], tr, s));
    }
    p.dt = dt;
    p.uOld = c->d_oldSol;
    p.cStiff = cst;
    p.rkWu = c->d_wU;
    p.rkWq = c->d_wQ;
    p.rkWl = c->d_wL;
  }
  const bool affine = c->assemblyPath == 0 && c->affineMesh && c->kappaCellConstant && c->d_atab && c->d_prep;
  c->timer.begin(K_LOCAL, s);
  if (affine) HFX_CUDA(c, launch_local_affine(c->dim, c->order, p, c->d_atab, c->d_geo, c->d_prep, s));
  else HFX_CUDA(c, launch_local_condense(c->dim, c->order, p, s));
  c->timer.end(K_LOCAL, s);
  c->lastAffine = affine;
  c->qValid = !affine;
  ScatterParams sp{};
  sp.nFaces = c->topo.nFaces;
  sp.NF = c->re.nNodesFace;
  sp.LL = c->re.nFaces * c->re.nNodesFace;
  sp.browptr = c->d_browptr;
  sp.brow = c->d_brow;
  sp.nBlocks = (int64_t)c->bp.col.size();
  sp.src0 = c->d_src0;
  sp.src1 = c->d_src1;
  sp.loc0 = c->d_loc0;
  sp.loc1 = c->d_loc1;
  sp.perm = c->d_perm;
  sp.S = c->d_S;
  sp.S0 = c->d_S0;
  sp.cell2face = c->d_cell2face;
  sp.face2cell = c->d_face2cell;
  sp.F = c->re.nFaces;
  sp.val = c->d_val;
  sp.rhs = c->d_rhs;
  c->timer.begin(K_SCATTER, s);
  HFX_CUDA(c, launch_scatter(sp, s));
  c->timer.end(K_SCATTER, s);
  int status = 0;
  HFX_CUDA(c, cudaMemcpyAsync(&status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  HFX_CUDA(c, cudaStreamSynchronize(s));
  if (status == 2) return set_err(c, HFX_ERR_CUDA, "assemble: a bulk-copy or tensor-core wait ran out");
  if (status != 0) return set_err(c, HFX_ERR_SINGULAR, "assemble: singular element block in condensation");
  c->assembled = true;
  c->solved = false;
  c->mixedMode = false;
  return HFX_OK;
}

static int ensure_workspace(hfx_ctx* c, bool mixed, int restart);

static LocalParams local_params(hfx_ctx* c) {
  LocalParams p{};
  p.nCells = c->nCells;
  p.coords = c->d_coords;
  p.cells = c->d_cells;
  p.cell2face = c->d_cell2face;
  p.perm = c->d_perm;
  p.face2cell = c->d_face2cell;
  p.isBoundary = c->d_isBnd;
  p.tau = c->tau.p;
  p.tauVals = c->tauVals;
  p.kappa = c->kappa.p;
  p.kc = c->kc;
  p.kappaLayout = c->kLayout;
  p.srcMode = c->srcMode;
  p.src = c->src.p;
  p.srcParam = c->srcParam;
  p.dirichlet = c->dir.p;
  p.dt = c->dt;
  p.uOld = c->uold.p;
  p.tab = c->d_tab;
  p.tab32 = c->d_tab32;
  p.itab = c->d_itab;
  p.status = c->d_status;
  return p;
}

// FP64 residual of the full HDG system at the current (u, q, lambda); returns ||r||^2.
static int mixed_residual(hfx_ctx* c, double* rr) {
  const int NF = c->re.nNodesFace, F = c->re.nFaces, LL = F * NF;
  ResidualParams p{};
  p.nCells = c->nCells;
  p.coords = c->d_coords;
  p.cells = c->d_cells;
  p.cell2face = c->d_cell2face;
  p.perm = c->d_perm;
  p.face2cell = c->d_face2cell;
  p.tau = c->tau.p;
  p.tauVals = c->tauVals;
  p.kappa = c->kappa.p;
  p.kc = c->kc;
  p.kappaLayout = c->kLayout;
  p.srcMode = c->srcMode;
  p.src = c->src.p;
  p.srcParam = c->srcParam;
  p.dt = c->dt;
  p.uOld = c->uold.p;
  p.tab = c->d_tab;
  p.itab = c->d_itab;
  p.sol = c->d_sol;
  p.flux = c->d_flux;
  p.trace = c->d_trace;
  p.ru = c->d_ru;
  p.rq = c->d_rq;
  p.rl = c->d_rl;
  FaceResidualParams fp{c->topo.nFaces, NF, F, LL, c->d_face2cell, c->d_cell2face, c->d_perm, c->d_isBnd,
                        c->d_rl, c->dir.p, c->d_trace, c->d_rtrace};
  c->timer.begin(K_RESIDUAL, c->stream);
  HFX_CUDA(c, launch_residual(c->dim, c->order, p, fp, c->stream));
  c->timer.end(K_RESIDUAL, c->stream);
  const int grid = 1024;
  const int64_t LU = c->re.nNodes, LQ = (int64_t)c->dim * c->re.nNodes;
  HFX_CUDA(c, launch_sumsq(c->d_ru, c->nCells * LU, c->d_rq, c->nCells * LQ, c->d_rtrace, c->ndofs(), c->d_part, grid,
                           c->stream));
  std::vector<double> hp(grid);
  HFX_CUDA(c, cudaMemcpyAsync(hp.data(), c->d_part, sizeof(double) * grid, cudaMemcpyDeviceToHost, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  double acc = 0.0;
  for (double v : hp) acc += v;
  *rr = acc;
  return HFX_OK;
}

// FP32 element condensation with the residual rows as right-hand side
static int mixed_condense(hfx_ctx* c, bool writeOps) {
  LocalParams p = local_params(c);
  p.fp32 = 1;
  p.rhsU = c->d_ru;
  p.rhsQ = c->d_rq;
  p.writeOps = writeOps ? 1 : 0;
  p.S = c->d_S32;
  p.S0 = c->d_S032;
  p.U = c->d_U32;
  p.Q = c->d_Q32;
  p.U0 = c->d_U032;
  p.Q0 = c->d_Q032;
  if (c->lastTensor) {
    p.tcBlocks = c->d_tcb;
    p.tcStride = tc_blocks_stride(c->dim, c->order);
  }
  c->timer.begin(K_LOCAL, c->stream);
  HFX_CUDA(c, launch_local_condense(c->dim, c->order, p, c->stream));
  c->timer.end(K_LOCAL, c->stream);
  Scatter32Params sp{};
  sp.nFaces = c->topo.nFaces;
  sp.NF = c->re.nNodesFace;
  sp.LL = c->re.nFaces * c->re.nNodesFace;
  sp.F = c->re.nFaces;
  sp.nBlocks = (int64_t)c->bp.col.size();
  sp.browptr = c->d_browptr;
  sp.brow = c->d_brow;
  sp.src0 = c->d_src0;
  sp.src1 = c->d_src1;
  sp.loc0 = c->d_loc0;
  sp.loc1 = c->d_loc1;
  sp.perm = c->d_perm;
  sp.cell2face = c->d_cell2face;
  sp.face2cell = c->d_face2cell;
  sp.S = c->d_S32;
  sp.S0 = c->d_S032;
  sp.rtrace = c->d_rtrace;
  sp.val = c->ws.val32;
  sp.rhs = c->ws.rhs32;
  c->timer.begin(K_SCATTER, c->stream);
  HFX_CUDA(c, launch_scatter32(sp, writeOps, c->stream));
  c->timer.end(K_SCATTER, c->stream);
  return HFX_OK;
}

static int assemble_mixed(hfx_ctx* c) {
  int rc = ensure_outputs(c);
  if (rc) return rc;
  if ((rc = ensure_workspace(c, true, 0))) return rc;
  const int64_t E = c->nCells;
  const int LU = c->re.nNodes, LQ = c->dim * c->re.nNodes, LL = c->re.nFaces * c->re.nNodesFace;
  if (!c->d_S32) {
    DevMem& m = c->mixMem;
    HFX_CUDA(c, dalloc(m, &c->d_S32, (size_t)E * LL * LL));
    HFX_CUDA(c, dalloc(m, &c->d_S032, (size_t)E * LL));
    HFX_CUDA(c, dalloc(m, &c->d_U32, (size_t)E * LU * LL));
    HFX_CUDA(c, dalloc(m, &c->d_Q32, (size_t)E * LQ * LL));
    HFX_CUDA(c, dalloc(m, &c->d_U032, (size_t)E * LU));
    HFX_CUDA(c, dalloc(m, &c->d_Q032, (size_t)E * LQ));
    HFX_CUDA(c, dalloc(m, &c->d_dl32, (size_t)c->ndofs()));
    HFX_CUDA(c, dalloc(m, &c->d_ru, (size_t)E * LU));
    HFX_CUDA(c, dalloc(m, &c->d_rq, (size_t)E * LQ));
    HFX_CUDA(c, dalloc(m, &c->d_rl, (size_t)E * LL));
    HFX_CUDA(c, dalloc(m, &c->d_rtrace, (size_t)c->ndofs()));
    HFX_CUDA(c, dalloc(m, &c->d_part, 1024));
  }
  cudaStream_t s = c->stream;
  HFX_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
  HFX_CUDA(c, cudaMemsetAsync(c->d_sol, 0, sizeof(double) * E * LU, s));
  HFX_CUDA(c, cudaMemsetAsync(c->d_flux, 0, sizeof(double) * E * LQ, s));
  HFX_CUDA(c, cudaMemsetAsync(c->d_trace, 0, sizeof(double) * c->ndofs(), s));
  // element blocks contracted on the tensor cores once per assembly; every condensation of
  // this assembly (the first one and those of the refinement steps) loads them
  c->lastTensor = false;
  if (c->assemblyPath == 0 && tc_blocks_supported(c->dim, c->order)) {
    if (!c->d_tctab) {
      std::vector<double> tab;
      tab.insert(tab.end(), c->re.phi.begin(), c->re.phi.end());
      tab.insert(tab.end(), c->re.dphi.begin(), c->re.dphi.end());
      tab.insert(tab.end(), c->re.ipW.begin(), c->re.ipW.end());
      tab.insert(tab.end(), c->re.fPhi.begin(), c->re.fPhi.end());
      tab.insert(tab.end(), c->re.fDphi.begin(), c->re.fDphi.end());
      tab.insert(tab.end(), c->re.fIpW.begin(), c->re.fIpW.end());
      std::vector<float> t = tc_table(c->dim, c->order, tab.data());
      HFX_CUDA(c, upload(c->mixMem, &c->d_tctab, t.data(), t.size(), s));
      HFX_CUDA(c, dalloc(c->mixMem, &c->d_tcb, (size_t)E * tc_blocks_stride(c->dim, c->order)));
    }
    LocalParams lp = local_params(c);
    TcBlockParams tp{};
    tp.nCells = E;
    tp.coords = lp.coords;
    tp.cells = lp.cells;
    tp.cell2face = lp.cell2face;
    tp.perm = lp.perm;
    tp.face2cell = lp.face2cell;
    tp.tau = lp.tau;
    tp.tauVals = lp.tauVals;
    tp.kappa = lp.kappa;
    tp.kc = lp.kc;
    tp.kappaLayout = lp.kappaLayout;
    tp.srcMode = lp.srcMode;
    tp.src = lp.src;
    tp.srcParam = lp.srcParam;
    tp.itab = lp.itab;
    tp.tctab = c->d_tctab;
    tp.out = c->d_tcb;
    tp.status = c->d_status;
    c->timer.begin(K_TENSOR, s);
    HFX_CUDA(c, launch_tc_blocks(c->dim, c->order, tp, s));
    c->timer.end(K_TENSOR, s);
    c->lastTensor = true;
  }
  // residual at zero = the right-hand side b of the full system
  if ((rc = mixed_residual(c, &c->mixedBB))) return rc;
  c->mixedRR = c->mixedBB;
  if ((rc = mixed_condense(c, true))) return rc;
  int status = 0;
  HFX_CUDA(c, cudaMemcpyAsync(&status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  HFX_CUDA(c, cudaStreamSynchronize(s));
  if (status == 2) return set_err(c, HFX_ERR_CUDA, "assemble: a tensor-core wait ran out");
  if (status == 2) return set_err(c, HFX_ERR_CUDA, "assemble: a bulk-copy or tensor-core wait ran out");
  if (status != 0) return set_err(c, HFX_ERR_SINGULAR, "assemble: singular element block in condensation");
  c->assembled = true;
  c->solved = false;
  c->mixedMode = true;
  return HFX_OK;
}

int hfx_assemble_ex(hfx_ctx* c, int precision) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "assemble: upload a mesh first");
  if (precision != HFX_PREC_FP64 && precision != HFX_PREC_MIXED) return set_err(c, HFX_ERR_ARG, "assemble: unknown precision");
  cudaSetDevice(c->device);
  c->coarse.ready = false;  // the coarse operator follows the element matrices
  if (precision == HFX_PREC_MIXED && c->solverType != HFX_IMPLICIT)
    return set_err(c, HFX_ERR_UNSUPPORTED, "assemble: the explicit modes assemble in FP64");
  if (precision == HFX_PREC_MIXED && c->rkStages > 0)
    return set_err(c, HFX_ERR_UNSUPPORTED, "assemble: Runge-Kutta stages assemble in FP64");
  return precision == HFX_PREC_MIXED ? assemble_mixed(c) : assemble_fp64(c);
}

int hfx_assemble(hfx_ctx* c) { return hfx_assemble_ex(c, HFX_PREC_FP64); }

int hfx_set_assembly_path(hfx_ctx* c, int path) {
  if (!c) return HFX_ERR_ARG;
  if (path != 0 && path != 1) return set_err(c, HFX_ERR_ARG, "set_assembly_path: 0 (automatic) or 1 (quadrature)");
  c->lastTensor = false;
  c->assemblyPath = path;
  c->assembled = false;
  return HFX_OK;
}

int hfx_set_solver_type(hfx_ctx* c, int type) {
  if (!c) return HFX_ERR_ARG;
  if (type != HFX_IMPLICIT && type != HFX_WEXPLICIT && type != HFX_SEXPLICIT)
    return set_err(c, HFX_ERR_ARG, "set_solver_type: HFX_IMPLICIT, HFX_WEXPLICIT or HFX_SEXPLICIT");
  c->solverType = type;
  c->assembled = false;
  return HFX_OK;
}

int hfx_set_state(hfx_ctx* c, const double* solution, const double* flux) {
  if (!c || !solution || !flux) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "set_state: upload a mesh first");
  cudaSetDevice(c->device);
  int rc = ensure_outputs(c);
  if (rc) return rc;
  const size_t E = (size_t)c->nCells;
  HFX_CUDA(c, cudaMemcpyAsync(c->d_sol, solution, sizeof(double) * E * c->re.nNodes, cudaMemcpyHostToDevice, c->stream));
  HFX_CUDA(c, cudaMemcpyAsync(c->d_flux, flux, sizeof(double) * E * c->re.nNodes * c->dim, cudaMemcpyHostToDevice,
                              c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  c->assembled = false;
  return HFX_OK;
}

int hfx_set_trace(hfx_ctx* c, const double* trace) {
  if (!c || !trace) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "set_trace: upload a mesh first");
  cudaSetDevice(c->device);
  int rc = ensure_outputs(c);
  if (rc) return rc;
  HFX_CUDA(c, cudaMemcpyAsync(c->d_trace, trace, sizeof(double) * c->ndofs(), cudaMemcpyHostToDevice, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

int hfx_get_state(hfx_ctx* c, double* solution, double* flux, double* trace) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "get_state: upload a mesh first");
  cudaSetDevice(c->device);
  int rc = ensure_outputs(c);
  if (rc) return rc;
  const size_t E = (size_t)c->nCells;
  if (solution)
    HFX_CUDA(c, cudaMemcpyAsync(solution, c->d_sol, sizeof(double) * E * c->re.nNodes, cudaMemcpyDeviceToHost,
                                c->stream));
  if (flux)
    HFX_CUDA(c, cudaMemcpyAsync(flux, c->d_flux, sizeof(double) * E * c->re.nNodes * c->dim, cudaMemcpyDeviceToHost,
                                c->stream));
  if (trace)
    HFX_CUDA(c, cudaMemcpyAsync(trace, c->d_trace, sizeof(double) * c->ndofs(), cudaMemcpyDeviceToHost, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

// Butcher tables of RungeKutta::setUpDB (RungeKutta.cpp:215-286), the published
// coefficients of each scheme; rows [c_i | a_i0 .. a_i(s-1)], last row [0 | b].
int hfx_rk_butcher(int type, int* nStages, double* table) {
  if (!nStages) return HFX_ERR_ARG;
  const double g = 1.0 - std::sqrt(2.0) / 2.0;
  std::vector<double> t;
  int S = 0;
  switch (type) {
    case HFX_RK_FEULER: S = 1; t = {0, 0, 0, 1}; break;
    case HFX_RK_EMIDPOINT: S = 2; t = {0, 0, 0, 0.5, 0.5, 0, 0, 0, 1}; break;
    case HFX_RK_HEUN: S = 2; t = {0, 0, 0, 1, 1, 0, 0, 0.5, 0.5}; break;
    case HFX_RK_KUTTA3: S = 3; t = {0, 0, 0, 0, 0.5, 0.5, 0, 0, 1, -1, 2, 0, 0, 1.0 / 6, 2.0 / 3, 1.0 / 6}; break;
    case HFX_RK_HEUN3: S = 3; t = {0, 0, 0, 0, 1.0 / 3, 1.0 / 3, 0, 0, 2.0 / 3, 0, 2.0 / 3, 0, 0, 0.25, 0, 0.75}; break;
    case HFX_RK_SSPRK3: S = 3; t = {0, 0, 0, 0, 1, 1, 0, 0, 0.5, 0.25, 0.25, 0, 0, 1.0 / 6, 1.0 / 6, 2.0 / 3}; break;
    case HFX_RK_RK4:
      S = 4;
      t = {0, 0, 0, 0, 0, 0.5, 0.5, 0, 0, 0, 0.5, 0, 0.5, 0, 0, 1, 0, 0, 1, 0, 0, 1.0 / 6, 1.0 / 3, 1.0 / 3, 1.0 / 6};
      break;
    case HFX_RK_BEULER: S = 1; t = {1, 1, 0, 1}; break;
    case HFX_RK_IMIDPOINT: S = 1; t = {0.5, 0.5, 0, 1}; break;
    case HFX_RK_CRANKNICOLSON: S = 2; t = {0, 0, 0, 1, 0.5, 0.5, 0, 0.5, 0.5}; break;
    case HFX_RK_KS2: S = 2; t = {0.5, 0.5, 0, 1.5, -0.5, 2, 0, -0.5, 1.5}; break;
    case HFX_RK_QZ2: S = 2; t = {0.25, 0.25, 0, 0.75, 0.5, 0.25, 0, 0.5, 0.5}; break;
    case HFX_RK_ALX2: S = 2; t = {g, g, 0, 1, 1 - g, g, 0, 1 - g, g}; break;
    case HFX_RK_RK43:
      S = 4;
      t = {0.5, 0.5, 0, 0, 0, 2.0 / 3, 1.0 / 6, 0.5, 0, 0, 0.5, -0.5, 0.5, 0.5, 0, 1, 1.5, -1.5, 0.5, 0.5,
           0, 1.5, -1.5, 0.5, 0.5};
      break;
    default: return HFX_ERR_ARG;
  }
  *nStages = S;
  if (table) std::copy(t.begin(), t.end(), table);
  return HFX_OK;
}

static void rk_clear(hfx_ctx* c) {
  cudaStreamSynchronize(c->stream);
  c->rkStages = c->rkStage = 0;
  c->rkMem.release();
  c->d_kSol.clear();
  c->d_kFlux.clear();
  c->d_kTrace.clear();
  c->d_oldSol = c->d_oldFlux = c->d_oldTrace = c->d_wU = c->d_wQ = c->d_wL = nullptr;
}

static int rk_configure(hfx_ctx* c, int nStages, const double* table, double dt) {
  if (!(dt > 0.0)) return set_err(c, HFX_ERR_ARG, "rk_set: the time step needs to be set and it should not be 0");
  const int W = nStages + 1;
  cudaSetDevice(c->device);
  int rc = ensure_outputs(c);
  if (rc) return rc;
  rk_clear(c);
  c->d_kSol.assign(nStages, nullptr);
  c->d_kFlux.assign(nStages, nullptr);
  c->d_kTrace.assign(nStages, nullptr);
  const size_t E = (size_t)c->nCells, LU = c->re.nNodes, LQ = (size_t)c->dim * c->re.nNodes, n = c->ndofs();
  DevMem& m = c->rkMem;
  HFX_CUDA(c, dalloc(m, &c->d_oldSol, E * LU));
  HFX_CUDA(c, dalloc(m, &c->d_oldFlux, E * LQ));
  HFX_CUDA(c, dalloc(m, &c->d_oldTrace, n));
  HFX_CUDA(c, dalloc(m, &c->d_wU, E * LU));
  HFX_CUDA(c, dalloc(m, &c->d_wQ, E * LQ));
  HFX_CUDA(c, dalloc(m, &c->d_wL, n));
  for (int k = 0; k < nStages; ++k) {
    HFX_CUDA(c, dalloc(m, &c->d_kSol[k], E * LU));
    HFX_CUDA(c, dalloc(m, &c->d_kFlux[k], E * LQ));
    HFX_CUDA(c, dalloc(m, &c->d_kTrace[k], n));
  }
  c->rkTable.assign(table, table + (size_t)W * W);
  c->rkStages = nStages;
  c->rkStage = 0;
  c->rkDt = dt;
  c->assembled = false;
  // Old* = the current fields until the first begin_step
  HFX_CUDA(c, cudaMemcpyAsync(c->d_oldSol, c->d_sol, sizeof(double) * E * LU, cudaMemcpyDeviceToDevice, c->stream));
  HFX_CUDA(c, cudaMemcpyAsync(c->d_oldFlux, c->d_flux, sizeof(double) * E * LQ, cudaMemcpyDeviceToDevice, c->stream));
  HFX_CUDA(c, cudaMemcpyAsync(c->d_oldTrace, c->d_trace, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

// RungeKutta::setButcherTable(EMatrix) (RungeKutta.cpp:18-32): a square table
// whose strictly upper part (first column included) is zero; 0 stages = off.
int hfx_rk_set(hfx_ctx* c, int nStages, const double* table, double dt) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "rk_set: upload a mesh first");
  if (nStages == 0) {
    rk_clear(c);
    c->assembled = false;
    return HFX_OK;
  }
  if (nStages < 0 || nStages > RkTerms::MAX || !table) return set_err(c, HFX_ERR_ARG, "rk_set: 1..8 stages and a table");
  const int W = nStages + 1;
  for (int i = 0; i < W; ++i)
    for (int j = i + 1; j < W; ++j)
      if (table[i * W + j] != 0.0)
        return set_err(c, HFX_ERR_ARG,
                       "rk_set: the upper triangular part of the Butcher table should be null (no fully implicit "
                       "implementation as of yet)");
  return rk_configure(c, nStages, table, dt);
}

// RungeKutta(re, RKType) (RungeKutta.cpp:5-16): a named table, taken as is.
int hfx_rk_set_type(hfx_ctx* c, int type, double dt) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "rk_set_type: upload a mesh first");
  int S = 0;
  if (hfx_rk_butcher(type, &S, nullptr)) return set_err(c, HFX_ERR_ARG, "rk_set_type: unknown Runge-Kutta type");
  std::vector<double> t((size_t)(S + 1) * (S + 1));
  hfx_rk_butcher(type, &S, t.data());
  return rk_configure(c, S, t.data(), dt);
}

int hfx_rk_begin_step(hfx_ctx* c) {
  if (!c) return HFX_ERR_ARG;
  if (c->rkStages == 0) return set_err(c, HFX_ERR_STATE, "rk_begin_step: no Runge-Kutta scheme set");
  if (c->rkStage != 0) return set_err(c, HFX_ERR_STATE, "rk_begin_step: the previous step has stages left");
  const size_t E = (size_t)c->nCells, LU = c->re.nNodes, LQ = (size_t)c->dim * c->re.nNodes, n = c->ndofs();
  HFX_CUDA(c, cudaMemcpyAsync(c->d_oldSol, c->d_sol, sizeof(double) * E * LU, cudaMemcpyDeviceToDevice, c->stream));
  HFX_CUDA(c, cudaMemcpyAsync(c->d_oldFlux, c->d_flux, sizeof(double) * E * LQ, cudaMemcpyDeviceToDevice, c->stream));
  HFX_CUDA(c, cudaMemcpyAsync(c->d_oldTrace, c->d_trace, sizeof(double) * n, cudaMemcpyDeviceToDevice, c->stream));
  c->assembled = false;
  return HFX_OK;
}

// RungeKutta::computeStage (RungeKutta.cpp:131-170): k_s = (x - x_old) / dt,
// x = x_old + dt sum_{j<=s} a_sj k_j for Solution, Flux and Trace.
int hfx_rk_compute_stage(hfx_ctx* c) {
  if (!c) return HFX_ERR_ARG;
  if (c->rkStages == 0) return set_err(c, HFX_ERR_STATE, "rk_compute_stage: no Runge-Kutta scheme set");
  if (c->rkStage >= c->rkStages)
    return set_err(c, HFX_ERR_STATE,
                   "rk_compute_stage: cannot compute more stages than the method allows, think about computing the "
                   "solution");
  const int S = c->rkStages, st = c->rkStage;
  const double dt = c->rkDt;
  const int64_t E = c->nCells, LU = c->re.nNodes, LQ = (int64_t)c->dim * c->re.nNodes;
  double* xs[3] = {c->d_sol, c->d_flux, c->d_trace};
  const double* olds[3] = {c->d_oldSol, c->d_oldFlux, c->d_oldTrace};
  std::vector<double*>* ks[3] = {&c->d_kSol, &c->d_kFlux, &c->d_kTrace};
  const int64_t len[3] = {E * LU, E * LQ, c->ndofs()};
  for (int f = 0; f < 3; ++f) {
    RkTerms d{};
    d.n = 1;
    d.coef[0] = -1.0 / dt;
    d.ptr[0] = olds[f];
    HFX_CUDA(c, launch_rk_lincomb(len[f], (*ks[f])[st], 1.0 / dt, xs[f], d, c->stream));
    RkTerms u{};
    for (int j = 0; j <= st; ++j) {
      u.coef[u.n] = dt * c->rkTable[(size_t)st * (S + 1) + 1 + j];
      u.ptr[u.n++] = (*ks[f])[j];
    }
    HFX_CUDA(c, launch_rk_lincomb(len[f], xs[f], 1.0, olds[f], u, c->stream));
  }
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  c->rkStage += 1;
  c->assembled = false;
  c->qValid = false;
  return HFX_OK;
}

// RungeKutta::computeSolution (RungeKutta.cpp:172-213): x = x_old + dt sum_k b_k k_k.
int hfx_rk_compute_solution(hfx_ctx* c) {
  if (!c) return HFX_ERR_ARG;
  if (c->rkStages == 0) return set_err(c, HFX_ERR_STATE, "rk_compute_solution: no Runge-Kutta scheme set");
  if (c->rkStage != c->rkStages)
    return set_err(c, HFX_ERR_STATE, "rk_compute_solution: all stages must be computed before computing the solution");
  const int S = c->rkStages;
  const double dt = c->rkDt;
  const int64_t E = c->nCells, LU = c->re.nNodes, LQ = (int64_t)c->dim * c->re.nNodes;
  double* xs[3] = {c->d_sol, c->d_flux, c->d_trace};
  const double* olds[3] = {c->d_oldSol, c->d_oldFlux, c->d_oldTrace};
  std::vector<double*>* ks[3] = {&c->d_kSol, &c->d_kFlux, &c->d_kTrace};
  const int64_t len[3] = {E * LU, E * LQ, c->ndofs()};
  for (int f = 0; f < 3; ++f) {
    RkTerms u{};
    for (int k = 0; k < S; ++k) {
      u.coef[u.n] = dt * c->rkTable[(size_t)S * (S + 1) + 1 + k];
      u.ptr[u.n++] = (*ks[f])[k];
    }
    HFX_CUDA(c, launch_rk_lincomb(len[f], xs[f], 1.0, olds[f], u, c->stream));
  }
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  c->rkStage = 0;
  c->assembled = false;
  c->qValid = false;
  return HFX_OK;
}

int hfx_assembly_info(hfx_ctx* c, int* affine) {
  if (!c || !affine) return HFX_ERR_ARG;
  *affine = c->lastAffine ? 1 : 0;
  return HFX_OK;
}

int hfx_cg_operators(hfx_ctx* c, int which, int precision, const double* velocity, int velLayout, double* out) {
  if (!c || !out || which <= 0 || which > 7) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "cg_operators: upload a mesh first");
  if (precision != HFX_PREC_FP64 && precision != HFX_PREC_MIXED)
    return set_err(c, HFX_ERR_ARG, "cg_operators: precision is HFX_PREC_FP64 or HFX_PREC_MIXED");
  if ((which & HFX_OP_CONVECTION) && (!velocity || (velLayout != 0 && velLayout != 1)))
    return set_err(c, HFX_ERR_ARG, "cg_operators: convection needs a velocity (layout 0 or 1)");
  if (!local_condense_supported(c->dim, c->order))
    return set_err(c, HFX_ERR_UNSUPPORTED, "cg_operators: order not supported");
  cudaSetDevice(c->device);
  cudaStream_t s = c->stream;
  const int N = c->re.nNodes;
  const size_t outN = (size_t)c->nCells * 3 * N * N;
  if (!c->d_cgout) HFX_CUDA(c, dalloc(c->cgMem, &c->d_cgout, outN));
  const double* dvel = nullptr;
  if (which & HFX_OP_CONVECTION) {
    const size_t nv = (velLayout == 0 ? (size_t)c->nNodes : (size_t)c->nCells * N) * c->dim;
    if (nv > c->cgVelCap) {
      HFX_CUDA(c, dalloc(c->cgMem, &c->d_cgvel, nv));
      c->cgVelCap = nv;
    }
    HFX_CUDA(c, cudaMemcpyAsync(c->d_cgvel, velocity, sizeof(double) * nv, cudaMemcpyHostToDevice, s));
    dvel = c->d_cgvel;
  }
  CgOpParams p{};
  p.nCells = c->nCells;
  p.coords = c->d_coords;
  p.cells = c->d_cells;
  p.kappa = c->kappa.p;
  p.kc = c->kc;
  p.kappaLayout = c->kLayout;
  p.vel = dvel;
  p.velLayout = velLayout;
  p.tab = c->d_tab;
  p.which = which;
  p.out = c->d_cgout;
  p.status = c->d_status;
  if (precision == HFX_PREC_MIXED) {
    if (!c->d_cgtab) {
      std::vector<double> tab;
      tab.insert(tab.end(), c->re.phi.begin(), c->re.phi.end());
      tab.insert(tab.end(), c->re.dphi.begin(), c->re.dphi.end());
      tab.insert(tab.end(), c->re.ipW.begin(), c->re.ipW.end());
      std::vector<float> t = tc_cg_table(c->dim, c->order, tab.data());
      HFX_CUDA(c, upload(c->cgMem, &c->d_cgtab, t.data(), t.size(), s));
    }
    if (!c->d_status) HFX_CUDA(c, dalloc(c->outMem, &c->d_status, 1));
    p.status = c->d_status;
    p.tctab = c->d_cgtab;
    HFX_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), s));
    c->timer.begin(K_TENSOR, s);
    HFX_CUDA(c, launch_cg_operators_tc(c->dim, c->order, p, s));
    c->timer.end(K_TENSOR, s);
  } else {
    c->timer.begin(K_LOCAL, s);
    HFX_CUDA(c, launch_cg_operators_f64(c->dim, c->order, p, s));
    c->timer.end(K_LOCAL, s);
  }
  HFX_CUDA(c, cudaMemcpyAsync(out, c->d_cgout, sizeof(double) * outN, cudaMemcpyDeviceToHost, s));
  int status = 0;
  if (precision == HFX_PREC_MIXED)
    HFX_CUDA(c, cudaMemcpyAsync(&status, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
  HFX_CUDA(c, cudaStreamSynchronize(s));
  if (status == 2) return set_err(c, HFX_ERR_CUDA, "cg_operators: a tensor-core wait ran out");
  return HFX_OK;
}

int hfx_test_coarse_barrier(hfx_ctx* c) {
  if (!c) return HFX_ERR_ARG;
  if (!c->coarseBuilt || !c->coarse.dev.testHold)
    return set_err(c, HFX_ERR_STATE, "test_coarse_barrier: no two-level solve has run yet");
  const int one = 1;
  c->coarse.forceCoop = true;  // the next solve takes the cooperative kernel, whose barrier is tested
  HFX_CUDA(c, cudaMemcpyAsync(c->coarse.dev.testHold, &one, sizeof(int), cudaMemcpyHostToDevice, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

int hfx_set_tuning(hfx_ctx* c, int spmvKernel) {
  if (!c || spmvKernel < -1 || spmvKernel > 3) return HFX_ERR_ARG;
  c->spmvChoice = spmvKernel;
  return HFX_OK;
}

int hfx_tuning_info(hfx_ctx* c, int* spmvKernel, float* spmvMs) {
  if (!c) return HFX_ERR_ARG;
  if (spmvKernel) *spmvKernel = c->spmvChoice;
  if (spmvMs)
    for (int k = 0; k < 4; ++k) spmvMs[k] = c->spmvTimes[k];
  return HFX_OK;
}

int hfx_mixed_assembly_info(hfx_ctx* c, int* tensorCores) {
  if (!c || !tensorCores) return HFX_ERR_ARG;
  *tensorCores = (c->mixedMode && c->lastTensor) ? 1 : 0;
  return HFX_OK;
}

int hfx_get_tc_blocks(hfx_ctx* c, int count, const int* cells, float* out, int64_t* stride) {
  if (!c || count < 0 || (count > 0 && (!cells || !out))) return HFX_ERR_ARG;
  const int64_t st = tc_blocks_stride(c->dim, c->order);
  if (stride) *stride = st;
  if (!c->assembled || !c->mixedMode || !c->lastTensor)
    return set_err(c, HFX_ERR_STATE, "get_tc_blocks: no tensor-core mixed assembly");
  for (int k = 0; k < count; ++k) {
    if (cells[k] < 0 || cells[k] >= c->nCells) return set_err(c, HFX_ERR_ARG, "get_tc_blocks: cell out of range");
    HFX_CUDA(c, cudaMemcpyAsync(out + (size_t)k * st, c->d_tcb + (size_t)cells[k] * st, sizeof(float) * st,
                                cudaMemcpyDeviceToHost, c->stream));
  }
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

int hfx_get_condensed(hfx_ctx* c, double* S, double* S0, double* U, double* Q, double* U0, double* Q0) {
  if (!c) return HFX_ERR_ARG;
  if (!c->assembled) return set_err(c, HFX_ERR_STATE, "get_condensed: assemble first");
  if (c->mixedMode) return set_err(c, HFX_ERR_STATE, "get_condensed: the mixed assembly keeps FP32 blocks; use hfx_assemble");
  const int64_t E = c->nCells;
  const int LU = c->re.nNodes, LQ = c->dim * c->re.nNodes, LL = c->re.nFaces * c->re.nNodesFace;
  cudaStream_t s = c->stream;
  auto cp = [&](double* h, const double* d, size_t n) {
    return h ? cudaMemcpyAsync(h, d, sizeof(double) * n, cudaMemcpyDeviceToHost, s) : cudaSuccess;
  };
  if ((Q || Q0) && !c->qValid) {
    // the affine path keeps Q, Q0 implicit: form them from U, U0 and the element factors
    HFX_CUDA(c, launch_q_from_u(c->dim, c->order, c->nCells, c->d_U, c->d_U0, c->d_atab, c->d_geo, c->d_Q, c->d_Q0, s));
    c->qValid = true;
  }
  HFX_CUDA(c, cp(S, c->d_S, (size_t)E * LL * LL));
  HFX_CUDA(c, cp(S0, c->d_S0, (size_t)E * LL));
  HFX_CUDA(c, cp(U, c->d_U, (size_t)E * LU * LL));
  HFX_CUDA(c, cp(Q, c->d_Q, (size_t)E * LQ * LL));
  HFX_CUDA(c, cp(U0, c->d_U0, (size_t)E * LU));
  HFX_CUDA(c, cp(Q0, c->d_Q0, (size_t)E * LQ));
  HFX_CUDA(c, cudaStreamSynchronize(s));
  return HFX_OK;
}

int hfx_get_csr(hfx_ctx* c, int64_t* rowptr, int* col, double* val, double* rhs) {
  if (!c) return HFX_ERR_ARG;
  if (!c->assembled && (val || rhs)) return set_err(c, HFX_ERR_STATE, "get_csr: assemble first");
  if (c->mixedMode && (val || rhs)) return set_err(c, HFX_ERR_STATE, "get_csr: the mixed assembly keeps FP32 values; use hfx_assemble");
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "get_csr: no mesh");
  const int NF = c->re.nNodesFace;
  const int nF = c->topo.nFaces;
  if (rowptr || col) {
    int64_t pos = 0;
    if (rowptr) rowptr[0] = 0;
    for (int f = 0; f < nF; ++f) {
      int64_t b0 = c->bp.rowptr[f], nb = c->bp.rowptr[f + 1] - b0;
      for (int a = 0; a < NF; ++a) {
        if (col)
          for (int64_t k = 0; k < nb; ++k)
            for (int b = 0; b < NF; ++b) col[pos + k * NF + b] = c->bp.col[b0 + k] * NF + b;
        pos += nb * NF;
        if (rowptr) rowptr[(int64_t)f * NF + a + 1] = pos;
      }
    }
  }
  cudaStream_t s = c->stream;
  std::vector<double> blocks;
  if (val) {
    blocks.resize((size_t)c->nnz());
    HFX_CUDA(c, cudaMemcpyAsync(blocks.data(), c->d_val, sizeof(double) * c->nnz(), cudaMemcpyDeviceToHost, s));
  }
  if (rhs) HFX_CUDA(c, cudaMemcpyAsync(rhs, c->d_rhs, sizeof(double) * c->ndofs(), cudaMemcpyDeviceToHost, s));
  HFX_CUDA(c, cudaStreamSynchronize(s));
  if (val) {
    // device blocks are column-major per Nf x Nf block; AIJ rows are row-major
    int64_t pos = 0;
    for (int f = 0; f < nF; ++f) {
      int64_t b0 = c->bp.rowptr[f], nb = c->bp.rowptr[f + 1] - b0;
      for (int a = 0; a < NF; ++a)
        for (int64_t k = 0; k < nb; ++k)
          for (int b = 0; b < NF; ++b) val[pos++] = blocks[(b0 + k) * NF * NF + (int64_t)b * NF + a];
    }
  }
  return HFX_OK;
}

int hfx_get_condensed_sample(hfx_ctx* c, int count, const int* cells, double* S, double* S0, double* U, double* Q,
                             double* U0, double* Q0) {
  if (!c || count < 0 || (count > 0 && !cells)) return HFX_ERR_ARG;
  if (!c->assembled) return set_err(c, HFX_ERR_STATE, "get_condensed_sample: assemble first");
  if (c->mixedMode)
    return set_err(c, HFX_ERR_STATE, "get_condensed_sample: the mixed assembly keeps FP32 blocks; use hfx_assemble");
  for (int k = 0; k < count; ++k)
    if (cells[k] < 0 || cells[k] >= c->nCells) return set_err(c, HFX_ERR_ARG, "get_condensed_sample: cell out of range");
  const int64_t LU = c->re.nNodes, LQ = c->dim * c->re.nNodes, LL = c->re.nFaces * c->re.nNodesFace;
  cudaStream_t s = c->stream;
  if ((Q || Q0) && !c->qValid) {
    HFX_CUDA(c, launch_q_from_u(c->dim, c->order, c->nCells, c->d_U, c->d_U0, c->d_atab, c->d_geo, c->d_Q, c->d_Q0, s));
    c->qValid = true;
  }
  auto cp = [&](double* h, const double* d, int64_t n, int k) {
    return h ? cudaMemcpyAsync(h + (size_t)k * n, d + (size_t)cells[k] * n, sizeof(double) * n, cudaMemcpyDeviceToHost, s)
             : cudaSuccess;
  };
  for (int k = 0; k < count; ++k) {
    HFX_CUDA(c, cp(S, c->d_S, LL * LL, k));
    HFX_CUDA(c, cp(S0, c->d_S0, LL, k));
    HFX_CUDA(c, cp(U, c->d_U, LU * LL, k));
    HFX_CUDA(c, cp(Q, c->d_Q, LQ * LL, k));
    HFX_CUDA(c, cp(U0, c->d_U0, LU, k));
    HFX_CUDA(c, cp(Q0, c->d_Q0, LQ, k));
  }
  HFX_CUDA(c, cudaStreamSynchronize(s));
  return HFX_OK;
}

int hfx_get_csr_rows(hfx_ctx* c, int count, const int* faces, int* rowlen, int* col, double* val, double* rhs,
                     int64_t cap) {
  if (!c || count < 0 || (count > 0 && (!faces || !rowlen))) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "get_csr_rows: no mesh");
  if (!c->assembled && (val || rhs)) return set_err(c, HFX_ERR_STATE, "get_csr_rows: assemble first");
  if (c->mixedMode && (val || rhs))
    return set_err(c, HFX_ERR_STATE, "get_csr_rows: the mixed assembly keeps FP32 values; use hfx_assemble");
  const int NF = c->re.nNodesFace;
  const int nF = c->topo.nFaces;
  int64_t total = 0;
  std::vector<char> seen;
  for (int k = 0; k < count; ++k) {
    const int f = faces[k];
    if (f < 0 || f >= nF) return set_err(c, HFX_ERR_ARG, "get_csr_rows: face out of range");
    total += (c->bp.rowptr[f + 1] - c->bp.rowptr[f]) * NF * NF;
  }
  {
    std::vector<int> sorted(faces, faces + count);
    std::sort(sorted.begin(), sorted.end());
    if (std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end())
      return set_err(c, HFX_ERR_ARG, "get_csr_rows: face listed twice");
  }
  if ((col || val) && total > cap) return set_err(c, HFX_ERR_ARG, "get_csr_rows: cap too small");
  cudaStream_t s = c->stream;
  std::vector<double> blocks(val ? (size_t)total : 0);
  int64_t pos = 0;
  for (int k = 0; k < count; ++k) {
    const int f = faces[k];
    const int64_t b0 = c->bp.rowptr[f], nb = c->bp.rowptr[f + 1] - b0;
    if (val)
      HFX_CUDA(c, cudaMemcpyAsync(blocks.data() + pos, c->d_val + b0 * NF * NF, sizeof(double) * nb * NF * NF,
                                  cudaMemcpyDeviceToHost, s));
    if (rhs)
      HFX_CUDA(c, cudaMemcpyAsync(rhs + (size_t)k * NF, c->d_rhs + (int64_t)f * NF, sizeof(double) * NF,
                                  cudaMemcpyDeviceToHost, s));
    pos += nb * NF * NF;
  }
  HFX_CUDA(c, cudaStreamSynchronize(s));
  // device blocks are column-major per Nf x Nf block; AIJ rows are row-major
  pos = 0;
  for (int k = 0; k < count; ++k) {
    const int f = faces[k];
    const int64_t b0 = c->bp.rowptr[f], nb = c->bp.rowptr[f + 1] - b0;
    for (int a = 0; a < NF; ++a) {
      rowlen[(size_t)k * NF + a] = (int)(nb * NF);
      for (int64_t kb = 0; kb < nb; ++kb)
        for (int b = 0; b < NF; ++b) {
          const int64_t o = pos + (int64_t)a * nb * NF + kb * NF + b;
          if (col) col[o] = c->bp.col[b0 + kb] * NF + b;
          if (val) val[o] = blocks[pos + kb * NF * NF + (int64_t)b * NF + a];
        }
    }
    pos += nb * NF * NF;
  }
  return HFX_OK;
}

// Coarse space of the two-level preconditioner: host structure and device
// buffers on first use (mesh-dependent), the operator after every assembly.
static int ensure_coarse(hfx_ctx* c, double target, int maxDeg = 64) {
  cudaStream_t s = c->stream;
  if (!c->coarseBuilt) {
    std::string err;
    CoarseHost h;
    if (!build_coarse_host(c->re, c->nCells, c->cellVerts.data(), c->topo, &h, &err))
      return set_err(c, HFX_ERR_ARG, err);
    DevMem& m = c->coarseMem;
    m.release();
    CoarseDev& d = c->coarse.dev;
    d = CoarseDev{};
    d.nV = h.nV;
    d.dim = h.dim;
    d.NF = h.NF;
    d.F = h.F;
    d.LL = h.LL;
    d.NV1 = h.NV1;
    d.nFaces = c->topo.nFaces;
    d.nCells = c->nCells;
    d.nnz = (int64_t)h.col.size();
    int *rowptr, *col, *cptr, *cidx, *rptr, *ridx, *faceV;
    HFX_CUDA(c, upload(m, &rowptr, h.rowptr.data(), h.rowptr.size(), s));
    HFX_CUDA(c, upload(m, &col, h.col.data(), h.col.size(), s));
    HFX_CUDA(c, upload(m, &cptr, h.cptr.data(), h.cptr.size(), s));
    HFX_CUDA(c, upload(m, &cidx, h.cidx.data(), h.cidx.size(), s));
    HFX_CUDA(c, upload(m, &rptr, h.rptr.data(), h.rptr.size(), s));
    HFX_CUDA(c, upload(m, &ridx, h.ridx.data(), h.ridx.size(), s));
    HFX_CUDA(c, upload(m, &faceV, h.faceV.data(), h.faceV.size(), s));
    HFX_CUDA(c, upload(m, &d.Wf, h.Wf.data(), h.Wf.size(), s));
    int *ellCol, *ellSrc;
    HFX_CUDA(c, upload(m, &ellCol, h.ellCol.data(), h.ellCol.size(), s));
    HFX_CUDA(c, upload(m, &ellSrc, h.ellSrc.data(), h.ellSrc.size(), s));
    HFX_CUDA(c, dalloc(m, &d.ellVal, h.ellCol.size()));
    d.ellW = h.ellW;
    d.ellCol = ellCol;
    d.ellSrc = ellSrc;
    HFX_CUDA(c, upload(m, &d.Wc, h.Wc.data(), h.Wc.size(), s));
    d.rowptr = rowptr;
    d.col = col;
    d.cptr = cptr;
    d.cidx = cidx;
    d.rptr = rptr;
    d.ridx = ridx;
    d.faceV = faceV;
    d.cell2face = c->d_cell2face;
    d.isBnd = c->d_isBnd;
    const size_t nV = (size_t)h.nV;
    HFX_CUDA(c, dalloc(m, &d.Ce, (size_t)c->nCells * h.NV1 * h.NV1));
    HFX_CUDA(c, dalloc(m, &d.val, h.col.size()));
    HFX_CUDA(c, dalloc(m, &d.dinv, nV));
    HFX_CUDA(c, dalloc(m, &d.rc, nV));
    HFX_CUDA(c, dalloc(m, &d.yc, nV));
    HFX_CUDA(c, dalloc(m, &d.cr, nV));
    HFX_CUDA(c, dalloc(m, &d.cd0, nV));
    HFX_CUDA(c, dalloc(m, &d.cd1, nV));
    HFX_CUDA(c, dalloc(m, &d.lz, nV));
    HFX_CUDA(c, dalloc(m, &d.partials, (size_t)152 * 32 + 64));
    HFX_CUDA(c, dalloc(m, &d.barrier, 2));
    HFX_CUDA(c, dalloc(m, &d.error, 1));
    HFX_CUDA(c, dalloc(m, &d.testHold, 1));
    HFX_CUDA(c, dalloc(m, &d.lanczosOut, 2 * 30 + 3));
    HFX_CUDA(c, cudaMemsetAsync(d.barrier, 0, 2 * sizeof(unsigned), s));
    HFX_CUDA(c, cudaMemsetAsync(d.error, 0, sizeof(int), s));
    HFX_CUDA(c, cudaMemsetAsync(d.testHold, 0, sizeof(int), s));
    c->coarseHost = std::move(h);
    c->coarseBuilt = true;
    c->coarse.ready = false;
  }
  if (!c->coarse.ready || c->coarseTarget != target || c->coarseMaxDeg != maxDeg) {
    c->coarseTarget = target;
    c->coarseMaxDeg = maxDeg;
    c->timer.begin(K_COARSE, s);
    cudaError_t e = coarse_setup<double>(&c->coarse, c->d_S, maxDeg, target, s);
    c->timer.end(K_COARSE, s);
    if (e != cudaSuccess) return cuda_err(c, e, "coarse setup");
  }
  return HFX_OK;
}

void hfx_solve_opts_default(hfx_solve_opts* o) {
  if (!o) return;
  o->method = HFX_KSP_AUTO;
  o->precond = HFX_PC_BLOCK_JACOBI;
  o->precision = HFX_PREC_FP64;
  o->rtol = 1e-10;
  o->maxits = 20000;
  o->restart = 30;
  o->inner_rtol = 1e-2;
  o->use_initial_guess = 0;
  o->coarse_guess = 0;
  o->coarse_rtol = 0.1;
  o->coarse_mode = HFX_COARSE_CHEBYSHEV;
  o->coarse_degree = 0;
}

static int ensure_workspace(hfx_ctx* c, bool mixed, int restart) {
  const size_t n = (size_t)c->ndofs(), nnz = (size_t)c->nnz();
  const int NF = c->re.nNodesFace;
  DevMem& m = c->wsMem;
  TraceWorkspace& w = c->ws;
  if (restart > c->wsRestart) {
    // GMRES bases grow on demand (restart+1 vectors per precision)
    HFX_CUDA(c, dalloc(m, &w.V64, n * (restart + 1)));
    HFX_CUDA(c, dalloc(m, &w.V32, n * (restart + 1)));
    HFX_CUDA(c, dalloc(m, &w.hdev, (size_t)restart + 1));
    c->wsRestart = restart;
  }
  if (c->wsReady && (!mixed || c->wsMixed)) return HFX_OK;
  if (!c->wsReady) {
    HFX_CUDA(c, dalloc(m, &w.bS, n));
    HFX_CUDA(c, dalloc(m, &w.r, n));
    HFX_CUDA(c, dalloc(m, &w.z, n));
    HFX_CUDA(c, dalloc(m, &w.p0, n));
    HFX_CUDA(c, dalloc(m, &w.p1, n));
    HFX_CUDA(c, dalloc(m, &w.q, n));
    HFX_CUDA(c, dalloc(m, &w.pc64, (size_t)c->topo.nFaces * NF * NF));
    HFX_CUDA(c, dalloc(m, &w.partials, trace_partials_needed()));
    HFX_CUDA(c, dalloc(m, &w.state, 1));
    HFX_CUDA(c, cudaMemsetAsync(w.p0, 0, sizeof(double) * n, c->stream));
    HFX_CUDA(c, cudaMemsetAsync(w.p1, 0, sizeof(double) * n, c->stream));
    c->wsReady = true;
  }
  if (mixed && !c->wsMixed) {
    HFX_CUDA(c, dalloc(m, &w.val32, nnz));
    w.val32h = nullptr;
    if (c->nHalf > 0) HFX_CUDA(c, dalloc(m, &w.val32h, (size_t)c->nHalf * NF * NF));
    HFX_CUDA(c, dalloc(m, &w.pc32, (size_t)c->topo.nFaces * NF * NF));
    HFX_CUDA(c, dalloc(m, &w.r32, n));
    HFX_CUDA(c, dalloc(m, &w.z32, n));
    HFX_CUDA(c, dalloc(m, &w.p032, n));
    HFX_CUDA(c, dalloc(m, &w.p132, n));
    HFX_CUDA(c, dalloc(m, &w.q32, n));
    HFX_CUDA(c, dalloc(m, &w.d32, n));
    HFX_CUDA(c, dalloc(m, &w.rhs32, n));
    HFX_CUDA(c, dalloc(m, &w.bS32, n));
    HFX_CUDA(c, cudaMemsetAsync(w.p032, 0, sizeof(float) * n, c->stream));
    HFX_CUDA(c, cudaMemsetAsync(w.p132, 0, sizeof(float) * n, c->stream));
    c->wsMixed = true;
  }
  return HFX_OK;
}

// Iterative refinement of the full HDG system: FP64 residual, FP32 condensed
// correction (element condensation, trace solve, recovery), FP64 update.
static int solve_mixed(hfx_ctx* c, const hfx_solve_opts& o, int method, int restart, double* trace,
                       hfx_solve_info* info) {
  cudaStream_t s = c->stream;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  F32SolveArgs a{};
  a.dim = c->dim;
  a.A = TraceView{c->topo.nFaces, c->re.nNodesFace, c->d_browptr, c->d_bcol, c->d_isBnd};
  a.val = c->ws.val32;
  a.rhs = c->ws.rhs32;
  a.x = c->d_dl32;
  a.precond = o.precond;
  a.gmres = method == HFX_KSP_GMRES;
  a.restart = restart;
  a.ws = c->ws;
  a.stream = s;
  a.timer = &c->timer;
  const int LU = c->re.nNodes, LQ = c->dim * c->re.nNodes, LL = c->re.nFaces * c->re.nNodesFace;
  Correct32Params cp{c->nCells, c->re.nFaces, c->re.nNodesFace, LU, LQ, LL, c->ndofs(), c->d_cell2face, c->d_perm,
                     c->d_U32, c->d_Q32, c->d_U032, c->d_Q032, c->d_dl32, c->d_sol, c->d_flux, c->d_trace};
  const double inner = o.inner_rtol > 0 ? o.inner_rtol : 1e-4;
  int its = 0, refinements = 0, status = 0, rc;
  double rr = c->mixedRR, bb = c->mixedBB;
  bool first = true;
  while (true) {
    if (!first) {
      if ((rc = mixed_residual(c, &rr))) return rc;
      if (!std::isfinite(rr)) {
        status = HFX_ERR_NAN;
        break;
      }
    }
    if (rr <= o.rtol * o.rtol * bb) break;
    if (its >= o.maxits || refinements >= 60) {
      status = HFX_ERR_NOT_CONVERGED;
      break;
    }
    if (!first && (rc = mixed_condense(c, false))) return rc;
    a.rtol = std::max(inner, 0.5 * o.rtol * std::sqrt(bb / std::max(rr, 1e-300)));
    a.maxits = o.maxits - its;
    a.rebuildPrecond = first;
    int st = trace_solve_f32(a, &its);
    if (st != 0 && st != HFX_ERR_NOT_CONVERGED) {
      status = st;
      break;
    }
    c->timer.begin(K_RECOVER, s);
    HFX_CUDA(c, launch_correct32(cp, s));
    c->timer.end(K_RECOVER, s);
    refinements += 1;
    first = false;
  }
  c->mixedRR = rr;
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (info) {
    info->status = status;
    info->iterations = its;
    info->refinements = refinements;
    info->rel_residual = bb > 0 ? std::sqrt(rr / bb) : std::sqrt(rr);
    info->solve_ms = ms;
    info->fallback = 0;
    info->coarse_degree = 0;
    info->coarse_learned = 0;
  }
  if (trace) HFX_CUDA(c, cudaMemcpy(trace, c->d_trace, sizeof(double) * c->ndofs(), cudaMemcpyDeviceToHost));
  c->solved = true;
  if (status == HFX_ERR_NOT_CONVERGED) return set_err(c, status, "solve: mixed refinement not converged");
  if (status != 0) return set_err(c, status, "solve: mixed refinement failed");
  return HFX_OK;
}

int hfx_solve(hfx_ctx* c, const hfx_solve_opts* opts, double* trace, hfx_solve_info* info) {
  if (!c) return HFX_ERR_ARG;
  if (!c->assembled) return set_err(c, HFX_ERR_STATE, "solve: system must be assembled before solving");
  hfx_solve_opts o;
  if (opts) o = *opts;
  else hfx_solve_opts_default(&o);
  if (o.method < HFX_KSP_CG || o.method > HFX_KSP_AUTO) return set_err(c, HFX_ERR_ARG, "solve: unknown method");
  if (o.precond < HFX_PC_NONE || o.precond > HFX_PC_TWOLEVEL || o.rtol <= 0.0 || o.maxits <= 0)
    return set_err(c, HFX_ERR_ARG, "solve: bad options");
  int method = o.method;
  if (method == HFX_KSP_AUTO) method = c->kappaCellConstant ? HFX_KSP_CG : HFX_KSP_GMRES;
  if (method == HFX_KSP_CG && !c->kappaCellConstant)
    return set_err(c, HFX_ERR_ARG,
                   "solve: CG needs a symmetric trace system; the diffusion tensor varies inside cells (use GMRES)");
  if (o.precond == HFX_PC_TWOLEVEL && (method != HFX_KSP_CG || c->mixedMode))
    return set_err(c, HFX_ERR_UNSUPPORTED,
                   "solve: the two-level preconditioner needs CG on the trace system assembled in FP64");
  const int restart = o.restart > 0 ? o.restart : 30;
  cudaSetDevice(c->device);
  bool mixed = o.precision == HFX_PREC_MIXED;
  int rc = ensure_workspace(c, mixed, method == HFX_KSP_GMRES ? restart : 0);
  if (rc) return rc;
  if (c->mixedMode) return solve_mixed(c, o, method, restart, trace, info);
  if (c->solverType == HFX_SEXPLICIT) {
    // no global solve: each face solves its own block
    cudaEvent_t f0, f1;
    cudaEventCreate(&f0);
    cudaEventCreate(&f1);
    cudaEventRecord(f0, c->stream);
    HFX_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
    c->timer.begin(K_OTHER, c->stream);
    HFX_CUDA(c, launch_face_block_solve(c->topo.nFaces, c->re.nNodesFace, c->d_browptr, c->d_bcol, c->d_val,
                                        c->d_rhs, c->d_trace, c->d_status, c->stream));
    c->timer.end(K_OTHER, c->stream);
    cudaEventRecord(f1, c->stream);
    int fst = 0;
    HFX_CUDA(c, cudaMemcpyAsync(&fst, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    HFX_CUDA(c, cudaStreamSynchronize(c->stream));
    float fms = 0.f;
    cudaEventElapsedTime(&fms, f0, f1);
    cudaEventDestroy(f0);
    cudaEventDestroy(f1);
    if (info) {
      *info = hfx_solve_info{};
      info->status = fst ? HFX_ERR_SINGULAR : HFX_OK;
      info->solve_ms = fms;
    }
    if (fst) return set_err(c, HFX_ERR_SINGULAR, "solve: singular face block (SEXPLICIT)");
    if (trace) HFX_CUDA(c, cudaMemcpy(trace, c->d_trace, sizeof(double) * c->ndofs(), cudaMemcpyDeviceToHost));
    c->solved = true;
    return HFX_OK;
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->stream);
  // a fixed Chebyshev degree K: the reduction target is out of reach, so the cap K decides
  int cdeg = o.coarse_degree > 0 ? std::min(o.coarse_degree, 64) : 0;
  // learned mode without an accepted polynomial: Chebyshev of the trained degree (the
  // polynomial the training started from), not the reduction target's degree
  if (!cdeg && o.precond == HFX_PC_TWOLEVEL && o.coarse_mode == HFX_COARSE_LEARNED && c->coarse.thetaHat.empty())
    cdeg = c->learnDegree;
  const double ctarget = cdeg ? 1e-300 : (o.coarse_rtol > 0.0 && o.coarse_rtol < 1.0 ? o.coarse_rtol : 0.1);
  if (o.precond == HFX_PC_TWOLEVEL && (rc = ensure_coarse(c, ctarget, cdeg ? cdeg : 64))) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return rc;
  }
  TraceSolveArgs a{};
  a.dim = c->dim;
  a.A = TraceView{c->topo.nFaces, c->re.nNodesFace, c->d_browptr, c->d_bcol, c->d_isBnd};
  if (method == HFX_KSP_CG && c->kappaCellConstant) {
    a.A.hidx = c->d_hidx;  // symmetric operator: FP32 copy in half storage
    a.A.ell = c->d_ell;
    a.A.ellWidth = c->ellWidth;
    a.A.nHalf = c->nHalf;
  }
  a.val = c->d_val;
  a.rhs = c->d_rhs;
  a.x = c->d_trace;
  a.precond = o.precond;
  a.mixed = mixed;
  a.rtol = o.rtol;
  a.inner_rtol = o.inner_rtol > 0 ? o.inner_rtol : 1e-2;
  a.maxits = o.maxits;
  a.max_refinements = 50;
  a.check_every = 25;
  a.use_initial_guess = o.use_initial_guess;
  a.ws = c->ws;
  a.stream = c->stream;
  a.timer = &c->timer;
  a.restart = restart;
  a.coarse = o.precond == HFX_PC_TWOLEVEL ? &c->coarse : nullptr;
  a.coarse_guess = o.coarse_guess;
  a.spmvChoice = &c->spmvChoice;
  a.spmvTimes = c->spmvTimes;
  a.stretchHint = &c->stretchHint;
  const bool learned = o.precond == HFX_PC_TWOLEVEL && o.coarse_mode == HFX_COARSE_LEARNED &&
                       !c->coarse.thetaHat.empty();
  c->coarse.useLearned = learned;
  TraceSolveResult res;
  int st = method == HFX_KSP_CG ? trace_solve(a, &res) : trace_gmres(a, &res);
  int fallback = 0;
  if (o.precond == HFX_PC_TWOLEVEL && st != 3) {
    // a coarse-solve barrier that gave up invalidates the two-level iterates
    int berr = 0;
    HFX_CUDA(c, cudaMemcpy(&berr, c->coarse.dev.error, sizeof(int), cudaMemcpyDeviceToHost));
    if (berr) {
      HFX_CUDA(c, cudaMemset(c->coarse.dev.error, 0, sizeof(int)));
      HFX_CUDA(c, cudaMemset(c->coarse.dev.barrier, 0, 2 * sizeof(unsigned)));
      c->coarse.coopGrid = 0;  // one-cluster or launch-per-step coarse solve from now on
      c->coarse.forceCoop = false;
      st = HFX_ERR_BREAKDOWN;
    }
  }
  if (o.precond == HFX_PC_TWOLEVEL &&
      (st == HFX_ERR_BREAKDOWN || st == HFX_ERR_NAN || st == HFX_ERR_NOT_CONVERGED)) {
    // the plain block-Jacobi solve finishes what the two-level solve could not
    const int its = res.iterations;
    a.precond = HFX_PC_BLOCK_JACOBI;
    a.coarse = nullptr;
    a.maxits = std::max(1, o.maxits - its);
    a.use_initial_guess = 0;
    res = TraceSolveResult{};
    st = trace_solve(a, &res);
    res.iterations += its;
    fallback = 1;
  }
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (info) {
    info->status = st;
    info->iterations = res.iterations;
    info->refinements = res.refinements;
    info->rel_residual = res.rel_residual;
    info->solve_ms = ms;
    info->fallback = fallback;
    info->coarse_degree =
        o.precond != HFX_PC_TWOLEVEL ? 0 : (learned ? (int)c->coarse.thetaHat.size() : c->coarse.degree);
    info->coarse_learned = learned ? 1 : 0;
  }
  c->coarse.useLearned = false;
  if (st == 3) return cuda_err(c, res.cudaErr, "solve");
  if (trace) HFX_CUDA(c, cudaMemcpy(trace, c->d_trace, sizeof(double) * c->ndofs(), cudaMemcpyDeviceToHost));
  c->solved = true;
  if (st == HFX_ERR_NOT_CONVERGED) return set_err(c, st, "solve: not converged within maxits");
  if (st == HFX_ERR_BREAKDOWN) return set_err(c, st, "solve: CG breakdown (non-positive curvature)");
  if (st == HFX_ERR_NAN) return set_err(c, st, "solve: NaN or Inf in the Krylov iteration");
  if (st != 0) return set_err(c, st, "solve: failed");
  return HFX_OK;
}

int hfx_coarse_operator(hfx_ctx* c, int* nV, int64_t* nnz, int* rowptr, int* col, float* val, int* vertexNode) {
  if (!c || !nV || !nnz) return HFX_ERR_ARG;
  if (!c->assembled || c->mixedMode)
    return set_err(c, HFX_ERR_STATE, "coarse_operator: needs a trace system assembled in FP64");
  cudaSetDevice(c->device);
  int rc = ensure_coarse(c, c->coarseTarget > 0.0 ? c->coarseTarget : 0.1, c->coarseMaxDeg);
  if (rc) return rc;
  const CoarseHost& h = c->coarseHost;
  *nV = h.nV;
  *nnz = (int64_t)h.col.size();
  if (!rowptr) return HFX_OK;
  std::copy(h.rowptr.begin(), h.rowptr.end(), rowptr);
  if (col) std::copy(h.col.begin(), h.col.end(), col);
  if (vertexNode) std::copy(h.vertexNode.begin(), h.vertexNode.end(), vertexNode);
  if (val) HFX_CUDA(c, cudaMemcpy(val, c->coarse.dev.val, sizeof(float) * h.col.size(), cudaMemcpyDeviceToHost));
  return HFX_OK;
}

int hfx_coarse_bounds(hfx_ctx* c, double* out) {
  if (!c || !out) return HFX_ERR_ARG;
  if (!c->assembled || c->mixedMode)
    return set_err(c, HFX_ERR_STATE, "coarse_bounds: needs a trace system assembled in FP64");
  cudaSetDevice(c->device);
  int rc = ensure_coarse(c, c->coarseTarget > 0.0 ? c->coarseTarget : 0.1, c->coarseMaxDeg);
  if (rc) return rc;
  const CoarseSolver& cs = c->coarse;
  out[0] = cs.lmin;
  out[1] = cs.lmax;
  out[2] = cs.ritzMin;
  out[3] = cs.ritzMax;
  out[4] = cs.rowBound;
  return HFX_OK;
}

int hfx_coarse_train(hfx_ctx* c, int degree, int samples, int steps, hfx_train_info* info) {
  if (!c) return HFX_ERR_ARG;
  if (degree < 1 || degree > 16 || samples < 1 || samples > 32 || steps < 0)
    return set_err(c, HFX_ERR_ARG, "coarse_train: degree 1..16, samples 1..32, steps >= 0");
  if (!c->assembled || c->mixedMode)
    return set_err(c, HFX_ERR_STATE, "coarse_train: needs a trace system assembled in FP64");
  if (!c->kappaCellConstant)
    return set_err(c, HFX_ERR_UNSUPPORTED, "coarse_train: the two-level preconditioner needs a symmetric system");
  cudaSetDevice(c->device);
  auto t0 = std::chrono::steady_clock::now();
  int rc = ensure_workspace(c, false, 0);
  if (rc) return rc;
  if ((rc = ensure_coarse(c, c->coarseTarget > 0.0 ? c->coarseTarget : 0.1, c->coarseMaxDeg))) return rc;
  c->learnDegree = degree;
  const int64_t nV = c->coarse.dev.nV;
  float* buf = nullptr;
  HFX_CUDA(c, cudaMalloc(&buf, sizeof(float) * (size_t)samples * nV));
  // samples: the coarse residuals of a two-level CG run on this system (Chebyshev coarse solve)
  TraceSolveArgs a{};
  a.dim = c->dim;
  a.A = TraceView{c->topo.nFaces, c->re.nNodesFace, c->d_browptr, c->d_bcol, c->d_isBnd};
  a.val = c->d_val;
  a.rhs = c->d_rhs;
  a.x = c->d_trace;
  a.precond = HFX_PC_TWOLEVEL;
  a.mixed = 0;
  a.rtol = 1e-300;
  a.maxits = 2 * samples;
  a.check_every = 25;
  a.ws = c->ws;
  a.stream = c->stream;
  a.timer = &c->timer;
  a.coarse = &c->coarse;
  a.sampleBuf = buf;
  a.sampleCap = samples;
  a.sampleStride = 2;
  int taken = 0;
  a.sampleCount = &taken;
  c->coarse.useLearned = false;
  TraceSolveResult res;
  int st = trace_solve(a, &res);
  c->solved = false;
  if (st == 3) {
    cudaFree(buf);
    return cuda_err(c, res.cudaErr, "coarse_train samples");
  }
  const int S = std::min(taken, samples);
  CoarseTrainResult tr;
  cudaError_t e = coarse_train(&c->coarse, buf, S, degree, steps, 0.05, c->stream, &tr);
  if (e == cudaSuccess && !tr.accepted && steps > 0) {
    // no accepted improvement (every lower-loss step left the residual polynomial above 1):
    // one more round from Chebyshev that keeps each step inside that bound; a rejected
    // round leaves the coarse solve as it was
    CoarseTrainResult tr2;
    e = coarse_train(&c->coarse, buf, S, degree, steps, 0.05, c->stream, &tr2, true);
    if (e == cudaSuccess) {
      tr2.lowerSteps += tr.lowerSteps;
      tr2.rejectedSteps += tr.rejectedSteps;
      tr = tr2;
    }
  }
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_err(c, e, "coarse_train");
  if (info) {
    info->degree = tr.degree;
    info->samples = S;
    info->steps = tr.steps;
    info->accepted = tr.accepted;
    info->loss_chebyshev = tr.lossChebyshev;
    info->loss_learned = tr.lossLearned;
    info->max_poly = tr.maxGain;
    info->train_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    info->loss_first_step = tr.lossFirstStep;
    info->lower_steps = tr.lowerSteps;
    info->rejected_steps = tr.rejectedSteps;
  }
  return HFX_OK;
}

int hfx_coarse_loss_grad(hfx_ctx* c, int degree, const double* theta, int samples, const float* values, double* loss,
                         double* grad) {
  if (!c || !theta || !values || !loss || !grad || degree < 1 || degree > 16 || samples < 1) return HFX_ERR_ARG;
  if (!c->assembled || c->mixedMode)
    return set_err(c, HFX_ERR_STATE, "coarse_loss_grad: needs a trace system assembled in FP64");
  cudaSetDevice(c->device);
  int rc = ensure_coarse(c, c->coarseTarget > 0.0 ? c->coarseTarget : 0.1, c->coarseMaxDeg);
  if (rc) return rc;
  const int64_t nV = c->coarse.dev.nV;
  float* buf = nullptr;
  HFX_CUDA(c, cudaMalloc(&buf, sizeof(float) * (size_t)samples * nV));
  cudaError_t e = cudaMemcpy(buf, values, sizeof(float) * (size_t)samples * nV, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = coarse_loss_grad(c->coarse, buf, samples, degree, theta, loss, grad, c->stream);
  cudaFree(buf);
  if (e != cudaSuccess) return cuda_err(c, e, "coarse_loss_grad");
  return HFX_OK;
}

int hfx_recover(hfx_ctx* c, double* solution, double* flux) {
  if (!c) return HFX_ERR_ARG;
  if (!c->solved) return set_err(c, HFX_ERR_STATE, "recover: solve first");
  cudaSetDevice(c->device);
  const int LU = c->re.nNodes, LQ = c->dim * c->re.nNodes, LL = c->re.nFaces * c->re.nNodesFace;
  const int64_t E = c->nCells;
  if (!c->mixedMode) {  // mixed mode: Solution and Flux are the refined FP64 state
    RecoverParams p{c->nCells, c->re.nFaces, c->re.nNodesFace, LU, LQ, LL, c->d_cell2face, c->d_perm,
                    c->d_U, c->d_Q, c->d_U0, c->d_Q0, c->d_trace, c->d_sol, c->d_flux};
    c->timer.begin(K_RECOVER, c->stream);
    if (c->lastAffine) HFX_CUDA(c, launch_recover_affine(c->dim, c->order, p, c->d_atab, c->d_geo, c->stream));
    else HFX_CUDA(c, launch_recover(p, c->stream));
    c->timer.end(K_RECOVER, c->stream);
  }
  // NULL outputs keep Solution and Flux on the device only
  if (solution) HFX_CUDA(c, cudaMemcpyAsync(solution, c->d_sol, sizeof(double) * E * LU, cudaMemcpyDeviceToHost, c->stream));
  if (flux) HFX_CUDA(c, cudaMemcpyAsync(flux, c->d_flux, sizeof(double) * E * LQ, cudaMemcpyDeviceToHost, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

int hfx_profile_enable(hfx_ctx* c, int on) {
  if (!c) return HFX_ERR_ARG;
  cudaStreamSynchronize(c->stream);
  c->timer.reset();
  c->timer.enable(on != 0);
  return HFX_OK;
}

int hfx_kernel_time(hfx_ctx* c, int kernel, int* launches, double* ms) {
  if (!c || !launches || !ms || kernel < 0 || kernel >= K_COUNT) return HFX_ERR_ARG;
  c->timer.read(kernel, launches, ms);
  return HFX_OK;
}

int hfx_mark(hfx_ctx* c, int slot) {
  if (!c || slot < 0 || slot >= 8) return HFX_ERR_ARG;
  if (!c->marks[slot]) HFX_CUDA(c, cudaEventCreate(&c->marks[slot]));
  HFX_CUDA(c, cudaEventRecord(c->marks[slot], c->stream));
  return HFX_OK;
}

int hfx_elapsed_ms(hfx_ctx* c, int slot0, int slot1, double* ms) {
  if (!c || !ms || slot0 < 0 || slot0 >= 8 || slot1 < 0 || slot1 >= 8 || !c->marks[slot0] || !c->marks[slot1])
    return HFX_ERR_ARG;
  HFX_CUDA(c, cudaEventSynchronize(c->marks[slot1]));
  float x = 0.f;
  HFX_CUDA(c, cudaEventElapsedTime(&x, c->marks[slot0], c->marks[slot1]));
  *ms = x;
  return HFX_OK;
}

int hfx_elapsed_between(hfx_ctx* c0, int slot0, hfx_ctx* c1, int slot1, double* ms) {
  if (!c0 || !c1 || !ms || slot0 < 0 || slot0 >= 8 || slot1 < 0 || slot1 >= 8 || !c0->marks[slot0] ||
      !c1->marks[slot1] || c0->device != c1->device)
    return HFX_ERR_ARG;
  HFX_CUDA(c0, cudaEventSynchronize(c0->marks[slot0]));
  HFX_CUDA(c1, cudaEventSynchronize(c1->marks[slot1]));
  float x = 0.f;
  HFX_CUDA(c1, cudaEventElapsedTime(&x, c0->marks[slot0], c1->marks[slot1]));
  *ms = x;
  return HFX_OK;
}

int hfx_synchronize(hfx_ctx* c) {
  if (!c) return HFX_ERR_ARG;
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

// ---- generic sparse system --------------------------------------------------
int hfx_la_create(hfx_ctx* c, hfx_la** out) {
  if (!c || !out) return HFX_ERR_ARG;
  *out = new hfx_la{c, LaSystem()};
  return HFX_OK;
}

int hfx_la_destroy(hfx_la* la) {
  delete la;
  return HFX_OK;
}

int hfx_la_allocate(hfx_la* la, int ndofs) {
  if (!la) return HFX_ERR_ARG;
  if (ndofs <= 0) return set_err(la->ctx, HFX_ERR_ARG, "la_allocate: ndofs must be positive");
  la->sys.allocate(ndofs);
  return HFX_OK;
}

int hfx_la_set_values(hfx_la* la, int nr, const int* rows, int nc, const int* cols, const double* vals, int insert) {
  if (!la) return HFX_ERR_ARG;
  if (!la->sys.allocated()) return set_err(la->ctx, HFX_ERR_STATE, "la_set_values: allocate first");
  std::string err;
  if (!la->sys.add_block(nr, rows, nc, cols, vals, insert != 0, &err)) return set_err(la->ctx, HFX_ERR_ARG, err);
  return HFX_OK;
}

int hfx_la_set_rhs(hfx_la* la, int n, const int* idx, const double* vals, int insert) {
  if (!la) return HFX_ERR_ARG;
  if (!la->sys.allocated()) return set_err(la->ctx, HFX_ERR_STATE, "la_set_rhs: allocate first");
  std::string err;
  if (!la->sys.add_rhs(n, idx, vals, insert != 0, &err)) return set_err(la->ctx, HFX_ERR_ARG, err);
  return HFX_OK;
}

int hfx_la_zero_rows(hfx_la* la, int n, const int* rows) {
  if (!la) return HFX_ERR_ARG;
  if (!la->sys.allocated()) return set_err(la->ctx, HFX_ERR_STATE, "la_zero_rows: allocate first");
  std::string err;
  if (!la->sys.zero_rows(n, rows, &err)) return set_err(la->ctx, HFX_ERR_ARG, err);
  return HFX_OK;
}

int hfx_la_assemble(hfx_la* la) {
  if (!la) return HFX_ERR_ARG;
  if (!la->sys.allocated()) return set_err(la->ctx, HFX_ERR_STATE, "la_assemble: allocate first");
  la->sys.assemble();
  return HFX_OK;
}

int hfx_la_clear(hfx_la* la) {
  if (!la) return HFX_ERR_ARG;
  if (!la->sys.assembled()) return set_err(la->ctx, HFX_ERR_STATE, "la_clear: assemble at least once first");
  la->sys.clear();
  return HFX_OK;
}

int hfx_la_nnz(hfx_la* la, int64_t* nnz) {
  if (!la || !nnz) return HFX_ERR_ARG;
  *nnz = la->sys.nnz();
  return HFX_OK;
}

int hfx_la_solve(hfx_la* la, const hfx_solve_opts* opts, double* x, hfx_solve_info* info) {
  if (!la || !x) return HFX_ERR_ARG;
  if (!la->sys.assembled()) return set_err(la->ctx, HFX_ERR_STATE, "la_solve: assemble before solving");
  hfx_solve_opts o;
  if (opts) o = *opts;
  else {
    hfx_solve_opts_default(&o);
    o.method = HFX_KSP_GMRES;
    o.precond = HFX_PC_JACOBI;
  }
  cudaSetDevice(la->ctx->device);
  LaSolveResult r;
  std::string err;
  int st = la->sys.solve(o.rtol, o.maxits, o.restart > 0 ? o.restart : 30, o.precond == HFX_PC_NONE ? 0 : 1,
                         la->ctx->stream, x, &r, &err);
  if (info) {
    info->status = st;
    info->iterations = r.iterations;
    info->refinements = 0;
    info->rel_residual = r.rel_residual;
    info->solve_ms = r.ms;
    info->fallback = 0;
    info->coarse_degree = 0;
    info->coarse_learned = 0;
  }
  if (st != 0) return set_err(la->ctx, st, err);
  return HFX_OK;
}

// ---------------------------------------------------------------- Burgers
// HDGSolver with HDGBurgersModel and NonLinearWrapper (HDGSolver.cpp:81-175,677-779,
// HDGBurgersModel.cpp:35-125, NonLinearWrapper.cpp:41-79): nd = dim unknowns per node.
// The trace system is the scalar path's face-block pattern with Nf*nd x Nf*nd blocks:
// the global DOF (face*Nf + node)*nd + k is face*(Nf*nd) + (node*nd + k).

static int burgers_ready(hfx_ctx* c, const char* who) {
  if (!c) return HFX_ERR_ARG;
  if (!c->burgers.ready) return set_err(c, HFX_ERR_STATE, std::string(who) + ": call hfx_burgers_setup first");
  cudaSetDevice(c->device);
  return HFX_OK;
}

int hfx_burgers_setup(hfx_ctx* c) {
  if (!c) return HFX_ERR_ARG;
  if (!c->haveMesh) return set_err(c, HFX_ERR_STATE, "burgers_setup: upload a mesh first");
  if (!burgers_supported(c->dim, c->order))
    return set_err(c, HFX_ERR_UNSUPPORTED, "burgers_setup: the Burgers element kernel is built for 2D cells, p <= 5");
  cudaSetDevice(c->device);
  BurgersState& B = c->burgers;
  B.release();
  const int nd = c->dim, N = c->re.nNodes, F = c->re.nFaces, Nf = c->re.nNodesFace;
  B.nd = nd;
  B.NLF = Nf * nd;
  B.NU = N * nd;
  B.NQ = c->dim * N * nd;
  B.NL = F * Nf * nd;
  B.nDofs = (int64_t)c->topo.nFaces * B.NLF;
  B.nnz = (int64_t)c->bp.col.size() * B.NLF * B.NLF;
  if (B.NLF > 16) return set_err(c, HFX_ERR_UNSUPPORTED, "burgers_setup: more than 16 trace values per face");
  const int64_t E = c->nCells;
  cudaStream_t s = c->stream;
  DevMem& m = B.mem;
  HFX_CUDA(c, dalloc(m, &B.buf, (size_t)E * B.NU));
  HFX_CUDA(c, dalloc(m, &B.sol, (size_t)E * B.NU));
  HFX_CUDA(c, dalloc(m, &B.old, (size_t)E * B.NU));
  HFX_CUDA(c, dalloc(m, &B.flux, (size_t)E * B.NQ));
  HFX_CUDA(c, dalloc(m, &B.trace, (size_t)B.nDofs));
  HFX_CUDA(c, dalloc(m, &B.S, (size_t)E * B.NL * B.NL));
  HFX_CUDA(c, dalloc(m, &B.S0, (size_t)E * B.NL));
  HFX_CUDA(c, dalloc(m, &B.U, (size_t)E * B.NU * B.NL));
  HFX_CUDA(c, dalloc(m, &B.Q, (size_t)E * B.NQ * B.NL));
  HFX_CUDA(c, dalloc(m, &B.U0, (size_t)E * B.NU));
  HFX_CUDA(c, dalloc(m, &B.Q0, (size_t)E * B.NQ));
  HFX_CUDA(c, dalloc(m, &B.val, (size_t)B.nnz));
  HFX_CUDA(c, dalloc(m, &B.rhs, (size_t)B.nDofs));
  HFX_CUDA(c, dalloc(m, &B.partials, newton_partials_needed()));
  HFX_CUDA(c, dalloc(m, &B.red, 2));
  HFX_CUDA(c, dalloc(m, &B.status, 1));
  HFX_CUDA(c, dalloc(m, &B.ticket, 1));
  HFX_CUDA(c, dalloc(m, &B.cache, (size_t)E * burgers_cache_doubles(c->dim, c->order)));
  B.cacheValid = false;
  HFX_CUDA(c, cudaMemsetAsync(B.ticket, 0, sizeof(unsigned), s));
  for (double* p : {B.buf, B.sol, B.old})
    HFX_CUDA(c, cudaMemsetAsync(p, 0, sizeof(double) * E * B.NU, s));
  HFX_CUDA(c, cudaMemsetAsync(B.flux, 0, sizeof(double) * E * B.NQ, s));
  HFX_CUDA(c, cudaMemsetAsync(B.trace, 0, sizeof(double) * B.nDofs, s));
  std::vector<uint8_t> px((size_t)E * F * B.NLF);
  for (int64_t e = 0; e < E; ++e)
    for (int f = 0; f < F; ++f)
      for (int a = 0; a < Nf; ++a)
        for (int k = 0; k < nd; ++k)
          px[((size_t)e * F + f) * B.NLF + a * nd + k] = (uint8_t)(c->perm[((size_t)e * F + f) * Nf + a] * nd + k);
  HFX_CUDA(c, upload(m, &B.permx, px.data(), px.size(), s));
  std::vector<double> tau((size_t)c->topo.nFaces * Nf * nd * nd, 0.0);
  for (size_t k = 0; k < (size_t)c->topo.nFaces * Nf; ++k)
    for (int q = 0; q < nd; ++q) tau[k * nd * nd + q * nd + q] = 1.0;
  HFX_CUDA(c, B.tau.set(tau.data(), tau.size(), s));
  std::vector<double> zeros((size_t)B.nDofs, 0.0);
  HFX_CUDA(c, B.dir.set(zeros.data(), zeros.size(), s));
  B.tauSides = 1;
  B.kc = 0;
  B.haveSrc = false;
  B.dt = 0.0;
  HFX_CUDA(c, cudaStreamSynchronize(s));
  B.ready = true;
  return HFX_OK;
}

int hfx_burgers_set_tau(hfx_ctx* c, const double* tau, int sides) {
  if (int rc = burgers_ready(c, "burgers_set_tau")) return rc;
  if (!tau || (sides != 1 && sides != 2)) return set_err(c, HFX_ERR_ARG, "burgers_set_tau: tau and sides 1 or 2");
  BurgersState& B = c->burgers;
  B.tauSides = sides;
  B.cacheValid = false;
  HFX_CUDA(c, B.tau.set(tau, (size_t)c->topo.nFaces * c->re.nNodesFace * sides * B.nd * B.nd, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

int hfx_burgers_set_diffusion(hfx_ctx* c, const double* nu, int comps, int layout) {
  if (int rc = burgers_ready(c, "burgers_set_diffusion")) return rc;
  BurgersState& B = c->burgers;
  B.cacheValid = false;
  if (!nu || comps == 0) {
    B.kc = 0;
    return HFX_OK;
  }
  if ((comps != 1 && comps != c->dim * c->dim) || (layout != 0 && layout != 1))
    return set_err(c, HFX_ERR_ARG, "burgers_set_diffusion: comps 1 or dim*dim, layout 0 (mesh nodes) or 1 (cell nodes)");
  const size_t n = (size_t)(layout == 0 ? c->nNodes : (int64_t)c->nCells * c->re.nNodes) * comps;
  HFX_CUDA(c, B.nu.set(nu, n, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  B.kc = comps;
  B.nuLayout = layout;
  return HFX_OK;
}

int hfx_burgers_set_source(hfx_ctx* c, const double* values) {
  if (int rc = burgers_ready(c, "burgers_set_source")) return rc;
  BurgersState& B = c->burgers;
  B.haveSrc = values != nullptr;
  if (values) {
    HFX_CUDA(c, B.src.set(values, (size_t)c->nCells * c->re.nIP * B.nd, c->stream));
    HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  return HFX_OK;
}

int hfx_burgers_set_dirichlet(hfx_ctx* c, const double* values) {
  if (int rc = burgers_ready(c, "burgers_set_dirichlet")) return rc;
  if (!values) return set_err(c, HFX_ERR_ARG, "burgers_set_dirichlet: values");
  HFX_CUDA(c, c->burgers.dir.set(values, (size_t)c->burgers.nDofs, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  return HFX_OK;
}

int hfx_burgers_set_time_step(hfx_ctx* c, double dt) {
  if (int rc = burgers_ready(c, "burgers_set_time_step")) return rc;
  if (!(dt >= 0.0)) return set_err(c, HFX_ERR_ARG, "burgers_set_time_step: dt >= 0");
  c->burgers.dt = dt;
  return HFX_OK;
}

int hfx_burgers_set_state(hfx_ctx* c, const double* solution, const double* buffer, const double* trace,
                          const double* oldSolution) {
  if (int rc = burgers_ready(c, "burgers_set_state")) return rc;
  BurgersState& B = c->burgers;
  const size_t nu = (size_t)c->nCells * B.NU;
  cudaStream_t s = c->stream;
  if (solution) HFX_CUDA(c, cudaMemcpyAsync(B.sol, solution, sizeof(double) * nu, cudaMemcpyHostToDevice, s));
  if (buffer) HFX_CUDA(c, cudaMemcpyAsync(B.buf, buffer, sizeof(double) * nu, cudaMemcpyHostToDevice, s));
  if (oldSolution) HFX_CUDA(c, cudaMemcpyAsync(B.old, oldSolution, sizeof(double) * nu, cudaMemcpyHostToDevice, s));
  if (trace) {
    HFX_CUDA(c, cudaMemcpyAsync(B.trace, trace, sizeof(double) * B.nDofs, cudaMemcpyHostToDevice, s));
    B.histCount = 0;  // a new trace: the earlier solutions may no longer span it
  }
  HFX_CUDA(c, cudaStreamSynchronize(s));
  return HFX_OK;
}

int hfx_burgers_get_state(hfx_ctx* c, double* solution, double* flux, double* trace, double* buffer) {
  if (int rc = burgers_ready(c, "burgers_get_state")) return rc;
  BurgersState& B = c->burgers;
  const size_t nu = (size_t)c->nCells * B.NU;
  cudaStream_t s = c->stream;
  if (solution) HFX_CUDA(c, cudaMemcpyAsync(solution, B.sol, sizeof(double) * nu, cudaMemcpyDeviceToHost, s));
  if (flux)
    HFX_CUDA(c, cudaMemcpyAsync(flux, B.flux, sizeof(double) * c->nCells * B.NQ, cudaMemcpyDeviceToHost, s));
  if (trace) HFX_CUDA(c, cudaMemcpyAsync(trace, B.trace, sizeof(double) * B.nDofs, cudaMemcpyDeviceToHost, s));
  if (buffer) HFX_CUDA(c, cudaMemcpyAsync(buffer, B.buf, sizeof(double) * nu, cudaMemcpyDeviceToHost, s));
  HFX_CUDA(c, cudaStreamSynchronize(s));
  return HFX_OK;
}

int hfx_burgers_begin_step(hfx_ctx* c) {
  if (int rc = burgers_ready(c, "burgers_begin_step")) return rc;
  BurgersState& B = c->burgers;
  const size_t nu = (size_t)c->nCells * B.NU;
  HFX_CUDA(c, cudaMemcpyAsync(B.buf, B.sol, sizeof(double) * nu, cudaMemcpyDeviceToDevice, c->stream));
  HFX_CUDA(c, cudaMemcpyAsync(B.old, B.sol, sizeof(double) * nu, cudaMemcpyDeviceToDevice, c->stream));
  return HFX_OK;
}

// Element kernel + scatter, queued on the stream; *status is read by the caller.
static int burgers_assemble_async(hfx_ctx* c) {
  BurgersState& B = c->burgers;
  cudaStream_t s = c->stream;
  BurgersParams p{};
  p.nCells = c->nCells;
  p.coords = c->d_coords;
  p.cells = c->d_cells;
  p.cell2face = c->d_cell2face;
  p.perm = c->d_perm;
  p.face2cell = c->d_face2cell;
  p.isBoundary = c->d_isBnd;
  p.tau = B.tau.p;
  p.tauSides = B.tauSides;
  p.nu = B.kc ? B.nu.p : nullptr;
  p.kc = B.kc;
  p.nuLayout = B.nuLayout;
  p.src = B.haveSrc ? B.src.p : nullptr;
  p.dirichlet = B.dir.p;
  p.dt = B.dt;
  p.uOld = B.old;
  p.buf = B.buf;
  p.trace = B.trace;
  p.tab = c->d_tab;
  p.itab = c->d_itab;
  p.S = B.S;
  p.S0 = B.S0;
  p.U = B.U;
  p.U0 = B.U0;
  p.status = B.status;
  p.cache = B.cache;
  p.cacheMode = B.cacheValid ? 2 : 1;
  HFX_CUDA(c, cudaMemsetAsync(B.status, 0, sizeof(int), s));
  c->timer.begin(K_LOCAL, s);
  HFX_CUDA(c, launch_burgers_local(c->dim, c->order, p, s));
  c->timer.end(K_LOCAL, s);
  B.cacheValid = true;  // every element stores its blocks before its Schur solve
  ScatterParams sp{};
  sp.nFaces = c->topo.nFaces;
  sp.NF = B.NLF;
  sp.LL = B.NL;
  sp.browptr = c->d_browptr;
  sp.brow = c->d_brow;
  sp.nBlocks = (int64_t)c->bp.col.size();
  sp.src0 = c->d_src0;
  sp.src1 = c->d_src1;
  sp.loc0 = c->d_loc0;
  sp.loc1 = c->d_loc1;
  sp.perm = B.permx;
  sp.S = B.S;
  sp.S0 = B.S0;
  sp.cell2face = c->d_cell2face;
  sp.face2cell = c->d_face2cell;
  sp.F = c->re.nFaces;
  sp.val = B.val;
  sp.rhs = B.rhs;
  c->timer.begin(K_SCATTER, s);
  HFX_CUDA(c, launch_scatter(sp, s));
  c->timer.end(K_SCATTER, s);
  return HFX_OK;
}

int hfx_burgers_assemble(hfx_ctx* c) {
  if (int rc = burgers_ready(c, "burgers_assemble")) return rc;
  BurgersState& B = c->burgers;
  if (int rc = burgers_assemble_async(c)) return rc;
  int status = 0;
  HFX_CUDA(c, cudaMemcpyAsync(&status, B.status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  HFX_CUDA(c, cudaStreamSynchronize(c->stream));
  if (status) return set_err(c, HFX_ERR_SINGULAR, "burgers_assemble: singular Schur block in condensation");
  B.assembled = true;
  B.solved = false;
  return HFX_OK;
}

static int burgers_check_opts(hfx_ctx* c, const hfx_solve_opts& o) {
  if (o.method == HFX_KSP_CG)
    return set_err(c, HFX_ERR_ARG, "burgers_solve: the Burgers trace system is not symmetric (use GMRES)");
  if (o.precision != HFX_PREC_FP64 && o.precision != HFX_PREC_MIXED)
    return set_err(c, HFX_ERR_ARG, "burgers_solve: precision is HFX_PREC_FP64 or HFX_PREC_MIXED");
  if (o.precond < HFX_PC_NONE || o.precond > HFX_PC_BLOCK_JACOBI || o.rtol <= 0.0 || o.maxits <= 0)
    return set_err(c, HFX_ERR_ARG, "burgers_solve: precond none / Jacobi / block Jacobi, rtol > 0, maxits > 0");
  return HFX_OK;
}

// GMRES + recovery, queued on the stream; returns the Krylov status. history > 0: the
// initial guess is the least-squares fit of the last `history` solutions (then the
// solution joins them).
static int burgers_solve_core(hfx_ctx* c, const hfx_solve_opts& o, TraceSolveResult* res, int* kst,
                              int history = 0) {
  BurgersState& B = c->burgers;
  const int restart = o.restart > 0 ? o.restart : 30;
  DevMem& m = B.wsMem;
  TraceWorkspace& w = B.ws;
  const size_t n = (size_t)B.nDofs;
  if (restart > B.wsRestart) {
    HFX_CUDA(c, dalloc(m, &w.V64, n * (restart + 1)));
    HFX_CUDA(c, dalloc(m, &w.hdev, (size_t)restart + 1));
    B.wsRestart = restart;
  }
  if (!B.wsReady) {
    HFX_CUDA(c, dalloc(m, &w.bS, n));
    HFX_CUDA(c, dalloc(m, &w.r, n));
    HFX_CUDA(c, dalloc(m, &w.z, n));
    HFX_CUDA(c, dalloc(m, &w.q, n));
    HFX_CUDA(c, dalloc(m, &w.p0, n));
    HFX_CUDA(c, dalloc(m, &w.pc64, (size_t)c->topo.nFaces * B.NLF * B.NLF));
    HFX_CUDA(c, dalloc(m, &w.partials, trace_partials_needed()));
    HFX_CUDA(c, dalloc(m, &w.state, 1));
    B.wsReady = true;
  }
  // mixed precision: FP32 GMRES on an FP32 copy of the system inside FP64 residual refinement
  const bool mixed = o.precision == HFX_PREC_MIXED;
  if (mixed && !B.wsMixed) {
    HFX_CUDA(c, dalloc(m, &w.val32, (size_t)B.nnz));
    HFX_CUDA(c, dalloc(m, &w.pc32, (size_t)c->topo.nFaces * B.NLF * B.NLF));
    HFX_CUDA(c, dalloc(m, &w.rhs32, n));
    HFX_CUDA(c, dalloc(m, &w.d32, n));
    HFX_CUDA(c, dalloc(m, &w.q32, n));
    HFX_CUDA(c, dalloc(m, &w.p032, n));
    B.wsMixed = true;
  }
  if (mixed && restart > B.wsRestart32) {
    HFX_CUDA(c, dalloc(m, &w.V32, n * (restart + 1)));
    B.wsRestart32 = restart;
  }
  TraceSolveArgs a{};
  a.dim = c->dim;
  a.A = TraceView{c->topo.nFaces, B.NLF, c->d_browptr, c->d_bcol, c->d_isBnd};
  a.val = B.val;
  a.rhs = B.rhs;
  a.x = B.trace;
  a.precond = o.precond;
  a.mixed = mixed ? 1 : 0;
  a.rtol = o.rtol;
  // FP32 GMRES reduces the residual by inner_rtol (FP32 keeps about 1e-6 of it) between the
  // FP64 residual replacements
  a.inner_rtol = mixed ? std::min(std::max(o.inner_rtol, 1e-5), 0.5) : 1e-2;
  a.maxits = o.maxits;
  a.max_refinements = mixed ? 100 : 1;
  a.check_every = 25;
  a.use_initial_guess = o.use_initial_guess;
  a.ws = B.ws;
  a.stream = c->stream;
  a.timer = &c->timer;
  a.restart = restart;
  if (history > 0) {
    if (B.histCap < history) {
      HFX_CUDA(c, dalloc(m, &B.hist, n * (size_t)history));
      HFX_CUDA(c, dalloc(m, &B.histY, n * (size_t)history));
      B.histCap = history;
      B.histCount = B.histHead = 0;
    }
    const int cnt = std::min(B.histCount, history);
    if (cnt > 0) {
      trace_prepare(a);
      a.prepared = 1;
      const double* X[8];
      for (int i = 0; i < cnt; ++i) X[i] = B.hist + (size_t)((B.histHead - 1 - i + B.histCap) % B.histCap) * n;
      if (trace_projection_guess(a, X, cnt, B.histY) > 0) a.use_initial_guess = 1;
    }
  }
  *kst = trace_gmres(a, res);
  if (*kst == 3) return cuda_err(c, res->cudaErr, "burgers_solve");
  if (history > 0 && *kst == 0) {
    HFX_CUDA(c, cudaMemcpyAsync(B.hist + (size_t)B.histHead * n, B.trace, sizeof(double) * n,
                                cudaMemcpyDeviceToDevice, c->stream));
    B.histHead = (B.histHead + 1) % B.histCap;
    B.histCount = std::min(B.histCount + 1, B.histCap);
  }
  BurgersRecoverParams rp{c->nCells, c->d_cell2face, B.permx, B.U, B.U0, B.cache, B.trace, B.sol, B.flux};
  c->timer.begin(K_RECOVER, c->stream);
  HFX_CUDA(c, launch_burgers_recover(c->dim, c->order, rp, c->stream));
  c->timer.end(K_RECOVER, c->stream);
  return HFX_OK;
}

static int burgers_krylov_err(hfx_ctx* c, int st) {
  if (st == HFX_ERR_NOT_CONVERGED) return set_err(c, st, "burgers_solve: GMRES not converged within maxits");
  if (st == HFX_ERR_BREAKDOWN) return set_err(c, st, "burgers_solve: GMRES breakdown");
  if (st == HFX_ERR_NAN) return set_err(c, st, "burgers_solve: NaN or Inf in GMRES");
  if (st == HFX_ERR_UNSUPPORTED) return set_err(c, st, "burgers_solve: trace block size not built into GMRES");
  return set_err(c, st, "burgers_solve: failed");
}

int hfx_burgers_solve(hfx_ctx* c, const hfx_solve_opts* opts, hfx_solve_info* info) {
  if (int rc = burgers_ready(c, "burgers_solve")) return rc;
  BurgersState& B = c->burgers;
  if (!B.assembled) return set_err(c, HFX_ERR_STATE, "burgers_solve: assemble first");
  hfx_solve_opts o;
  if (opts) o = *opts;
  else {
    hfx_solve_opts_default(&o);
    o.method = HFX_KSP_GMRES;
  }
  if (int rc = burgers_check_opts(c, o)) return rc;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, c->stream);
  TraceSolveResult res;
  int st = 0;
  int rc = burgers_solve_core(c, o, &res, &st);
  cudaEventRecord(e1, c->stream);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  if (info) {
    *info = hfx_solve_info{};
    info->status = st;
    info->iterations = res.iterations;
    info->rel_residual = res.rel_residual;
    info->solve_ms = ms;
  }
  B.solved = true;
  if (st != 0) return burgers_krylov_err(c, st);
  return HFX_OK;
}

void hfx_newton_opts_default(hfx_newton_opts* o) {
  if (!o) return;
  o->res_tol = 1e-6;
  o->max_iters = 20;
  o->dampening = 0.0;
  hfx_solve_opts_default(&o->lin);
  o->lin.method = HFX_KSP_GMRES;
  o->lin.rtol = 1e-12;
  o->warm_start = 0;
  o->history = 0;
}

int hfx_burgers_newton(hfx_ctx* c, const hfx_newton_opts* opts, hfx_newton_info* info) {
  if (int rc = burgers_ready(c, "burgers_newton")) return rc;
  BurgersState& B = c->burgers;
  hfx_newton_opts o;
  if (opts) o = *opts;
  else hfx_newton_opts_default(&o);
  if (!(o.res_tol > 0.0) || o.max_iters <= 0 || !(o.dampening >= 0.0 && o.dampening < 1.0) || o.history < 0 ||
      o.history > 8)
    return set_err(c, HFX_ERR_ARG,
                   "burgers_newton: res_tol > 0, max_iters > 0, 0 <= dampening < 1, 0 <= history <= 8");
  if (int rc = burgers_check_opts(c, o.lin)) return rc;
  hfx_solve_opts lin = o.lin;
  lin.use_initial_guess = o.warm_start ? 1 : 0;
  cudaStream_t s = c->stream;
  const int64_t nu = (int64_t)c->nCells * B.NU;
  cudaEvent_t ev[4];
  for (auto& e : ev) cudaEventCreate(&e);
  hfx_newton_info out{};
  int rc = HFX_OK;
  for (int it = 0; it < o.max_iters; ++it) {
    cudaEventRecord(ev[0], s);
    if ((rc = burgers_assemble_async(c))) break;
    cudaEventRecord(ev[1], s);
    TraceSolveResult res;
    int st = 0;
    if ((rc = burgers_solve_core(c, lin, &res, &st, o.history))) break;
    cudaEventRecord(ev[2], s);
    if (cudaError_t e = launch_newton_residual(nu, B.sol, B.buf, B.partials, B.ticket, B.red, s)) {
      rc = cuda_err(c, e, "burgers_newton: residual");
      break;
    }
    double red[2] = {0.0, 0.0};
    int kstatus = 0;
    cudaMemcpyAsync(red, B.red, sizeof(red), cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(&kstatus, B.status, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaEventRecord(ev[3], s);
    if (cudaError_t e = cudaStreamSynchronize(s)) {
      rc = cuda_err(c, e, "burgers_newton");
      break;
    }
    float ta = 0.f, ts = 0.f;
    cudaEventElapsedTime(&ta, ev[0], ev[1]);
    cudaEventElapsedTime(&ts, ev[1], ev[2]);
    out.assemble_ms += ta;
    out.solve_ms += ts;
    out.krylov_iterations += res.iterations;
    out.iterations = it + 1;
    if (kstatus) {
      rc = set_err(c, HFX_ERR_SINGULAR, "burgers_newton: singular Schur block in condensation");
      break;
    }
    if (st != 0) {
      rc = burgers_krylov_err(c, st);
      break;
    }
    out.residual = red[1] != 0.0 ? std::sqrt(red[0] / red[1]) : std::sqrt(red[0]);
    if (out.residual < o.res_tol) break;
    if (cudaError_t e = launch_newton_update(nu, o.dampening, B.sol, B.buf, s)) {
      rc = cuda_err(c, e, "burgers_newton: update");
      break;
    }
  }
  for (auto& e : ev) cudaEventDestroy(e);
  out.status = rc;
  B.assembled = true;
  B.solved = rc == HFX_OK;
  if (info) *info = out;
  return rc;
}

int hfx_burgers_get_condensed(hfx_ctx* c, double* S, double* S0, double* U, double* Q, double* U0, double* Q0) {
  if (int rc = burgers_ready(c, "burgers_get_condensed")) return rc;
  BurgersState& B = c->burgers;
  if (!B.assembled) return set_err(c, HFX_ERR_STATE, "burgers_get_condensed: assemble first");
  const size_t E = (size_t)c->nCells;
  cudaStream_t s = c->stream;
  auto cp = [&](double* h, const double* d, size_t n) {
    return h ? cudaMemcpyAsync(h, d, sizeof(double) * n, cudaMemcpyDeviceToHost, s) : cudaSuccess;
  };
  if (Q || Q0)  // the element kernel does not store Q: form it from U, U0 and the cache
    HFX_CUDA(c, launch_burgers_q(c->dim, c->order, (int64_t)E, B.U, B.U0, B.cache, B.Q, B.Q0, s));
  HFX_CUDA(c, cp(S, B.S, E * B.NL * B.NL));
  HFX_CUDA(c, cp(S0, B.S0, E * B.NL));
  HFX_CUDA(c, cp(U, B.U, E * B.NU * B.NL));
  HFX_CUDA(c, cp(Q, B.Q, E * B.NQ * B.NL));
  HFX_CUDA(c, cp(U0, B.U0, E * B.NU));
  HFX_CUDA(c, cp(Q0, B.Q0, E * B.NQ));
  HFX_CUDA(c, cudaStreamSynchronize(s));
  return HFX_OK;
}

int hfx_burgers_nnz(hfx_ctx* c, int64_t* nnz) {
  if (int rc = burgers_ready(c, "burgers_nnz")) return rc;
  if (!nnz) return set_err(c, HFX_ERR_ARG, "burgers_nnz: nnz");
  *nnz = c->burgers.nnz;
  return HFX_OK;
}

int hfx_burgers_get_csr(hfx_ctx* c, int64_t* rowptr, int* col, double* val, double* rhs) {
  if (int rc = burgers_ready(c, "burgers_get_csr")) return rc;
  BurgersState& B = c->burgers;
  if (!B.assembled && (val || rhs)) return set_err(c, HFX_ERR_STATE, "burgers_get_csr: assemble first");
  const int NB = B.NLF;
  const int nF = c->topo.nFaces;
  if (rowptr || col) {
    int64_t pos = 0;
    if (rowptr) rowptr[0] = 0;
    for (int f = 0; f < nF; ++f) {
      int64_t b0 = c->bp.rowptr[f], nb = c->bp.rowptr[f + 1] - b0;
      for (int a = 0; a < NB; ++a) {
        if (col)
          for (int64_t k = 0; k < nb; ++k)
            for (int b = 0; b < NB; ++b) col[pos + k * NB + b] = c->bp.col[b0 + k] * NB + b;
        pos += nb * NB;
        if (rowptr) rowptr[(int64_t)f * NB + a + 1] = pos;
      }
    }
  }
  cudaStream_t s = c->stream;
  std::vector<double> blocks;
  if (val) {
    blocks.resize((size_t)B.nnz);
    HFX_CUDA(c, cudaMemcpyAsync(blocks.data(), B.val, sizeof(double) * B.nnz, cudaMemcpyDeviceToHost, s));
  }
  if (rhs) HFX_CUDA(c, cudaMemcpyAsync(rhs, B.rhs, sizeof(double) * B.nDofs, cudaMemcpyDeviceToHost, s));
  HFX_CUDA(c, cudaStreamSynchronize(s));
  if (val) {
    int64_t pos = 0;
    for (int f = 0; f < nF; ++f) {
      int64_t b0 = c->bp.rowptr[f], nb = c->bp.rowptr[f + 1] - b0;
      for (int a = 0; a < NB; ++a)
        for (int64_t k = 0; k < nb; ++k)
          for (int b = 0; b < NB; ++b) val[pos++] = blocks[(b0 + k) * NB * NB + (int64_t)b * NB + a];
    }
  }
  return HFX_OK;
}

}  // extern "C"
