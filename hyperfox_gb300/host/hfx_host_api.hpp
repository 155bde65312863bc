// C++ host API over the C ABI, mirroring HyperFox's own interfaces so that a
// HyperFox user keeps the same calls:
//   hfx::gpu::GpuLinAlgebraInterface  ~ LinAlgebraInterface / PetscInterface
//                                       (LinAlgebraInterface.h:23-162, PetscInterface.cpp:33-265)
//   hfx::gpu::GpuHDGSolver            ~ HDGSolver (HDGSolver.h:16-87) with the
//                                       field map Solution/Flux/Trace/Tau/Dirichlet
//   hfx::gpu::Mesh / Field / models   ~ the parts of Mesh, Field, HDGDiffusionSource,
//                                       HDGLaplaceModel and DirichletModel the path reads
//   hfx::gpu::MeshUnion               ~ many independent Meshes of one order as one
//   hfx::gpu::GpuBurgersSolver        ~ HDGSolver with HDGBurgersModel (vector Burgers)
//   hfx::gpu::NonLinearWrapper        ~ NonLinearWrapper (NonLinearWrapper.h:14-128)
// Errors throw ErrorHandle(class, method, message) exactly where HyperFox
// throws (calls out of order, missing fields); device failures carry the
// library's message.
#pragma once
#include <cmath>
#include <cstdio>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "hfx_gb300.h"

namespace hfx {
namespace gpu {

class ErrorHandle : public std::exception {
 public:
  ErrorHandle(std::string cls, std::string method, std::string msg)
      : what_(cls + "::" + method + ": " + msg) {}
  const char* what() const noexcept override { return what_.c_str(); }

 private:
  std::string what_;
};

// One device context shared by the objects of a thread.
class Device {
 public:
  explicit Device(int device = 0) {
    if (hfx_ctx_create(device, &ctx_) != HFX_OK) throw ErrorHandle("Device", "Device", "no CUDA device");
  }
  ~Device() { hfx_ctx_destroy(ctx_); }
  Device(const Device&) = delete;
  Device& operator=(const Device&) = delete;
  hfx_ctx* ctx() const { return ctx_; }
  void check(int rc, const char* cls, const char* method) const {
    if (rc != HFX_OK) throw ErrorHandle(cls, method, hfx_last_error(ctx_));
  }

 private:
  hfx_ctx* ctx_ = nullptr;
};

// ---------------------------------------------------------------- LinAlgebraInterface
struct GpuSolverOpts {  // PetscOpts (PetscOpts.h:8-29) analogue
  int method = HFX_KSP_GMRES;
  int precond = HFX_PC_JACOBI;
  int precision = HFX_PREC_FP64;
  double rtol = 1e-6;
  int maxits = 1000;
  int restart = 30;
  // HFX_PC_TWOLEVEL only: coarse solve, and the degree of the learned coarse
  // polynomial GpuHDGSolver trains on its first solve (HFX_COARSE_LEARNED)
  int coarseMode = HFX_COARSE_CHEBYSHEV;
  int learnedDegree = 8;
};

class GpuLinAlgebraInterface {
 public:
  explicit GpuLinAlgebraInterface(Device* dev, GpuSolverOpts opts = GpuSolverOpts()) : dev_(dev), opts_(opts) {}
  ~GpuLinAlgebraInterface() { destroySystem(); }

  void initialize() {
    if (!initialized) {
      dev_->check(hfx_la_create(dev_->ctx(), &la_), "GpuLinAlgebraInterface", "initialize");
      initialized = true;
    }
  }
  void configure() {
    if (!initialized) throw ErrorHandle("GpuLinAlgebraInterface", "configure", "the object was not initialized before being configured.");
    configured = true;
  }
  void allocate(int ndofs, const std::vector<int>* diag = nullptr, const std::vector<int>* off = nullptr) {
    (void)diag;
    (void)off;  // the device CSR is built from the values given, no preallocation needed
    if (!(initialized && configured))
      throw ErrorHandle("GpuLinAlgebraInterface", "allocate", "the object was not initialized and configured before being allocated.");
    dev_->check(hfx_la_allocate(la_, ndofs), "GpuLinAlgebraInterface", "allocate");
    nDOFs = ndofs;
    allocated = true;
  }
  void addValMatrix(int i, int j, const double& v) { vals("addValMatrix", 1, &i, 1, &j, &v, 0); }
  void addValsMatrix(std::vector<int>& is, std::vector<int>& js, const double* v) {
    vals("addValsMatrix", (int)is.size(), is.data(), (int)js.size(), js.data(), v, 0);
  }
  void addValRHS(int i, const double& v) { rhs("addValRHS", 1, &i, &v, 0); }
  void addValsRHS(std::vector<int>& is, const double* v) { rhs("addValsRHS", (int)is.size(), is.data(), v, 0); }
  void setValMatrix(int i, int j, const double& v) { vals("setValMatrix", 1, &i, 1, &j, &v, 1); }
  void setValsMatrix(std::vector<int>& is, std::vector<int>& js, const double* v) {
    vals("setValsMatrix", (int)is.size(), is.data(), (int)js.size(), js.data(), v, 1);
  }
  void setValRHS(int i, const double& v) { rhs("setValRHS", 1, &i, &v, 1); }
  void setValsRHS(std::vector<int>& is, const double* v) { rhs("setValsRHS", (int)is.size(), is.data(), v, 1); }
  void zeroOutRows(std::vector<int>& is) {
    if (!allocated) throw ErrorHandle("GpuLinAlgebraInterface", "zeroOutRows", "the matrix must be allocated before zeroing out rows.");
    dev_->check(hfx_la_zero_rows(la_, (int)is.size(), is.data()), "GpuLinAlgebraInterface", "zeroOutRows");
  }
  void assemble() {
    if (!allocated) throw ErrorHandle("GpuLinAlgebraInterface", "assemble", "the matrix should at least be allocated before assembling.");
    dev_->check(hfx_la_assemble(la_), "GpuLinAlgebraInterface", "assemble");
    assembled = true;
  }
  void assembleFlush() { assemble(); }
  void solve(std::vector<double>* solution) {
    if (!assembled) throw ErrorHandle("GpuLinAlgebraInterface", "solve", "the matrix needs to be assembled before solving.");
    solution->resize(nDOFs);
    hfx_solve_opts o;
    hfx_solve_opts_default(&o);
    o.method = opts_.method;
    o.precond = opts_.precond;
    o.precision = opts_.precision;
    o.rtol = opts_.rtol;
    o.maxits = opts_.maxits;
    o.restart = opts_.restart;
    hfx_solve_info info;
    dev_->check(hfx_la_solve(la_, &o, solution->data(), &info), "GpuLinAlgebraInterface", "solve");
    lastInfo = info;
  }
  void getSolutionOwnership(std::vector<int>* range) {
    if (!assembled) throw ErrorHandle("GpuLinAlgebraInterface", "getRowOwnership", "the matrix needs to be assembled before querying ownership.");
    range->resize(nDOFs);
    for (int i = 0; i < nDOFs; ++i) (*range)[i] = i;
  }
  void clearSystem() {
    if (!assembled) throw ErrorHandle("GpuLinAlgebraInterface", "clearSystem", "the matrix needs to be assembled at least once before clearing.");
    dev_->check(hfx_la_clear(la_), "GpuLinAlgebraInterface", "clearSystem");
  }
  void destroySystem() {
    if (la_) hfx_la_destroy(la_);
    la_ = nullptr;
    initialized = configured = allocated = assembled = false;
  }
  int getNumDofs() const { return nDOFs; }
  hfx_solve_info lastInfo{};
  hfx_train_info trainInfo{};

 private:
  void vals(const char* m, int nr, const int* r, int nc, const int* cc, const double* v, int insert) {
    if (!allocated) throw ErrorHandle("GpuLinAlgebraInterface", m, "the matrix must be allocated before adding values.");
    dev_->check(hfx_la_set_values(la_, nr, r, nc, cc, v, insert), "GpuLinAlgebraInterface", m);
  }
  void rhs(const char* m, int n, const int* i, const double* v, int insert) {
    if (!allocated) throw ErrorHandle("GpuLinAlgebraInterface", m, "the RHS must be allocated before adding values.");
    dev_->check(hfx_la_set_rhs(la_, n, i, v, insert), "GpuLinAlgebraInterface", m);
  }
  Device* dev_;
  GpuSolverOpts opts_;
  hfx_la* la_ = nullptr;
  int nDOFs = 0;
  bool initialized = false, configured = false, allocated = false, assembled = false;
};

// ---------------------------------------------------------------- mesh, fields, models
enum FieldType { None = -1, Node = 0, Edge = 1, Face = 2, Cell = 3 };  // FieldTypes.h

// Simplex mesh: nodes [nNodes][dim], cells [nCells][N] (vertices first).
struct Mesh {
  int dim = 0, order = 0;
  std::vector<double> nodes;
  std::vector<int> cells;
  // face topology (filled by GpuHDGSolver::allocate with the MOAB rule)
  std::vector<int> cell2face, face2cell, faces, boundary;
  int nFaces = 0;
  int numCells() const { return (int)(cells.size() / nodesPerCell()); }
  int numNodes() const { return (int)(nodes.size() / dim); }
  int nodesPerCell() const { hfx_refel_info i; hfx_refel_query(dim, order, &i); return i.nNodes; }
  int nodesPerFace() const { hfx_refel_info i; hfx_refel_query(dim, order, &i); return i.nNodesFace; }
  void computeFaces() {
    int nF = 0, nB = 0;
    if (hfx_mesh_compute_topology(dim, order, numCells(), cells.data(), &nF, &nB, nullptr, nullptr, nullptr, nullptr))
      throw ErrorHandle("Mesh", "computeFaces", "invalid mesh");
    cell2face.resize((size_t)numCells() * (dim + 1));
    face2cell.resize(2 * (size_t)nF);
    faces.resize((size_t)nF * nodesPerFace());
    boundary.resize(nB);
    hfx_mesh_compute_topology(dim, order, numCells(), cells.data(), &nF, &nB, cell2face.data(), face2cell.data(),
                              faces.data(), boundary.data());
    nFaces = nF;
  }
};

// Independent problems of one order as ONE mesh (HyperFox runs one problem per Mesh,
// and a Mesh has one ReferenceElement, Mesh.cpp:24-29). The nodes, cells and faces of
// problem k follow those of problems 0..k-1. The union's own topology (computeFaces,
// the MOAB creation-order rule) numbers the faces problem by problem, so problem k's
// faces are [faceOffset[k], faceOffset[k+1]) in its own order. No face or vertex is
// shared, so the trace system is block diagonal: one GpuHDGSolver on `mesh` serves every
// problem. Its Krylov tolerance groupTolerance(rtol, rhs, valsPerFace) bounds every
// problem's own relative residual by rtol: |r_k| <= |r| <= rtol min_j |b_j| <= rtol |b_k|,
// over the problems whose part b_k of the right-hand side is non-zero.
struct MeshUnion {
  Mesh mesh;
  std::vector<long long> nodeOffset{0}, cellOffset{0}, faceOffset{0};
  explicit MeshUnion(const std::vector<const Mesh*>& parts) {
    if (parts.empty()) throw ErrorHandle("MeshUnion", "MeshUnion", "no problems");
    mesh.dim = parts[0]->dim;
    mesh.order = parts[0]->order;
    for (const Mesh* m : parts) {
      if (m->dim != mesh.dim || m->order != mesh.order)
        throw ErrorHandle("MeshUnion", "MeshUnion", "all problems of one union have one dimension and one order");
      int nF = 0, nB = 0;
      if (hfx_mesh_compute_topology(m->dim, m->order, m->numCells(), m->cells.data(), &nF, &nB, nullptr, nullptr,
                                    nullptr, nullptr))
        throw ErrorHandle("MeshUnion", "MeshUnion", "invalid mesh");
      const long long shift = nodeOffset.back();
      mesh.nodes.insert(mesh.nodes.end(), m->nodes.begin(), m->nodes.end());
      for (int v : m->cells) mesh.cells.push_back((int)(v + shift));
      nodeOffset.push_back(shift + m->numNodes());
      cellOffset.push_back(cellOffset.back() + m->numCells());
      faceOffset.push_back(faceOffset.back() + nF);
      if (nodeOffset.back() >= (1LL << 31) || faceOffset.back() >= (1LL << 31))
        throw ErrorHandle("MeshUnion", "MeshUnion", "more than 2^31 - 1 nodes or faces");
    }
    mesh.computeFaces();
    if (mesh.nFaces != faceOffset.back())
      throw ErrorHandle("MeshUnion", "MeshUnion", "the problems share faces");
  }
  int numProblems() const { return (int)cellOffset.size() - 1; }
  double groupTolerance(double rtol, const std::vector<double>& rhs, int valsPerFace) const {
    double total = 0.0, least = -1.0;
    for (int k = 0; k < numProblems(); ++k) {
      double sq = 0.0;
      for (long long i = faceOffset[k] * valsPerFace; i < faceOffset[k + 1] * valsPerFace; ++i) sq += rhs[i] * rhs[i];
      total += sq;
      if (sq > 0.0 && (least < 0.0 || sq < least)) least = sq;
    }
    return (total == 0.0 || least < 0.0) ? rtol : rtol * std::sqrt(least / total);
  }
};

struct Field {  // Field.h:14-34: values[entity][objPerEnt][valsPerObj]
  Field(const Mesh* m, FieldType t, int objPerEnt, int valsPerObj) : type(t), obj(objPerEnt), vals(valsPerObj) {
    size_t ents = t == Cell ? m->numCells() : (t == Node ? m->numNodes() : 0);
    if (t == Face) {
      const_cast<Mesh*>(m)->computeFaces();
      ents = m->nFaces;
    }
    values.assign(ents * obj * vals, 0.0);
  }
  FieldType type;
  int obj, vals;
  std::vector<double> values;
  std::vector<double>* getValues() { return &values; }
};

struct DirichletModel {};  // Set-type boundary model: identity rows + Dirichlet values

// RungeKutta (src/operator/RungeKutta.h, RKType.h) with the auxiliary fields
// {"Flux", "Trace"}: the stages run on the device. A model with this time scheme
// has its U rows modified at every assemble (RungeKutta::apply); at the first
// stage of a step the solver takes the field map's Solution, Flux and Trace as
// the Old fields (the reference's tests copy them into OldSolution/OldFlux/
// OldTrace by hand), and computeStage / computeSolution update the device fields
// and copy Solution, Flux and Trace back into the field map.
enum RKType { FEuler, EMidpoint, Heun, Kutta3, Heun3, SSPRK3, RK4, BEuler, IMidpoint, CrankNicolson, KS2, QZ2, ALX2, RK43 };

class RungeKutta {
 public:
  explicit RungeKutta(RKType type = CrankNicolson) { setButcherTable(type); }
  void setButcherTable(RKType type) {
    int S = 0;
    if (hfx_rk_butcher((int)type, &S, nullptr)) throw ErrorHandle("RungeKutta", "setButcherTable", "unknown RKType");
    table_.assign((size_t)(S + 1) * (S + 1), 0.0);
    hfx_rk_butcher((int)type, &S, table_.data());
    type_ = (int)type;
    dirty_ = true;
  }
  // row-major (S+1) x (S+1); the strictly upper part must be zero (RungeKutta.cpp:18-32)
  void setButcherTable(const std::vector<double>& table, int rows, int cols) {
    if (rows != cols || (int)table.size() != rows * cols)
      throw ErrorHandle("RungeKutta", "setButcherTable", "the Butcher table should be square");
    for (int i = 0; i < rows; ++i)
      for (int j = i + 1; j < cols; ++j)
        if (table[(size_t)i * cols + j] != 0.0)
          throw ErrorHandle("RungeKutta", "setButcherTable",
                            "the upper triangular part of the Butcher table should be null (no fully implicit "
                            "implementation as of yet)");
    table_ = table;
    type_ = -1;
    dirty_ = true;
  }
  void setTimeStep(double dt) {
    dt_ = dt;
    dirty_ = true;
  }
  int getNumStages() const { return (int)std::lround(std::sqrt((double)table_.size())) - 1; }
  int getStage() const { return stage_; }
  void computeStage(std::map<std::string, Field*>* fm) {
    if (!ctx_) throw ErrorHandle("RungeKutta", "computeStage", "the scheme must be assembled by a solver first");
    if (stage_ >= getNumStages())
      throw ErrorHandle("RungeKutta", "computeStage",
                        "cannot compute more stages than the method allows, think about computing the solution");
    check(hfx_rk_compute_stage(ctx_), "computeStage");
    ++stage_;
    download(fm, "computeStage");
  }
  void computeSolution(std::map<std::string, Field*>* fm) {
    if (!ctx_ || stage_ != getNumStages())
      throw ErrorHandle("RungeKutta", "computeSolution", "all stages must be computed before computing the solution");
    check(hfx_rk_compute_solution(ctx_), "computeSolution");
    stage_ = 0;
    download(fm, "computeSolution");
  }

 private:
  friend class GpuHDGSolver;
  void check(int rc, const char* where) {
    if (rc) throw ErrorHandle("RungeKutta", where, ctx_ ? hfx_last_error(ctx_) : "no device context");
  }
  // called by the solver before each assemble
  void prepare(hfx_ctx* ctx, std::map<std::string, Field*>* fm) {
    if (dt_ == 0.0) throw ErrorHandle("RungeKutta", "apply", "the time step needs to be set before applying and it should not be 0");
    ctx_ = ctx;
    if (dirty_) {
      const int S = getNumStages();
      check(type_ >= 0 ? hfx_rk_set_type(ctx, type_, dt_) : hfx_rk_set(ctx, S, table_.data(), dt_), "apply");
      dirty_ = false;
      stage_ = 0;
    }
    if (stage_ == 0) {  // a new step: the field map's state becomes the Old fields
      check(hfx_set_state(ctx, fm->at("Solution")->values.data(), fm->at("Flux")->values.data()), "apply");
      check(hfx_set_trace(ctx, fm->at("Trace")->values.data()), "apply");
      check(hfx_rk_begin_step(ctx), "apply");
    }
  }
  void download(std::map<std::string, Field*>* fm, const char* where) {
    check(hfx_get_state(ctx_, fm->at("Solution")->values.data(), fm->at("Flux")->values.data(),
                        fm->at("Trace")->values.data()),
          where);
  }
  std::vector<double> table_;
  int type_ = -1;
  double dt_ = 0.0;
  int stage_ = 0;
  bool dirty_ = true;
  hfx_ctx* ctx_ = nullptr;
};

struct HDGDiffusionSource {  // HDGDiffusionSource.h; HDGLaplaceModel = no source
  int sourceMode = HFX_SRC_NONE;
  double sourceParam = 0.0;
  std::vector<double> sourceValues;  // [nCells][nIP] for HFX_SRC_VALUES
  double dt = 0.0;                   // implicit Euler when > 0 (Euler.cpp:18-34)
  RungeKutta* timeScheme = nullptr;  // Model::setTimeScheme; replaces dt when set
  void setTimeScheme(RungeKutta* ts) { timeScheme = ts; }
};
struct HDGLaplaceModel : HDGDiffusionSource {};

// ---------------------------------------------------------------- HDGSolver
class GpuHDGSolver {
 public:
  explicit GpuHDGSolver(Device* dev) : dev_(dev) {}
  void setMesh(Mesh* m) { mesh_ = m; }
  void setFieldMap(std::map<std::string, Field*>* fm) { fields_ = fm; }
  void setModel(HDGDiffusionSource* m) { model_ = m; }
  void setBoundaryModel(DirichletModel* b) { bnd_ = b; }
  void setLinSystem(GpuSolverOpts opts) { opts_ = opts; haveLin_ = true; }
  void initialize() { initialized_ = true; }

  void allocate() {  // HDGSolver.cpp:5-106 checks
    if (!initialized_) throw ErrorHandle("HDGSolver", "allocate", "must initialize the solver before allocating.");
    if (!mesh_) throw ErrorHandle("HDGSolver", "allocate", "must set the Mesh before allocating.");
    if (!haveLin_) throw ErrorHandle("HDGSolver", "allocate", "must set the linear system before allocating.");
    if (!model_) throw ErrorHandle("HDGSolver", "allocate", "must set the model before allocating.");
    if (!bnd_) throw ErrorHandle("HDGSolver", "allocate", "must set the boundary model before allocating.");
    if (!fields_ || fields_->empty()) throw ErrorHandle("HDGSolver", "allocate", "must set the fields before allocating.");
    for (const char* f : {"Solution", "Flux", "Tau", "Trace"})
      if (!fields_->count(f)) throw ErrorHandle("HDGSolver", "allocate", std::string("the field map must have a ") + f + " field.");
    if (fields_->at("Solution")->type != Cell) throw ErrorHandle("HDGSolver", "allocate", "the Solution field must be a cell field.");
    if (fields_->at("Flux")->type != Cell) throw ErrorHandle("HDGSolver", "allocate", "the Flux field must be a cell field.");
    if (fields_->at("Tau")->type != Face) throw ErrorHandle("HDGSolver", "allocate", "the Tau field must be a face field.");
    if (fields_->at("Trace")->type != Face) throw ErrorHandle("HDGSolver", "allocate", "the Trace field must be a face field.");
    mesh_->computeFaces();
    dev_->check(hfx_mesh_upload(dev_->ctx(), mesh_->dim, mesh_->order, mesh_->numNodes(), mesh_->nodes.data(),
                                mesh_->numCells(), mesh_->cells.data(), mesh_->nFaces, mesh_->cell2face.data(),
                                mesh_->face2cell.data(), mesh_->faces.data(), (int)mesh_->boundary.size(),
                                mesh_->boundary.data()),
                "HDGSolver", "allocate");
    allocated_ = true;
  }

  void assemble() {
    if (!(initialized_ && allocated_)) throw ErrorHandle("HDGSolver", "assemble", "the solver must be initialized and allocated before assembling.");
    Field* tau = fields_->at("Tau");
    dev_->check(hfx_set_tau(dev_->ctx(), tau->values.data(), tau->vals), "HDGSolver", "assemble");
    if (fields_->count("Dirichlet"))
      dev_->check(hfx_set_dirichlet(dev_->ctx(), fields_->at("Dirichlet")->values.data()), "HDGSolver", "assemble");
    if (fields_->count("DiffusionTensor")) {
      Field* k = fields_->at("DiffusionTensor");
      dev_->check(hfx_set_kappa(dev_->ctx(), k->values.data(), k->vals, k->type == Node ? 0 : 1), "HDGSolver", "assemble");
    }
    dev_->check(hfx_set_source(dev_->ctx(), model_->sourceMode,
                               model_->sourceValues.empty() ? nullptr : model_->sourceValues.data(), model_->sourceParam),
                "HDGSolver", "assemble");
    if (model_->timeScheme)
      model_->timeScheme->prepare(dev_->ctx(), fields_);
    else if (model_->dt > 0.0)
      dev_->check(hfx_set_time_scheme(dev_->ctx(), model_->dt, fields_->at("Solution")->values.data()), "HDGSolver", "assemble");
    dev_->check(hfx_assemble(dev_->ctx()), "HDGSolver", "assemble");
    assembled_ = true;
  }

  void solve() {
    if (!assembled_) throw ErrorHandle("HDGSolver", "solve", "system must be assembled before solving");
    hfx_solve_opts o;
    hfx_solve_opts_default(&o);
    o.precond = opts_.precond;
    o.precision = opts_.precision;
    o.rtol = opts_.rtol;
    o.maxits = opts_.maxits;
    o.restart = opts_.restart;
    o.method = opts_.method;
    o.coarse_mode = opts_.coarseMode;
    if (opts_.precond == HFX_PC_TWOLEVEL && opts_.coarseMode == HFX_COARSE_LEARNED && !trained_) {
      // the learned coarse solve is trained once per mesh, on this system's own coarse errors
      dev_->check(hfx_coarse_train(dev_->ctx(), opts_.learnedDegree, 16, 300, &trainInfo), "HDGSolver", "solve");
      trained_ = true;
    }
    dev_->check(hfx_solve(dev_->ctx(), &o, fields_->at("Trace")->values.data(), &lastInfo), "HDGSolver", "solve");
    dev_->check(hfx_recover(dev_->ctx(), fields_->at("Solution")->values.data(), fields_->at("Flux")->values.data()),
                "HDGSolver", "solve");
  }
  hfx_solve_info lastInfo{};
  hfx_train_info trainInfo{};

 private:
  Device* dev_;
  Mesh* mesh_ = nullptr;
  std::map<std::string, Field*>* fields_ = nullptr;
  HDGDiffusionSource* model_ = nullptr;
  DirichletModel* bnd_ = nullptr;
  GpuSolverOpts opts_;
  bool haveLin_ = false, initialized_ = false, allocated_ = false, assembled_ = false, trained_ = false;
};

// ---------------------------------------------------------------- Burgers / Newton
// Euler (src/operator/Euler.h): implicit Euler on the U rows; the model reads the
// field map's OldSolution as u_old when there is one, else its Solution (the field
// Euler::setFieldMap takes, Euler.cpp:7-16).
struct Euler {
  double dt = 0.0;
  void setTimeStep(double t) { dt = t; }
};

// HDGBurgersModel (src/model/HDGBurgersModel.h): vector Burgers, nd = dim unknowns
// per node; one Source per component given at the volume IPs ([nCells][nIP][nd],
// the values HDGBurgersModel::setSourceFunction's functor would return there).
struct HDGBurgersModel {
  std::vector<double> sourceValues;
  Euler* timeScheme = nullptr;
  void setTimeScheme(Euler* ts) { timeScheme = ts; }
};

// HDGSolver with HDGBurgersModel (HDGSolver.cpp:5-175,677-779): the field map needs
// Solution, BufferSolution, Flux, Trace, Tau and Dirichlet with nd values per node
// (HDGBurgersModel::setFieldMap, HDGBurgersModel.cpp:5-33); DiffusionTensor (Node or
// Cell field, 1 or dim*dim values) adds the diffusion operator. Tau may be double
// valued (2*nd*nd values per face node). assemble() linearises about BufferSolution
// and Trace; solve() writes Trace, Solution and Flux back into the field map.
class GpuBurgersSolver {
 public:
  explicit GpuBurgersSolver(Device* dev) : dev_(dev) {}
  void setMesh(Mesh* m) { mesh_ = m; }
  void setFieldMap(std::map<std::string, Field*>* fm) { fields_ = fm; }
  void setModel(HDGBurgersModel* m) { model_ = m; }
  void setBoundaryModel(DirichletModel* b) { bnd_ = b; }
  void setLinSystem(GpuSolverOpts opts) { opts_ = opts; haveLin_ = true; }
  void initialize() { initialized_ = true; }

  void allocate() {
    if (!initialized_) throw ErrorHandle("HDGSolver", "allocate", "must initialize the solver before allocating.");
    if (!mesh_) throw ErrorHandle("HDGSolver", "allocate", "must set the Mesh before allocating.");
    if (!haveLin_) throw ErrorHandle("HDGSolver", "allocate", "must set the linear system before allocating.");
    if (!model_) throw ErrorHandle("HDGSolver", "allocate", "must set the model before allocating.");
    if (!bnd_) throw ErrorHandle("HDGSolver", "allocate", "must set the boundary model before allocating.");
    if (!fields_ || fields_->empty()) throw ErrorHandle("HDGSolver", "allocate", "must set the fields before allocating.");
    for (const char* f : {"Solution", "BufferSolution", "Flux", "Tau", "Trace", "Dirichlet"})
      if (!fields_->count(f))
        throw ErrorHandle("HDGBurgersModel", "setFieldMap", std::string("the field map must have a ") + f + " field");
    const int nd = mesh_->dim;
    if (fields_->at("BufferSolution")->vals != nd || fields_->at("Solution")->vals != nd)
      throw ErrorHandle("HDGBurgersModel", "setFieldMap",
                        "the BufferSolution must have the same number of DOFs per node as spatial dimensions for the "
                        "Burgers equation");
    if (fields_->at("Trace")->vals != nd)
      throw ErrorHandle("HDGBurgersModel", "setFieldMap",
                        "the Trace must have the same number of DOFs per node as spatial dimensions for the Burgers "
                        "equation");
    const int tv = fields_->at("Tau")->vals;
    if (tv != nd * nd && tv != 2 * nd * nd)
      throw ErrorHandle("HDGBurgersModel", "setFieldMap", "the Tau field holds nd*nd (or 2*nd*nd) values per node");
    mesh_->computeFaces();
    dev_->check(hfx_mesh_upload(dev_->ctx(), mesh_->dim, mesh_->order, mesh_->numNodes(), mesh_->nodes.data(),
                                mesh_->numCells(), mesh_->cells.data(), mesh_->nFaces, mesh_->cell2face.data(),
                                mesh_->face2cell.data(), mesh_->faces.data(), (int)mesh_->boundary.size(),
                                mesh_->boundary.data()),
                "HDGSolver", "allocate");
    dev_->check(hfx_burgers_setup(dev_->ctx()), "HDGSolver", "allocate");
    allocated_ = true;
  }

  // every field of the map to the device (HDGSolver::assemble's field gather)
  void upload() {
    hfx_ctx* c = dev_->ctx();
    const int nd = mesh_->dim;
    Field* tau = fields_->at("Tau");
    dev_->check(hfx_burgers_set_tau(c, tau->values.data(), tau->vals / (nd * nd)), "HDGSolver", "assemble");
    dev_->check(hfx_burgers_set_dirichlet(c, fields_->at("Dirichlet")->values.data()), "HDGSolver", "assemble");
    if (fields_->count("DiffusionTensor")) {
      Field* k = fields_->at("DiffusionTensor");
      dev_->check(hfx_burgers_set_diffusion(c, k->values.data(), k->vals, k->type == Node ? 0 : 1), "HDGSolver",
                  "assemble");
    } else {
      dev_->check(hfx_burgers_set_diffusion(c, nullptr, 0, 0), "HDGSolver", "assemble");
    }
    dev_->check(hfx_burgers_set_source(c, model_->sourceValues.empty() ? nullptr : model_->sourceValues.data()),
                "HDGSolver", "assemble");
    const double dt = model_->timeScheme ? model_->timeScheme->dt : 0.0;
    if (model_->timeScheme && dt == 0.0)
      throw ErrorHandle("Euler", "apply", "the time step needs to be set before applying and it should not be 0");
    dev_->check(hfx_burgers_set_time_step(c, dt), "HDGSolver", "assemble");
    const Field* old = dt > 0.0 ? (fields_->count("OldSolution") ? fields_->at("OldSolution") : fields_->at("Solution"))
                                : nullptr;
    dev_->check(hfx_burgers_set_state(c, fields_->at("Solution")->values.data(),
                                      fields_->at("BufferSolution")->values.data(), fields_->at("Trace")->values.data(),
                                      old ? old->values.data() : nullptr),
                "HDGSolver", "assemble");
  }

  void assemble() {
    if (!(initialized_ && allocated_))
      throw ErrorHandle("HDGSolver", "assemble", "the solver must be initialized and allocated before assembling.");
    upload();
    dev_->check(hfx_burgers_assemble(dev_->ctx()), "HDGSolver", "assemble");
    assembled_ = true;
  }

  void solve() {
    if (!assembled_) throw ErrorHandle("HDGSolver", "solve", "system must be assembled before solving");
    hfx_solve_opts o = linOpts();
    dev_->check(hfx_burgers_solve(dev_->ctx(), &o, &lastInfo), "HDGSolver", "solve");
    download(false);
  }

  hfx_solve_opts linOpts() const {
    hfx_solve_opts o;
    hfx_solve_opts_default(&o);
    o.method = HFX_KSP_GMRES;
    o.precond = opts_.precond;
    o.rtol = opts_.rtol;
    o.maxits = opts_.maxits;
    o.restart = opts_.restart;
    return o;
  }
  // Solution, Flux, Trace (and BufferSolution) back into the field map
  void download(bool withBuffer) {
    dev_->check(hfx_burgers_get_state(dev_->ctx(), fields_->at("Solution")->values.data(),
                                      fields_->at("Flux")->values.data(), fields_->at("Trace")->values.data(),
                                      withBuffer ? fields_->at("BufferSolution")->values.data() : nullptr),
                "HDGSolver", "solve");
  }
  bool allocated() const { return allocated_; }
  Device* device() { return dev_; }
  std::map<std::string, Field*>* fieldMap() { return fields_; }
  hfx_solve_info lastInfo{};

 private:
  Device* dev_;
  Mesh* mesh_ = nullptr;
  std::map<std::string, Field*>* fields_ = nullptr;
  HDGBurgersModel* model_ = nullptr;
  DirichletModel* bnd_ = nullptr;
  GpuSolverOpts opts_;
  bool haveLin_ = false, initialized_ = false, allocated_ = false, assembled_ = false;
};

// NonLinearWrapper (src/solver/NonLinearWrapper.h, NonLinearWrapper.cpp:5-79). With
// the vanilla linearised solver and residual computer and the solver's own
// Solution / BufferSolution as the solution fields, solve() runs the whole loop on
// the device (hfx_burgers_newton) and copies the fields back at the end; a user
// linearised solver or residual computer runs the reference's loop on the host.
class NonLinearWrapper {
 public:
  void solve() {
    if (!mySolver) throw ErrorHandle("NonLinearWrapper", "solve", "the Solver must be set before attempting to solve");
    if (!currentSolution || !previousSolution)
      throw ErrorHandle("NonLinearWrapper", "solve", "the current and previous Solutions should be set before attempting to solve");
    std::map<std::string, Field*>* fm = mySolver->fieldMap();
    const bool deviceLoop = !linearizedSolver && !residualComputer && mySolver->allocated() && fm &&
                            fm->count("Solution") && fm->at("Solution") == currentSolution &&
                            fm->count("BufferSolution") && fm->at("BufferSolution") == previousSolution;
    if (deviceLoop) {
      mySolver->upload();
      hfx_newton_opts o;
      hfx_newton_opts_default(&o);
      o.res_tol = resTol;
      o.max_iters = maxIters;
      o.dampening = dampening;
      o.lin = mySolver->linOpts();
      o.warm_start = warmStart ? 1 : 0;
      o.history = history;
      mySolver->device()->check(hfx_burgers_newton(mySolver->device()->ctx(), &o, &lastInfo), "NonLinearWrapper",
                                "solve");
      residual = lastInfo.residual;
      mySolver->download(true);
      return;
    }
    for (int i = 0; i < maxIters; ++i) {
      if (linearizedSolver) linearizedSolver(mySolver);
      else {
        mySolver->assemble();
        mySolver->solve();
      }
      residual = residualComputer ? residualComputer(currentSolution, previousSolution)
                                  : vanillaResidual(currentSolution, previousSolution);
      if (verbose) std::printf("\rIteration %d at residual value %f", i + 1, residual);
      if (residual < resTol) break;
      std::vector<double>& cur = currentSolution->values;
      std::vector<double>& prev = previousSolution->values;
      for (size_t k = 0; k < cur.size(); ++k) {
        const double v = (1.0 - dampening) * cur[k] + dampening * prev[k];
        cur[k] = v;
        prev[k] = v;
      }
    }
    if (verbose) std::printf("\n");
  }
  double getResidual() const { return residual; }
  void setResidualTolerance(double tol) { resTol = tol; }
  void setMaxIterations(int iters) { maxIters = iters; }
  void setVerbosity(bool v) { verbose = v; }
  void setSolutionFields(Field* currentSol, Field* prevSol) {
    currentSolution = currentSol;
    previousSolution = prevSol;
  }
  void setSolver(GpuBurgersSolver* solver) { mySolver = solver; }
  void setResidualComputer(std::function<double(Field*, Field*)> f) { residualComputer = f; }
  void setLinearizedSolver(std::function<void(GpuBurgersSolver*)> f) { linearizedSolver = f; }
  void setDampening(double d) { dampening = d; }
  // start every Krylov solve from the current trace (PETSc starts from zero)
  void setWarmStart(bool on) { warmStart = on; }
  // start every Krylov solve from the least-squares fit of the last k (<= 8) trace
  // solutions to the new system (device loop only; 0 = off)
  void setKrylovHistory(int k) { history = k; }
  hfx_newton_info lastInfo{};

  // NonLinearWrapper::vanillaResidualComputer (NonLinearWrapper.cpp:14-34), one rank
  static double vanillaResidual(Field* cur, Field* prev) {
    double diff = 0.0, ref = 0.0;
    for (size_t i = 0; i < cur->values.size(); ++i) {
      diff += (cur->values[i] - prev->values[i]) * (cur->values[i] - prev->values[i]);
      ref += prev->values[i] * prev->values[i];
    }
    return ref != 0.0 ? std::sqrt(diff / ref) : std::sqrt(diff);
  }

 private:
  GpuBurgersSolver* mySolver = nullptr;
  Field* currentSolution = nullptr;
  Field* previousSolution = nullptr;
  std::function<double(Field*, Field*)> residualComputer;
  std::function<void(GpuBurgersSolver*)> linearizedSolver;
  double residual = 0.0, resTol = 1e-6, dampening = 0.0;
  int maxIters = 20, history = 0;
  bool verbose = false, warmStart = false;
};

// ---------------------------------------------------------------- HDF5Io
// HDF5Io (src/io/HDF5Io.cpp:13-393) on the host reader/writer: load() fills the
// mesh from /Mesh when present and every registered field from /FieldData (the
// field's type and shape come from the file); write() stores the mesh and the
// registered fields. The mesh's dim and order select the reference element, as
// for Mesh(dim, order, "simplex") before HDF5Io::load.
class HDF5Io {
 public:
  HDF5Io() = default;
  explicit HDF5Io(Mesh* m) : mesh_(m) {}
  void setMesh(Mesh* m) { mesh_ = m; }
  void setField(const std::string& name, Field* f) { fields_[name] = f; }
  void load(const std::string& path) {
    if (!mesh_) throw ErrorHandle("HDF5Io", "load", "must enter a mesh into the io before loading a file.");
    int nd = 0, nn = 0, nc = 0, npc = 0;
    int rc = hfx_h5_read_mesh(path.c_str(), &nd, &nn, &nc, &npc, nullptr, nullptr);
    const bool haveMesh = rc == HFX_OK;
    if (haveMesh) {
      if (nd != mesh_->dim || npc != mesh_->nodesPerCell())
        throw ErrorHandle("HDF5Io", "load", "the file's mesh does not match the mesh's dimension and order");
      mesh_->nodes.assign((size_t)nn * nd, 0.0);
      mesh_->cells.assign((size_t)nc * npc, 0);
      check(hfx_h5_read_mesh(path.c_str(), &nd, &nn, &nc, &npc, mesh_->nodes.data(), mesh_->cells.data()), "load");
      mesh_->nFaces = 0;
    }
    int nf = 0, need = 0;
    const bool haveFields = hfx_h5_field_names(path.c_str(), nullptr, 0, &nf, &need) == HFX_OK && nf > 0;
    if (!haveMesh && !haveFields)
      throw ErrorHandle("HDF5Io", "load", "could not find Mesh or FieldData groups in file: " + std::string(hfx_mesh_io_error()));
    for (auto& kv : fields_) {
      int ft = 0;
      int64_t shape[3] = {0, 0, 0};
      check(hfx_h5_read_field(path.c_str(), kv.first.c_str(), &ft, shape, nullptr), "load");
      Field* f = kv.second;
      f->type = (FieldType)ft;
      f->obj = (int)shape[1];
      f->vals = (int)shape[2];
      f->values.assign((size_t)(shape[0] * shape[1] * shape[2]), 0.0);
      check(hfx_h5_read_field(path.c_str(), kv.first.c_str(), &ft, shape, f->values.data()), "load");
    }
  }
  void write(const std::string& path) {
    std::vector<const char*> names;
    std::vector<int> types;
    std::vector<int64_t> shapes;
    std::vector<const double*> vals;
    for (auto& kv : fields_) {
      const Field* f = kv.second;
      const int64_t per = (int64_t)f->obj * f->vals;
      names.push_back(kv.first.c_str());
      types.push_back((int)f->type);
      shapes.insert(shapes.end(), {per ? (int64_t)f->values.size() / per : 0, (int64_t)f->obj, (int64_t)f->vals});
      vals.push_back(f->values.data());
    }
    const bool m = mesh_ && !mesh_->cells.empty();
    check(hfx_h5_write(path.c_str(), m ? mesh_->dim : 0, m ? mesh_->numNodes() : 0, m ? mesh_->nodes.data() : nullptr,
                       m ? mesh_->numCells() : 0, m ? mesh_->nodesPerCell() : 0, m ? mesh_->cells.data() : nullptr,
                       (int)names.size(), names.data(), types.data(), shapes.data(), vals.data()),
          "write");
  }

 private:
  static void check(int rc, const char* where) {
    if (rc) throw ErrorHandle("HDF5Io", where, hfx_mesh_io_error());
  }
  Mesh* mesh_ = nullptr;
  std::map<std::string, Field*> fields_;
};

}  // namespace gpu
}  // namespace hfx
