// The reference's own unit tests, re-expressed against the C++ host API
// (TestLinAlgebraInterfaces.cpp:23-150, TestHDGSolver.cpp:14-101, TestHDF5Io.cpp
// write mesh / write field sections).
// Exits non-zero on the first failed check.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <functional>
#include <string>
#include <vector>

#include "../../hyperfox_gb300/host/hfx_host_api.hpp"

using namespace hfx::gpu;

static int failures = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAILED %s:%d: %s\n", __FILE__, __LINE__, #c);   \
      ++failures;                                                  \
    }                                                              \
  } while (0)
static bool throws(const std::function<void()>& f) {
  try {
    f();
  } catch (const ErrorHandle&) {
    return true;
  }
  return false;
}

int main(int argc, char** argv) {
  {  // HDF5Io write then load of a mesh and two fields (TestHDF5Io.cpp "Test write mesh file", "Write test field")
    const std::string path = std::string(argc > 1 ? argv[1] : ".") + "/tmp.h5";
    Mesh m;
    m.dim = 2;
    m.order = 1;
    m.nodes = {0, 0, 1, 0, 1, 1, 0, 1, 0.5, 0.5, 0.5, 0, 1, 0.5, 0.5, 1, 0, 0.5};
    m.cells = {0, 5, 4, 5, 1, 4, 1, 6, 4, 6, 2, 4, 2, 7, 4, 7, 3, 4, 3, 8, 4, 8, 0, 4};
    Field nodeField(&m, Node, 1, 1), cellField(&m, Cell, 2, 1);
    for (int i = 0; i < 9; ++i) nodeField.values[i] = i;
    for (int i = 0; i < 8; ++i) {
      cellField.values[2 * i] = i;
      cellField.values[2 * i + 1] = -i;
    }
    HDF5Io io(&m);
    io.setField("NodeField", &nodeField);
    io.setField("CellField", &cellField);
    io.write(path);
    Mesh m2;
    m2.dim = 2;
    m2.order = 1;
    Field nf2(&m2, None, 1, 1), cf2(&m2, None, 1, 1);
    HDF5Io io2(&m2);
    io2.setField("NodeField", &nf2);
    io2.setField("CellField", &cf2);
    io2.load(path);
    CHECK(m2.nodes == m.nodes && m2.cells == m.cells);
    CHECK(nf2.type == Node && nf2.values == nodeField.values);
    CHECK(cf2.type == Cell && cf2.obj == 2 && cf2.values == cellField.values);
    Field missing(&m2, None, 1, 1);
    io2.setField("Solution", &missing);
    CHECK(throws([&] { io2.load(path); }));
    HDF5Io noMesh;
    CHECK(throws([&] { noMesh.load(path); }));
    Mesh wrongOrder;
    wrongOrder.dim = 2;
    wrongOrder.order = 2;
    HDF5Io io3(&wrongOrder);
    CHECK(throws([&] { io3.load(path); }));
  }
  Device dev(0);
  {  // ordering of initialize -> configure -> allocate (TestLinAlgebraInterfaces.cpp:23-67)
    GpuSolverOpts o;
    o.rtol = 1e-16;
    GpuLinAlgebraInterface L(&dev, o);
    int i = 0, j = 0;
    double val = 1;
    std::vector<double> dv = {1};
    std::vector<int> iv = {0};
    CHECK(throws([&] { L.solve(&dv); }));
    CHECK(throws([&] { L.assemble(); }));
    CHECK(throws([&] { L.setValsRHS(iv, dv.data()); }));
    CHECK(throws([&] { L.setValMatrix(i, j, val); }));
    CHECK(throws([&] { L.allocate(1); }));
    CHECK(throws([&] { L.configure(); }));
    L.initialize();
    CHECK(throws([&] { L.solve(&dv); }));
    CHECK(throws([&] { L.allocate(1); }));
    L.configure();
    CHECK(throws([&] { L.setValRHS(i, val); }));
    L.allocate(1);
    L.setValsRHS(iv, dv.data());
    L.setValRHS(i, val);
    L.setValsMatrix(iv, iv, dv.data());
    L.setValMatrix(i, j, val);
    L.assemble();
    L.solve(&dv);
    CHECK(std::fabs(dv[0] - 1.0) < 1e-12);
    L.clearSystem();
  }
  {  // identity and triangular systems (TestLinAlgebraInterfaces.cpp:70-120)
    GpuSolverOpts o;
    o.rtol = 1e-16;
    o.maxits = 5000;
    GpuLinAlgebraInterface L(&dev, o);
    for (int k = 1; k <= 40; k += 13) {
      L.destroySystem();
      L.initialize();
      L.configure();
      L.allocate(k);
      for (int r = 0; r < k; ++r) {
        for (int c = 0; c <= r; ++c) L.setValMatrix(r, c, 1.0);
        L.setValRHS(r, 1.0);
      }
      L.assemble();
      std::vector<double> sol;
      L.solve(&sol);
      for (int r = 0; r < k; ++r) CHECK(std::fabs(sol[r] - (r == 0 ? 1.0 : 0.0)) < 1e-12);
    }
  }
  {  // HDGSolver setup sequence and the constant Dirichlet solve (TestHDGSolver.cpp:14-101)
    Mesh m;
    m.dim = 2;
    m.order = 2;
    // 4x4 squares, two triangles each, p=2 nodes built from the reference nodes
    const int n = 4;
    hfx_refel_info info;
    hfx_refel_query(2, 2, &info);
    std::vector<double> rn(info.nNodes * 2);
    hfx_refel_tables(2, 2, rn.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    std::vector<double> pts;
    std::vector<int> cells;
    auto node_id = [&](double x, double y) {
      for (size_t k = 0; k < pts.size() / 2; ++k)
        if (std::fabs(pts[2 * k] - x) < 1e-12 && std::fabs(pts[2 * k + 1] - y) < 1e-12) return (int)k;
      pts.push_back(x);
      pts.push_back(y);
      return (int)(pts.size() / 2 - 1);
    };
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double h = 1.0 / n, x0 = i * h, y0 = j * h;
        double tri[2][3][2] = {{{x0, y0}, {x0 + h, y0}, {x0, y0 + h}}, {{x0 + h, y0 + h}, {x0, y0 + h}, {x0 + h, y0}}};
        for (auto& t : tri)
          for (int a = 0; a < info.nNodes; ++a) {
            double l1 = 0.5 * (rn[2 * a] + 1), l2 = 0.5 * (rn[2 * a + 1] + 1);
            double x = t[0][0] + l1 * (t[1][0] - t[0][0]) + l2 * (t[2][0] - t[0][0]);
            double y = t[0][1] + l1 * (t[1][1] - t[0][1]) + l2 * (t[2][1] - t[0][1]);
            cells.push_back(node_id(x, y));
          }
      }
    m.nodes = pts;
    m.cells = cells;
    Field sol(&m, Cell, info.nNodes, 1), flux(&m, Cell, info.nNodes, 2);
    Field dir(&m, Face, info.nNodesFace, 1), lambda(&m, Face, info.nNodesFace, 1), tau(&m, Face, info.nNodesFace, 1);
    std::fill(dir.values.begin(), dir.values.end(), 3.0);
    std::fill(tau.values.begin(), tau.values.end(), 1.0);
    std::map<std::string, Field*> fm;
    DirichletModel dirMod;
    HDGLaplaceModel lap;
    GpuSolverOpts o;
    o.rtol = 1e-14;
    o.maxits = 20000;
    o.method = HFX_KSP_CG;
    GpuHDGSolver s(&dev);
    CHECK(throws([&] { s.solve(); }));
    CHECK(throws([&] { s.assemble(); }));
    CHECK(throws([&] { s.allocate(); }));
    s.setMesh(&m);
    fm["Solution"] = &sol;
    fm["Flux"] = &flux;
    fm["Trace"] = &lambda;
    fm["Dirichlet"] = &dir;
    fm["Tau"] = &tau;
    s.setFieldMap(&fm);
    s.setLinSystem(o);
    s.setModel(&lap);
    CHECK(throws([&] { s.allocate(); }));
    s.setBoundaryModel(&dirMod);
    CHECK(throws([&] { s.allocate(); }));  // not initialized
    s.initialize();
    s.allocate();
    CHECK(throws([&] { s.solve(); }));
    s.assemble();
    s.solve();
    for (double v : sol.values) CHECK(std::fabs(v - 3.0) < 1e-12);
    for (double v : flux.values) CHECK(std::fabs(v) < 1e-11);
    for (double v : lambda.values) CHECK(std::fabs(v - 3.0) < 1e-12);
    // the same solve with the two-level preconditioner, mixed precision and the learned coarse solve
    GpuSolverOpts o2 = o;
    o2.precond = HFX_PC_TWOLEVEL;
    o2.precision = HFX_PREC_MIXED;
    o2.coarseMode = HFX_COARSE_LEARNED;
    o2.learnedDegree = 4;
    o2.rtol = 1e-13;
    GpuHDGSolver s2(&dev);
    s2.setMesh(&m);
    s2.setFieldMap(&fm);
    s2.setLinSystem(o2);
    s2.setModel(&lap);
    s2.setBoundaryModel(&dirMod);
    s2.initialize();
    s2.allocate();
    s2.assemble();
    s2.solve();
    CHECK(s2.lastInfo.status == 0 && s2.lastInfo.fallback == 0);
    for (double v : sol.values) CHECK(std::fabs(v - 3.0) < 1e-11);
    for (double v : lambda.values) CHECK(std::fabs(v - 3.0) < 1e-11);

    // RungeKutta through the host API (TestHDGDiffusionSource.cpp:213-249 loop): the
    // steady state Solution = Trace = 3, Flux = 0 is a fixed point of every scheme
    // (dt within RK4's explicit stability limit on this mesh: rounding must not grow)
    RungeKutta ts(RK4);
    CHECK(ts.getNumStages() == 4);
    CHECK(throws([&] { ts.setButcherTable(std::vector<double>(4, 1.0), 2, 2); }));
    CHECK(throws([&] { ts.computeSolution(&fm); }));
    ts.setTimeStep(1e-3);
    HDGLaplaceModel lapT;
    lapT.setTimeScheme(&ts);
    GpuHDGSolver s3(&dev);
    s3.setMesh(&m);
    s3.setFieldMap(&fm);
    s3.setLinSystem(o);
    s3.setModel(&lapT);
    s3.setBoundaryModel(&dirMod);
    s3.initialize();
    s3.allocate();
    for (int step = 0; step < 2; ++step) {
      for (int k = 0; k < ts.getNumStages(); ++k) {
        s3.assemble();
        s3.solve();
        ts.computeStage(&fm);
      }
      CHECK(throws([&] { ts.computeStage(&fm); }));
      ts.computeSolution(&fm);
      CHECK(ts.getStage() == 0);
    }
    for (double v : sol.values) CHECK(std::fabs(v - 3.0) < 1e-10);
    for (double v : lambda.values) CHECK(std::fabs(v - 3.0) < 1e-10);
    for (double v : flux.values) CHECK(std::fabs(v) < 1e-9);
  }
  {  // NonLinearWrapper with a user linearised solver (TestNonLinearWrapper.cpp:10-47):
     // x <- x - x^2 / (2x) halves x, the relative change stays 1/2, max iterations end the loop
    Mesh m;
    m.dim = 2;
    m.order = 1;
    m.nodes = {0, 0, 1, 0, 0, 1};
    m.cells = {0, 1, 2};
    Field sol(&m, Node, 1, 1), interSol(&m, Node, 1, 1);
    GpuBurgersSolver dummy(&dev);
    NonLinearWrapper wrap;
    CHECK(throws([&] { wrap.solve(); }));
    wrap.setVerbosity(false);
    wrap.setSolver(&dummy);
    CHECK(throws([&] { wrap.solve(); }));
    wrap.setSolutionFields(&sol, &interSol);
    wrap.setLinearizedSolver([&](GpuBurgersSolver*) {
      for (size_t i = 0; i < sol.values.size(); ++i)
        sol.values[i] = interSol.values[i] - interSol.values[i] * interSol.values[i] / (2.0 * interSol.values[i]);
    });
    for (double start : {1.0, 2.0, -1.0, 0.25, 42.0, 1e-8}) {
      std::fill(interSol.values.begin(), interSol.values.end(), start);
      std::fill(sol.values.begin(), sol.values.end(), 0.0);
      wrap.solve();
      CHECK(std::fabs(wrap.getResidual() - 0.5) < 1e-12);
      for (double v : interSol.values) CHECK(std::fabs(v) < 1e-4 * std::max(1.0, std::fabs(start)) * 50);
    }
  }
  {  // stationary Burgers, Cole-Hopf solution (TestHDGBurgersStat.cpp:107-399) through
     // GpuBurgersSolver + NonLinearWrapper: the device loop and the host loop agree
    const int p = 2, n = 4;
    Mesh m;
    m.dim = 2;
    m.order = p;
    hfx_refel_info info;
    hfx_refel_query(2, p, &info);
    std::vector<double> rn(info.nNodes * 2);
    hfx_refel_tables(2, p, rn.data(), nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr);
    auto node_id = [&](double x, double y) {
      for (size_t k = 0; k < m.nodes.size() / 2; ++k)
        if (std::fabs(m.nodes[2 * k] - x) < 1e-12 && std::fabs(m.nodes[2 * k + 1] - y) < 1e-12) return (int)k;
      m.nodes.push_back(x);
      m.nodes.push_back(y);
      return (int)(m.nodes.size() / 2 - 1);
    };
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double h = 1.0 / n, x0 = i * h, y0 = j * h;
        double tri[2][3][2] = {{{x0, y0}, {x0 + h, y0}, {x0, y0 + h}}, {{x0 + h, y0 + h}, {x0, y0 + h}, {x0 + h, y0}}};
        for (auto& t : tri)
          for (int a = 0; a < info.nNodes; ++a) {
            double l1 = 0.5 * (rn[2 * a] + 1), l2 = 0.5 * (rn[2 * a + 1] + 1);
            m.cells.push_back(node_id(t[0][0] + l1 * (t[1][0] - t[0][0]) + l2 * (t[2][0] - t[0][0]),
                                      t[0][1] + l1 * (t[1][1] - t[0][1]) + l2 * (t[2][1] - t[0][1])));
          }
      }
    const double D = 1.0, A = 0.5;
    auto exact = [&](double x, double y, double* u) {
      const double ep = std::exp(A * (x - 1.0)), em = std::exp(-A * (x - 1.0));
      const double phi = 0.001 * A * std::exp(2.0 * A) * (1 + x) + (ep + em) * std::cos(A * y);
      u[0] = -2 * D * (0.001 * A * std::exp(2.0 * A) + A * (ep - em) * std::cos(A * y)) / phi;
      u[1] = -2 * D * (-A * (ep + em) * std::sin(A * y)) / phi;
    };
    Field sol(&m, Cell, info.nNodes, 2), buf(&m, Cell, info.nNodes, 2), flux(&m, Cell, info.nNodes, 4);
    Field trace(&m, Face, info.nNodesFace, 2), dir(&m, Face, info.nNodesFace, 2), tau(&m, Face, info.nNodesFace, 8);
    Field nu(&m, Node, 1, 1);
    std::fill(nu.values.begin(), nu.values.end(), D);
    for (int f = 0; f < m.nFaces; ++f)
      for (int a = 0; a < info.nNodesFace; ++a) {
        const int node = m.faces[(size_t)f * info.nNodesFace + a];
        exact(m.nodes[2 * node], m.nodes[2 * node + 1], &dir.values[((size_t)f * info.nNodesFace + a) * 2]);
        for (int side = 0; side < 2; ++side) {
          double* t = &tau.values[(((size_t)f * info.nNodesFace + a) * 2 + side) * 4];
          t[0] = t[3] = 2.0 * D * n;  // (D / h) * 2 * I
        }
      }
    std::map<std::string, Field*> fm{{"Solution", &sol}, {"BufferSolution", &buf}, {"Flux", &flux},
                                     {"Trace", &trace}, {"Tau", &tau}, {"Dirichlet", &dir},
                                     {"DiffusionTensor", &nu}};
    DirichletModel dirMod;
    HDGBurgersModel bm;
    GpuSolverOpts o;
    o.precond = HFX_PC_BLOCK_JACOBI;
    o.rtol = 1e-13;
    o.maxits = 20000;
    GpuBurgersSolver s(&dev);
    CHECK(throws([&] { s.assemble(); }));
    s.setMesh(&m);
    s.setFieldMap(&fm);
    s.setLinSystem(o);
    s.setModel(&bm);
    s.setBoundaryModel(&dirMod);
    s.initialize();
    s.allocate();
    NonLinearWrapper w;
    w.setSolver(&s);
    w.setSolutionFields(&sol, &buf);
    w.setMaxIterations(10);
    w.setResidualTolerance(1e-8);
    w.solve();  // vanilla: the loop runs on the device
    CHECK(w.lastInfo.iterations > 1 && w.lastInfo.iterations < 10 && w.getResidual() < 1e-8);
    std::vector<double> devSol = sol.values;
    double err2 = 0.0, ref2 = 0.0;
    for (int e = 0; e < m.numCells(); ++e)
      for (int a = 0; a < info.nNodes; ++a) {
        const int node = m.cells[(size_t)e * info.nNodes + a];
        double u[2];
        exact(m.nodes[2 * node], m.nodes[2 * node + 1], u);
        for (int k = 0; k < 2; ++k) {
          const double d = sol.values[((size_t)e * info.nNodes + a) * 2 + k] - u[k];
          err2 += d * d;
          ref2 += u[k] * u[k];
        }
      }
    CHECK(std::sqrt(err2 / ref2) < 1e-3);  // the reference asserts l2Err < 1
    // the same loop on the host (a user residual computer selects it)
    std::fill(sol.values.begin(), sol.values.end(), 0.0);
    std::fill(buf.values.begin(), buf.values.end(), 0.0);
    std::fill(trace.values.begin(), trace.values.end(), 0.0);
    NonLinearWrapper wh;
    wh.setSolver(&s);
    wh.setSolutionFields(&sol, &buf);
    wh.setMaxIterations(10);
    wh.setResidualTolerance(1e-8);
    wh.setResidualComputer(NonLinearWrapper::vanillaResidual);
    wh.solve();
    double dmax = 0.0, smax = 0.0;
    for (size_t i = 0; i < sol.values.size(); ++i) {
      dmax = std::max(dmax, std::fabs(sol.values[i] - devSol[i]));
      smax = std::max(smax, std::fabs(devSol[i]));
    }
    CHECK(dmax < 1e-10 * smax);
    CHECK(std::fabs(wh.getResidual() - w.getResidual()) < 1e-3 * w.getResidual() + 1e-12);
  }
  std::printf("%s (%d failures)\n", failures ? "FAIL" : "OK", failures);
  return failures ? 1 : 0;
}
