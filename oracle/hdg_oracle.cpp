// HDG oracle: TEST INFRASTRUCTURE ONLY.
//
// A CPU, FP64, single-file restatement of HyperFox's HDG element-local path and
// the trace solve behind it. Only the tests, the smoke check and the bench's CPU
// baseline load it, always as the reference the CUDA path is compared with; the
// CUDA library never links it.
//
// Every function names the HyperFox file:line it restates. The reference
// cannot be built here (Eigen, Boost.Math, PETSc, MOAB are absent), so parity
// is pinned through the reference's own known-answer tests (re-expressed in
// tests/test_oracle_*.py) and, for the cubature tables, through the reference's
// own Cubature.cpp compiled by oracle/build_ref.sh. Face numbering follows the
// MOAB creation-order rule restated below and is "parity unpinned" against a
// real MOAB build (no reference test pins face order).
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <set>
#include <stdexcept>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../hyperfox_gb300/csrc/cubature_tables.inc"

namespace orc {

// ---------------------------------------------------------------- dense helpers
// Column-major dense matrix (the reference's EMatrix is column-major Eigen).
struct Mat {
  int r = 0, c = 0;
  std::vector<double> a;
  Mat() {}
  Mat(int r_, int c_) : r(r_), c(c_), a((size_t)r_ * c_, 0.0) {}
  double& operator()(int i, int j) { return a[i + (size_t)j * r]; }
  double operator()(int i, int j) const { return a[i + (size_t)j * r]; }
};

// LU with partial pivoting, in place. Returns false on an exactly singular pivot.
static bool lu_factor(Mat& A, std::vector<int>& piv) {
  int n = A.r;
  piv.resize(n);
  for (int k = 0; k < n; ++k) {
    int p = k;
    double best = std::fabs(A(k, k));
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A(i, k)) > best) { best = std::fabs(A(i, k)); p = i; }
    piv[k] = p;
    if (best == 0.0) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) std::swap(A(k, j), A(p, j));
    double inv = 1.0 / A(k, k);
    for (int i = k + 1; i < n; ++i) A(i, k) *= inv;
    for (int j = k + 1; j < n; ++j) {
      double akj = A(k, j);
      if (akj == 0.0) continue;
      for (int i = k + 1; i < n; ++i) A(i, j) -= A(i, k) * akj;
    }
  }
  return true;
}

// Solve A X = B in place in B (B is n x m) with a factored A.
static void lu_solve(const Mat& LU, const std::vector<int>& piv, Mat& B) {
  int n = LU.r;
  for (int col = 0; col < B.c; ++col) {
    double* b = &B.a[(size_t)col * n];
    for (int k = 0; k < n; ++k) std::swap(b[k], b[piv[k]]);
    for (int k = 0; k < n; ++k)
      for (int i = k + 1; i < n; ++i) b[i] -= LU(i, k) * b[k];
    for (int k = n - 1; k >= 0; --k) {
      b[k] /= LU(k, k);
      for (int i = 0; i < k; ++i) b[i] -= LU(i, k) * b[k];
    }
  }
}

static Mat inverse(const Mat& A) {
  Mat LU = A;
  std::vector<int> piv;
  if (!lu_factor(LU, piv)) throw std::runtime_error("singular matrix");
  Mat I(A.r, A.r);
  for (int i = 0; i < A.r; ++i) I(i, i) = 1.0;
  lu_solve(LU, piv, I);
  return I;
}

static double det_small(const Mat& A) {
  Mat LU = A;
  std::vector<int> piv;
  if (!lu_factor(LU, piv)) return 0.0;
  double d = 1.0;
  for (int k = 0; k < A.r; ++k) {
    d *= LU(k, k);
    if (piv[k] != k) d = -d;
  }
  return d;
}

// C = alpha*A*B + beta*C (all column-major)
static void gemm(double alpha, const Mat& A, const Mat& B, double beta, Mat& C) {
  for (int j = 0; j < C.c; ++j)
    for (int i = 0; i < C.r; ++i) {
      double s = 0.0;
      for (int k = 0; k < A.c; ++k) s += A(i, k) * B(k, j);
      C(i, j) = alpha * s + beta * C(i, j);
    }
}

static Mat block(const Mat& A, int r0, int c0, int nr, int nc) {
  Mat B(nr, nc);
  for (int j = 0; j < nc; ++j)
    for (int i = 0; i < nr; ++i) B(i, j) = A(r0 + i, c0 + j);
  return B;
}

// ------------------------------------------------------ Jacobi polynomials
// Standard Jacobi polynomials P_n^{(a,b)} by the three-term recurrence, as
// Boost.Math's jacobi() used at ReferenceElement.cpp:280-310 defines them.
static double jacobi(int n, double a, double b, double x) {
  if (n == 0) return 1.0;
  double p0 = 1.0, p1 = (a + 1.0) + (a + b + 2.0) * (x - 1.0) / 2.0;
  for (int k = 2; k <= n; ++k) {
    double c1 = 2.0 * k * (k + a + b) * (2.0 * k + a + b - 2.0);
    double c2 = (2.0 * k + a + b - 1.0) * ((2.0 * k + a + b) * (2.0 * k + a + b - 2.0) * x + a * a - b * b);
    double c3 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * (2.0 * k + a + b);
    double p2 = (c2 * p1 - c3 * p0) / c1;
    p0 = p1;
    p1 = p2;
  }
  return p1;
}
// First derivative (Boost.Math jacobi_derivative(n,a,b,x,1)).
static double jacobi_d(int n, double a, double b, double x) {
  if (n == 0) return 0.0;
  return 0.5 * (n + a + b + 1.0) * jacobi(n - 1, a + 1.0, b + 1.0, x);
}

// Gauss-Lobatto-Legendre interior points (roots of P'_p), ascending.
static std::vector<double> gll_interior(int p) {
  std::vector<double> r;
  for (int k = 1; k < p; ++k) {
    double x = -std::cos(M_PI * k / p);
    for (int it = 0; it < 100; ++it) {
      // P'_p roots = roots of P_{p-1}^{(1,1)}
      double f = jacobi(p - 1, 1.0, 1.0, x);
      double df = jacobi_d(p - 1, 1.0, 1.0, x);
      double dx = f / df;
      x -= dx;
      if (std::fabs(dx) < 1e-17) break;
    }
    r.push_back(x);
  }
  std::sort(r.begin(), r.end());
  return r;
}

// Gauss-Legendre rule with n points, in the point order Cubature.cpp:109-280 lists.
static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
  std::vector<double> pos;  // positive roots ascending
  for (int k = 1; k <= n; ++k) {
    double t = std::cos(M_PI * (k - 0.25) / (n + 0.5));
    for (int it = 0; it < 100; ++it) {
      double f = jacobi(n, 0, 0, t), df = jacobi_d(n, 0, 0, t);
      double dt = f / df;
      t -= dt;
      if (std::fabs(dt) < 1e-17) break;
    }
    if (t > 1e-14) pos.push_back(t);
  }
  std::sort(pos.begin(), pos.end());
  // signed indices into pos (1-based), 0 = the zero root
  static const std::vector<std::vector<int>> order = {
      {}, {0}, {-1, 1}, {0, -1, 1}, {1, -1, 2, -2}, {0, 1, -1, 2, -2},
      {2, -2, -1, 1, -3, 3}, {0, 1, -1, -2, 2, -3, 3}, {-1, 1, -2, 2, -3, 3, -4, 4},
      {0, -3, 3, -4, 4, -1, 1, -2, 2}, {-1, 1, -2, 2, -3, 3, -4, 4, -5, 5},
      {0, -1, 1, -2, 2, -3, 3, -4, 4, -5, 5}};
  if (n < 1 || n > 11) throw std::runtime_error("Gauss-Legendre size");
  x.clear();
  w.clear();
  for (int s : order[n]) {
    double t = (s == 0) ? 0.0 : (s > 0 ? pos[s - 1] : -pos[-s - 1]);
    double dp = jacobi_d(n, 0, 0, t);
    x.push_back(t);
    w.push_back(2.0 / ((1.0 - t * t) * dp * dp));
  }
}

// Simplex cubature of a given polynomial order (Cubature.cpp nIPMap).
static void simplex_cubature(int dim, int order, std::vector<std::vector<double>>& X,
                             std::vector<double>& W) {
  X.clear();
  W.clear();
  if (dim == 1) {
    std::vector<double> x, w;
    int n = (int)std::ceil((order + 1.0) / 2.0);
    gauss_legendre(n, x, w);
    for (size_t i = 0; i < x.size(); ++i) {
      X.push_back({x[i]});
      W.push_back(w[i]);
    }
    return;
  }
  for (int k = 0; k < kNumCubatureRules; ++k) {
    const auto& e = kCubatureRules[k];
    if (e.dim == dim && e.order == order) {
      for (int i = 0; i < e.npts; ++i) {
        std::vector<double> p(dim);
        for (int d = 0; d < dim; ++d) p[d] = e.data[i * (dim + 1) + d];
        X.push_back(p);
        W.push_back(e.data[i * (dim + 1) + dim]);
      }
      return;
    }
  }
  throw std::runtime_error("cubature order not tabulated");
}

// ------------------------------------------------------ reference element
using NodeList = std::vector<std::vector<double>>;
using FaceList = std::vector<std::vector<int>>;

// Principal vertices and face lists (ReferenceElement.cpp:1012-1060).
static void simplex_topology(int dim, NodeList& nodes, FaceList& faces) {
  if (dim == 1) {
    nodes = {{-1.0}, {1.0}};
    faces = {{0}, {1}};
  } else if (dim == 2) {
    nodes = {{-1.0, -1.0}, {1.0, -1.0}, {-1.0, 1.0}};
    faces = {{0, 1}, {1, 2}, {2, 0}};
  } else {
    nodes = {{-1.0, -1.0, -1.0}, {1.0, -1.0, -1.0}, {-1.0, 1.0, -1.0}, {-1.0, -1.0, 1.0}};
    faces = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 1}, {3, 2},
             {3, 1, 0}, {2, 1, 3}, {2, 3, 0}, {0, 1, 2}};
  }
}

static std::vector<std::vector<int>> combos_with_repetition(const std::vector<int>& set, int size) {
  // ReferenceElement.cpp:577-610: Cartesian product, first position slowest.
  std::vector<std::vector<int>> out;
  if (size == 1) {
    for (int v : set) out.push_back({v});
    return out;
  }
  auto inner = combos_with_repetition(set, size - 1);
  for (int v : set)
    for (auto& c : inner) {
      std::vector<int> n(1, v);
      n.insert(n.end(), c.begin(), c.end());
      out.push_back(n);
    }
  return out;
}

static NodeList remove_duplicates(const NodeList& v) {
  // ReferenceElement.cpp:1159-1183: keep first occurrences (tolerance 1e-12).
  std::set<int> dup;
  int s = (int)v.size();
  for (int i = 0; i < s; ++i)
    for (int j = i + 1; j < s; ++j) {
      bool isDup = true;
      for (size_t d = 0; d < v[i].size(); ++d)
        if (!(std::fabs(v[i][d] - v[j][d]) < 1e-12)) { isDup = false; break; }
      if (isDup) dup.insert(j);
    }
  NodeList r;
  for (int i = 0; i < s; ++i)
    if (!dup.count(i)) r.push_back(v[i]);
  return r;
}

static std::map<std::pair<int, int>, NodeList> g_nodeDB;

// Node database (ReferenceElement.cpp:614-1150): Lobatto points in 1D, the
// recursive simplex construction with the warped interior formula in 2D/3D.
static const NodeList& node_db(int dim, int p) {
  auto key = std::make_pair(dim, p);
  auto it = g_nodeDB.find(key);
  if (it != g_nodeDB.end()) return it->second;
  NodeList val;
  if (dim == 1) {
    if (p == 0) val = {{0.0}};
    else {
      val = {{-1.0}, {1.0}};
      for (double x : gll_interior(p)) val.push_back({x});
    }
  } else if (p == 0) {
    val = {std::vector<double>(dim, 0.0)};
  } else {
    NodeList principal;
    FaceList faceList;
    simplex_topology(dim, principal, faceList);
    val = principal;
    for (int q = 1; q < dim; ++q) {
      NodeList nm1;
      FaceList dummy;
      simplex_topology(q, nm1, dummy);
      Mat inter(q, q);
      for (int k = 0; k < q; ++k)
        for (int l = 0; l < q; ++l) inter(k, l) = nm1[l + 1][k] - nm1[0][k];
      Mat invInter = inverse(inter);
      const NodeList fen = node_db(q, p);
      for (auto& face : faceList) {
        if ((int)face.size() != (int)nm1.size()) continue;
        Mat T(dim, q);
        for (int l = 0; l < q; ++l)
          for (int d = 0; d < dim; ++d) T(d, l) = principal[face[l + 1]][d] - principal[face[0]][d];
        Mat Ti(dim, q);
        gemm(1.0, T, invInter, 0.0, Ti);
        for (auto& fn : fen) {
          std::vector<double> nv(dim);
          for (int d = 0; d < dim; ++d) {
            double s = 0.0;
            for (int l = 0; l < q; ++l) s += Ti(d, l) * (fn[l] - nm1[0][l]);
            nv[d] = s + principal[face[0]][d];
          }
          val.push_back(nv);
        }
      }
    }
    int nFaceNodes = (int)val.size();
    if (p > 1) {
      const NodeList& one = node_db(1, p);
      std::vector<double> L;
      for (int k = 0; k < p + 1; ++k) L.push_back(one[k][0]);
      double endCorner = L[1];
      L.erase(L.begin() + 1);
      L.push_back(endCorner);
      std::vector<int> idx;
      for (int k = 1; k < p; ++k) idx.push_back(k);
      auto combos = combos_with_repetition(idx, dim);
      std::vector<std::vector<int>> reduced;
      for (auto& c : combos) {
        int s = 0;
        for (int v : c) s += v;
        if (s < p) reduced.push_back(c);
      }
      std::map<std::vector<int>, double> coef;
      for (auto& c : reduced) {
        int s = 0;
        for (int v : c) s += v;
        double cf = 2.0 + dim * L[c[0]];
        for (int l = 1; l < dim; ++l) cf -= L[c[l]];
        cf -= L[p - s];
        cf *= 1.0 / (dim + 1.0);
        cf -= 1.0;
        coef[c] = cf;
      }
      val.resize(nFaceNodes + reduced.size());
      for (size_t k = 0; k < reduced.size(); ++k) {
        auto& c = reduced[k];
        std::vector<double> nv(dim);
        if (dim == 2) {
          nv[0] = coef[c];
          nv[1] = coef[{c[1], c[0]}];
        } else {
          nv[0] = coef[c];
          nv[1] = coef[{c[1], c[0], c[2]}];
          nv[2] = coef[{c[2], c[1], c[0]}];
        }
        val[nFaceNodes + k] = nv;
      }
    }
    val = remove_duplicates(val);
  }
  g_nodeDB[key] = val;
  return g_nodeDB[key];
}

struct RefEl {
  int dim = 0, order = 0, nNodes = 0, nFaces = 0, nIP = 0;
  NodeList nodes;
  FaceList faceNodes;
  std::vector<std::vector<int>> modes;
  Mat invV;
  NodeList ipX;
  std::vector<double> ipW;
  NodeList phi;                                  // [ip][node]
  std::vector<std::vector<std::vector<double>>> dphi;  // [ip][node][dim]
  RefEl* face = nullptr;
  ~RefEl() { delete face; }

  std::vector<double> mapped(const std::vector<double>& x) const {
    // ReferenceElement.cpp:232-265 (collapsed coordinates)
    std::vector<double> m(dim);
    if (dim == 1) m = x;
    else if (dim == 2) {
      m[0] = (x[1] != 1.0) ? 2.0 * (1.0 + x[0]) / (1.0 - x[1]) - 1.0 : -1.0;
      m[1] = x[1];
    } else {
      m[0] = ((x[1] + x[2]) != 0.0) ? -2.0 * (1.0 + x[0]) / (x[1] + x[2]) - 1.0 : -1.0;
      m[1] = (x[2] != 1.0) ? 2.0 * (1.0 + x[1]) / (1.0 - x[2]) - 1.0 : -1.0;
      m[2] = x[2];
    }
    return m;
  }

  // Dubiner modes at a point (ReferenceElement.cpp:267-316).
  std::vector<double> compute_modes(const std::vector<double>& x) const {
    std::vector<double> res(nNodes, 1.0);
    auto m = mapped(x);
    for (int j = 0; j < nNodes; ++j) {
      const auto& md = modes[j];
      for (int k = 0; k < dim; ++k) {
        if (k == 0) res[j] *= jacobi(md[0], 0.0, 0.0, m[0]);
        else if (k == 1)
          res[j] *= std::sqrt(2.0) * jacobi(md[1], 2.0 * md[0] + 1.0, 0.0, m[1]) * std::pow(1 - m[1], md[0]);
        else
          res[j] *= 2.0 * jacobi(md[2], 2.0 * (md[1] + md[0] + 1.0), 0.0, m[2]) *
                    std::pow(1 - m[2], md[1] + md[0]);
      }
    }
    return res;
  }

  // Gradients of the modes (ReferenceElement.cpp:319-445).
  std::vector<std::vector<double>> compute_dmodes(const std::vector<double>& x) const {
    std::vector<std::vector<double>> res(nNodes, std::vector<double>(dim, 1.0));
    auto m = mapped(x);
    Mat J(dim, dim);
    const double eps = 1e-6;
    if (dim == 1) J(0, 0) = 1.0;
    else if (dim == 2) {
      if (x[1] != 1.0) {
        J(0, 0) = 2.0 / (1.0 - x[1]);
        J(1, 0) = 2.0 * (1.0 + x[0]) * (1.0 / std::pow(1.0 - x[1], 2.0));
      } else {
        J(0, 0) = 2.0 / eps;
        J(1, 0) = 0.0;
      }
      J(0, 1) = 0.0;
      J(1, 1) = 1.0;
    } else {
      if ((x[1] + x[2]) != 0.0) {
        J(0, 0) = -2.0 / (x[1] + x[2]);
        J(1, 0) = 2.0 * (1.0 + x[0]) * (1.0 / std::pow(x[1] + x[2], 2.0));
        J(2, 0) = 2.0 * (1.0 + x[0]) * (1.0 / std::pow(x[1] + x[2], 2.0));
      } else {
        J(0, 0) = -2.0 / eps;
        J(1, 0) = 0.0;
        J(2, 0) = 0.0;
      }
      if (x[2] != 1.0) {
        J(1, 1) = 2.0 / (1.0 - x[2]);
        J(2, 1) = 2.0 * (1.0 + x[1]) * (1.0 / std::pow(1.0 - x[2], 2.0));
      } else {
        J(1, 1) = 2.0 / eps;
        J(2, 1) = 0.0;
      }
      J(0, 1) = 0.0;
      J(0, 2) = 0.0;
      J(1, 2) = 0.0;
      J(2, 2) = 1.0;
    }
    for (int j = 0; j < nNodes; ++j) {
      const auto& md = modes[j];
      std::vector<double> g(dim, 1.0);
      for (int k = 0; k < dim; ++k)
        for (int l = 0; l < dim; ++l) {
          if (l == 0) {
            g[k] *= (l != k) ? jacobi(md[0], 0.0, 0.0, m[0]) : jacobi_d(md[0], 0.0, 0.0, m[0]);
          } else if (l == 1) {
            if (l != k)
              g[k] *= std::sqrt(2.0) * jacobi(md[1], 2.0 * md[0] + 1.0, 0.0, m[1]) * std::pow(1 - m[1], md[0]);
            else {
              int power = std::max(md[0] - 1, 0);
              g[k] *= std::sqrt(2.0) * jacobi_d(md[1], 2.0 * md[0] + 1.0, 0.0, m[1]) * std::pow(1 - m[1], md[0]) +
                      std::sqrt(2.0) * jacobi(md[1], 2.0 * md[0] + 1.0, 0.0, m[1]) *
                          (-md[0] * std::pow(1 - m[1], power));
            }
          } else {
            double a2 = 2.0 * (md[1] + md[0] + 1.0);
            if (k != l)
              g[k] *= 2.0 * jacobi(md[2], a2, 0.0, m[2]) * std::pow(1 - m[2], md[1] + md[0]);
            else {
              int power = std::max(md[1] + md[0] - 1, 0);
              g[k] *= 2.0 * jacobi_d(md[2], a2, 0.0, m[2]) * std::pow(1 - m[2], md[1] + md[0]) +
                      2.0 * jacobi(md[2], a2, 0.0, m[2]) * (-(md[1] + md[0]) * std::pow(1 - m[2], power));
            }
          }
        }
      std::vector<double> gg(dim, 0.0);
      for (int a = 0; a < dim; ++a)
        for (int b = 0; b < dim; ++b) gg[a] += J(a, b) * g[b];
      res[j] = gg;
    }
    return res;
  }

  std::vector<double> interpolate(const std::vector<double>& x) const {
    auto mv = compute_modes(x);
    std::vector<double> r(nNodes, 0.0);
    for (int j = 0; j < nNodes; ++j)
      for (int i = 0; i < nNodes; ++i) r[j] += mv[i] * invV(i, j);
    return r;
  }
  std::vector<std::vector<double>> interpolate_d(const std::vector<double>& x) const {
    auto dm = compute_dmodes(x);
    std::vector<std::vector<double>> r(nNodes, std::vector<double>(dim, 0.0));
    for (int k = 0; k < dim; ++k)
      for (int j = 0; j < nNodes; ++j)
        for (int i = 0; i < nNodes; ++i) r[j][k] += dm[i][k] * invV(i, j);
    return r;
  }

  RefEl(int dim_, int p) : dim(dim_), order(p) {
    // ReferenceElement.cpp:5-26 (simplex only)
    nodes = node_db(dim, p);
    nNodes = (int)nodes.size();
    nFaces = dim + 1;
    simplex_cubature(dim, 2 * p, ipX, ipW);
    nIP = (int)ipX.size();
    if (dim > 1) face = new RefEl(dim - 1, p);
    // face nodes (ReferenceElement.cpp:136-202)
    faceNodes.assign(nFaces, {});
    if (dim == 1) {
      faceNodes[0] = {0};
      faceNodes[1] = {1};
    } else {
      NodeList nm1, principal;
      FaceList dummy, faceList;
      simplex_topology(dim - 1, nm1, dummy);
      simplex_topology(dim, principal, faceList);
      Mat inter(dim - 1, dim - 1);
      for (int k = 0; k < dim - 1; ++k)
        for (int l = 0; l < dim - 1; ++l) inter(k, l) = nm1[l + 1][k] - nm1[0][k];
      Mat invInter = inverse(inter);
      int fi = 0;
      for (auto& fl : faceList) {
        if (fl.size() != nm1.size()) continue;
        Mat T(dim, dim - 1);
        for (int l = 0; l < dim - 1; ++l)
          for (int d = 0; d < dim; ++d) T(d, l) = principal[fl[l + 1]][d] - principal[fl[0]][d];
        Mat Ti(dim, dim - 1);
        gemm(1.0, T, invInter, 0.0, Ti);
        for (auto& fn : face->nodes) {
          std::vector<double> nv(dim);
          for (int d = 0; d < dim; ++d) {
            double s = 0.0;
            for (int l = 0; l < dim - 1; ++l) s += Ti(d, l) * (fn[l] - nm1[0][l]);
            nv[d] = s + principal[fl[0]][d];
          }
          int found = -1;
          for (int n = 0; n < nNodes && found < 0; ++n) {
            bool eq = true;
            for (int d = 0; d < dim; ++d)
              if (std::fabs(nodes[n][d] - nv[d]) > 1e-12) { eq = false; break; }
            if (eq) found = n;
          }
          if (found < 0) throw std::runtime_error("face node not found");
          faceNodes[fi].push_back(found);
        }
        ++fi;
      }
    }
    // node to mode map (ReferenceElement.cpp:204-218)
    std::vector<int> ords;
    for (int k = 0; k <= p; ++k) ords.push_back(k);
    for (auto& c : combos_with_repetition(ords, dim)) {
      int s = 0;
      for (int v : c) s += v;
      if (s <= p) modes.push_back(c);
    }
    // inverse Vandermonde (ReferenceElement.cpp:447-455)
    Mat V(nNodes, nNodes);
    for (int i = 0; i < nNodes; ++i) {
      auto row = compute_modes(nodes[i]);
      for (int j = 0; j < nNodes; ++j) V(i, j) = row[j];
    }
    invV = inverse(V);
    for (int i = 0; i < nIP; ++i) {
      phi.push_back(interpolate(ipX[i]));
      dphi.push_back(interpolate_d(ipX[i]));
    }
  }
};

static std::map<std::pair<int, int>, RefEl*> g_refels;
static RefEl* get_refel(int dim, int p) {
  auto k = std::make_pair(dim, p);
  auto it = g_refels.find(k);
  if (it != g_refels.end()) return it->second;
  RefEl* r = new RefEl(dim, p);
  g_refels[k] = r;
  return r;
}

// ------------------------------------------------------------------ mesh faces
// Restatement of Mesh::computeFaces (Mesh.cpp:183-274) without MOAB. MOAB creates
// a missing face the first time a cell asks for its sides, cell by cell in handle
// order, sides in MOAB's canonical order (triangle edges (0,1),(1,2),(2,0); tet
// faces (0,1,3),(1,2,3),(0,3,2),(0,2,1)); face IDs are creation order.
struct MeshFaces {
  int nFaces = 0;
  std::vector<int> cell2face, face2cell, faces, boundary;
};

static MeshFaces compute_faces(int dim, int order, int nCells, const int* cells) {
  RefEl* re = get_refel(dim, order);
  RefEl* skel = get_refel(dim, 1);
  int N = re->nNodes, F = re->nFaces, Nf = re->face->nNodes;
  static const int tri[3][2] = {{0, 1}, {1, 2}, {2, 0}};
  static const int tet[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};
  MeshFaces m;
  std::map<std::vector<int>, int> lookup;
  std::vector<std::vector<int>> adj;
  m.cell2face.assign((size_t)nCells * F, -1);
  for (int c = 0; c < nCells; ++c) {
    for (int s = 0; s < F; ++s) {
      std::vector<int> loc(dim);
      for (int k = 0; k < dim; ++k) loc[k] = (dim == 2) ? tri[s][k] : tet[s][k];
      std::vector<int> key(dim);
      for (int k = 0; k < dim; ++k) key[k] = cells[(size_t)c * N + loc[k]];
      std::sort(key.begin(), key.end());
      int id;
      auto it = lookup.find(key);
      if (it == lookup.end()) {
        id = m.nFaces++;
        lookup[key] = id;
        adj.push_back({});
      } else id = it->second;
      adj[id].push_back(c);
      // Mesh::getFaceIndex (Mesh.cpp:454-494): first skeleton face holding all vertices
      int index = -1;
      for (int i = 0; i < F && index < 0; ++i) {
        bool isFace = true;
        for (int k = 0; k < dim; ++k)
          if (std::find(skel->faceNodes[i].begin(), skel->faceNodes[i].end(), loc[k]) ==
              skel->faceNodes[i].end()) { isFace = false; break; }
        if (isFace) index = i;
      }
      m.cell2face[(size_t)c * F + index] = id;
    }
  }
  // Mesh::computeFace2CellMap (Mesh.cpp:377-402): lower cell first, -1 on the boundary
  m.face2cell.assign((size_t)m.nFaces * 2, -1);
  for (int f = 0; f < m.nFaces; ++f) {
    std::sort(adj[f].begin(), adj[f].end());
    m.face2cell[2 * f] = adj[f][0];
    if (adj[f].size() == 2) m.face2cell[2 * f + 1] = adj[f][1];
    else m.boundary.push_back(f);  // Mesh::computeBoundary (Mesh.cpp:496-511), sorted
  }
  // Mesh::computeFaceConnectivity (Mesh.cpp:517-537): from the first adjacent cell
  m.faces.assign((size_t)m.nFaces * Nf, -1);
  for (int f = 0; f < m.nFaces; ++f) {
    int c = m.face2cell[2 * f];
    int loc = 0;
    while (m.cell2face[(size_t)c * F + loc] != f) ++loc;
    for (int j = 0; j < Nf; ++j) m.faces[(size_t)f * Nf + j] = cells[(size_t)c * N + re->faceNodes[loc][j]];
  }
  return m;
}

// ------------------------------------------------------------------ problem
struct Problem {
  int dim, order, nNodes, nCells;
  RefEl* re;
  std::vector<double> coords;
  std::vector<int> cells;
  MeshFaces mf;
  // fields
  std::vector<double> tau;  // face field: nFaces*Nf*tauVals
  int tauVals = 1;          // 1 or 2 (double valued)
  std::vector<double> kappa;  // cell-nodal: nCells*N*kc
  int kc = 0;                 // 0 = none, 1 = scalar, dim*dim = tensor
  int srcMode = 0;            // 0 none, 1 values at IPs, 2 d*pi^2*prod sin(pi x)
  std::vector<double> src;    // nCells*nI
  std::vector<double> dirichlet;  // face field nFaces*Nf
  double dt = 0.0;            // > 0: implicit Euler (Euler.cpp:18-34)
  std::vector<double> uOld;   // nCells*N
  // Runge-Kutta stage (RungeKutta::apply, RungeKutta.cpp:90-129): rkDt > 0 turns it
  // on; rkDiag = a_ss; rkOld* = OldSolution/OldFlux/OldTrace; rkComb* = sum_{i<s}
  // a_si RKStage_*_i (cell fields nCells*N, nCells*N*d node-major; face field nFaces*Nf)
  double rkDt = 0.0, rkDiag = 0.0;
  std::vector<double> rkOldU, rkOldQ, rkOldL, rkCombU, rkCombQ, rkCombL;
  // HDGSolverType (HDGSolverOpts.h:6-10): 0 IMPLICIT, 1 WEXPLICIT, 2 SEXPLICIT; the
  // explicit modes build S, S0 from the current Solution and Flux (HDGSolver.cpp:349-354)
  int solverType = 0;
  std::vector<double> solState;   // nCells*N
  std::vector<double> fluxState;  // nCells*N*dim, node-major (i, d)
  // outputs
  int lenU, lenQ, lenL, nloc;
  std::vector<double> S, S0, U, Q, U0, Q0;
  std::vector<int> rowptr, col;
  std::vector<double> val, rhs;
  double t_local = 0, t_bc = 0, t_scatter = 0, t_solve = 0, t_recover = 0;
  int iters = 0;
};

// RungeKutta::apply (RungeKutta.cpp:90-129) on the first lenU rows of A (all n
// columns) and of rhs: uj = dt comb + ut (comb = sum_{i<s} a_si k_i), then
// s = dt s - dt K uj; K = dt a_ss K; K[:, :lenU] += M; s += K ut.
static void rk_apply(Mat& A, std::vector<double>& rhs, int lenU, int n, const Mat& M, const std::vector<double>& ut,
                     const std::vector<double>& comb, double dt, double aDiag) {
  std::vector<double> uj(n);
  for (int j = 0; j < n; ++j) uj[j] = dt * comb[j] + ut[j];
  for (int i = 0; i < lenU; ++i) {
    double kuj = 0.0;
    for (int j = 0; j < n; ++j) kuj += A(i, j) * uj[j];
    rhs[i] = dt * rhs[i] - dt * kuj;
    for (int j = 0; j < n; ++j) A(i, j) *= dt * aDiag;
    for (int j = 0; j < lenU; ++j) A(i, j) += M(i, j);
    double kut = 0.0;
    for (int j = 0; j < n; ++j) kut += A(i, j) * ut[j];
    rhs[i] += kut;
  }
}

// Local matrix + RHS for one element (HDGDiffusionSource::computeLocalMatrix /
// computeLocalRHS, HDGDiffusionSource.cpp:43-85, HDGModel.cpp:35-85).
static void local_system(const Problem& P, int iEl, Mat& A, std::vector<double>& rhs,
                         std::vector<int>* f2cOut = nullptr) {
  const RefEl* re = P.re;
  const RefEl* fe = re->face;
  int d = P.dim, N = re->nNodes, F = re->nFaces, Nf = fe->nNodes, nI = re->nIP, nIf = fe->nIP;
  int lenU = N, lenQ = d * N, startL = lenU + lenQ, n = P.nloc;
  const int* cell = &P.cells[(size_t)iEl * N];
  NodeList X(N, std::vector<double>(d));
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < d; ++k) X[i][k] = P.coords[(size_t)cell[i] * d + k];
  // face2CellMap (HDGSolver.cpp:258-275)
  std::vector<int> facesIn(F), f2c(F * Nf);
  for (int i = 0; i < F; ++i) facesIn[i] = P.mf.cell2face[(size_t)iEl * F + i];
  for (int i = 0; i < F; ++i) {
    const int* face = &P.mf.faces[(size_t)facesIn[i] * Nf];
    for (int j = 0; j < Nf; ++j) {
      int node = cell[re->faceNodes[i][j]];
      int pos = -1;
      for (int q = 0; q < Nf; ++q)
        if (face[q] == node) { pos = q; break; }
      if (pos < 0) throw std::runtime_error("couldn't find cell node in face");
      f2c[i * Nf + j] = pos;
    }
  }
  if (f2cOut) *f2cOut = f2c;
  // tau: double-valued side select then reorder to local order (HDGSolver.cpp:276-326)
  std::vector<double> tauLoc(F * Nf);
  for (int i = 0; i < F; ++i) {
    int f = facesIn[i];
    int side = (P.mf.face2cell[2 * f] == iEl) ? 0 : 1;
    for (int j = 0; j < Nf; ++j) {
      int q = f2c[i * Nf + j];
      tauLoc[i * Nf + j] = P.tau[((size_t)f * Nf + q) * P.tauVals + (P.tauVals == 2 ? side : 0)];
    }
  }
  // Jacobians, measures (Operator.cpp:14-84, HDGModel.cpp:53-85)
  int nJ = nI + F * nIf;
  std::vector<Mat> invJ(nI);
  std::vector<double> dV(nJ);
  for (int q = 0; q < nI; ++q) {
    Mat J(d, d);
    for (int i = 0; i < N; ++i)
      for (int r = 0; r < d; ++r)
        for (int s = 0; s < d; ++s) J(r, s) += re->dphi[q][i][r] * X[i][s];
    dV[q] = re->ipW[q] * det_small(J);
    invJ[q] = inverse(J);
  }
  std::vector<std::vector<double>> normals(F * nIf, std::vector<double>(d));
  for (int f = 0; f < F; ++f) {
    // HDGBase::calcNormals (HDGBase.cpp:34-65)
    int v0 = re->faceNodes[f][0], vn = -1;
    for (int k = 0; k < N; ++k)
      if (std::find(re->faceNodes[f].begin(), re->faceNodes[f].end(), k) == re->faceNodes[f].end()) {
        vn = k;
        break;
      }
    std::vector<double> test(d);
    for (int k = 0; k < d; ++k) test[k] = X[vn][k] - X[v0][k];
    for (int q = 0; q < nIf; ++q) {
      Mat J(d - 1, d);
      for (int i = 0; i < Nf; ++i)
        for (int r = 0; r < d - 1; ++r)
          for (int s = 0; s < d; ++s) J(r, s) += fe->dphi[q][i][r] * X[re->faceNodes[f][i]][s];
      Mat JJt(d - 1, d - 1);
      for (int a = 0; a < d - 1; ++a)
        for (int b = 0; b < d - 1; ++b)
          for (int s = 0; s < d; ++s) JJt(a, b) += J(a, s) * J(b, s);
      dV[nI + f * nIf + q] = fe->ipW[q] * std::sqrt(det_small(JJt));
      std::vector<double> nv(d);
      if (d == 2) {
        nv[0] = -J(0, 1);
        nv[1] = J(0, 0);
      } else {
        nv[0] = J(0, 1) * J(1, 2) - J(0, 2) * J(1, 1);
        nv[1] = J(0, 2) * J(1, 0) - J(0, 0) * J(1, 2);
        nv[2] = J(0, 0) * J(1, 1) - J(0, 1) * J(1, 0);
      }
      double nrm = 0.0;
      for (double v : nv) nrm += v * v;
      nrm = std::sqrt(nrm);
      double prod = 0.0;
      for (int k = 0; k < d; ++k) {
        nv[k] /= nrm;
        prod += test[k] * nv[k];
      }
      if (prod > 0)
        for (int k = 0; k < d; ++k) nv[k] = -nv[k];
      normals[f * nIf + q] = nv;
    }
  }
  // diffusion tensor at IPs (HDGDiffusion.cpp:31-72, HDGDiffusionSource.cpp:60-79)
  std::vector<Mat> Dn(N, Mat(d, d));
  for (int i = 0; i < N; ++i) {
    if (P.kc == 0) {
      for (int k = 0; k < d; ++k) Dn[i](k, k) = 1.0;
    } else if (P.kc == 1) {
      for (int k = 0; k < d; ++k) Dn[i](k, k) = P.kappa[(size_t)iEl * N + i];
    } else {
      for (int a = 0; a < d * d; ++a) Dn[i].a[a] = P.kappa[((size_t)iEl * N + i) * d * d + a];
    }
  }
  std::vector<Mat> Ds(nJ, Mat(d, d));
  for (int q = 0; q < nI; ++q)
    for (int a = 0; a < d * d; ++a) {
      double s = 0.0;
      for (int i = 0; i < N; ++i) s += re->phi[q][i] * Dn[i].a[a];
      Ds[q].a[a] = s;
    }
  for (int f = 0; f < F; ++f)
    for (int q = 0; q < nIf; ++q)
      for (int a = 0; a < d * d; ++a) {
        double s = 0.0;
        for (int i = 0; i < Nf; ++i) s += fe->phi[q][i] * Dn[re->faceNodes[f][i]].a[a];
        Ds[nI + f * nIf + q].a[a] = s;
      }
  A = Mat(n, n);
  Mat B(n, n);  // HDGBase part
  // HDGBase::assemble (HDGBase.cpp:67-158), face integrals
  for (int q = 0; q < nIf; ++q) {
    const auto& sh = fe->phi[q];
    for (int f = 0; f < F; ++f) {
      int off = f * nIf + q;
      double tq = 0.0;  // HDGBase::setTau (HDGBase.cpp:18-32)
      for (int i = 0; i < Nf; ++i) tq += tauLoc[f * Nf + i] * sh[i];
      double mm = dV[nI + off] * tq;
      std::vector<double> vm(d);
      for (int k = 0; k < d; ++k) vm[k] = dV[nI + off] * normals[off][k];
      for (int iN = 0; iN < Nf; ++iN)
        for (int jN = 0; jN < Nf; ++jN) {
          double ss = sh[iN] * sh[jN];
          double v = mm * ss;
          int li = startL + f * Nf + iN, lj = startL + f * Nf + jN;
          int ui = re->faceNodes[f][iN], uj = re->faceNodes[f][jN];
          B(li, lj) -= v;
          B(li, uj) += v;
          B(ui, uj) += v;
          B(ui, lj) -= v;
          for (int k = 0; k < d; ++k) B(lenU + ui * d + k, lj) -= vm[k] * ss;
        }
    }
  }
  for (int q = 0; q < nI; ++q) {
    const auto& sh = re->phi[q];
    for (int iN = 0; iN < N; ++iN) {
      std::vector<double> vm(d, 0.0);
      for (int a = 0; a < d; ++a) {
        for (int b = 0; b < d; ++b) vm[a] += invJ[q](a, b) * re->dphi[q][iN][b];
        vm[a] *= dV[q];
      }
      for (int k = 0; k < d; ++k)
        for (int jN = 0; jN < N; ++jN) {
          B(lenU + iN * d + k, jN) += vm[k] * sh[jN];
          B(lenU + iN * d + k, lenU + jN * d + k) += dV[q] * sh[iN] * sh[jN];
        }
    }
  }
  // HDGDiffusion::assemble (HDGDiffusion.cpp:74-145)
  Mat D(n, n);
  for (int f = 0; f < F; ++f)
    for (int q = 0; q < nIf; ++q) {
      const auto& sh = fe->phi[q];
      int off = f * nIf + q;
      std::vector<double> bv(d, 0.0);
      for (int a = 0; a < d; ++a) {
        for (int b = 0; b < d; ++b) bv[a] += Ds[nI + off](a, b) * normals[off][b];
        bv[a] *= dV[nI + off];
      }
      for (int iN = 0; iN < Nf; ++iN)
        for (int jN = 0; jN < Nf; ++jN)
          for (int k = 0; k < d; ++k) {
            double v = bv[k] * sh[iN] * sh[jN];
            D(startL + f * Nf + iN, lenU + re->faceNodes[f][jN] * d + k) -= v;
            D(re->faceNodes[f][iN], lenU + re->faceNodes[f][jN] * d + k) -= v;
          }
    }
  for (int q = 0; q < nI; ++q) {
    const auto& sh = re->phi[q];
    for (int iN = 0; iN < N; ++iN) {
      std::vector<double> g(d, 0.0), bv(d, 0.0);
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) g[a] += invJ[q](a, b) * re->dphi[q][iN][b];
      for (int a = 0; a < d; ++a) {
        for (int b = 0; b < d; ++b) bv[a] += Ds[q](a, b) * g[b];
        bv[a] *= dV[q];
      }
      for (int jN = 0; jN < N; ++jN)
        for (int k = 0; k < d; ++k) D(iN, lenU + jN * d + k) += bv[k] * sh[jN];
    }
  }
  for (size_t i = 0; i < A.a.size(); ++i) A.a[i] = B.a[i] + D.a[i];
  // Source (Source.cpp:5-48), RHS of the U rows
  rhs.assign(n, 0.0);
  if (P.srcMode != 0) {
    for (int q = 0; q < nI; ++q) {
      double fq;
      if (P.srcMode == 1) fq = P.src[(size_t)iEl * nI + q];
      else {
        std::vector<double> x(d, 0.0);
        for (int i = 0; i < N; ++i)
          for (int k = 0; k < d; ++k) x[k] += X[i][k] * re->phi[q][i];
        fq = d * M_PI * M_PI;
        for (int k = 0; k < d; ++k) fq *= std::sin(M_PI * x[k]);
      }
      double lm = fq * dV[q];
      for (int i = 0; i < N; ++i) rhs[i] += re->phi[q][i] * lm;
    }
  }
  if (P.rkDt > 0.0) {
    // RungeKutta::apply on the U rows of the local system (HDGModel.cpp:39-47):
    // s = dt s - dt K uj; K = dt a_ss K; K[:, U] += M; s += K ut
    const double dt = P.rkDt;
    Mat M(N, N);
    for (int q = 0; q < nI; ++q)
      for (int i = 0; i < N; ++i)
        for (int j = 0; j < N; ++j) M(i, j) += re->phi[q][i] * re->phi[q][j] * dV[q];
    std::vector<double> ut(n, 0.0), uj(n, 0.0);
    for (int i = 0; i < N; ++i) {
      ut[i] = P.rkOldU[(size_t)iEl * N + i];
      uj[i] = P.rkCombU[(size_t)iEl * N + i];
      for (int k = 0; k < d; ++k) {
        ut[lenU + i * d + k] = P.rkOldQ[((size_t)iEl * N + i) * d + k];
        uj[lenU + i * d + k] = P.rkCombQ[((size_t)iEl * N + i) * d + k];
      }
    }
    for (int fi = 0; fi < F; ++fi)
      for (int j = 0; j < Nf; ++j) {
        const size_t g = (size_t)facesIn[fi] * Nf + f2c[fi * Nf + j];
        ut[startL + fi * Nf + j] = P.rkOldL[g];
        uj[startL + fi * Nf + j] = P.rkCombL[g];
      }
    rk_apply(A, rhs, lenU, n, M, ut, uj, dt, P.rkDiag);
  } else if (P.dt > 0.0) {
    // implicit Euler on the U rows (HDGModel.cpp:39-47, Euler.cpp:18-34, Mass.cpp:5-38)
    Mat M(N, N);
    for (int q = 0; q < nI; ++q)
      for (int i = 0; i < N; ++i)
        for (int j = i; j < N; ++j) M(i, j) += re->phi[q][i] * re->phi[q][j] * dV[q];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < i; ++j) M(i, j) = M(j, i);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < lenU; ++i) A(i, j) *= P.dt;
    for (int i = 0; i < lenU; ++i) rhs[i] *= P.dt;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) {
        A(i, j) += M(i, j);
        rhs[i] += M(i, j) * P.uOld[(size_t)iEl * N + j];
      }
  }
}

// Static condensation (HDGSolver.cpp:331-348), IMPLICIT mode.
// Destination of one element's condensed blocks (column-major, as Problem's arrays).
struct CondensedOut {
  double *S, *S0, *U, *Q, *U0, *Q0;
};

static void condense_to(const Problem& P, int iEl, const Mat& A, const std::vector<double>& r, CondensedOut out);

static void condense(Problem& P, int iEl, const Mat& A, const std::vector<double>& r) {
  const size_t e = (size_t)iEl;
  condense_to(P, iEl, A, r,
              CondensedOut{&P.S[e * P.lenL * P.lenL], &P.S0[e * P.lenL], &P.U[e * P.lenU * P.lenL],
                           &P.Q[e * P.lenQ * P.lenL], &P.U0[e * P.lenU], &P.Q0[e * P.lenQ]});
}

static void condense_to(const Problem& P, int iEl, const Mat& A, const std::vector<double>& r, CondensedOut out) {
  int lenU = P.lenU, lenQ = P.lenQ, lenL = P.lenL;
  int sU = 0, sQ = lenU, sL = lenU + lenQ;
  Mat Sqq = block(A, sQ, sQ, lenQ, lenQ);
  std::vector<int> pq;
  if (!lu_factor(Sqq, pq)) throw std::runtime_error("singular Sqq");
  Mat Xu = block(A, sQ, sU, lenQ, lenU);
  lu_solve(Sqq, pq, Xu);
  Mat Xl = block(A, sQ, sL, lenQ, lenL);
  lu_solve(Sqq, pq, Xl);
  Mat Suq = block(A, sU, sQ, lenU, lenQ);
  Mat Am = block(A, sU, sU, lenU, lenU);
  gemm(-1.0, Suq, Xu, 1.0, Am);
  std::vector<int> pa;
  if (!lu_factor(Am, pa)) throw std::runtime_error("singular Schur block");
  Mat Ul = block(A, sU, sL, lenU, lenL);
  gemm(-1.0, Suq, Xl, 1.0, Ul);
  lu_solve(Am, pa, Ul);
  for (auto& v : Ul.a) v = -v;  // U
  Mat U0(lenU, 1);
  for (int i = 0; i < lenU; ++i) U0(i, 0) = r[sU + i];
  lu_solve(Am, pa, U0);
  Mat Qm(lenQ, lenL);
  gemm(-1.0, Xu, Ul, 0.0, Qm);
  for (size_t i = 0; i < Qm.a.size(); ++i) Qm.a[i] -= Xl.a[i];
  Mat Q0(lenQ, 1);
  gemm(-1.0, Xu, U0, 0.0, Q0);
  Mat S = block(A, sL, sL, lenL, lenL);
  Mat S0(lenL, 1);
  for (int i = 0; i < lenL; ++i) S0(i, 0) = r[sL + i];
  if (P.solverType == 0) {
    gemm(1.0, block(A, sL, sU, lenL, lenU), Ul, 1.0, S);
    gemm(1.0, block(A, sL, sQ, lenL, lenQ), Qm, 1.0, S);
    gemm(-1.0, block(A, sL, sU, lenL, lenU), U0, 1.0, S0);
    gemm(-1.0, block(A, sL, sQ, lenL, lenQ), Q0, 1.0, S0);
  } else {
    // explicit modes (HDGSolver.cpp:349-354): S = Sll, S0 = f_L - Slu sol - Slq flux
    Mat sol(lenU, 1), flux(lenQ, 1);
    for (int i = 0; i < lenU; ++i) sol(i, 0) = P.solState[(size_t)iEl * lenU + i];
    for (int i = 0; i < lenQ; ++i) flux(i, 0) = P.fluxState[(size_t)iEl * lenQ + i];
    gemm(-1.0, block(A, sL, sU, lenL, lenU), sol, 1.0, S0);
    gemm(-1.0, block(A, sL, sQ, lenL, lenQ), flux, 1.0, S0);
  }
  std::copy(S.a.begin(), S.a.end(), out.S);
  std::copy(S0.a.begin(), S0.a.end(), out.S0);
  if (out.U) std::copy(Ul.a.begin(), Ul.a.end(), out.U);
  if (out.Q) std::copy(Qm.a.begin(), Qm.a.end(), out.Q);
  if (out.U0) std::copy(U0.a.begin(), U0.a.end(), out.U0);
  if (out.Q0) std::copy(Q0.a.begin(), Q0.a.end(), out.Q0);
}

// The Dirichlet Set of apply_dirichlet on one element's S, S0 (its boundary faces).
static void dirichlet_element(const Problem& P, int c, double* S, double* S0) {
  int F = P.re->nFaces, Nf = P.re->face->nNodes, lenL = P.lenL;
  for (int loc = 0; loc < F; ++loc) {
    int f = P.mf.cell2face[(size_t)c * F + loc];
    if (!std::binary_search(P.mf.boundary.begin(), P.mf.boundary.end(), f)) continue;
    if (P.mf.face2cell[2 * f] != c) continue;
    for (int i = 0; i < Nf; ++i) {
      int row = loc * Nf + i;
      for (int j = 0; j < lenL; ++j) S[row + (size_t)j * lenL] = 0.0;
      S0[row] = 0.0;
    }
    for (int i = 0; i < Nf; ++i) {
      int row = loc * Nf + i;
      S[row + (size_t)row * lenL] += 1.0;
      S0[row] += P.dirichlet[(size_t)f * Nf + i];
    }
  }
}

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

template <class Fn>
static void parallel_for(int n, int nthreads, Fn fn) {
  if (nthreads <= 1 || n < 2) {
    for (int i = 0; i < n; ++i) fn(i);
    return;
  }
  std::vector<std::thread> th;
  for (int t = 0; t < nthreads; ++t)
    th.emplace_back([=]() {
      long lo = (long)n * t / nthreads, hi = (long)n * (t + 1) / nthreads;
      for (long i = lo; i < hi; ++i) fn((int)i);
    });
  for (auto& x : th) x.join();
}

static void element_loop(Problem& P, int nthreads, int first, int count) {
  parallel_for(count, nthreads, [&](int k) {
    int iEl = first + k;
    Mat A;
    std::vector<double> r;
    local_system(P, iEl, A, r);
    condense(P, iEl, A, r);
  });
}

// Dirichlet boundary model with Set assembly (HDGSolver.cpp:361-529,
// DirichletModel.cpp:19-44): zero the face rows of S and S0, add the identity
// and the Dirichlet values (face order).
static void apply_dirichlet(Problem& P) {
  int F = P.re->nFaces, Nf = P.re->face->nNodes, lenL = P.lenL;
  for (int f : P.mf.boundary) {
    int c = P.mf.face2cell[2 * f];
    int loc = 0;
    while (P.mf.cell2face[(size_t)c * F + loc] != f) ++loc;
    double* S = &P.S[(size_t)c * lenL * lenL];
    double* S0 = &P.S0[(size_t)c * lenL];
    for (int i = 0; i < Nf; ++i) {
      int row = loc * Nf + i;
      for (int j = 0; j < lenL; ++j) S[row + (size_t)j * lenL] = 0.0;
      S0[row] = 0.0;
    }
    for (int i = 0; i < Nf; ++i) {
      int row = loc * Nf + i;
      S[row + (size_t)row * lenL] += 1.0;
      S0[row] += P.dirichlet[(size_t)f * Nf + i];
    }
  }
}

// Trace DOF numbering (HDGSolver.cpp:589-598) and the PETSc AIJ pattern:
// sorted columns, every entry of every element block kept (explicit zeros too).
static void build_csr(Problem& P) {
  int F = P.re->nFaces, Nf = P.re->face->nNodes, N = P.re->nNodes, lenL = P.lenL;
  int ndofs = P.mf.nFaces * Nf;
  std::vector<std::set<int>> faceNbr(P.mf.nFaces);
  for (int c = 0; c < P.nCells; ++c)
    for (int i = 0; i < F; ++i)
      for (int j = 0; j < F; ++j) faceNbr[P.mf.cell2face[(size_t)c * F + i]].insert(P.mf.cell2face[(size_t)c * F + j]);
  P.rowptr.assign(ndofs + 1, 0);
  for (int f = 0; f < P.mf.nFaces; ++f)
    for (int a = 0; a < Nf; ++a) P.rowptr[f * Nf + a + 1] = (int)faceNbr[f].size() * Nf;
  for (int r = 0; r < ndofs; ++r) P.rowptr[r + 1] += P.rowptr[r];
  P.col.assign(P.rowptr[ndofs], 0);
  for (int f = 0; f < P.mf.nFaces; ++f)
    for (int a = 0; a < Nf; ++a) {
      int k = P.rowptr[f * Nf + a];
      for (int g : faceNbr[f])
        for (int b = 0; b < Nf; ++b) P.col[k++] = g * Nf + b;
    }
  P.val.assign(P.col.size(), 0.0);
  P.rhs.assign(ndofs, 0.0);
  std::vector<int> rc(lenL);
  for (int c = 0; c < P.nCells; ++c) {
    const int* cell = &P.cells[(size_t)c * N];
    for (int i = 0; i < F; ++i) {
      int f = P.mf.cell2face[(size_t)c * F + i];
      const int* face = &P.mf.faces[(size_t)f * Nf];
      for (int j = 0; j < Nf; ++j) {
        int node = cell[P.re->faceNodes[i][j]], pos = 0;
        while (face[pos] != node) ++pos;
        rc[i * Nf + j] = f * Nf + pos;
      }
    }
    const double* S = &P.S[(size_t)c * lenL * lenL];
    for (int i = 0; i < lenL; ++i) {
      int row = rc[i];
      int* cb = &P.col[P.rowptr[row]];
      int len = P.rowptr[row + 1] - P.rowptr[row];
      for (int j = 0; j < lenL; ++j) {
        int k = (int)(std::lower_bound(cb, cb + len, rc[j]) - cb);
        P.val[P.rowptr[row] + k] += S[i + (size_t)j * lenL];
      }
      P.rhs[row] += P.S0[(size_t)c * lenL + i];
    }
  }
}

// Restarted GMRES(30) with a Jacobi preconditioner (PETSc KSPGMRES + PCJACOBI,
// PetscOpts.h:12-28), zero initial guess, relative tolerance on the
// preconditioned residual as PETSc's default left preconditioning does.
static int gmres(const Problem& P, std::vector<double>& x, double rtol, int maxit, int nthreads) {
  int n = (int)P.rhs.size(), m = 30;
  std::vector<double> dinv(n, 1.0);
  for (int r = 0; r < n; ++r)
    for (int k = P.rowptr[r]; k < P.rowptr[r + 1]; ++k)
      if (P.col[k] == r && P.val[k] != 0.0) dinv[r] = 1.0 / P.val[k];
  auto spmv = [&](const std::vector<double>& v, std::vector<double>& out) {
    parallel_for(nthreads, nthreads, [&](int t) {
      long lo = (long)n * t / nthreads, hi = (long)n * (t + 1) / nthreads;
      for (long r = lo; r < hi; ++r) {
        double s = 0.0;
        for (int k = P.rowptr[r]; k < P.rowptr[r + 1]; ++k) s += P.val[k] * v[P.col[k]];
        out[r] = s * dinv[r];
      }
    });
  };
  x.assign(n, 0.0);
  std::vector<double> r(n), w(n);
  std::vector<std::vector<double>> V(m + 1, std::vector<double>(n));
  std::vector<double> H((m + 1) * m), cs(m), sn(m), g(m + 1);
  double bnorm = 0.0;
  for (int i = 0; i < n; ++i) bnorm += (P.rhs[i] * dinv[i]) * (P.rhs[i] * dinv[i]);
  bnorm = std::sqrt(bnorm);
  if (bnorm == 0.0) return 0;
  int it = 0;
  while (it < maxit) {
    spmv(x, w);
    for (int i = 0; i < n; ++i) r[i] = P.rhs[i] * dinv[i] - w[i];
    double beta = 0.0;
    for (double v : r) beta += v * v;
    beta = std::sqrt(beta);
    if (beta <= rtol * bnorm) return it;
    for (int i = 0; i < n; ++i) V[0][i] = r[i] / beta;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m && it < maxit; ++j, ++it) {
      spmv(V[j], w);
      for (int i = 0; i <= j; ++i) {
        double h = 0.0;
        for (int k = 0; k < n; ++k) h += w[k] * V[i][k];
        H[i + j * (m + 1)] = h;
        for (int k = 0; k < n; ++k) w[k] -= h * V[i][k];
      }
      double hn = 0.0;
      for (double v : w) hn += v * v;
      hn = std::sqrt(hn);
      H[j + 1 + j * (m + 1)] = hn;
      if (hn != 0.0)
        for (int k = 0; k < n; ++k) V[j + 1][k] = w[k] / hn;
      for (int i = 0; i < j; ++i) {
        double a = H[i + j * (m + 1)], b = H[i + 1 + j * (m + 1)];
        H[i + j * (m + 1)] = cs[i] * a + sn[i] * b;
        H[i + 1 + j * (m + 1)] = -sn[i] * a + cs[i] * b;
      }
      double a = H[j + j * (m + 1)], b = H[j + 1 + j * (m + 1)];
      double den = std::sqrt(a * a + b * b);
      cs[j] = a / den;
      sn[j] = b / den;
      H[j + j * (m + 1)] = den;
      H[j + 1 + j * (m + 1)] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      if (std::fabs(g[j + 1]) <= rtol * bnorm) { ++j; ++it; break; }
    }
    std::vector<double> y(j);
    for (int i = j - 1; i >= 0; --i) {
      double s = g[i];
      for (int k = i + 1; k < j; ++k) s -= H[i + k * (m + 1)] * y[k];
      y[i] = s / H[i + i * (m + 1)];
    }
    for (int i = 0; i < j; ++i)
      for (int k = 0; k < n; ++k) x[k] += y[i] * V[i][k];
    if (j > 0 && std::fabs(g[j]) <= rtol * bnorm) return it;
  }
  return -it;
}

// Local recovery (HDGSolver.cpp:741-775).
static void recover(const Problem& P, const double* trace, double* sol, double* flux) {
  int F = P.re->nFaces, Nf = P.re->face->nNodes, N = P.re->nNodes;
  int lenU = P.lenU, lenQ = P.lenQ, lenL = P.lenL;
  std::vector<double> lam(lenL);
  for (int c = 0; c < P.nCells; ++c) {
    const int* cell = &P.cells[(size_t)c * N];
    for (int i = 0; i < F; ++i) {
      int f = P.mf.cell2face[(size_t)c * F + i];
      const int* face = &P.mf.faces[(size_t)f * Nf];
      for (int j = 0; j < Nf; ++j) {
        int node = cell[P.re->faceNodes[i][j]], pos = 0;
        while (face[pos] != node) ++pos;
        lam[i * Nf + j] = trace[(size_t)f * Nf + pos];
      }
    }
    const double* U = &P.U[(size_t)c * lenU * lenL];
    const double* Q = &P.Q[(size_t)c * lenQ * lenL];
    for (int i = 0; i < lenU; ++i) {
      double s = 0.0;
      for (int j = 0; j < lenL; ++j) s += U[i + (size_t)j * lenU] * lam[j];
      sol[(size_t)c * lenU + i] = s + P.U0[(size_t)c * lenU + i];
    }
    for (int i = 0; i < lenQ; ++i) {
      double s = 0.0;
      for (int j = 0; j < lenL; ++j) s += Q[i + (size_t)j * lenQ] * lam[j];
      flux[(size_t)c * lenQ + i] = s + P.Q0[(size_t)c * lenQ + i];
    }
  }
}

// ============================================================ Burgers (vector unknowns)
// HDGBurgersModel (HDGBurgersModel.cpp:35-125): nd = dim unknowns per node, local
// matrix = HDGBase + HDGUNabU (+ HDGDiffusion when a diffusion tensor is given), RHS =
// HDGUNabU's RHS + one scalar Source per component, implicit Euler (Euler.cpp:18-34)
// with the mass multiplied over the components (Mass.cpp:5-38, Operator.cpp:86-97).
// Local index layout (HDGBase.cpp:85-91): U (i*nd + c), Q ((i*d + k)*nd + c),
// L ((f*Nf + a)*nd + c).
struct BurgersFields {
  std::vector<double> tau;    // [nFaces][Nf][sides][nd*nd] column-major nd x nd
  int tauSides = 1;
  std::vector<double> nu;     // [nCells][N][kc] (kc 0 = no diffusion operator, 1, d*d)
  int kc = 0;
  std::vector<double> src;    // [nCells][nI][nd] values at the integration points, or empty
  std::vector<double> dir;    // [nFaces][Nf][nd]
  double dt = 0.0;
  std::vector<double> old;    // "Solution" read by Euler: [nCells][N*nd]
  std::vector<double> buf;    // BufferSolution [nCells][N*nd]
  std::vector<double> trace;  // Trace [nFaces][Nf*nd]
};
static std::map<const Problem*, BurgersFields> g_burgers;

struct ElemGeo {
  NodeList X;
  std::vector<Mat> invJ;
  std::vector<double> dV;
  std::vector<std::vector<double>> normals;
  std::vector<int> facesIn, f2c;
};

// Element nodes, face2CellMap (HDGSolver.cpp:258-275), volume and face Jacobians
// (Operator.cpp:14-84, HDGModel.cpp:53-85) and outward normals (HDGBase.cpp:34-65):
// the same arithmetic as in local_system above.
static void element_geometry(const Problem& P, int iEl, ElemGeo& g) {
  const RefEl* re = P.re;
  const RefEl* fe = re->face;
  int d = P.dim, N = re->nNodes, F = re->nFaces, Nf = fe->nNodes, nI = re->nIP, nIf = fe->nIP;
  const int* cell = &P.cells[(size_t)iEl * N];
  g.X.assign(N, std::vector<double>(d));
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < d; ++k) g.X[i][k] = P.coords[(size_t)cell[i] * d + k];
  g.facesIn.assign(F, 0);
  g.f2c.assign(F * Nf, 0);
  for (int i = 0; i < F; ++i) g.facesIn[i] = P.mf.cell2face[(size_t)iEl * F + i];
  for (int i = 0; i < F; ++i) {
    const int* face = &P.mf.faces[(size_t)g.facesIn[i] * Nf];
    for (int j = 0; j < Nf; ++j) {
      int node = cell[re->faceNodes[i][j]], pos = -1;
      for (int q = 0; q < Nf; ++q)
        if (face[q] == node) { pos = q; break; }
      if (pos < 0) throw std::runtime_error("couldn't find cell node in face");
      g.f2c[i * Nf + j] = pos;
    }
  }
  g.invJ.assign(nI, Mat());
  g.dV.assign(nI + F * nIf, 0.0);
  for (int q = 0; q < nI; ++q) {
    Mat J(d, d);
    for (int i = 0; i < N; ++i)
      for (int r = 0; r < d; ++r)
        for (int s = 0; s < d; ++s) J(r, s) += re->dphi[q][i][r] * g.X[i][s];
    g.dV[q] = re->ipW[q] * det_small(J);
    g.invJ[q] = inverse(J);
  }
  g.normals.assign(F * nIf, std::vector<double>(d));
  for (int f = 0; f < F; ++f) {
    int v0 = re->faceNodes[f][0], vn = -1;
    for (int k = 0; k < N; ++k)
      if (std::find(re->faceNodes[f].begin(), re->faceNodes[f].end(), k) == re->faceNodes[f].end()) {
        vn = k;
        break;
      }
    std::vector<double> test(d);
    for (int k = 0; k < d; ++k) test[k] = g.X[vn][k] - g.X[v0][k];
    for (int q = 0; q < nIf; ++q) {
      Mat J(d - 1, d);
      for (int i = 0; i < Nf; ++i)
        for (int r = 0; r < d - 1; ++r)
          for (int s = 0; s < d; ++s) J(r, s) += fe->dphi[q][i][r] * g.X[re->faceNodes[f][i]][s];
      Mat JJt(d - 1, d - 1);
      for (int a = 0; a < d - 1; ++a)
        for (int b = 0; b < d - 1; ++b)
          for (int s = 0; s < d; ++s) JJt(a, b) += J(a, s) * J(b, s);
      g.dV[nI + f * nIf + q] = fe->ipW[q] * std::sqrt(det_small(JJt));
      std::vector<double> nv(d);
      if (d == 2) {
        nv[0] = -J(0, 1);
        nv[1] = J(0, 0);
      } else {
        nv[0] = J(0, 1) * J(1, 2) - J(0, 2) * J(1, 1);
        nv[1] = J(0, 2) * J(1, 0) - J(0, 0) * J(1, 2);
        nv[2] = J(0, 0) * J(1, 1) - J(0, 1) * J(1, 0);
      }
      double nrm = 0.0;
      for (double v : nv) nrm += v * v;
      nrm = std::sqrt(nrm);
      double prod = 0.0;
      for (int k = 0; k < d; ++k) {
        nv[k] /= nrm;
        prod += test[k] * nv[k];
      }
      if (prod > 0)
        for (int k = 0; k < d; ++k) nv[k] = -nv[k];
      g.normals[f * nIf + q] = nv;
    }
  }
}

// HDGBase::assemble with nd unknowns per node (HDGBase.cpp:67-158); tauIP holds the
// nd x nd tau (column-major) at every face integration point (HDGBase::setTau,
// HDGBase.cpp:18-32).
static void base_nd(const RefEl* re, int nd, const std::vector<double>& dV, const std::vector<Mat>& invJ,
                    const std::vector<std::vector<double>>& normals, const std::vector<double>& tauIP, Mat& op) {
  const RefEl* fe = re->face;
  int d = re->dim, N = re->nNodes, F = re->nFaces, Nf = fe->nNodes, nI = re->nIP, nIf = fe->nIP;
  int sQ = N * nd, sL = N * (d + 1) * nd, n = sL + F * Nf * nd, st = nd * nd;
  op = Mat(n, n);
  for (int q = 0; q < nIf; ++q) {
    const auto& sh = fe->phi[q];
    for (int f = 0; f < F; ++f) {
      int off = f * nIf + q;
      const auto& fn = re->faceNodes[f];
      double ds = dV[nI + off];
      for (int iN = 0; iN < Nf; ++iN)
        for (int c = 0; c < nd; ++c)
          for (int jN = 0; jN < Nf; ++jN) {
            double ss = sh[iN] * sh[jN];
            for (int m = 0; m < nd; ++m) {
              double val = ds * tauIP[(size_t)off * st + m * nd + c] * ss;
              op(sL + (f * Nf + iN) * nd + c, sL + (f * Nf + jN) * nd + m) -= val;
              op(sL + (f * Nf + iN) * nd + c, fn[jN] * nd + m) += val;
              op(fn[iN] * nd + c, fn[jN] * nd + m) += val;
              op(fn[iN] * nd + c, sL + (f * Nf + jN) * nd + m) -= val;
            }
            for (int k = 0; k < d; ++k)
              op(sQ + (fn[iN] * d + k) * nd + c, sL + (f * Nf + jN) * nd + c) -= ds * normals[off][k] * ss;
          }
    }
  }
  for (int q = 0; q < nI; ++q) {
    const auto& sh = re->phi[q];
    for (int iN = 0; iN < N; ++iN) {
      std::vector<double> vm(d, 0.0);
      for (int a = 0; a < d; ++a) {
        for (int b = 0; b < d; ++b) vm[a] += invJ[q](a, b) * re->dphi[q][iN][b];
        vm[a] *= dV[q];
      }
      for (int k = 0; k < d; ++k)
        for (int c = 0; c < nd; ++c)
          for (int jN = 0; jN < N; ++jN) {
            op(sQ + (iN * d + k) * nd + c, jN * nd + c) += vm[k] * sh[jN];
            op(sQ + (iN * d + k) * nd + c, sQ + (jN * d + k) * nd + c) += dV[q] * sh[iN] * sh[jN];
          }
    }
  }
}

// HDGDiffusion::assemble with nd unknowns per node (HDGDiffusion.cpp:74-145); Ds =
// the d x d tensor (column-major) at the volume then the face integration points
// (HDGDiffusion::setDiffusionTensor, HDGDiffusion.cpp:31-72).
static void diffusion_nd(const RefEl* re, int nd, const std::vector<double>& dV, const std::vector<Mat>& invJ,
                         const std::vector<std::vector<double>>& normals, const std::vector<Mat>& Ds, Mat& op) {
  const RefEl* fe = re->face;
  int d = re->dim, N = re->nNodes, F = re->nFaces, Nf = fe->nNodes, nI = re->nIP, nIf = fe->nIP;
  int lenU = N * nd, lenQ = d * lenU, n = lenU + lenQ + F * Nf * nd;
  op = Mat(n, n);
  for (int f = 0; f < F; ++f) {
    const auto& fn = re->faceNodes[f];
    for (int q = 0; q < nIf; ++q) {
      const auto& sh = fe->phi[q];
      int off = f * nIf + q;
      std::vector<double> bv(d, 0.0);
      for (int a = 0; a < d; ++a) {
        for (int b = 0; b < d; ++b) bv[a] += Ds[nI + off](a, b) * normals[off][b];
        bv[a] *= dV[nI + off];
      }
      for (int iN = 0; iN < Nf; ++iN)
        for (int c = 0; c < nd; ++c)
          for (int jN = 0; jN < Nf; ++jN)
            for (int k = 0; k < d; ++k) {
              double v = bv[k] * sh[iN] * sh[jN];
              op(lenU + lenQ + (f * Nf + iN) * nd + c, lenU + (fn[jN] * d + k) * nd + c) -= v;
              op(fn[iN] * nd + c, lenU + (fn[jN] * d + k) * nd + c) -= v;
            }
    }
  }
  for (int q = 0; q < nI; ++q) {
    const auto& sh = re->phi[q];
    for (int iN = 0; iN < N; ++iN) {
      std::vector<double> g(d, 0.0), bv(d, 0.0);
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) g[a] += invJ[q](a, b) * re->dphi[q][iN][b];
      for (int a = 0; a < d; ++a) {
        for (int b = 0; b < d; ++b) bv[a] += Ds[q](a, b) * g[b];
        bv[a] *= dV[q];
      }
      for (int c = 0; c < nd; ++c)
        for (int jN = 0; jN < N; ++jN)
          for (int k = 0; k < d; ++k) op(iN * nd + c, lenU + (jN * d + k) * nd + c) += bv[k] * sh[jN];
    }
  }
}

// HDGUNabU (HDGUNabU.cpp:27-193): the u.grad(u) term linearised about the nodal
// solution sol[N][nd] and the local-order trace tr[F*Nf][nd]; face terms into the L
// rows, those rows summed into the U rows of their face nodes, volume terms into the
// U-U block, RHS = op [u; 0; t] / 2 on the U and L rows.
static void unabu_nd(const RefEl* re, int nd, const std::vector<double>& dV, const std::vector<Mat>& invJ,
                     const std::vector<std::vector<double>>& normals, const std::vector<double>& sol,
                     const std::vector<double>& tr, Mat& op, std::vector<double>& rhs) {
  const RefEl* fe = re->face;
  int d = re->dim, N = re->nNodes, F = re->nFaces, Nf = fe->nNodes, nI = re->nIP, nIf = fe->nIP;
  int lenU = N * nd, sL = N * (d + 1) * nd, lenL = F * Nf * nd, n = sL + lenL;
  op = Mat(n, n);
  // setSolution / setTrace (HDGUNabU.cpp:27-99): values at the integration points
  std::vector<double> sols((size_t)nI * nd, 0.0), fsols((size_t)F * nIf * nd, 0.0), trs((size_t)F * nIf * nd, 0.0);
  for (int q = 0; q < nI; ++q)
    for (int i = 0; i < N; ++i)
      for (int c = 0; c < nd; ++c) sols[q * nd + c] += re->phi[q][i] * sol[i * nd + c];
  for (int f = 0; f < F; ++f)
    for (int q = 0; q < nIf; ++q)
      for (int a = 0; a < Nf; ++a)
        for (int c = 0; c < nd; ++c) {
          fsols[(f * nIf + q) * nd + c] += fe->phi[q][a] * sol[re->faceNodes[f][a] * nd + c];
          trs[(f * nIf + q) * nd + c] += fe->phi[q][a] * tr[(f * Nf + a) * nd + c];
        }
  // face integrals (HDGUNabU.cpp:126-145)
  for (int f = 0; f < F; ++f)
    for (int q = 0; q < nIf; ++q) {
      const auto& sh = fe->phi[q];
      int off = f * nIf + q;
      double ds = dV[nI + off], tn = 0.0;
      for (int k = 0; k < d; ++k) tn += trs[off * nd + k] * normals[off][k];
      tn *= ds;
      for (int iN = 0; iN < Nf; ++iN)
        for (int c = 0; c < nd; ++c)
          for (int jN = 0; jN < Nf; ++jN) {
            op(sL + (f * Nf + iN) * nd + c, sL + (f * Nf + jN) * nd + c) += tn * sh[jN] * sh[iN];
            for (int m = 0; m < nd; ++m)
              op(sL + (f * Nf + iN) * nd + c, sL + (f * Nf + jN) * nd + m) +=
                  fsols[off * nd + c] * sh[jN] * sh[iN] * normals[off][m] * ds;
          }
    }
  // face rows summed into the U rows of the face's nodes (HDGUNabU.cpp:147-152)
  for (int f = 0; f < F; ++f)
    for (int iN = 0; iN < Nf; ++iN)
      for (int c = 0; c < nd; ++c)
        for (int j = 0; j < lenL; ++j)
          op(re->faceNodes[f][iN] * nd + c, sL + j) += op(sL + (f * Nf + iN) * nd + c, sL + j);
  // volume integrals (HDGUNabU.cpp:153-177)
  for (int q = 0; q < nI; ++q) {
    const auto& sh = re->phi[q];
    std::vector<double> G((size_t)N * d, 0.0);
    for (int i = 0; i < N; ++i)
      for (int a = 0; a < d; ++a)
        for (int b = 0; b < d; ++b) G[i * d + a] += invJ[q](a, b) * re->dphi[q][i][b];
    double divSol = 0.0;  // trace of sum_i grad(phi_i) u_i^T (needs nd == d)
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < d; ++k) divSol += G[i * d + k] * sol[i * nd + k];
    for (int iN = 0; iN < N; ++iN) {
      double sg = 0.0;
      for (int k = 0; k < d; ++k) sg += sols[q * nd + k] * G[iN * d + k];
      for (int c = 0; c < nd; ++c)
        for (int jN = 0; jN < N; ++jN) {
          op(iN * nd + c, jN * nd + c) -= (divSol * sh[iN] + sg) * dV[q] * sh[jN];
          for (int m = 0; m < nd; ++m)
            op(iN * nd + c, jN * nd + m) -=
                sols[q * nd + c] * (G[jN * d + m] * sh[iN] + G[iN * d + m] * sh[jN]) * dV[q];
        }
    }
  }
  // RHS (HDGUNabU.cpp:178-190)
  rhs.assign(n, 0.0);
  for (int i = 0; i < lenU; ++i) {
    double s = 0.0;
    for (int j = 0; j < lenU; ++j) s += op(i, j) * sol[j] / 2.0;
    for (int j = 0; j < lenL; ++j) s += op(i, sL + j) * tr[j] / 2.0;
    rhs[i] += s;
  }
  for (int i = 0; i < lenL; ++i) {
    double s = 0.0;
    for (int j = 0; j < lenU; ++j) s += op(sL + i, j) * sol[j] / 2.0;
    for (int j = 0; j < lenL; ++j) s += op(sL + i, sL + j) * tr[j] / 2.0;
    rhs[sL + i] += s;
  }
}

// HDGBurgersModel::computeLocalMatrix / computeLocalRHS (HDGBurgersModel.cpp:93-125)
// for one element of the mesh, then HDGModel::compute's time scheme (HDGModel.cpp:35-51).
static void burgers_local_system(const Problem& P, const BurgersFields& B, int iEl, Mat& A,
                                 std::vector<double>& rhs) {
  const RefEl* re = P.re;
  const RefEl* fe = re->face;
  int d = P.dim, nd = d, N = re->nNodes, F = re->nFaces, Nf = fe->nNodes, nI = re->nIP, nIf = fe->nIP;
  int lenU = N * nd, st = nd * nd, n = P.nloc;
  ElemGeo g;
  element_geometry(P, iEl, g);
  // local fields (HDGSolver.cpp:276-326): tau side select, face fields in local order
  std::vector<double> tauLoc((size_t)F * Nf * st), trLoc((size_t)F * Nf * nd);
  for (int i = 0; i < F; ++i) {
    int f = g.facesIn[i];
    int side = (P.mf.face2cell[2 * f] == iEl) ? 0 : 1;
    for (int j = 0; j < Nf; ++j) {
      int qn = g.f2c[i * Nf + j];
      for (int v = 0; v < st; ++v)
        tauLoc[(i * Nf + j) * st + v] = B.tau[(((size_t)f * Nf + qn) * B.tauSides + (B.tauSides == 2 ? side : 0)) * st + v];
      for (int c = 0; c < nd; ++c) trLoc[(i * Nf + j) * nd + c] = B.trace[((size_t)f * Nf + qn) * nd + c];
    }
  }
  std::vector<double> tauIP((size_t)F * nIf * st, 0.0);
  for (int f = 0; f < F; ++f)
    for (int q = 0; q < nIf; ++q)
      for (int a = 0; a < Nf; ++a)
        for (int v = 0; v < st; ++v) tauIP[(f * nIf + q) * st + v] += tauLoc[(f * Nf + a) * st + v] * fe->phi[q][a];
  std::vector<double> sol(B.buf.begin() + (size_t)iEl * lenU, B.buf.begin() + (size_t)(iEl + 1) * lenU);
  Mat Ab, Ac, Ad;
  std::vector<double> rc;
  base_nd(re, nd, g.dV, g.invJ, g.normals, tauIP, Ab);
  unabu_nd(re, nd, g.dV, g.invJ, g.normals, sol, trLoc, Ac, rc);
  A = Mat(n, n);
  for (size_t i = 0; i < A.a.size(); ++i) A.a[i] = Ab.a[i] + Ac.a[i];
  if (B.kc != 0) {
    // parseDiffusionVals (HDGBurgersModel.cpp:128-150): scalar times identity or a d x d tensor
    std::vector<Mat> Dn(N, Mat(d, d));
    for (int i = 0; i < N; ++i) {
      if (B.kc == 1)
        for (int k = 0; k < d; ++k) Dn[i](k, k) = B.nu[(size_t)iEl * N + i];
      else
        for (int a = 0; a < d * d; ++a) Dn[i].a[a] = B.nu[((size_t)iEl * N + i) * d * d + a];
    }
    std::vector<Mat> Ds(nI + F * nIf, Mat(d, d));
    for (int q = 0; q < nI; ++q)
      for (int a = 0; a < d * d; ++a) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) s += re->phi[q][i] * Dn[i].a[a];
        Ds[q].a[a] = s;
      }
    for (int f = 0; f < F; ++f)
      for (int q = 0; q < nIf; ++q)
        for (int a = 0; a < d * d; ++a) {
          double s = 0.0;
          for (int i = 0; i < Nf; ++i) s += fe->phi[q][i] * Dn[re->faceNodes[f][i]].a[a];
          Ds[nI + f * nIf + q].a[a] = s;
        }
    diffusion_nd(re, nd, g.dV, g.invJ, g.normals, Ds, Ad);
    for (size_t i = 0; i < A.a.size(); ++i) A.a[i] += Ad.a[i];
  }
  rhs = rc;
  if (!B.src.empty()) {
    // one scalar Source per component (Source.cpp:24-48, HDGBurgersModel.cpp:114-123)
    for (int c = 0; c < nd; ++c)
      for (int q = 0; q < nI; ++q) {
        double lm = B.src[((size_t)iEl * nI + q) * nd + c] * g.dV[q];
        for (int i = 0; i < N; ++i) rhs[i * nd + c] += re->phi[q][i] * lm;
      }
  }
  if (B.dt > 0.0) {
    // Euler::apply (Euler.cpp:18-34), implicit: U rows times dt, plus M (x) I_nd
    Mat M(N, N);
    for (int q = 0; q < nI; ++q)
      for (int i = 0; i < N; ++i)
        for (int j = i; j < N; ++j) M(i, j) += re->phi[q][i] * re->phi[q][j] * g.dV[q];
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < i; ++j) M(i, j) = M(j, i);
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < lenU; ++i) A(i, j) *= B.dt;
    for (int i = 0; i < lenU; ++i) rhs[i] *= B.dt;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j)
        for (int c = 0; c < nd; ++c) {
          A(i * nd + c, j * nd + c) += M(i, j);
          rhs[i * nd + c] += M(i, j) * B.old[(size_t)iEl * lenU + j * nd + c];
        }
  }
}

// Dirichlet Set on the boundary faces with nd values per node (HDGSolver.cpp:361-529,
// DirichletModel.cpp:19-44): the model's identity and its face-ordered values are
// added to the element's local face rows as they are, without the face2CellMap
// permutation (HDGSolver.cpp:493-497), as apply_dirichlet above.
static void apply_dirichlet_nd(Problem& P, int nd, const std::vector<double>& dir) {
  int F = P.re->nFaces, Nf = P.re->face->nNodes, lenL = P.lenL, lenT = Nf * nd;
  for (int f : P.mf.boundary) {
    int c = P.mf.face2cell[2 * f];
    int loc = 0;
    while (P.mf.cell2face[(size_t)c * F + loc] != f) ++loc;
    double* S = &P.S[(size_t)c * lenL * lenL];
    double* S0 = &P.S0[(size_t)c * lenL];
    for (int i = 0; i < lenT; ++i) {
      int row = loc * lenT + i;
      for (int j = 0; j < lenL; ++j) S[row + (size_t)j * lenL] = 0.0;
      S0[row] = 0.0;
    }
    for (int i = 0; i < lenT; ++i) {
      int row = loc * lenT + i;
      S[row + (size_t)row * lenL] += 1.0;
      S0[row] += dir[(size_t)f * lenT + i];
    }
  }
}

// Global trace index (faceID*Nf + face2CellMap)*nd + k (HDGSolver.cpp:589-598) and
// the AIJ pattern with every entry of every element block kept.
static void build_csr_nd(Problem& P, int nd) {
  int F = P.re->nFaces, Nf = P.re->face->nNodes, N = P.re->nNodes, lenL = P.lenL, B = Nf * nd;
  int ndofs = P.mf.nFaces * B;
  std::vector<std::set<int>> faceNbr(P.mf.nFaces);
  for (int c = 0; c < P.nCells; ++c)
    for (int i = 0; i < F; ++i)
      for (int j = 0; j < F; ++j) faceNbr[P.mf.cell2face[(size_t)c * F + i]].insert(P.mf.cell2face[(size_t)c * F + j]);
  P.rowptr.assign(ndofs + 1, 0);
  for (int f = 0; f < P.mf.nFaces; ++f)
    for (int a = 0; a < B; ++a) P.rowptr[f * B + a + 1] = (int)faceNbr[f].size() * B;
  for (int r = 0; r < ndofs; ++r) P.rowptr[r + 1] += P.rowptr[r];
  P.col.assign(P.rowptr[ndofs], 0);
  for (int f = 0; f < P.mf.nFaces; ++f)
    for (int a = 0; a < B; ++a) {
      int k = P.rowptr[f * B + a];
      for (int g : faceNbr[f])
        for (int b = 0; b < B; ++b) P.col[k++] = g * B + b;
    }
  P.val.assign(P.col.size(), 0.0);
  P.rhs.assign(ndofs, 0.0);
  std::vector<int> rc(lenL);
  for (int c = 0; c < P.nCells; ++c) {
    const int* cell = &P.cells[(size_t)c * N];
    for (int i = 0; i < F; ++i) {
      int f = P.mf.cell2face[(size_t)c * F + i];
      const int* face = &P.mf.faces[(size_t)f * Nf];
      for (int j = 0; j < Nf; ++j) {
        int node = cell[P.re->faceNodes[i][j]], pos = 0;
        while (face[pos] != node) ++pos;
        for (int k = 0; k < nd; ++k) rc[(i * Nf + j) * nd + k] = (f * Nf + pos) * nd + k;
      }
    }
    const double* S = &P.S[(size_t)c * lenL * lenL];
    for (int i = 0; i < lenL; ++i) {
      int row = rc[i];
      int* cb = &P.col[P.rowptr[row]];
      int len = P.rowptr[row + 1] - P.rowptr[row];
      for (int j = 0; j < lenL; ++j) {
        int k = (int)(std::lower_bound(cb, cb + len, rc[j]) - cb);
        P.val[P.rowptr[row] + k] += S[i + (size_t)j * lenL];
      }
      P.rhs[row] += P.S0[(size_t)c * lenL + i];
    }
  }
}

// Local recovery (HDGSolver.cpp:741-775) with nd values per trace node.
static void recover_nd(const Problem& P, int nd, const double* trace, double* sol, double* flux) {
  int F = P.re->nFaces, Nf = P.re->face->nNodes, N = P.re->nNodes;
  int lenU = P.lenU, lenQ = P.lenQ, lenL = P.lenL;
  std::vector<double> lam(lenL);
  for (int c = 0; c < P.nCells; ++c) {
    const int* cell = &P.cells[(size_t)c * N];
    for (int i = 0; i < F; ++i) {
      int f = P.mf.cell2face[(size_t)c * F + i];
      const int* face = &P.mf.faces[(size_t)f * Nf];
      for (int j = 0; j < Nf; ++j) {
        int node = cell[P.re->faceNodes[i][j]], pos = 0;
        while (face[pos] != node) ++pos;
        for (int k = 0; k < nd; ++k) lam[(i * Nf + j) * nd + k] = trace[((size_t)f * Nf + pos) * nd + k];
      }
    }
    const double* U = &P.U[(size_t)c * lenU * lenL];
    const double* Q = &P.Q[(size_t)c * lenQ * lenL];
    for (int i = 0; i < lenU; ++i) {
      double s = 0.0;
      for (int j = 0; j < lenL; ++j) s += U[i + (size_t)j * lenU] * lam[j];
      sol[(size_t)c * lenU + i] = s + P.U0[(size_t)c * lenU + i];
    }
    for (int i = 0; i < lenQ; ++i) {
      double s = 0.0;
      for (int j = 0; j < lenL; ++j) s += Q[i + (size_t)j * lenQ] * lam[j];
      flux[(size_t)c * lenQ + i] = s + P.Q0[(size_t)c * lenQ + i];
    }
  }
}

}  // namespace orc

using namespace orc;

static std::string g_err;

#define ORC_TRY(...)               \
  try {                            \
    __VA_ARGS__;                   \
    return 0;                      \
  } catch (const std::exception& e) { \
    g_err = e.what();              \
    return -1;                     \
  }

extern "C" {

const char* orc_last_error() { return g_err.c_str(); }

int orc_refel_sizes(int dim, int order, int* out /* nNodes,nFaces,nNodesFace,nIP,nIPFace */) {
  ORC_TRY({
    RefEl* r = get_refel(dim, order);
    out[0] = r->nNodes;
    out[1] = r->nFaces;
    out[2] = r->face ? r->face->nNodes : 1;
    out[3] = r->nIP;
    out[4] = r->face ? r->face->nIP : 0;
  })
}

// nodes[N*d], faceNodes[F*Nf], ipX[nI*d], ipW[nI], phi[nI*N], dphi[nI*N*d]
int orc_refel_tables(int dim, int order, double* nodes, int* faceNodes, double* ipX, double* ipW,
                     double* phi, double* dphi) {
  ORC_TRY({
    RefEl* r = get_refel(dim, order);
    for (int i = 0; i < r->nNodes; ++i)
      for (int k = 0; k < dim; ++k) nodes[i * dim + k] = r->nodes[i][k];
    int Nf = r->face ? r->face->nNodes : 1;
    for (int f = 0; f < r->nFaces; ++f)
      for (int j = 0; j < Nf; ++j) faceNodes[f * Nf + j] = r->faceNodes[f][j];
    for (int q = 0; q < r->nIP; ++q) {
      for (int k = 0; k < dim; ++k) ipX[q * dim + k] = r->ipX[q][k];
      ipW[q] = r->ipW[q];
      for (int i = 0; i < r->nNodes; ++i) {
        phi[q * r->nNodes + i] = r->phi[q][i];
        for (int k = 0; k < dim; ++k) dphi[(q * r->nNodes + i) * dim + k] = r->dphi[q][i][k];
      }
    }
  })
}

// Cubature rule of a given polynomial order (Cubature.cpp nIPMap); returns the
// number of points (negative if cap is too small).
int orc_cubature(int dim, int order, double* X, double* W, int cap) {
  try {
    std::vector<std::vector<double>> x;
    std::vector<double> w;
    simplex_cubature(dim, order, x, w);
    int n = (int)w.size();
    if (n > cap) return -n;
    for (int i = 0; i < n; ++i) {
      for (int k = 0; k < dim; ++k) X[i * dim + k] = x[i][k];
      W[i] = w[i];
    }
    return n;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1000000;
  }
}

// Lagrange basis / gradients at arbitrary reference points (for the reference's
// Lagrange-property and monomial tests, TestReferenceElement.cpp:117-236).
int orc_refel_eval(int dim, int order, int npts, const double* pts, double* phi, double* dphi) {
  ORC_TRY({
    RefEl* r = get_refel(dim, order);
    for (int p = 0; p < npts; ++p) {
      std::vector<double> x(pts + p * dim, pts + (p + 1) * dim);
      auto v = r->interpolate(x);
      auto g = r->interpolate_d(x);
      for (int i = 0; i < r->nNodes; ++i) {
        phi[p * r->nNodes + i] = v[i];
        for (int k = 0; k < dim; ++k) dphi[(p * r->nNodes + i) * dim + k] = g[i][k];
      }
    }
  })
}

void* orc_problem_create(int dim, int order, int nNodes, const double* coords, int nCells,
                         const int* cells) {
  try {
    Problem* P = new Problem();
    P->dim = dim;
    P->order = order;
    P->nNodes = nNodes;
    P->nCells = nCells;
    P->re = get_refel(dim, order);
    int N = P->re->nNodes;
    P->coords.assign(coords, coords + (size_t)nNodes * dim);
    P->cells.assign(cells, cells + (size_t)nCells * N);
    P->mf = compute_faces(dim, order, nCells, cells);
    P->lenU = N;
    P->lenQ = dim * N;
    P->lenL = P->re->nFaces * P->re->face->nNodes;
    P->nloc = P->lenU + P->lenQ + P->lenL;
    int Nf = P->re->face->nNodes;
    P->tau.assign((size_t)P->mf.nFaces * Nf, 1.0);
    P->dirichlet.assign((size_t)P->mf.nFaces * Nf, 0.0);
    return P;
  } catch (const std::exception& e) {
    g_err = e.what();
    return nullptr;
  }
}

void orc_problem_destroy(void* h) { delete (Problem*)h; }

// out: nFaces, nBoundary
int orc_problem_face_counts(void* h, int* out) {
  Problem* P = (Problem*)h;
  out[0] = P->mf.nFaces;
  out[1] = (int)P->mf.boundary.size();
  return 0;
}

int orc_problem_faces(void* h, int* cell2face, int* face2cell, int* faces, int* boundary) {
  Problem* P = (Problem*)h;
  std::copy(P->mf.cell2face.begin(), P->mf.cell2face.end(), cell2face);
  std::copy(P->mf.face2cell.begin(), P->mf.face2cell.end(), face2cell);
  std::copy(P->mf.faces.begin(), P->mf.faces.end(), faces);
  std::copy(P->mf.boundary.begin(), P->mf.boundary.end(), boundary);
  return 0;
}

// tau: nFaces*Nf*tauVals (tauVals 1 or 2); kappa: nCells*N*kc (kc 0,1,d*d);
// srcMode 0/1/2 with src nCells*nI for mode 1; dirichlet: nFaces*Nf;
// dt > 0 turns on implicit Euler with uOld nCells*N.
int orc_problem_set_fields(void* h, const double* tau, int tauVals, const double* kappa, int kc,
                           int srcMode, const double* src, const double* dirichlet, double dt,
                           const double* uOld) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    int Nf = P->re->face->nNodes, N = P->re->nNodes;
    P->tauVals = tauVals;
    P->tau.assign(tau, tau + (size_t)P->mf.nFaces * Nf * tauVals);
    P->kc = kc;
    if (kc) P->kappa.assign(kappa, kappa + (size_t)P->nCells * N * kc);
    P->srcMode = srcMode;
    if (srcMode == 1) P->src.assign(src, src + (size_t)P->nCells * P->re->nIP);
    if (dirichlet) P->dirichlet.assign(dirichlet, dirichlet + (size_t)P->mf.nFaces * Nf);
    P->dt = dt;
    if (dt > 0.0) P->uOld.assign(uOld, uOld + (size_t)P->nCells * N);
  })
}

// RungeKutta::apply on a given stiffness K (lenU x n, column-major) and rhs (lenU),
// mass M (lenU x lenU): the same algebra the element systems get.
int orc_rk_apply(int lenU, int n, double* K, double* rhs, const double* M, const double* ut, const double* comb,
                 double dt, double aDiag) {
  ORC_TRY({
    Mat A(lenU, n), Mm(lenU, lenU);
    std::copy(K, K + (size_t)lenU * n, A.a.begin());
    std::copy(M, M + (size_t)lenU * lenU, Mm.a.begin());
    std::vector<double> r(rhs, rhs + lenU), u(ut, ut + n), c(comb, comb + n);
    rk_apply(A, r, lenU, n, Mm, u, c, dt, aDiag);
    std::copy(A.a.begin(), A.a.end(), K);
    std::copy(r.begin(), r.end(), rhs);
  })
}

// Runge-Kutta stage on the U rows (RungeKutta.cpp:90-129); dt <= 0 switches it off.
int orc_problem_set_rk(void* h, double dt, double aDiag, const double* oldU, const double* oldQ,
                       const double* oldL, const double* combU, const double* combQ, const double* combL) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    P->rkDt = dt;
    P->rkDiag = aDiag;
    if (dt > 0.0) {
      const size_t nu = (size_t)P->nCells * P->re->nNodes, nq = nu * P->dim,
                   nl = (size_t)P->mf.nFaces * P->re->face->nNodes;
      P->rkOldU.assign(oldU, oldU + nu);
      P->rkOldQ.assign(oldQ, oldQ + nq);
      P->rkOldL.assign(oldL, oldL + nl);
      P->rkCombU.assign(combU, combU + nu);
      P->rkCombQ.assign(combQ, combQ + nq);
      P->rkCombL.assign(combL, combL + nl);
    }
  })
}

// Physical coordinates of the volume integration points, nCells*nI*d.
int orc_problem_ip_coords(void* h, double* out) {
  Problem* P = (Problem*)h;
  const RefEl* re = P->re;
  int N = re->nNodes, d = P->dim;
  for (int c = 0; c < P->nCells; ++c)
    for (int q = 0; q < re->nIP; ++q)
      for (int k = 0; k < d; ++k) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) s += re->phi[q][i] * P->coords[(size_t)P->cells[(size_t)c * N + i] * d + k];
        out[((size_t)c * re->nIP + q) * d + k] = s;
      }
  return 0;
}

// Element-local stage over elements [first, first+count) (count <= 0: all).
int orc_problem_local(void* h, int nthreads, int first, int count) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    if (P->S.empty()) {
      P->S.assign((size_t)P->nCells * P->lenL * P->lenL, 0.0);
      P->S0.assign((size_t)P->nCells * P->lenL, 0.0);
      P->U.assign((size_t)P->nCells * P->lenU * P->lenL, 0.0);
      P->Q.assign((size_t)P->nCells * P->lenQ * P->lenL, 0.0);
      P->U0.assign((size_t)P->nCells * P->lenU, 0.0);
      P->Q0.assign((size_t)P->nCells * P->lenQ, 0.0);
    }
    if (count <= 0) {
      first = 0;
      count = P->nCells;
    }
    double t0 = now();
    element_loop(*P, nthreads, first, count);
    P->t_local = now() - t0;
  })
}

// Full assemble: local + Dirichlet + CSR (HDGSolver::assemble, HDGSolver.cpp:166-174).
int orc_problem_assemble(void* h, int nthreads) {
  Problem* P = (Problem*)h;
  if (orc_problem_local(h, nthreads, 0, 0)) return -1;
  ORC_TRY({
    double t0 = now();
    apply_dirichlet(*P);
    double t1 = now();
    build_csr(*P);
    double t2 = now();
    P->t_bc = t1 - t0;
    P->t_scatter = t2 - t1;
  })
}

// Local matrix and RHS of one element (column-major n*n, n) before condensation.
int orc_problem_local_matrix(void* h, int iEl, double* A, double* rhs, int* face2cellmap) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    Mat M;
    std::vector<double> r;
    std::vector<int> f2c;
    local_system(*P, iEl, M, r, &f2c);
    std::copy(M.a.begin(), M.a.end(), A);
    std::copy(r.begin(), r.end(), rhs);
    if (face2cellmap) std::copy(f2c.begin(), f2c.end(), face2cellmap);
  })
}

// Condensed blocks of a list of elements only (compact outputs [count][...], the
// Dirichlet Set applied to their boundary faces as the full assembly applies it):
// element-block parity on meshes too large to condense whole.
int orc_problem_sample(void* h, int nthreads, int count, const int* ids, double* S, double* S0, double* U,
                       double* Q, double* U0, double* Q0) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    const size_t lU = P->lenU, lQ = P->lenQ, lL = P->lenL;
    for (int k = 0; k < count; ++k)
      if (ids[k] < 0 || ids[k] >= P->nCells) throw std::runtime_error("element id out of range");
    parallel_for(count, nthreads, [&](int k) {
      Mat A;
      std::vector<double> r;
      local_system(*P, ids[k], A, r);
      const size_t e = (size_t)k;
      condense_to(*P, ids[k], A, r,
                  CondensedOut{S + e * lL * lL, S0 + e * lL, U ? U + e * lU * lL : nullptr,
                               Q ? Q + e * lQ * lL : nullptr, U0 ? U0 + e * lU : nullptr, Q0 ? Q0 + e * lQ : nullptr});
      dirichlet_element(*P, ids[k], S + e * lL * lL, S0 + e * lL);
    });
  })
}

// The trace-system rows of a list of faces (all Nf rows of each, in face order),
// built as build_csr builds them but from the condensed blocks of the cells that
// touch those faces only. Outputs: rowlen[nsel*Nf], then col/val of the rows back
// to back (cap entries at most) and rhs[nsel*Nf]. Returns the entry count.
long orc_problem_face_rows(void* h, int nthreads, int nsel, const int* faceIds, int* rowlen, int* col, double* val,
                           double* rhs, long cap) {
  try {
    Problem* P = (Problem*)h;
    const int F = P->re->nFaces, Nf = P->re->face->nNodes, N = P->re->nNodes, lenL = P->lenL;
    std::vector<int> cellsOf;  // cells touching the selected faces, ascending (build_csr's order)
    for (int k = 0; k < nsel; ++k) {
      int f = faceIds[k];
      if (f < 0 || f >= P->mf.nFaces) throw std::runtime_error("face id out of range");
      for (int sd = 0; sd < 2; ++sd)
        if (P->mf.face2cell[2 * f + sd] >= 0) cellsOf.push_back(P->mf.face2cell[2 * f + sd]);
    }
    std::sort(cellsOf.begin(), cellsOf.end());
    cellsOf.erase(std::unique(cellsOf.begin(), cellsOf.end()), cellsOf.end());
    const int nc = (int)cellsOf.size();
    std::vector<double> S((size_t)nc * lenL * lenL), S0((size_t)nc * lenL);
    parallel_for(nc, nthreads, [&](int k) {
      Mat A;
      std::vector<double> r;
      local_system(*P, cellsOf[k], A, r);
      condense_to(*P, cellsOf[k], A, r,
                  CondensedOut{&S[(size_t)k * lenL * lenL], &S0[(size_t)k * lenL], nullptr, nullptr, nullptr, nullptr});
      dirichlet_element(*P, cellsOf[k], &S[(size_t)k * lenL * lenL], &S0[(size_t)k * lenL]);
    });
    // row layout: the sorted set of faces of the cells touching f
    std::vector<std::vector<int>> cols(nsel);
    long total = 0;
    std::map<int, int> selIndex;
    for (int k = 0; k < nsel; ++k) {
      int f = faceIds[k];
      if (!selIndex.emplace(f, k).second) throw std::runtime_error("face listed twice");
      std::set<int> nb;
      for (int sd = 0; sd < 2; ++sd) {
        int c = P->mf.face2cell[2 * f + sd];
        if (c < 0) continue;
        for (int i = 0; i < F; ++i) nb.insert(P->mf.cell2face[(size_t)c * F + i]);
      }
      for (int g : nb)
        for (int b = 0; b < Nf; ++b) cols[k].push_back(g * Nf + b);
      total += (long)cols[k].size() * Nf;
    }
    if (total > cap) return -total;
    std::vector<long> start(nsel + 1, 0);
    for (int k = 0; k < nsel; ++k) start[k + 1] = start[k] + (long)cols[k].size() * Nf;
    for (int k = 0; k < nsel; ++k)
      for (int a = 0; a < Nf; ++a) {
        rowlen[k * Nf + a] = (int)cols[k].size();
        std::copy(cols[k].begin(), cols[k].end(), col + start[k] + (long)a * cols[k].size());
        std::fill(val + start[k] + (long)a * cols[k].size(), val + start[k] + (long)(a + 1) * cols[k].size(), 0.0);
        rhs[k * Nf + a] = 0.0;
      }
    std::vector<int> rc(lenL);
    for (int kc = 0; kc < nc; ++kc) {
      int c = cellsOf[kc];
      const int* cell = &P->cells[(size_t)c * N];
      for (int i = 0; i < F; ++i) {
        int f = P->mf.cell2face[(size_t)c * F + i];
        const int* face = &P->mf.faces[(size_t)f * Nf];
        for (int j = 0; j < Nf; ++j) {
          int node = cell[P->re->faceNodes[i][j]], pos = 0;
          while (face[pos] != node) ++pos;
          rc[i * Nf + j] = f * Nf + pos;
        }
      }
      const double* Se = &S[(size_t)kc * lenL * lenL];
      for (int i = 0; i < lenL; ++i) {
        auto it = selIndex.find(rc[i] / Nf);
        if (it == selIndex.end()) continue;
        int k = it->second, a = rc[i] % Nf;
        const std::vector<int>& cb = cols[k];
        long base = start[k] + (long)a * cb.size();
        for (int j = 0; j < lenL; ++j) {
          int pos = (int)(std::lower_bound(cb.begin(), cb.end(), rc[j]) - cb.begin());
          val[base + pos] += Se[i + (size_t)j * lenL];
        }
        rhs[k * Nf + a] += S0[(size_t)kc * lenL + i];
      }
    }
    return total;
  } catch (const std::exception& e) {
    g_err = e.what();
    return -1;
  }
}

// CG element operators of one DOF per node, element by element, restated loop for loop:
// Mass::assemble (Mass.cpp:5-38), Diffusion::assemble (Diffusion.cpp:5-43) with the nodal
// diffusion field interpolated to the IPs as Diffusion::setDiffTensor does (Diffusion.cpp:59-69;
// scalar kc = 1 times the identity, or a d x d tensor stored column-major, kc = d*d; none:
// identity), Convection::assemble (Convection.cpp:21-46) with the nodal velocity interpolated
// as Convection::setVelocity does (Convection.cpp:5-19). vel: [nCells][N][d] (may be null when
// bit 2 is not asked). out: [nCells][3][N*N], op(i, j) at j*N + i; which: bit 0 mass, bit 1
// diffusion, bit 2 convection (the others are left untouched).
int orc_problem_cg_operators(void* h, int which, const double* vel, double* out) {
  ORC_TRY({
    Problem& P = *(Problem*)h;
    const RefEl* re = P.re;
    const int d = P.dim, N = re->nNodes, nI = re->nIP;
    if ((which & 4) && !vel) throw std::runtime_error("convection needs a velocity");
    for (int e = 0; e < P.nCells; ++e) {
      const int* cell = &P.cells[(size_t)e * N];
      double* oM = out + ((size_t)e * 3 + 0) * N * N;
      double* oD = out + ((size_t)e * 3 + 1) * N * N;
      double* oC = out + ((size_t)e * 3 + 2) * N * N;
      for (int k = 0; k < 3; ++k)
        if (which & (1 << k)) std::fill(out + ((size_t)e * 3 + k) * N * N, out + ((size_t)e * 3 + k + 1) * N * N, 0.0);
      for (int q = 0; q < nI; ++q) {
        Mat J(d, d);
        for (int i = 0; i < N; ++i)
          for (int r = 0; r < d; ++r)
            for (int t = 0; t < d; ++t) J(r, t) += re->dphi[q][i][r] * P.coords[(size_t)cell[i] * d + t];
        const double dv = re->ipW[q] * det_small(J);
        const Mat iJ = inverse(J);
        // gradShapes.col(i) = invJ * dphi_i
        std::vector<std::vector<double>> g(N, std::vector<double>(d, 0.0));
        for (int i = 0; i < N; ++i)
          for (int a = 0; a < d; ++a)
            for (int r = 0; r < d; ++r) g[i][a] += iJ(a, r) * re->dphi[q][i][r];
        if (which & 1)
          for (int j = 0; j < N; ++j)
            for (int k = 0; k < N; ++k) oM[k * N + j] += re->phi[q][j] * re->phi[q][k] * dv;
        if (which & 2) {
          Mat K(d, d);
          for (int a = 0; a < d; ++a) K(a, a) = P.kc == 0 ? 1.0 : 0.0;
          if (P.kc > 0)
            for (int j = 0; j < N; ++j) {
              const double* kn = &P.kappa[((size_t)e * N + j) * P.kc];
              for (int a = 0; a < d; ++a)
                for (int b = 0; b < d; ++b)
                  K(a, b) += re->phi[q][j] * (P.kc == 1 ? (a == b ? kn[0] : 0.0) : kn[a + b * d]);
            }
          for (int i = 0; i < N; ++i)
            for (int j = 0; j < N; ++j) {
              double v = 0.0;  // (K grad phi_i)^T grad phi_j
              for (int a = 0; a < d; ++a) {
                double kg = 0.0;
                for (int b = 0; b < d; ++b) kg += K(a, b) * g[i][b];
                v += kg * g[j][a];
              }
              oD[j * N + i] += v * dv;
            }
        }
        if (which & 4) {
          std::vector<double> vq(d, 0.0), meas(d, 0.0);
          for (int j = 0; j < N; ++j)
            for (int a = 0; a < d; ++a) vq[a] += vel[((size_t)e * N + j) * d + a] * re->phi[q][j];
          for (int r = 0; r < d; ++r)
            for (int a = 0; a < d; ++a) meas[r] += dv * vq[a] * iJ(a, r);  // dV (v^T invJ)^T
          for (int k = 0; k < N; ++k)
            for (int l = 0; l < N; ++l) {
              double dot = 0.0;
              for (int r = 0; r < d; ++r) dot += meas[r] * re->dphi[q][l][r];
              oC[l * N + k] += dot * re->phi[q][k];
            }
        }
      }
    }
  })
}

int orc_problem_condensed(void* h, double* S, double* S0, double* U, double* Q, double* U0, double* Q0) {
  Problem* P = (Problem*)h;
  std::copy(P->S.begin(), P->S.end(), S);
  std::copy(P->S0.begin(), P->S0.end(), S0);
  if (U) std::copy(P->U.begin(), P->U.end(), U);
  if (Q) std::copy(P->Q.begin(), P->Q.end(), Q);
  if (U0) std::copy(P->U0.begin(), P->U0.end(), U0);
  if (Q0) std::copy(P->Q0.begin(), P->Q0.end(), Q0);
  return 0;
}

long orc_problem_nnz(void* h) { return (long)((Problem*)h)->col.size(); }

int orc_problem_csr(void* h, int* rowptr, int* col, double* val, double* rhs) {
  Problem* P = (Problem*)h;
  std::copy(P->rowptr.begin(), P->rowptr.end(), rowptr);
  std::copy(P->col.begin(), P->col.end(), col);
  std::copy(P->val.begin(), P->val.end(), val);
  std::copy(P->rhs.begin(), P->rhs.end(), rhs);
  return 0;
}

// GMRES(30)+Jacobi solve; returns iterations (negative if not converged).
int orc_problem_solve(void* h, double rtol, int maxit, int nthreads, double* x) {
  Problem* P = (Problem*)h;
  std::vector<double> sol;
  double t0 = now();
  int it = gmres(*P, sol, rtol, maxit, nthreads);
  P->t_solve = now() - t0;
  P->iters = it;
  std::copy(sol.begin(), sol.end(), x);
  return it;
}

int orc_problem_recover(void* h, const double* trace, double* sol, double* flux) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    double t0 = now();
    recover(*P, trace, sol, flux);
    P->t_recover = now() - t0;
  })
}

// Stage timings in seconds: local, dirichlet, scatter, solve, recover.
int orc_problem_set_solver(void* h, int type, const double* sol, const double* flux) {
  ORC_TRY({
    Problem& P = *(Problem*)h;
    if (type < 0 || type > 2) throw std::runtime_error("solver type 0..2");
    P.solverType = type;
    if (type != 0) {
      if (!sol || !flux) throw std::runtime_error("explicit modes need Solution and Flux");
      P.solState.assign(sol, sol + (size_t)P.nCells * P.lenU);
      P.fluxState.assign(flux, flux + (size_t)P.nCells * P.lenQ);
    }
  });
  return 0;
}

// SEXPLICIT trace (HDGSolver.cpp:709-729): every face solves its own assembled
// block, trace_f = S_f^{-1} S0_f. The per-face S_f, S0_f are the sums of the
// element face blocks (Add), which here are the diagonal blocks of the CSR.
int orc_problem_solve_faces(void* h, double* x) {
  ORC_TRY({
    Problem& P = *(Problem*)h;
    const int Nf = P.re->face->nNodes;
    const int nF = (int)P.mf.face2cell.size() / 2;
    for (int f = 0; f < nF; ++f) {
      Mat B(Nf, Nf), b(Nf, 1);
      for (int a = 0; a < Nf; ++a) {
        const int row = f * Nf + a;
        b(a, 0) = P.rhs[row];
        for (int k = P.rowptr[row]; k < P.rowptr[row + 1]; ++k) {
          const int c = P.col[k];
          if (c / Nf == f) B(a, c % Nf) = P.val[k];
        }
      }
      std::vector<int> piv;
      if (!lu_factor(B, piv)) throw std::runtime_error("singular face block");
      lu_solve(B, piv, b);
      for (int a = 0; a < Nf; ++a) x[(size_t)f * Nf + a] = b(a, 0);
    }
  });
  return 0;
}

int orc_problem_timings(void* h, double* out) {
  Problem* P = (Problem*)h;
  out[0] = P->t_local;
  out[1] = P->t_bc;
  out[2] = P->t_scatter;
  out[3] = P->t_solve;
  out[4] = P->t_recover;
  return 0;
}

// ---------------------------------------------------------------- Burgers
// A problem with nd = dim unknowns per node (HDGBurgersModel.cpp:35-60). Defaults:
// tau = identity, no diffusion, no source, Dirichlet 0, stationary, buffer and trace 0.
void* orc_burgers_create(int dim, int order, int nNodes, const double* coords, int nCells, const int* cells) {
  Problem* P = (Problem*)orc_problem_create(dim, order, nNodes, coords, nCells, cells);
  if (!P) return nullptr;
  const int nd = dim, N = P->re->nNodes, F = P->re->nFaces, Nf = P->re->face->nNodes;
  P->lenU = N * nd;
  P->lenQ = dim * N * nd;
  P->lenL = F * Nf * nd;
  P->nloc = P->lenU + P->lenQ + P->lenL;
  BurgersFields& B = g_burgers[P];
  B.tau.assign((size_t)P->mf.nFaces * Nf * nd * nd, 0.0);
  for (size_t k = 0; k < (size_t)P->mf.nFaces * Nf; ++k)
    for (int c = 0; c < nd; ++c) B.tau[k * nd * nd + c * nd + c] = 1.0;
  B.dir.assign((size_t)P->mf.nFaces * Nf * nd, 0.0);
  B.buf.assign((size_t)nCells * N * nd, 0.0);
  B.trace.assign((size_t)P->mf.nFaces * Nf * nd, 0.0);
  return P;
}

void orc_burgers_destroy(void* h) {
  g_burgers.erase((Problem*)h);
  delete (Problem*)h;
}

// tau [nFaces][Nf][sides][nd*nd]; nu [nCells][N][kc] (kc 0, 1 or d*d); src
// [nCells][nI][nd] or null; dir [nFaces][Nf][nd]; dt > 0: implicit Euler on
// old [nCells][N*nd].
int orc_burgers_set_fields(void* h, const double* tau, int tauSides, const double* nu, int kc, const double* src,
                           const double* dir, double dt, const double* old) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    BurgersFields& B = g_burgers.at(P);
    const int nd = P->dim, N = P->re->nNodes, Nf = P->re->face->nNodes;
    if (tau) {
      B.tauSides = tauSides;
      B.tau.assign(tau, tau + (size_t)P->mf.nFaces * Nf * tauSides * nd * nd);
    }
    B.kc = kc;
    B.nu.assign(nu, nu + (kc ? (size_t)P->nCells * N * kc : 0));
    B.src.assign(src, src + (src ? (size_t)P->nCells * P->re->nIP * nd : 0));
    if (dir) B.dir.assign(dir, dir + (size_t)P->mf.nFaces * Nf * nd);
    B.dt = dt;
    B.old.assign(old, old + (dt > 0.0 ? (size_t)P->nCells * N * nd : 0));
  })
}

// BufferSolution [nCells][N*nd] and Trace [nFaces][Nf*nd] the operator is linearised about.
int orc_burgers_set_state(void* h, const double* buf, const double* trace) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    BurgersFields& B = g_burgers.at(P);
    if (buf) std::copy(buf, buf + B.buf.size(), B.buf.begin());
    if (trace) std::copy(trace, trace + B.trace.size(), B.trace.begin());
  })
}

int orc_burgers_local_matrix(void* h, int iEl, double* A, double* rhs) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    Mat M;
    std::vector<double> r;
    burgers_local_system(*P, g_burgers.at(P), iEl, M, r);
    std::copy(M.a.begin(), M.a.end(), A);
    std::copy(r.begin(), r.end(), rhs);
  })
}

// HDGSolver::assemble (HDGSolver.cpp:166-174) with the Burgers model: local systems,
// condensation, Dirichlet Set, CSR.
int orc_burgers_assemble(void* h, int nthreads) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    const BurgersFields& B = g_burgers.at(P);
    P->S.assign((size_t)P->nCells * P->lenL * P->lenL, 0.0);
    P->S0.assign((size_t)P->nCells * P->lenL, 0.0);
    P->U.assign((size_t)P->nCells * P->lenU * P->lenL, 0.0);
    P->Q.assign((size_t)P->nCells * P->lenQ * P->lenL, 0.0);
    P->U0.assign((size_t)P->nCells * P->lenU, 0.0);
    P->Q0.assign((size_t)P->nCells * P->lenQ, 0.0);
    P->solverType = 0;
    double t0 = now();
    parallel_for(P->nCells, nthreads, [&](int iEl) {
      Mat A;
      std::vector<double> r;
      burgers_local_system(*P, B, iEl, A, r);
      condense(*P, iEl, A, r);
    });
    double t1 = now();
    apply_dirichlet_nd(*P, P->dim, B.dir);
    build_csr_nd(*P, P->dim);
    P->t_local = t1 - t0;
    P->t_scatter = now() - t1;
  })
}

int orc_burgers_recover(void* h, const double* trace, double* sol, double* flux) {
  ORC_TRY({
    Problem* P = (Problem*)h;
    recover_nd(*P, P->dim, trace, sol, flux);
  })
}

// HDGUNabU assembled on the reference element the way its unit test sets it up
// (TestHDGUNabU.cpp:36-66): identity volume Jacobians with dV = the cubature weights,
// face measures from the face Jacobians of the reference faces, the reference normals
// (TestUtils.h getRefNormals). sol [N][nd], trace [F*Nf][nd] (nd = dim); op n x n
// column-major, rhs n.
int orc_unabu_refel(int dim, int order, const double* sol, const double* trace, double* op, double* rhs) {
  ORC_TRY({
    RefEl* re = get_refel(dim, order);
    const RefEl* fe = re->face;
    int nI = re->nIP, nIf = fe->nIP, F = re->nFaces, Nf = fe->nNodes, nd = dim;
    std::vector<double> dV(nI + F * nIf, 0.0);
    std::vector<Mat> invJ(nI, Mat(dim, dim));
    for (int q = 0; q < nI; ++q) {
      dV[q] = re->ipW[q];
      for (int k = 0; k < dim; ++k) invJ[q](k, k) = 1.0;
    }
    for (int f = 0; f < F; ++f)
      for (int q = 0; q < nIf; ++q) {
        Mat J(dim - 1, dim);
        for (int i = 0; i < Nf; ++i)
          for (int r = 0; r < dim - 1; ++r)
            for (int s = 0; s < dim; ++s) J(r, s) += fe->dphi[q][i][r] * re->nodes[re->faceNodes[f][i]][s];
        Mat JJt(dim - 1, dim - 1);
        for (int a = 0; a < dim - 1; ++a)
          for (int b = 0; b < dim - 1; ++b)
            for (int s = 0; s < dim; ++s) JJt(a, b) += J(a, s) * J(b, s);
        dV[nI + f * nIf + q] = fe->ipW[q] * std::sqrt(det_small(JJt));
      }
    std::vector<std::vector<double>> refN;
    if (dim == 2) {
      refN = {{0, -1}, {1.0 / std::sqrt(2.0), 1.0 / std::sqrt(2.0)}, {-1, 0}};
    } else {
      double s3 = 1.0 / std::sqrt(3.0);
      refN = {{0, -1, 0}, {s3, s3, s3}, {-1, 0, 0}, {0, 0, -1}};
    }
    std::vector<std::vector<double>> normals(F * nIf);
    for (int f = 0; f < F; ++f)
      for (int q = 0; q < nIf; ++q) normals[f * nIf + q] = refN[f];
    std::vector<double> u(sol, sol + (size_t)re->nNodes * nd), t(trace, trace + (size_t)F * Nf * nd);
    Mat A;
    std::vector<double> r;
    unabu_nd(re, nd, dV, invJ, normals, u, t, A, r);
    std::copy(A.a.begin(), A.a.end(), op);
    std::copy(r.begin(), r.end(), rhs);
  })
}

}  // extern "C"
