// Reference simplex element tables on the host (FP64), built once per (dim, p)
// and staged into device memory by the context.
//
// Replaces ReferenceElement(dim, ord, "simplex") (ReferenceElement.cpp:5-26).
// The node positions and their order, the face-node lists and the cubature
// rules must be those of HyperFox, because they fix the layout of every
// element block and the trace numbering; the Lagrange basis is the same
// polynomial space (P_p) evaluated through an orthonormal Proriol-Koornwinder-
// Dubiner basis instead of the reference's unnormalised Dubiner modes, which
// gives the same Lagrange functions up to round-off.
#include <algorithm>
#include <cmath>
#include <map>
#include <stdexcept>

#include "hfx_host.h"
#include "cubature_tables.inc"

namespace hfx {
namespace {

// ---- dense LU inverse (row-major n x n) ----
bool invert(std::vector<double>& A, int n) {
  std::vector<double> I(n * n, 0.0);
  for (int i = 0; i < n; ++i) I[i * n + i] = 1.0;
  for (int k = 0; k < n; ++k) {
    int p = k;
    for (int i = k + 1; i < n; ++i)
      if (std::fabs(A[i * n + k]) > std::fabs(A[p * n + k])) p = i;
    if (A[p * n + k] == 0.0) return false;
    if (p != k)
      for (int j = 0; j < n; ++j) {
        std::swap(A[k * n + j], A[p * n + j]);
        std::swap(I[k * n + j], I[p * n + j]);
      }
    double inv = 1.0 / A[k * n + k];
    for (int j = 0; j < n; ++j) {
      A[k * n + j] *= inv;
      I[k * n + j] *= inv;
    }
    for (int i = 0; i < n; ++i) {
      if (i == k) continue;
      double f = A[i * n + k];
      if (f == 0.0) continue;
      for (int j = 0; j < n; ++j) {
        A[i * n + j] -= f * A[k * n + j];
        I[i * n + j] -= f * I[k * n + j];
      }
    }
  }
  A.swap(I);
  return true;
}

// ---- orthonormal Jacobi polynomials (weight (1-x)^a (1+x)^b on [-1,1]) ----
double jacobi_n(double x, double a, double b, int n) {
  double g0 = std::pow(2.0, a + b + 1.0) / (a + b + 1.0) * std::tgamma(a + 1.0) * std::tgamma(b + 1.0) /
              std::tgamma(a + b + 1.0);
  double p0 = 1.0 / std::sqrt(g0);
  if (n == 0) return p0;
  double g1 = (a + 1.0) * (b + 1.0) / (a + b + 3.0) * g0;
  double p1 = ((a + b + 2.0) * x / 2.0 + (a - b) / 2.0) / std::sqrt(g1);
  if (n == 1) return p1;
  double aold = 2.0 / (2.0 + a + b) * std::sqrt((a + 1.0) * (b + 1.0) / (a + b + 3.0));
  for (int i = 1; i < n; ++i) {
    double h1 = 2.0 * i + a + b;
    double anew = 2.0 / (h1 + 2.0) *
                  std::sqrt((i + 1.0) * (i + 1.0 + a + b) * (i + 1.0 + a) * (i + 1.0 + b) / (h1 + 1.0) / (h1 + 3.0));
    double bnew = -(a * a - b * b) / h1 / (h1 + 2.0);
    double p2 = (-aold * p0 + (x - bnew) * p1) / anew;
    p0 = p1;
    p1 = p2;
    aold = anew;
  }
  return p1;
}
double djacobi_n(double x, double a, double b, int n) {
  if (n == 0) return 0.0;
  return std::sqrt(n * (n + a + b + 1.0)) * jacobi_n(x, a + 1.0, b + 1.0, n - 1);
}

struct Mode {
  int i, j, k;
};

std::vector<Mode> modes_of(int dim, int p) {
  std::vector<Mode> m;
  for (int i = 0; i <= p; ++i)
    for (int j = 0; j <= (dim > 1 ? p - i : 0); ++j)
      for (int k = 0; k <= (dim > 2 ? p - i - j : 0); ++k) m.push_back({i, j, k});
  return m;
}

// Value and gradient of an orthonormal simplex mode at reference point x.
void pkd(int dim, const Mode& m, const double* x, double* val, double* grad) {
  if (dim == 1) {
    *val = jacobi_n(x[0], 0, 0, m.i);
    if (grad) grad[0] = djacobi_n(x[0], 0, 0, m.i);
    return;
  }
  if (dim == 2) {
    double r = x[0], s = x[1];
    double a = (s != 1.0) ? 2.0 * (1.0 + r) / (1.0 - s) - 1.0 : -1.0, b = s;
    double fa = jacobi_n(a, 0, 0, m.i), gb = jacobi_n(b, 2.0 * m.i + 1.0, 0, m.j);
    *val = std::sqrt(2.0) * fa * gb * std::pow(1.0 - b, m.i);
    if (grad) {
      double dfa = djacobi_n(a, 0, 0, m.i), dgb = djacobi_n(b, 2.0 * m.i + 1.0, 0, m.j);
      double hb = 0.5 * (1.0 - b);
      double dr = dfa * gb, ds = dfa * gb * 0.5 * (1.0 + a);
      if (m.i > 0) {
        dr *= std::pow(hb, m.i - 1);
        ds *= std::pow(hb, m.i - 1);
      }
      double t = dgb * std::pow(hb, m.i);
      if (m.i > 0) t -= 0.5 * m.i * gb * std::pow(hb, m.i - 1);
      ds += fa * t;
      double sc = std::pow(2.0, m.i + 0.5);
      grad[0] = dr * sc;
      grad[1] = ds * sc;
    }
    return;
  }
  double r = x[0], s = x[1], t = x[2];
  double a = (s + t != 0.0) ? 2.0 * (1.0 + r) / (-s - t) - 1.0 : -1.0;
  double b = (t != 1.0) ? 2.0 * (1.0 + s) / (1.0 - t) - 1.0 : -1.0;
  double c = t;
  double fa = jacobi_n(a, 0, 0, m.i);
  double gb = jacobi_n(b, 2.0 * m.i + 1.0, 0, m.j);
  double hc = jacobi_n(c, 2.0 * (m.i + m.j) + 2.0, 0, m.k);
  *val = 2.0 * std::sqrt(2.0) * fa * gb * std::pow(1.0 - b, m.i) * hc * std::pow(1.0 - c, m.i + m.j);
  if (grad) {
    double dfa = djacobi_n(a, 0, 0, m.i);
    double dgb = djacobi_n(b, 2.0 * m.i + 1.0, 0, m.j);
    double dhc = djacobi_n(c, 2.0 * (m.i + m.j) + 2.0, 0, m.k);
    double hb = 0.5 * (1.0 - b), hcc = 0.5 * (1.0 - c);
    double vr = dfa * gb * hc;
    if (m.i > 0) vr *= std::pow(hb, m.i - 1);
    if (m.i + m.j > 0) vr *= std::pow(hcc, m.i + m.j - 1);
    double vs = 0.5 * (1.0 + a) * vr;
    double tmp = dgb * std::pow(hb, m.i);
    if (m.i > 0) tmp += -0.5 * m.i * gb * std::pow(hb, m.i - 1);
    if (m.i + m.j > 0) tmp *= std::pow(hcc, m.i + m.j - 1);
    tmp = fa * tmp * hc;
    vs += tmp;
    double vt = 0.5 * (1.0 + a) * vr + 0.5 * (1.0 + b) * tmp;
    double tmp2 = dhc * std::pow(hcc, m.i + m.j);
    if (m.i + m.j > 0) tmp2 -= 0.5 * (m.i + m.j) * hc * std::pow(hcc, m.i + m.j - 1);
    tmp2 = fa * gb * tmp2 * std::pow(hb, m.i);
    vt += tmp2;
    double sc = std::pow(2.0, 2 * m.i + m.j + 1.5);
    grad[0] = vr * sc;
    grad[1] = vs * sc;
    grad[2] = vt * sc;
  }
}

// Legendre-Gauss-Lobatto interior points for order p, ascending.
std::vector<double> lobatto_interior(int p) {
  std::vector<double> out;
  for (int k = 1; k < p; ++k) {
    double x = -std::cos(M_PI * k / p);
    for (int it = 0; it < 60; ++it) {
      double f = djacobi_n(x, 0, 0, p);                  // proportional to P_p'
      double df = std::sqrt(p * (p + 1.0)) * djacobi_n(x, 1, 1, p - 1);
      double dx = f / df;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    out.push_back(x);
  }
  std::sort(out.begin(), out.end());
  return out;
}

// n-point Gauss-Legendre rule listed in HyperFox's order (Cubature.cpp:109-280):
// entries are signed 1-based indices of the positive roots (0 = the zero root).
void gauss_rule(int n, std::vector<double>* x, std::vector<double>* w) {
  static const int kOrder[12][11] = {
      {0}, {0}, {-1, 1}, {0, -1, 1}, {1, -1, 2, -2}, {0, 1, -1, 2, -2},
      {2, -2, -1, 1, -3, 3}, {0, 1, -1, -2, 2, -3, 3}, {-1, 1, -2, 2, -3, 3, -4, 4},
      {0, -3, 3, -4, 4, -1, 1, -2, 2}, {-1, 1, -2, 2, -3, 3, -4, 4, -5, 5},
      {0, -1, 1, -2, 2, -3, 3, -4, 4, -5, 5}};
  std::vector<double> pos;
  for (int k = 1; k <= n; ++k) {
    double t = std::cos(M_PI * (k - 0.25) / (n + 0.5));
    for (int it = 0; it < 60; ++it) {
      double f = jacobi_n(t, 0, 0, n), df = djacobi_n(t, 0, 0, n);
      double dt = f / df;
      t -= dt;
      if (std::fabs(dt) < 1e-16) break;
    }
    if (t > 1e-13) pos.push_back(t);
  }
  std::sort(pos.begin(), pos.end());
  x->clear();
  w->clear();
  for (int q = 0; q < n; ++q) {
    int s = kOrder[n][q];
    double t = s == 0 ? 0.0 : (s > 0 ? pos[s - 1] : -pos[-s - 1]);
    // w = 2 / ((1-t^2) P_n'(t)^2) with the monic-normalised Legendre P_n
    double dp = djacobi_n(t, 0, 0, n) / std::sqrt((2.0 * n + 1.0) / 2.0);
    x->push_back(t);
    w->push_back(2.0 / ((1.0 - t * t) * dp * dp));
  }
}

bool cubature(int dim, int order, std::vector<double>* X, std::vector<double>* W) {
  X->clear();
  W->clear();
  if (dim == 1) {
    int n = (order + 2) / 2;  // ceil((order+1)/2)
    if (n < 1 || n > 11) return false;
    gauss_rule(n, X, W);
    return true;
  }
  for (int k = 0; k < kNumCubatureRules; ++k) {
    const CubatureRuleEntry& e = kCubatureRules[k];
    if (e.dim != dim || e.order != order) continue;
    for (int i = 0; i < e.npts; ++i) {
      for (int d = 0; d < dim; ++d) X->push_back(e.data[i * (dim + 1) + d]);
      W->push_back(e.data[i * (dim + 1) + dim]);
    }
    return true;
  }
  return false;
}

const double kV2[3][2] = {{-1, -1}, {1, -1}, {-1, 1}};
const double kV3[4][3] = {{-1, -1, -1}, {1, -1, -1}, {-1, 1, -1}, {-1, -1, 1}};
const int kEdges2[3][2] = {{0, 1}, {1, 2}, {2, 0}};
const int kEdges3[6][2] = {{0, 1}, {1, 2}, {2, 0}, {3, 0}, {3, 1}, {3, 2}};
const int kFaces3[4][3] = {{3, 1, 0}, {2, 1, 3}, {2, 3, 0}, {0, 1, 2}};

const double* vert(int dim, int v) { return dim == 2 ? kV2[v] : kV3[v]; }

// Node positions in HyperFox order (ReferenceElement.cpp:1012-1150):
// vertices, edge interiors (per edge, from its first vertex), face interiors
// (3D, per face in the 2D interior order), then the warped volume interior.
std::vector<double> simplex_nodes(int dim, int p) {
  std::vector<double> X;
  if (dim == 1) {
    if (p == 0) return {0.0};
    X = {-1.0, 1.0};
    for (double x : lobatto_interior(p)) X.push_back(x);
    return X;
  }
  if (p == 0) return std::vector<double>(dim, 0.0);
  for (int v = 0; v <= dim; ++v)
    for (int d = 0; d < dim; ++d) X.push_back(vert(dim, v)[d]);
  std::vector<double> gll = lobatto_interior(p);
  int nE = dim == 2 ? 3 : 6;
  for (int e = 0; e < nE; ++e) {
    int a = dim == 2 ? kEdges2[e][0] : kEdges3[e][0];
    int b = dim == 2 ? kEdges2[e][1] : kEdges3[e][1];
    for (double x : gll)
      for (int d = 0; d < dim; ++d)
        X.push_back(vert(dim, a)[d] + 0.5 * (x + 1.0) * (vert(dim, b)[d] - vert(dim, a)[d]));
  }
  if (dim == 3) {
    std::vector<double> tri = simplex_nodes(2, p);
    int nBoundary2 = 3 + 3 * (p - 1);
    for (int f = 0; f < 4; ++f) {
      const double *v0 = kV3[kFaces3[f][0]], *v1 = kV3[kFaces3[f][1]], *v2 = kV3[kFaces3[f][2]];
      for (size_t n = nBoundary2; n < tri.size() / 2; ++n) {
        double l1 = 0.5 * (tri[2 * n] + 1.0), l2 = 0.5 * (tri[2 * n + 1] + 1.0);
        for (int d = 0; d < 3; ++d) X.push_back(v0[d] + l1 * (v1[d] - v0[d]) + l2 * (v2[d] - v0[d]));
      }
    }
  }
  if (p > 1) {
    // Lobatto abscissae ascending including the ends.
    std::vector<double> L(1, -1.0);
    for (double x : gll) L.push_back(x);
    L.push_back(1.0);
    auto coef = [&](int c0, int c1, int c2) {
      int s = c0 + c1 + (dim == 3 ? c2 : 0);
      double v = 2.0 + dim * L[c0] - L[c1] - (dim == 3 ? L[c2] : 0.0) - L[p - s];
      return v / (dim + 1.0) - 1.0;
    };
    if (dim == 2) {
      for (int c0 = 1; c0 < p; ++c0)
        for (int c1 = 1; c1 < p; ++c1)
          if (c0 + c1 < p) {
            X.push_back(coef(c0, c1, 0));
            X.push_back(coef(c1, c0, 0));
          }
    } else {
      for (int c0 = 1; c0 < p; ++c0)
        for (int c1 = 1; c1 < p; ++c1)
          for (int c2 = 1; c2 < p; ++c2)
            if (c0 + c1 + c2 < p) {
              X.push_back(coef(c0, c1, c2));
              X.push_back(coef(c1, c0, c2));
              X.push_back(coef(c2, c1, c0));
            }
    }
  }
  return X;
}

// Lagrange basis (value, gradient) at points, through the orthonormal modes.
void lagrange_tables(int dim, int p, const std::vector<double>& nodes, const std::vector<double>& pts,
                     std::vector<double>* phi, std::vector<double>* dphi) {
  std::vector<Mode> ms = modes_of(dim, p);
  int N = (int)ms.size();
  std::vector<double> V(N * N);
  double v;
  for (int i = 0; i < N; ++i)
    for (int m = 0; m < N; ++m) {
      pkd(dim, ms[m], &nodes[i * dim], &v, nullptr);
      V[i * N + m] = v;
    }
  if (!invert(V, N)) throw std::runtime_error("singular Vandermonde");
  int nP = (int)pts.size() / dim;
  phi->assign(nP * N, 0.0);
  dphi->assign(nP * N * dim, 0.0);
  std::vector<double> mv(N), mg(N * dim);
  for (int q = 0; q < nP; ++q) {
    for (int m = 0; m < N; ++m) pkd(dim, ms[m], &pts[q * dim], &mv[m], &mg[m * dim]);
    for (int j = 0; j < N; ++j) {
      double s = 0.0;
      for (int m = 0; m < N; ++m) s += mv[m] * V[m * N + j];
      (*phi)[q * N + j] = s;
      for (int d = 0; d < dim; ++d) {
        double g = 0.0;
        for (int m = 0; m < N; ++m) g += mg[m * dim + d] * V[m * N + j];
        (*dphi)[(q * N + j) * dim + d] = g;
      }
    }
  }
}

}  // namespace

bool build_refel(int dim, int p, RefEl* out, std::string* err) {
  try {
    if (dim < 2 || dim > 3 || p < 1 || (dim == 2 && p > 10) || (dim == 3 && p > 5)) {
      *err = "reference element: only simplices with dim 2 (p<=10) or 3 (p<=5)";
      return false;
    }
    RefEl r;
    r.dim = dim;
    r.order = p;
    r.nodes = simplex_nodes(dim, p);
    r.nNodes = (int)r.nodes.size() / dim;
    r.nFaces = dim + 1;
    std::vector<double> fnodes = simplex_nodes(dim - 1, p);
    r.nNodesFace = (int)fnodes.size() / (dim - 1);
    // face nodes: map the face element's nodes and find them (ReferenceElement.cpp:136-202)
    for (int f = 0; f < r.nFaces; ++f) {
      for (int l = 0; l < r.nNodesFace; ++l) {
        double x[3];
        if (dim == 2) {
          const double *a = kV2[kEdges2[f][0]], *b = kV2[kEdges2[f][1]];
          double t = 0.5 * (fnodes[l] + 1.0);
          for (int d = 0; d < 2; ++d) x[d] = a[d] + t * (b[d] - a[d]);
        } else {
          const double *v0 = kV3[kFaces3[f][0]], *v1 = kV3[kFaces3[f][1]], *v2 = kV3[kFaces3[f][2]];
          double l1 = 0.5 * (fnodes[2 * l] + 1.0), l2 = 0.5 * (fnodes[2 * l + 1] + 1.0);
          for (int d = 0; d < 3; ++d) x[d] = v0[d] + l1 * (v1[d] - v0[d]) + l2 * (v2[d] - v0[d]);
        }
        int found = -1;
        for (int n = 0; n < r.nNodes && found < 0; ++n) {
          bool eq = true;
          for (int d = 0; d < dim; ++d)
            if (std::fabs(r.nodes[n * dim + d] - x[d]) > 1e-12) eq = false;
          if (eq) found = n;
        }
        if (found < 0) {
          *err = "reference element: face node not found";
          return false;
        }
        r.faceNodes.push_back(found);
      }
      int opp = -1;
      for (int k = 0; k < r.nNodes && opp < 0; ++k) {
        bool on = false;
        for (int l = 0; l < r.nNodesFace; ++l)
          if (r.faceNodes[f * r.nNodesFace + l] == k) on = true;
        if (!on) opp = k;
      }
      r.faceOpposite.push_back(opp);
    }
    if (!cubature(dim, 2 * p, &r.ipX, &r.ipW) || !cubature(dim - 1, 2 * p, &r.fIpX, &r.fIpW)) {
      *err = "reference element: cubature order not tabulated";
      return false;
    }
    r.nIP = (int)r.ipW.size();
    r.nIPFace = (int)r.fIpW.size();
    lagrange_tables(dim, p, r.nodes, r.ipX, &r.phi, &r.dphi);
    lagrange_tables(dim - 1, p, fnodes, r.fIpX, &r.fPhi, &r.fDphi);
    *out = std::move(r);
    return true;
  } catch (const std::exception& e) {
    *err = std::string("reference element: ") + e.what();
    return false;
  }
}

}  // namespace hfx
