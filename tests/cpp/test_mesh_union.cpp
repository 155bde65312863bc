// Host-only checks of hfx::gpu::MeshUnion (no GPU): the union's face topology is every
// problem's own topology shifted by its offsets, the group tolerance arithmetic, and the
// refusal of mixed orders.
#include <cstdio>
#include <vector>

#include "hfx_host_api.hpp"

using hfx::gpu::ErrorHandle;
using hfx::gpu::Mesh;
using hfx::gpu::MeshUnion;

static int fails = 0;
#define CHECK(c)                                                   \
  do {                                                             \
    if (!(c)) {                                                    \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c);      \
      ++fails;                                                     \
    }                                                              \
  } while (0)

// n x n squares of the unit square, two triangles each, high-order nodes of `order`
static Mesh square(int n, int order) {
  std::vector<double> v;
  std::vector<int> t;
  for (int i = 0; i <= n; ++i)
    for (int j = 0; j <= n; ++j) {
      v.push_back((double)i / n);
      v.push_back((double)j / n);
    }
  auto id = [n](int i, int j) { return i * (n + 1) + j; };
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) {
      int a = id(i, j), b = id(i + 1, j), c = id(i, j + 1), d = id(i + 1, j + 1);
      t.insert(t.end(), {a, b, c, d, c, b});
    }
  Mesh m;
  m.dim = 2;
  m.order = order;
  int nn = 0;
  int nc = (int)t.size() / 3;
  hfx_mesh_high_order(2, order, (int)v.size() / 2, v.data(), nc, t.data(), &nn, nullptr, nullptr);
  m.nodes.resize((size_t)nn * 2);
  m.cells.resize((size_t)nc * m.nodesPerCell());
  hfx_mesh_high_order(2, order, (int)v.size() / 2, v.data(), nc, t.data(), &nn, m.nodes.data(), m.cells.data());
  return m;
}

int main() {
  const int order = 2;
  std::vector<Mesh> parts = {square(2, order), square(3, order), square(1, order)};
  std::vector<const Mesh*> ptrs;
  for (auto& m : parts) ptrs.push_back(&m);
  MeshUnion u(ptrs);
  CHECK(u.numProblems() == 3);
  const int F = 3, Nf = u.mesh.nodesPerFace();
  size_t bpos = 0;
  for (int k = 0; k < 3; ++k) {
    Mesh& m = parts[k];
    m.computeFaces();
    CHECK(u.faceOffset[k + 1] - u.faceOffset[k] == m.nFaces);
    CHECK(u.cellOffset[k + 1] - u.cellOffset[k] == m.numCells());
    for (int c = 0; c < m.numCells(); ++c)
      for (int l = 0; l < F; ++l)
        CHECK(u.mesh.cell2face[(u.cellOffset[k] + c) * F + l] == m.cell2face[c * F + l] + u.faceOffset[k]);
    for (int f = 0; f < m.nFaces; ++f) {
      for (int s = 0; s < 2; ++s) {
        int a = m.face2cell[2 * f + s];
        CHECK(u.mesh.face2cell[2 * (u.faceOffset[k] + f) + s] == (a < 0 ? -1 : (int)(a + u.cellOffset[k])));
      }
      for (int j = 0; j < Nf; ++j)
        CHECK(u.mesh.faces[(u.faceOffset[k] + f) * Nf + j] == m.faces[f * Nf + j] + u.nodeOffset[k]);
    }
    for (int b : m.boundary) CHECK(u.mesh.boundary[bpos++] == b + u.faceOffset[k]);
  }
  CHECK(bpos == u.mesh.boundary.size());
  // group tolerance: problem k's right-hand side values all (k + 1); the smallest part wins
  std::vector<double> rhs((size_t)u.mesh.nFaces * Nf);
  double total = 0.0, least = -1.0;
  for (int k = 0; k < 3; ++k) {
    double sq = 0.0;
    for (long long i = u.faceOffset[k] * Nf; i < u.faceOffset[k + 1] * Nf; ++i) {
      rhs[i] = k + 1.0;
      sq += rhs[i] * rhs[i];
    }
    total += sq;
    if (least < 0 || sq < least) least = sq;
  }
  double tol = u.groupTolerance(1e-8, rhs, Nf);
  CHECK(std::fabs(tol - 1e-8 * std::sqrt(least / total)) <= 1e-22);
  CHECK(u.groupTolerance(1e-8, std::vector<double>(rhs.size(), 0.0), Nf) == 1e-8);
  // one order per union
  Mesh other = square(1, 3);
  bool threw = false;
  try {
    MeshUnion bad({&parts[0], &other});
  } catch (const ErrorHandle&) {
    threw = true;
  }
  CHECK(threw);
  if (fails) return 1;
  std::printf("OK\n");
  return 0;
}
