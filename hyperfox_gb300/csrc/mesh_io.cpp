// Mesh input on the host: a gmsh .msh (format 2.2, ASCII) reader for simplex
// meshes and the construction of a high-order node set from a linear mesh.
//
// Restates tools/convertGmsh2H5HO.cpp:117-257,367-398 without MOAB: every cell's
// reference nodes (ReferenceElement nodes, vertices first) are mapped by the
// cell's affine map x = x_0 + sum_k (xi_k + 1)/2 (x_{k+1} - x_0) and nodes that
// coincide (within 1e-10 of the mesh size, the tool matches within 1e-8) are
// merged. Nodes are numbered in order of first appearance, cell by cell and in
// reference-node order; the tool numbers vertices the same way and edge/face
// nodes in MOAB adjacency order, which only permutes node ids (cell node order,
// hence faces and trace DOFs, are the same).
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <fstream>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "hfx_gb300.h"
#include "hfx_host.h"

namespace hfx {
namespace {

thread_local std::string g_ioErr;

int io_fail(const std::string& m) {
  g_ioErr = m;
  return HFX_ERR_ARG;
}

// gmsh element types: number of nodes, topological dimension (simplices only)
bool gmsh_simplex(int type, int* nNodes, int* tdim) {
  switch (type) {
    case 1: *nNodes = 2; *tdim = 1; return true;    // 2-node line
    case 2: *nNodes = 3; *tdim = 2; return true;    // 3-node triangle
    case 4: *nNodes = 4; *tdim = 3; return true;    // 4-node tetrahedron
    case 8: *nNodes = 3; *tdim = 1; return true;    // 3-node line
    case 9: *nNodes = 6; *tdim = 2; return true;    // 6-node triangle
    case 11: *nNodes = 10; *tdim = 3; return true;  // 10-node tetrahedron
    case 15: *nNodes = 1; *tdim = 0; return true;   // point
    case 20: *nNodes = 9; *tdim = 2; return true;   // 9-node incomplete triangle
    case 21: *nNodes = 10; *tdim = 2; return true;  // 10-node triangle
    case 26: *nNodes = 4; *tdim = 1; return true;   // 4-node line
    case 29: *nNodes = 20; *tdim = 3; return true;  // 20-node tetrahedron
    default: return false;
  }
}

struct LinearMesh {
  std::vector<double> coords;  // [n][dim]
  std::vector<int> cells;      // [nCells][dim+1]
};

// Linear simplex mesh of dimension dim: the vertices (first dim+1 nodes) of the
// elements of that dimension; nodes renumbered in gmsh id order over the used ones.
int read_gmsh22(const std::string& path, int dim, LinearMesh* out) {
  std::ifstream in(path);
  if (!in) return io_fail("gmsh: cannot open " + path);
  std::string tok;
  std::vector<int64_t> ids;
  std::vector<double> xyz;
  std::vector<int> cellIds;  // gmsh node ids of the cells' vertices
  bool haveFormat = false;
  while (in >> tok) {
    if (tok == "$MeshFormat") {
      double ver;
      int ftype, dsize;
      if (!(in >> ver >> ftype >> dsize)) return io_fail("gmsh: bad $MeshFormat");
      if (ver < 2.0 || ver >= 3.0) return io_fail("gmsh: only format 2.x is read (found " + std::to_string(ver) + ")");
      if (ftype != 0) return io_fail("gmsh: only the ASCII format is read");
      haveFormat = true;
    } else if (tok == "$Nodes") {
      int64_t n;
      if (!(in >> n) || n < 0) return io_fail("gmsh: bad $Nodes count");
      ids.resize(n);
      xyz.resize(3 * n);
      for (int64_t i = 0; i < n; ++i)
        if (!(in >> ids[i] >> xyz[3 * i] >> xyz[3 * i + 1] >> xyz[3 * i + 2])) return io_fail("gmsh: truncated $Nodes");
    } else if (tok == "$Elements") {
      int64_t n;
      if (!(in >> n) || n < 0) return io_fail("gmsh: bad $Elements count");
      std::string line;
      std::getline(in, line);
      for (int64_t i = 0; i < n; ++i) {
        if (!std::getline(in, line)) return io_fail("gmsh: truncated $Elements");
        std::istringstream ls(line);
        int64_t id;
        int type, ntags;
        if (!(ls >> id >> type >> ntags)) return io_fail("gmsh: bad element line");
        for (int t = 0; t < ntags; ++t) {
          int64_t tag;
          if (!(ls >> tag)) return io_fail("gmsh: bad element tags");
        }
        int nn, tdim;
        if (!gmsh_simplex(type, &nn, &tdim)) return io_fail("gmsh: element type " + std::to_string(type) + " is not a simplex");
        std::vector<int64_t> nodes(nn);
        for (int k = 0; k < nn; ++k)
          if (!(ls >> nodes[k])) return io_fail("gmsh: element with missing nodes");
        if (tdim != dim) continue;
        for (int k = 0; k <= dim; ++k) cellIds.push_back((int)nodes[k]);
      }
    }
  }
  if (!haveFormat) return io_fail("gmsh: no $MeshFormat section");
  if (cellIds.empty()) return io_fail("gmsh: no element of dimension " + std::to_string(dim));
  std::unordered_map<int64_t, int64_t> pos;  // gmsh id -> index in ids
  for (int64_t i = 0; i < (int64_t)ids.size(); ++i) pos[ids[i]] = i;
  std::vector<int64_t> used;
  for (int g : cellIds) used.push_back(g);
  std::sort(used.begin(), used.end());
  used.erase(std::unique(used.begin(), used.end()), used.end());
  std::unordered_map<int64_t, int> newId;
  out->coords.clear();
  for (size_t k = 0; k < used.size(); ++k) {
    auto it = pos.find(used[k]);
    if (it == pos.end()) return io_fail("gmsh: element refers to a missing node");
    newId[used[k]] = (int)k;
    for (int c = 0; c < dim; ++c) out->coords.push_back(xyz[3 * it->second + c]);
  }
  out->cells.resize(cellIds.size());
  for (size_t k = 0; k < cellIds.size(); ++k) out->cells[k] = newId[cellIds[k]];
  return HFX_OK;
}

struct KeyHash {
  size_t operator()(const std::array<int64_t, 3>& k) const {
    uint64_t h = 1469598103934665603ull;
    for (int64_t v : k) {
      h ^= (uint64_t)v;
      h *= 1099511628211ull;
    }
    return (size_t)h;
  }
};

int high_order(int dim, int order, int nLin, const double* lin, int nCells, const int* cells,
               std::vector<double>* coords, std::vector<int>* hoCells) {
  RefEl re;
  std::string err;
  if (!build_refel(dim, order, &re, &err)) return io_fail(err);
  const int N = re.nNodes;
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int64_t i = 0; i < (int64_t)nLin; ++i)
    for (int k = 0; k < dim; ++k) {
      lo[k] = std::min(lo[k], lin[i * dim + k]);
      hi[k] = std::max(hi[k], lin[i * dim + k]);
    }
  double size = 0.0;
  for (int k = 0; k < dim; ++k) size = std::max(size, hi[k] - lo[k]);
  const double quantum = 1e-10 * (size > 0 ? size : 1.0);
  std::unordered_map<std::array<int64_t, 3>, int, KeyHash> ids;
  ids.reserve((size_t)nCells * N);
  coords->clear();
  hoCells->assign((size_t)nCells * N, 0);
  for (int64_t e = 0; e < nCells; ++e) {
    const int* cv = cells + e * (dim + 1);
    for (int k = 0; k <= dim; ++k)
      if (cv[k] < 0 || cv[k] >= nLin) return io_fail("high_order: cell vertex out of range");
    for (int i = 0; i < N; ++i) {
      double x[3] = {0, 0, 0};
      for (int c = 0; c < dim; ++c) {
        x[c] = lin[(int64_t)cv[0] * dim + c];
        if (i <= dim) x[c] = lin[(int64_t)cv[i] * dim + c];  // vertices reproduce exactly
        else
          for (int k = 0; k < dim; ++k)
            x[c] += 0.5 * (re.nodes[(size_t)i * dim + k] + 1.0) * (lin[(int64_t)cv[k + 1] * dim + c] - lin[(int64_t)cv[0] * dim + c]);
      }
      std::array<int64_t, 3> key = {0, 0, 0};
      for (int c = 0; c < dim; ++c) key[c] = (int64_t)std::llround(x[c] / quantum);
      auto it = ids.find(key);
      if (it == ids.end()) {
        // the same node computed from another cell can round to a neighbouring key (its
        // coordinates differ in the last bits and straddle a rounding boundary): look there
        // for a node within one quantum before creating a new one
        const int span = dim == 3 ? 27 : 9;
        for (int o = 0; o < span && it == ids.end(); ++o) {
          const int64_t d0 = o % 3 - 1, d1 = (o / 3) % 3 - 1, d2 = dim == 3 ? o / 9 - 1 : 0;
          if (d0 == 0 && d1 == 0 && d2 == 0) continue;
          const std::array<int64_t, 3> nk = {key[0] + d0, key[1] + d1, dim == 3 ? key[2] + d2 : 0};
          auto jt = ids.find(nk);
          if (jt == ids.end()) continue;
          bool close = true;
          for (int c = 0; c < dim; ++c)
            if (std::fabs((*coords)[(size_t)jt->second * dim + c] - x[c]) > quantum) close = false;
          if (close) it = jt;
        }
      }
      int id;
      if (it == ids.end()) {
        id = (int)(coords->size() / dim);
        ids.emplace(key, id);
        for (int c = 0; c < dim; ++c) coords->push_back(x[c]);
      } else {
        id = it->second;
      }
      (*hoCells)[(size_t)e * N + i] = id;
    }
  }
  return HFX_OK;
}

}  // namespace

void set_io_error(const std::string& m) { g_ioErr = m; }

}  // namespace hfx

using namespace hfx;

extern "C" {

int hfx_gmsh_read(const char* path, int dim, int* nNodes, int* nCells, double* coords, int* cells) {
  if (!path || !nNodes || !nCells || (dim != 2 && dim != 3)) return HFX_ERR_ARG;
  LinearMesh m;
  int rc = read_gmsh22(path, dim, &m);
  if (rc) return rc;
  *nNodes = (int)(m.coords.size() / dim);
  *nCells = (int)(m.cells.size() / (dim + 1));
  if (coords) std::copy(m.coords.begin(), m.coords.end(), coords);
  if (cells) std::copy(m.cells.begin(), m.cells.end(), cells);
  return HFX_OK;
}

int hfx_mesh_high_order(int dim, int order, int nLinNodes, const double* linCoords, int nCells, const int* linCells,
                        int* nNodes, double* coords, int* cells) {
  if (!linCoords || !linCells || !nNodes || nLinNodes <= 0 || nCells <= 0 || (dim != 2 && dim != 3))
    return HFX_ERR_ARG;
  std::vector<double> c;
  std::vector<int> hc;
  int rc = high_order(dim, order, nLinNodes, linCoords, nCells, linCells, &c, &hc);
  if (rc) return rc;
  *nNodes = (int)(c.size() / dim);
  if (coords) std::copy(c.begin(), c.end(), coords);
  if (cells) std::copy(hc.begin(), hc.end(), cells);
  return HFX_OK;
}

const char* hfx_mesh_io_error(void) { return hfx::g_ioErr.c_str(); }

}  // extern "C"
