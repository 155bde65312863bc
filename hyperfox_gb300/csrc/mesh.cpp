// Face topology, face-node orientation maps and the trace-system block pattern,
// on the host (integer work done once per mesh).
//
// Replaces Mesh::computeFaces and its maps (Mesh.cpp:183-537) without MOAB.
// HyperFox numbers faces by MOAB handle, i.e. creation order: MOAB creates a
// face the first time some cell asks for its sides, cells in order and sides
// in MOAB's canonical order (triangle edges (0,1),(1,2),(2,0); tetrahedron
// faces (0,1,3),(1,2,3),(0,3,2),(0,2,1)). That canonical side s contains the
// same vertices as HyperFox's reference face s (ReferenceElement.cpp:1024-1054),
// so side s is also the local face index found by Mesh::getFaceIndex.
// The rule is computed here by sorting (sorted vertex tuple, cell*F+side)
// records instead of a growing hash table.
#include <algorithm>
#include <array>
#include <numeric>

#include "hfx_host.h"

namespace hfx {

namespace {
const int kTriSides[3][2] = {{0, 1}, {1, 2}, {2, 0}};
const int kTetSides[4][3] = {{0, 1, 3}, {1, 2, 3}, {0, 3, 2}, {0, 2, 1}};

struct SideRec {
  std::array<int, 3> key;  // sorted vertex ids (unused slot = -1)
  int64_t rec;             // cell*F + side
};
}  // namespace

bool compute_topology(const RefEl& re, int nCells, const int* cells, Topology* out, std::string* err) {
  const int dim = re.dim, N = re.nNodes, F = re.nFaces, Nf = re.nNodesFace;
  const int64_t nRec = (int64_t)nCells * F;
  std::vector<SideRec> recs(nRec);
  for (int64_t c = 0; c < nCells; ++c) {
    const int* cell = cells + c * N;
    for (int s = 0; s < F; ++s) {
      std::array<int, 3> k = {-1, -1, -1};
      for (int v = 0; v < dim; ++v) {
        int lv = dim == 2 ? kTriSides[s][v] : kTetSides[s][v];
        k[v] = cell[lv];
      }
      std::sort(k.begin(), k.begin() + dim);
      recs[c * F + s] = {k, c * F + s};
    }
  }
  std::sort(recs.begin(), recs.end(), [](const SideRec& a, const SideRec& b) {
    return a.key != b.key ? a.key < b.key : a.rec < b.rec;
  });
  // groups of equal keys; a face is created at its group's first record
  std::vector<int64_t> groupStart;
  for (int64_t i = 0; i < nRec; ++i)
    if (i == 0 || recs[i].key != recs[i - 1].key) groupStart.push_back(i);
  int64_t nG = (int64_t)groupStart.size();
  std::vector<int64_t> order(nG);
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(),
            [&](int64_t a, int64_t b) { return recs[groupStart[a]].rec < recs[groupStart[b]].rec; });
  Topology t;
  t.nFaces = (int)nG;
  t.cell2face.assign(nRec, -1);
  t.face2cell.assign(2 * nG, -1);
  for (int64_t fid = 0; fid < nG; ++fid) {
    int64_t g = order[fid];
    int64_t lo = groupStart[g], hi = (g + 1 < nG) ? groupStart[g + 1] : nRec;
    if (hi - lo > 2) {
      *err = "mesh: a face is shared by more than two cells";
      return false;
    }
    for (int64_t i = lo; i < hi; ++i) {
      t.cell2face[recs[i].rec] = (int)fid;
      t.face2cell[2 * fid + (i - lo)] = (int)(recs[i].rec / F);
    }
    if (hi - lo == 1) t.boundary.push_back((int)fid);
  }
  // face connectivity from the first (lower) adjacent cell
  t.faces.assign((int64_t)nG * Nf, -1);
  for (int64_t f = 0; f < nG; ++f) {
    int c = t.face2cell[2 * f];
    int loc = 0;
    while (t.cell2face[(int64_t)c * F + loc] != f) ++loc;
    for (int j = 0; j < Nf; ++j) t.faces[f * Nf + j] = cells[(int64_t)c * N + re.faceNodes[loc * Nf + j]];
  }
  *out = std::move(t);
  return true;
}

bool compute_face_perm(const RefEl& re, int nCells, const int* cells, const Topology& t,
                       std::vector<uint8_t>* perm, std::string* err) {
  const int N = re.nNodes, F = re.nFaces, Nf = re.nNodesFace;
  perm->assign((int64_t)nCells * F * Nf, 0);
  for (int64_t c = 0; c < nCells; ++c)
    for (int i = 0; i < F; ++i) {
      int f = t.cell2face[c * F + i];
      if (f < 0 || f >= t.nFaces) {
        *err = "mesh: cell2face out of range";
        return false;
      }
      const int* face = &t.faces[(int64_t)f * Nf];
      for (int j = 0; j < Nf; ++j) {
        int node = cells[c * N + re.faceNodes[i * Nf + j]];
        int pos = -1;
        for (int q = 0; q < Nf; ++q)
          if (face[q] == node) {
            pos = q;
            break;
          }
        if (pos < 0) {
          *err = "mesh: couldn't find cell node in face";
          return false;
        }
        (*perm)[(c * F + i) * Nf + j] = (uint8_t)pos;
      }
    }
  return true;
}

bool compute_block_pattern(const RefEl& re, int nCells, const Topology& t, BlockPattern* out,
                           std::string* err) {
  const int F = re.nFaces;
  const int nF = t.nFaces;
  BlockPattern b;
  b.rowptr.assign(nF + 1, 0);
  // neighbours of face f: all faces of its (one or two) cells, sorted, unique
  std::vector<int> tmp;
  tmp.reserve(2 * F);
  for (int f = 0; f < nF; ++f) {
    tmp.clear();
    for (int s = 0; s < 2; ++s) {
      int c = t.face2cell[2 * f + s];
      if (c < 0) continue;
      for (int i = 0; i < F; ++i) tmp.push_back(t.cell2face[(int64_t)c * F + i]);
    }
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    b.rowptr[f + 1] = b.rowptr[f] + (int64_t)tmp.size();
  }
  int64_t nB = b.rowptr[nF];
  b.col.resize(nB);
  b.src0.assign(nB, -1);
  b.src1.assign(nB, -1);
  b.loc0.assign(nB, 0);
  b.loc1.assign(nB, 0);
  b.diag.assign(nF, -1);
  for (int f = 0; f < nF; ++f) {
    tmp.clear();
    for (int s = 0; s < 2; ++s) {
      int c = t.face2cell[2 * f + s];
      if (c < 0) continue;
      for (int i = 0; i < F; ++i) tmp.push_back(t.cell2face[(int64_t)c * F + i]);
    }
    std::sort(tmp.begin(), tmp.end());
    tmp.erase(std::unique(tmp.begin(), tmp.end()), tmp.end());
    std::copy(tmp.begin(), tmp.end(), b.col.begin() + b.rowptr[f]);
    for (int s = 0; s < 2; ++s) {
      int c = t.face2cell[2 * f + s];
      if (c < 0) continue;
      int li = -1;
      for (int i = 0; i < F; ++i)
        if (t.cell2face[(int64_t)c * F + i] == f) li = i;
      for (int j = 0; j < F; ++j) {
        int g = t.cell2face[(int64_t)c * F + j];
        int64_t k = b.rowptr[f] + (std::lower_bound(tmp.begin(), tmp.end(), g) - tmp.begin());
        uint8_t loc = (uint8_t)((li << 4) | j);
        if (b.src0[k] < 0) {
          b.src0[k] = c;
          b.loc0[k] = loc;
        } else if (b.src1[k] < 0) {
          b.src1[k] = c;
          b.loc1[k] = loc;
        } else {
          *err = "mesh: a trace block has more than two contributing cells";
          return false;
        }
        if (g == f) b.diag[f] = (int)k;
      }
    }
  }
  *out = std::move(b);
  return true;
}

}  // namespace hfx
