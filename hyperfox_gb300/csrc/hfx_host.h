// Host-side data structures shared by the C ABI and the CUDA launchers.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace hfx {

// Reference-element tables for a simplex of dimension dim and order p, with the
// face element's tables (dimension dim-1, same order).
struct RefEl {
  int dim = 0, order = 0;
  int nNodes = 0, nFaces = 0, nNodesFace = 0, nIP = 0, nIPFace = 0;
  std::vector<double> nodes;       // [N][dim]
  std::vector<int> faceNodes;      // [F][Nf]
  std::vector<int> faceOpposite;   // [F] first element node not on face f
  std::vector<double> ipX, ipW;    // [nIP][dim], [nIP]
  std::vector<double> phi, dphi;   // [nIP][N], [nIP][N][dim]
  std::vector<double> fIpX, fIpW;  // [nIPf][dim-1], [nIPf]
  std::vector<double> fPhi, fDphi; // [nIPf][Nf], [nIPf][Nf][dim-1]
};

// Builds the tables; returns false with a message on unsupported input.
bool build_refel(int dim, int order, RefEl* out, std::string* err);

// Face topology of a simplex mesh by the MOAB creation-order rule.
struct Topology {
  int nFaces = 0;
  std::vector<int> cell2face;  // [nCells][F]
  std::vector<int> face2cell;  // [nFaces][2]
  std::vector<int> faces;      // [nFaces][Nf]
  std::vector<int> boundary;   // ascending face ids
};
bool compute_topology(const RefEl& re, int nCells, const int* cells, Topology* out, std::string* err);

// Per element and local face: position of the element's j-th face node in the
// face connectivity (HDGSolver.cpp:258-275 face2CellMap), [nCells][F][Nf].
bool compute_face_perm(const RefEl& re, int nCells, const int* cells, const Topology& t,
                       std::vector<uint8_t>* perm, std::string* err);

// Face-block sparsity of the trace system: rows = faces, block columns = faces
// of every cell touching the row face, sorted. Each block is Nf x Nf.
struct BlockPattern {
  std::vector<int64_t> rowptr;  // [nFaces+1] in blocks
  std::vector<int> col;         // [nBlocks] face ids, ascending per row
  std::vector<int> diag;        // [nFaces] block index of (f,f)
  // For every block: contributing (cell, local face of row, local face of col),
  // first and optional second contributor (second cell = -1 when absent).
  std::vector<int> src0, src1;      // cell ids
  std::vector<uint8_t> loc0, loc1;  // packed (rowLocal<<4)|colLocal
};
bool compute_block_pattern(const RefEl& re, int nCells, const Topology& t, BlockPattern* out,
                           std::string* err);

// Reference operators of the affine element path (hdg_affine.cu), packed:
// M, R_rs, T_f, P_rf, T_ff', M^{-1} C_r, L_f. False if M is singular.
bool affine_tables(const RefEl& re, std::vector<double>* out);

}  // namespace hfx
