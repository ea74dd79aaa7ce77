// gt_refcell.cuh -- reference-cell tables (local faces, Lagrange nodes,
// quadrature) shared by the numbering and integration kernels.
//
// Local numbering follows GalerkinToolkit: unit square / cube local faces of
// src/domain.jl:213-268, tetrahedron faces src/domain.jl:439-469, Lagrange
// nodes from monomial exponents in CartesianIndices order (first index
// fastest, src/space.jl:1127-1177), component-major local DOFs
// (src/space.jl:1257-1286).
#pragma once
#include <stdint.h>

namespace gt {

struct RefTables {
  int D, nlv, nn;          // dimension, vertices per cell, space nodes per cell
  int nle, nlf, nlfv;      // local edges, local (D-1)-faces, vertices per (D-1)-face
  int nclosure;            // space nodes on one (D-1)-face
  int face_nodes, cell_node;  // order 2: nodes owned by 2-faces (hex: 1 each) / the cell (cubes: 1)
  int8_t vnode[8];         // space node of local vertex
  int8_t enode[12];        // space node at the midpoint of local edge (Q2)
  int8_t fnode[6];         // space node at the centre of local face (Q2 hex)
  int8_t cnode;            // space node at the cell centre (Q2)
  int8_t le_verts[12][2];  // local edge -> local vertices (0-based)
  int8_t lf_verts[6][4];   // local (D-1)-face -> local vertices
  int8_t closure[6][9];    // local (D-1)-face -> space nodes on its closure
};

// Host-side construction of the tables for a cell type and order.
inline RefTables make_ref_tables(int ctype, int order) {
  static const int QE[4][2] = {{1, 2}, {3, 4}, {1, 3}, {2, 4}};
  static const int HE[12][2] = {{1, 2}, {3, 4}, {1, 3}, {2, 4}, {5, 6}, {7, 8},
                                {5, 7}, {6, 8}, {1, 5}, {3, 7}, {2, 6}, {4, 8}};
  static const int HF[6][4] = {{1, 2, 3, 4}, {5, 6, 7, 8}, {1, 2, 5, 6},
                               {3, 4, 7, 8}, {1, 3, 5, 7}, {2, 4, 6, 8}};
  static const int TF[4][3] = {{1, 2, 3}, {1, 2, 4}, {1, 3, 4}, {2, 3, 4}};
  static const int TE[6][2] = {{1, 2}, {1, 3}, {2, 3}, {1, 4}, {2, 4}, {3, 4}};
  RefTables t{};
  if (ctype == 3 /*TET4*/) {
    t.D = 3; t.nlv = 4; t.nle = 6; t.nlf = 4; t.nlfv = 3;
    for (int e = 0; e < 6; e++) { t.le_verts[e][0] = TE[e][0] - 1; t.le_verts[e][1] = TE[e][1] - 1; }
    for (int f = 0; f < 4; f++)
      for (int i = 0; i < 3; i++) t.lf_verts[f][i] = TF[f][i] - 1;
    if (order == 1) {
      t.nn = 4; t.nclosure = 3;
      for (int v = 0; v < 4; v++) t.vnode[v] = (int8_t)v;
      for (int f = 0; f < 4; f++)
        for (int i = 0; i < 3; i++) t.closure[f][i] = TF[f][i] - 1;
      return t;
    }
    // P2: nodes are the exponents (a, b, c), a + b + c <= 2, first index
    // fastest: (000) (100) (200) (010) (110) (020) (001) (101) (011) (002)
    // -- vertices at nodes 0, 2, 5, 9, the midpoints of the local edges at
    // 1, 3, 4, 6, 7, 8 (edges 12, 13, 23, 14, 24, 34)
    static const int PV[4] = {0, 2, 5, 9}, PE[6] = {1, 3, 4, 6, 7, 8};
    t.nn = 10; t.nclosure = 6;
    for (int v = 0; v < 4; v++) t.vnode[v] = (int8_t)PV[v];
    for (int e = 0; e < 6; e++) t.enode[e] = (int8_t)PE[e];
    for (int f = 0; f < 4; f++) {
      // closure of face f: its 3 vertex nodes and the nodes of its 3 edges, ascending
      int nodes[6], cnt = 0;
      for (int i = 0; i < 3; i++) nodes[cnt++] = PV[TF[f][i] - 1];
      for (int e = 0; e < 6; e++) {
        int in = 0;
        for (int i = 0; i < 3; i++) in += (TE[e][0] == TF[f][i]) + (TE[e][1] == TF[f][i]);
        if (in == 2) nodes[cnt++] = PE[e];
      }
      for (int i = 0; i < 6; i++)
        for (int j = i + 1; j < 6; j++)
          if (nodes[j] < nodes[i]) { int tmp = nodes[i]; nodes[i] = nodes[j]; nodes[j] = tmp; }
      for (int i = 0; i < 6; i++) t.closure[f][i] = (int8_t)nodes[i];
    }
    return t;
  }
  int D = ctype == 1 ? 2 : 3, m = order + 1;
  t.D = D; t.nlv = 1 << D; t.nn = D == 2 ? m * m : m * m * m;
  t.nle = D == 2 ? 4 : 12; t.nlf = 2 * D; t.nlfv = D == 2 ? 2 : 4;
  auto qn = [&](int e0, int e1, int e2) { return D == 2 ? e0 + m * e1 : e0 + m * (e1 + m * e2); };
  for (int v = 0; v < t.nlv; v++)
    t.vnode[v] = (int8_t)qn((v & 1) * order, ((v >> 1) & 1) * order, ((v >> 2) & 1) * order);
  for (int e = 0; e < t.nle; e++) {
    const int* ev = D == 2 ? QE[e] : HE[e];
    t.le_verts[e][0] = (int8_t)(ev[0] - 1);
    t.le_verts[e][1] = (int8_t)(ev[1] - 1);
    int a = ev[0] - 1, b = ev[1] - 1;
    if (order == 2)
      t.enode[e] = (int8_t)qn((a & 1) + (b & 1), ((a >> 1) & 1) + ((b >> 1) & 1), ((a >> 2) & 1) + ((b >> 2) & 1));
  }
  for (int f = 0; f < t.nlf; f++) {
    int s[3] = {0, 0, 0};
    for (int i = 0; i < t.nlfv; i++) {
      int lv = (D == 2 ? QE[f][i] : HF[f][i]) - 1;
      t.lf_verts[f][i] = (int8_t)lv;
      for (int d = 0; d < 3; d++) s[d] += (lv >> d) & 1;
    }
    if (order == 2 && D == 3) t.fnode[f] = (int8_t)qn(s[0] / 2, s[1] / 2, s[2] / 2);
    // closure: nodes whose exponent in the face's fixed direction is 0 or order
    int dir = D == 2 ? (f < 2 ? 1 : 0) : 2 - f / 2, side = f & 1, cnt = 0;
    for (int k = 0; k < t.nn; k++) {
      int e[3] = {k % m, (k / m) % m, k / (m * m)};
      if (e[dir] == side * order) t.closure[f][cnt++] = (int8_t)k;
    }
    t.nclosure = cnt;
  }
  if (order == 2) {
    t.cnode = (int8_t)(D == 2 ? qn(1, 1, 0) : qn(1, 1, 1));
    t.face_nodes = D == 3 ? 1 : 0;
    t.cell_node = 1;
  }
  return t;
}

}  // namespace gt
