// Cell-to-node interpolation of node_interpolation.f90 as per-node gather
// lists, for the node-based Gauss gradient (gradients.f90:1491-1602).
//
// The reference computes weights once per mesh (set_interpolation_weights,
// :46-84): pseudo-Laplacian ('psl', :265-631, the default) or inverse
// distance ('ids', :88-260), for every (inner face, face node, owner /
// neighbour) and every (boundary face, face node) in its running order.
// interpolate_to_nodes (:635-700) then sums, per node, the inner
// contributions in that order; nodes on a boundary face are reset and get
// the boundary faces' contributions instead.  Here each node's list holds
// exactly the terms that survive, in the reference's order, so one thread
// per node sums them as the reference does.
#pragma once
#include <vector>

struct NodeInterp {
  int nNodes = 0;
  std::vector<int> ptr;     // [nNodes + 1]
  std::vector<int> src;     // field index: cell (0-based) or nC + boundary face (0-based)
  std::vector<double> w;    // weight of each term
};

// owner, neighbour, nodes 0-based; nodes[f * nomax + k], k < nnodes[f];
// x, y, z node coordinates; xc, yc, zc cell centroids; xf, yf, zf face
// centroids; method 0 'psl', 1 'ids'.  Every node must touch a face.
void build_node_interp(int nNodes, int nC, int nI, int nF, const int* owner, const int* neighbour,
                       const int* nnodes, const int* nodes, int nomax, const double* x, const double* y,
                       const double* z, const double* xc, const double* yc, const double* zc, const double* xf,
                       const double* yf, const double* zf, int method, NodeInterp& out);
