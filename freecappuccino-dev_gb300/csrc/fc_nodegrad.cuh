// Node-based Green-Gauss gradient (grad_node_based_gauss, gradients.f90:
// 1491-1602): node values from the per-node gather lists of
// host/fc_node_interp.hpp (interpolate_to_nodes, node_interpolation.f90:
// 635-700), face values as the average of the face's node values, then the
// Gauss sum per cell.  Written once per node and per cell for the CUDA
// kernels (fc_nodegrad.cu, no FMA contraction) and for the host replay that
// checks them against the oracle (tests/replay/nodegrad_replay.cpp).
// Arrays 0-based; the gradient is SoA: g[c], g[nT + c], g[2 nT + c].
#pragma once

#if defined(__CUDACC__)
#define FC_HD_NG __host__ __device__ __forceinline__
#else
#define FC_HD_NG inline
#endif

namespace fcng {

// phiN(v): the node's terms summed in the reference's order from 0
FC_HD_NG double node_value(int v, const int* ptr, const int* src, const double* w, const double* phi) {
  double s = 0.0;
  for (int e = ptr[v]; e < ptr[v + 1]; ++e) s = s + w[e] * phi[src[e]];
  return s;
}

// the gradient of cell c: its faces in ascending order (inner faces first,
// as the reference's face loop reaches them), + at the owner, - at the
// neighbour, times 1/vol
FC_HD_NG void node_gauss_cell(int c, const int* cf_ptr, const int* cf_face, const int* owner, const int* nnodes,
                              const int* nodes, int nomax, const double* uN, const double* arx, const double* ary,
                              const double* arz, const double* vol, double& gx, double& gy, double& gz) {
  gx = 0.0;
  gy = 0.0;
  gz = 0.0;
  for (int q = cf_ptr[c]; q < cf_ptr[c + 1]; ++q) {
    const int f = cf_face[q];
    double fie = 0.0;
    const int nn = nnodes[f];
    for (int k = 0; k < nn; ++k) fie = fie + uN[nodes[(size_t)f * nomax + k]];
    fie = fie / (double)nn;
    const double dfxe = fie * arx[f], dfye = fie * ary[f], dfze = fie * arz[f];
    if (owner[f] == c) {
      gx = gx + dfxe;
      gy = gy + dfye;
      gz = gz + dfze;
    } else {
      gx = gx - dfxe;
      gy = gy - dfye;
      gz = gz - dfze;
    }
  }
  const double volr = 1. / vol[c];
  gx = gx * volr;
  gy = gy * volr;
  gz = gz * volr;
}

}  // namespace fcng
