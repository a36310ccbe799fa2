// Node-based Green-Gauss gradients on the device (FC_GRAD_NODE_GAUSS;
// grad_node_based_gauss, gradients.f90:1491-1602, with the cell-to-node
// weights of node_interpolation.f90).  The weights are built once per mesh
// and method on the host (host/fc_node_interp.cpp, as the reference builds
// them at initialisation) and uploaded as per-node gather lists; each
// gradient is then one node pass and one cell pass.  Per-node and per-cell
// arithmetic: fc_nodegrad.cuh.  Built with --fmad=false.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "fc_fields.hpp"
#include "fc_fv.cuh"
#include "fc_internal.hpp"
#include "fc_node_interp.hpp"
#include "fc_nodegrad.cuh"

using namespace fcfv;

namespace {

__global__ void k_interp_nodes(int nNodes, const int* __restrict__ ptr, const int* __restrict__ src,
                               const double* __restrict__ w, const double* __restrict__ phi,
                               double* __restrict__ uN) {
  for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < nNodes; v += gridDim.x * blockDim.x)
    uN[v] = fcng::node_value(v, ptr, src, w, phi);
}

__global__ void k_grad_node(MeshView M, const int* __restrict__ nnodes, const int* __restrict__ nodes,
                            const double* __restrict__ uN, double* __restrict__ g) {
  const size_t nT = (size_t)M.nT;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double gx, gy, gz;
    fcng::node_gauss_cell(c, M.cf_ptr, M.cf_face, M.owner, nnodes, nodes, FC_NOMAX, uN, M.arx, M.ary, M.arz,
                          M.vol, gx, gy, gz);
    g[c] = gx;
    g[nT + c] = gy;
    g[2 * nT + c] = gz;
  }
}

inline int grid_for(int n) { return std::max(1, std::min(65535, (n + 255) / 256)); }

template <class T>
cudaError_t download(cudaStream_t s, std::vector<T>& h, const DVec<T>& d, size_t n) {
  h.resize(n);
  return fc_d2h(s, h.data(), d.p, n * sizeof(T));
}

// gather lists of the current mesh and method (built on first use)
int node_interp_prepare(fc_ctx* ctx) {
  if (ctx->ng_gen == ctx->mesh_gen && ctx->ng_method == ctx->node_interp) return FC_OK;
  const MeshDev& m = ctx->mesh;
  const int nN = m.numNodes, nC = m.numCells, nI = m.numInnerFaces, nF = m.numFaces;
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<int> nnodes, nodes;
  std::vector<double> x, y, z, xf, yf, zf;
  FC_CUDA_TRY(ctx, download(ctx->stream, nnodes, m.nnodes, nF));
  FC_CUDA_TRY(ctx, download(ctx->stream, nodes, m.nodes, (size_t)nF * FC_NOMAX));
  FC_CUDA_TRY(ctx, download(ctx->stream, x, m.x, nN));
  FC_CUDA_TRY(ctx, download(ctx->stream, y, m.y, nN));
  FC_CUDA_TRY(ctx, download(ctx->stream, z, m.z, nN));
  FC_CUDA_TRY(ctx, download(ctx->stream, xf, m.xf, nF));
  FC_CUDA_TRY(ctx, download(ctx->stream, yf, m.yf, nF));
  FC_CUDA_TRY(ctx, download(ctx->stream, zf, m.zf, nF));
  if (m.h_xyz.size() != (size_t)3 * nC || m.h_owner.size() != (size_t)nF || m.h_neighbour.size() != (size_t)nI)
    return fc_fail_msg(ctx, FC_ERR_STATE, "node-based gradient: host mesh arrays missing");
  const double* xc = m.h_xyz.data();
  NodeInterp ni;
  build_node_interp(nN, nC, nI, nF, m.h_owner.data(), m.h_neighbour.data(), nnodes.data(), nodes.data(), FC_NOMAX,
                    x.data(), y.data(), z.data(), xc, xc + nC, xc + 2 * (size_t)nC, xf.data(), yf.data(), zf.data(),
                    ctx->node_interp, ni);
  FC_CUDA_TRY(ctx, ctx->ng_ptr.alloc(ni.ptr.size()));
  FC_CUDA_TRY(ctx, ctx->ng_src.alloc(std::max<size_t>(1, ni.src.size())));
  FC_CUDA_TRY(ctx, ctx->ng_w.alloc(std::max<size_t>(1, ni.w.size())));
  FC_CUDA_TRY(ctx, ctx->ng_uN.alloc(std::max(1, nN)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, ctx->ng_ptr.p, ni.ptr.data(), ni.ptr.size() * sizeof(int)));
  if (!ni.src.empty()) {
    FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, ctx->ng_src.p, ni.src.data(), ni.src.size() * sizeof(int)));
    FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, ctx->ng_w.p, ni.w.data(), ni.w.size() * sizeof(double)));
  }
  ctx->ng_gen = ctx->mesh_gen;
  ctx->ng_method = ctx->node_interp;
  return FC_OK;
}

}  // namespace

int fv_grad_node(fc_ctx* ctx, const double* phi, double* g) {
  // face_mapping moves a twin face's owner and centre but not its nodes; the
  // node interpolation of such a mesh is not restated here
  if (ctx->mesh.nPer)
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "node-based gradients are not supported on meshes with periodic pairs");
  int st = node_interp_prepare(ctx);
  if (st) return st;
  MeshView M = mesh_view(ctx);
  const int nN = ctx->mesh.numNodes;
  k_interp_nodes<<<grid_for(nN), 256, 0, ctx->stream>>>(nN, ctx->ng_ptr.p, ctx->ng_src.p, ctx->ng_w.p, phi,
                                                         ctx->ng_uN.p);
  k_grad_node<<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, ctx->mesh.nnodes.p, ctx->mesh.nodes.p, ctx->ng_uN.p, g);
  ctx->kernel_launches += 2;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

extern "C" int fc_set_node_interpolation(fc_ctx* ctx, int method) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (method != FC_C2N_PSL && method != FC_C2N_IDS)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_set_node_interpolation: unknown method");
  ctx->node_interp = method;
  return FC_OK;
}
