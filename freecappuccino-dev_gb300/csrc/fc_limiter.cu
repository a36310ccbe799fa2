// Slope limiters of the cell gradients on the device (grad_scalar_field,
// gradients.f90:141-160): applied by fv_grad after the gradient when the
// context's limiter is set (fc_set_gradient_limiter).  One thread per cell;
// the arithmetic is fc_limiter.cuh's, shared with the host replay.  Built
// with --fmad=false so that every product and sum rounds as the reference's.
#include <cuda_runtime.h>

#include <algorithm>

#include "fc_fields.hpp"
#include "fc_fv.cuh"
#include "fc_internal.hpp"
#include "fc_limiter.cuh"

using namespace fcfv;

namespace {

constexpr int kMinMaxBlocks = 1024;

// per-block min and max of phi over the cells (minval/maxval(phi(1:numCells)))
__global__ void k_minmax_part(const double* __restrict__ phi, int nC, double* __restrict__ part) {
  __shared__ double smin[256], smax[256];
  double lo = phi[0], hi = phi[0];
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += gridDim.x * blockDim.x) {
    lo = fclim::dmin(lo, phi[c]);
    hi = fclim::dmax(hi, phi[c]);
  }
  smin[threadIdx.x] = lo;
  smax[threadIdx.x] = hi;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s) {
      smin[threadIdx.x] = fclim::dmin(smin[threadIdx.x], smin[threadIdx.x + s]);
      smax[threadIdx.x] = fclim::dmax(smax[threadIdx.x], smax[threadIdx.x + s]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    part[2 * blockIdx.x] = smin[0];
    part[2 * blockIdx.x + 1] = smax[0];
  }
}

// the block minima and maxima folded by one block, every thread sharing the
// loads (one thread's serial loop over them took ten times the pass itself)
constexpr int kMinMaxFinalThreads = 256;

__global__ void __launch_bounds__(kMinMaxFinalThreads) k_minmax_final(const double* __restrict__ part, int nb,
                                                                       double* __restrict__ mm) {
  __shared__ double smin[kMinMaxFinalThreads / 32], smax[kMinMaxFinalThreads / 32];
  double lo = part[0], hi = part[1];
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    lo = fclim::dmin(lo, part[2 * b]);
    hi = fclim::dmax(hi, part[2 * b + 1]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fclim::dmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fclim::dmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) {
    smin[threadIdx.x >> 5] = lo;
    smax[threadIdx.x >> 5] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      lo = fclim::dmin(lo, smin[w]);
      hi = fclim::dmax(hi, smax[w]);
    }
    mm[0] = lo;
    mm[1] = hi;
  }
}

template <int KIND>
__global__ void k_limit_scale(MeshView M, const int* __restrict__ ja, const double* __restrict__ phi,
                              const double* __restrict__ mm, double* __restrict__ g) {
  const double fimin = mm[0], fimax = mm[1];
  const size_t nT = (size_t)M.nT;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    const double gx = g[c], gy = g[nT + c], gz = g[2 * nT + c];
    const double s =
        fclim::limit_factor<KIND>(c, M.ia, ja, M.diag, M.xc, M.yc, M.zc, phi, gx, gy, gz, fimin, fimax);
    g[c] = s * gx;
    g[nT + c] = s * gy;
    g[2 * nT + c] = s * gz;
  }
}

__global__ void k_limit_md(MeshView M, const int* __restrict__ ja, const double* __restrict__ phi,
                           double* __restrict__ g) {
  const size_t nT = (size_t)M.nT;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double gx = g[c], gy = g[nT + c], gz = g[2 * nT + c];
    fclim::limit_md(c, M.ia, ja, M.cf_ptr, M.cf_face, M.nI, M.xf, M.yf, M.zf, M.xc, M.yc, M.zc, phi, gx, gy, gz);
    g[c] = gx;
    g[nT + c] = gy;
    g[2 * nT + c] = gz;
  }
}

inline int grid_for(int n) { return std::max(1, std::min(65535, (n + 255) / 256)); }

}  // namespace

// the context's slope limiter on the SoA gradient g of phi (cells only)
int fv_limit(fc_ctx* ctx, const double* phi, double* g) {
  const int kind = ctx->grad_limiter;
  if (kind == FC_LIMITER_NONE) return FC_OK;
  MeshView M = mesh_view(ctx);
  if (M.nC <= 0 || !M.ia || !M.diag) return fc_fail_msg(ctx, FC_ERR_STATE, "gradient limiter: no mesh system");
  const int* ja = ctx->sys_mesh->ja.p;
  const int gb = grid_for(M.nC);
  if (kind == FC_LIMITER_MD) {
    k_limit_md<<<gb, 256, 0, ctx->stream>>>(M, ja, phi, g);
    ctx->kernel_launches++;
  } else {
    DVec<double>& part = ctx->limiter_part;
    const int nb = std::min(kMinMaxBlocks, grid_for(M.nC));
    FC_CUDA_TRY(ctx, part.alloc((size_t)2 * kMinMaxBlocks + 2));
    double* mm = part.p + 2 * kMinMaxBlocks;
    k_minmax_part<<<nb, 256, 0, ctx->stream>>>(phi, M.nC, part.p);
    k_minmax_final<<<1, kMinMaxFinalThreads, 0, ctx->stream>>>(part.p, nb, mm);
    if (kind == FC_LIMITER_BJ) k_limit_scale<FC_LIMITER_BJ><<<gb, 256, 0, ctx->stream>>>(M, ja, phi, mm, g);
    else if (kind == FC_LIMITER_VENKAT) k_limit_scale<FC_LIMITER_VENKAT><<<gb, 256, 0, ctx->stream>>>(M, ja, phi, mm, g);
    else k_limit_scale<FC_LIMITER_R><<<gb, 256, 0, ctx->stream>>>(M, ja, phi, mm, g);
    ctx->kernel_launches += 3;
  }
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

extern "C" int fc_set_gradient_limiter(fc_ctx* ctx, int kind) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (kind < FC_LIMITER_NONE || kind > FC_LIMITER_MD)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_set_gradient_limiter: unknown limiter");
  ctx->grad_limiter = kind;
  return FC_OK;
}
