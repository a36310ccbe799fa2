// Discrete adjoint of steady scalar convection-diffusion (no counterpart in
// the reference; its operator is the implicit part of facefluxsc,
// scalar_fluxes.f90:32-141 and :256-337, with the main diagonal of
// temperature.f90:359-361).
//
// Forward model, A(gamma) phi = source * vol:
//   inner face f (owner P, neighbour N): gamma_f = gamma_P (1 - facint) +
//   gamma_N facint, de = gamma_f Df, a_PN = -de + min(F, 0),
//   a_NP = -de - max(F, 0) (upwind convection of the face flux F);
//   boundary face b: phi_b = 0, sp_P += gamma_P |S|^2 / (d_Pb . S);
//   a_PP = sp_P - sum of the row's off-diagonals.
// Adjoint: A^T lambda = dJ/dphi, solved by BiCGStab on the transposed values
// (same pattern: a_T[k] = a[transpose slot of k]); the gradient
//   dJ/dgamma_c = -lambda^T (dA/dgamma_c) phi
//              = -sum_f (lambda_P - lambda_N)(phi_P - phi_N) Df w_{c,f}
//                -sum_b lambda_c phi_c |S|^2 / (d . S),
// w_{c,f} = 1 - facint (c = P) or facint (c = N), is a reverse face loop that
// recomputes the face coefficients from the geometry instead of storing them.
//
// This translation unit is compiled with --fmad=false: the assembly and the
// gradient evaluate in the order of the oracle (oracle/oracle_fv.cpp), so both
// are compared bit for bit.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "fc_fields.hpp"
#include "fc_fv.cuh"
#include "fc_internal.hpp"

using namespace fcfv;

struct AdjState {
  int gen = -1;              // mesh generation of the buffers below
  DVec<int> tmap;            // transpose slot of every entry of the mesh pattern
  DVec<double> aT, gam, phi, lam, rhs, sf, grad;
};

void fc_adjoint_release(fc_ctx* ctx) {
  delete ctx->adj;
  ctx->adj = nullptr;
}

namespace {

__device__ __forceinline__ double bnd_dfi(const MeshView& M, int f, int ijp) {
  const double xpn = M.xf[f] - M.xc[ijp], ypn = M.yf[f] - M.yc[ijp], zpn = M.zf[f] - M.zc[ijp];
  const double arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
  return (arx * arx + ary * ary + arz * arz) / (xpn * arx + ypn * ary + zpn * arz);
}

__global__ void k_cd_face(MeshView M, const double* __restrict__ gamma, const double* __restrict__ flmass,
                          double* __restrict__ a) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double gf = gamma[ijp] * (1.0 - M.facint[i]) + gamma[ijn] * M.facint[i];
    const double de = gf * M.Df[i];
    const double fm = flmass[i];
    a[M.ijk[i]] = -de + fmin(fm, 0.0);
    a[M.jik[i]] = -de - fmax(fm, 0.0);
  }
}

// per cell: sp from its boundary faces (face order), the main diagonal, the
// right-hand side
__global__ void k_cd_cell(MeshView M, const double* __restrict__ gamma, const double* __restrict__ source,
                          double* __restrict__ a, double* __restrict__ su) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double sp = 0.0;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f >= M.nI) sp = sp + gamma[c] * bnd_dfi(M, f, c);
    }
    const int kd = M.diag[c];
    double s = 0.0;
    for (int k = M.ia[c]; k < M.ia[c + 1]; ++k) s += a[k];  // the diagonal slot holds 0 here
    const double off = s - a[kd];
    a[kd] = sp - off;
    su[c] = source[c] * M.vol[c];
  }
}

__global__ void k_transpose_values(int nnz, const int* __restrict__ tmap, const double* __restrict__ a,
                                   double* __restrict__ aT) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += gridDim.x * blockDim.x) aT[k] = a[tmap[k]];
}

__global__ void k_adj_face(MeshView M, const double* __restrict__ phi, const double* __restrict__ lam,
                           double* __restrict__ sf) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    sf[i] = (lam[ijp] - lam[ijn]) * (phi[ijp] - phi[ijn]) * M.Df[i];
  }
}

// reverse face loop, gathered per cell in face order (inner faces, then
// boundary faces)
__global__ void k_adj_cell(MeshView M, const double* __restrict__ phi, const double* __restrict__ lam,
                           const double* __restrict__ sf, double* __restrict__ out) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double g = 0.0;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f < M.nI) {
        if (M.owner[f] == c) g = g - sf[f] * (1.0 - M.facint[f]);
        else g = g - sf[f] * M.facint[f];
      } else {
        g = g - lam[c] * phi[c] * bnd_dfi(M, f, c);
      }
    }
    out[c] = g;
  }
}

inline int gridn(int n) { return std::max(1, std::min(65535, (n + 255) / 256)); }

}  // namespace

static int adj_state(fc_ctx* ctx, AdjState*& S) {
  if (!ctx->adj) ctx->adj = new AdjState();
  S = ctx->adj;
  if (S->gen == ctx->mesh_gen) return FC_OK;
  const CsrSystem* s = ctx->sys_mesh;
  const int n = s->n, nnz = s->nnz;
  // transpose slots of the (structurally symmetric) mesh pattern
  std::vector<int> tm(nnz);
  for (int i = 0; i < n; ++i)
    for (int k = s->h_ia[i]; k < s->h_ia[i + 1]; ++k) {
      const int j = s->h_ja[k];
      const int* b = s->h_ja.data() + s->h_ia[j];
      const int* e = s->h_ja.data() + s->h_ia[j + 1];
      const int* p = std::lower_bound(b, e, i);
      if (p == e || *p != i) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "adjoint: pattern is not symmetric");
      tm[k] = (int)(p - s->h_ja.data());
    }
  FC_CUDA_TRY(ctx, S->tmap.alloc(nnz));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, S->tmap.p, tm.data(), nnz * sizeof(int)));
  DVec<double>* nv[] = {&S->gam, &S->phi, &S->lam, &S->rhs, &S->grad};
  for (auto* v : nv) FC_CUDA_TRY(ctx, v->alloc(n));
  FC_CUDA_TRY(ctx, S->aT.alloc(nnz));
  FC_CUDA_TRY(ctx, S->sf.alloc(std::max(1, ctx->mesh.numInnerFaces)));
  S->gen = ctx->mesh_gen;
  return FC_OK;
}

// caller arrays of n doubles, host or device, to a device buffer
static int take(fc_ctx* ctx, const double* src, double* dst, size_t n) {
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDefault, ctx->stream));
  return FC_OK;
}

extern "C" int fc_cd_assemble(fc_ctx* ctx, const double* gamma, const double* source) {
  FC_RANGE();
  if (!ctx || !gamma || !source) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  AdjState* S;
  int st = adj_state(ctx, S);
  if (st) return st;
  FieldStore& F = ctx_fields(ctx);
  CsrSystem* sys = ctx->sys_mesh;
  MeshView M = mesh_view(ctx);
  // the source goes through rhs (free until the adjoint)
  if ((st = take(ctx, gamma, S->gam.p, M.nC)) || (st = take(ctx, source, S->rhs.p, M.nC))) return st;
  FC_CUDA_TRY(ctx, cudaMemsetAsync(sys->a.p, 0, (size_t)sys->nnz * sizeof(double), ctx->stream));
  if (M.nI) k_cd_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, S->gam.p, F.flmass.p, sys->a.p);
  k_cd_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, S->gam.p, S->rhs.p, sys->a.p, F.su.p);
  ctx->kernel_launches += 1 + (M.nI > 0);
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

static void info_of(const SolveResult& r, fc_solve_info* info) {
  if (!info) return;
  info->status = r.status; info->itr_used = r.itr_used; info->outer_iterations = r.outer; info->early_exit = r.early;
  info->res0_l1 = r.res0; info->resor = r.resor; info->resl = r.resl; info->factor = r.factor; info->ms = r.ms;
}

extern "C" int fc_cd_solve(fc_ctx* ctx, double* phi, int itr_max, double tol_rel, fc_solve_info* info) {
  FC_RANGE();
  if (!ctx || itr_max < 0) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh || !ctx->adj || ctx->adj->gen != ctx->mesh_gen)
    return fc_fail_msg(ctx, FC_ERR_STATE, "fc_cd_assemble not called for this mesh");
  AdjState* S = ctx->adj;
  CsrSystem* sys = ctx->sys_mesh;
  FC_CUDA_TRY(ctx, cudaMemsetAsync(S->phi.p, 0, (size_t)sys->n * sizeof(double), ctx->stream));
  SolveResult r;
  int st = sys_solve(ctx, sys, "bicgstab", sys->a.p, S->phi.p, ctx_fields(ctx).su.p, itr_max, 0.0, tol_rel, &r);
  if (!st) log_solve(ctx, "fc_cd_solve", "bicgstab", "phi", sys->n, r);
  info_of(r, info);
  if (st) return st;
  if (phi) FC_CUDA_TRY(ctx, cudaMemcpyAsync(phi, S->phi.p, sys->n * sizeof(double), cudaMemcpyDefault, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return r.status;
}

extern "C" int fc_cd_adjoint(fc_ctx* ctx, const double* dJdphi, double* lambda, double* dJdgamma, int itr_max,
                             double tol_rel, fc_solve_info* info) {
  FC_RANGE();
  if (!ctx || !dJdphi || itr_max < 0) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh || !ctx->adj || ctx->adj->gen != ctx->mesh_gen)
    return fc_fail_msg(ctx, FC_ERR_STATE, "fc_cd_assemble and fc_cd_solve not called for this mesh");
  AdjState* S = ctx->adj;
  CsrSystem* sys = ctx->sys_mesh;
  MeshView M = mesh_view(ctx);
  int st = take(ctx, dJdphi, S->rhs.p, M.nC);
  if (st) return st;
  k_transpose_values<<<gridn(sys->nnz), 256, 0, ctx->stream>>>(sys->nnz, S->tmap.p, sys->a.p, S->aT.p);
  ctx->kernel_launches++;
  FC_CUDA_TRY(ctx, cudaMemsetAsync(S->lam.p, 0, (size_t)sys->n * sizeof(double), ctx->stream));
  SolveResult r;
  st = sys_solve(ctx, sys, "bicgstab", S->aT.p, S->lam.p, S->rhs.p, itr_max, 0.0, tol_rel, &r);
  if (!st) log_solve(ctx, "fc_cd_adjoint", "bicgstab", "lambda", sys->n, r);
  info_of(r, info);
  if (st) return st;
  if (M.nI) k_adj_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, S->phi.p, S->lam.p, S->sf.p);
  k_adj_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, S->phi.p, S->lam.p, S->sf.p, S->grad.p);
  ctx->kernel_launches += 1 + (M.nI > 0);
  FC_CUDA_TRY(ctx, cudaGetLastError());
  if (lambda) FC_CUDA_TRY(ctx, cudaMemcpyAsync(lambda, S->lam.p, M.nC * sizeof(double), cudaMemcpyDefault, ctx->stream));
  if (dJdgamma)
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(dJdgamma, S->grad.p, M.nC * sizeof(double), cudaMemcpyDefault, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return r.status;
}
