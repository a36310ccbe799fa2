// Restarted GMRES(mr) with a true ILU(0) preconditioner (replaces
// pmgmres_ilu, ilu_cr, lus_cr, ax_cr and mult_givens of
// src/linearSolvers/linear_solvers.f90:789-1478).  The ILU(0) factorisation
// and its triangular solves are level scheduled (one cooperative kernel
// each); the Arnoldi vectors live on the device and the (mr+1) x mr
// Hessenberg/Givens algebra runs on the host, exactly as written in the
// reference, including rho being taken before the preconditioner is applied.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "fc_internal.hpp"
#include "fc_krylov.cuh"

using namespace fcdev;

namespace {

struct IluArgs {
  CsrView<double> S;
  GridCtl C;
  double* l;   // nnz: factors
  const double* r;
  double* w;   // in/out of the triangular solves
};

// ilu_cr, linear_solvers.f90:1267-1385 (row i after the rows it depends on)
__global__ void __launch_bounds__(FC_BLOCK) k_ilu0(IluArgs A) {
  const CsrView<double>& S = A.S;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  double* l = A.l;
  for (int lev = 0; lev < S.nlf; ++lev) {
    const int b = __ldg(S.lfp + lev), e = __ldg(S.lfp + lev + 1);
    for (int idx = b + gt; idx < e; idx += G) {
      const int i = __ldg(S.lfr + idx);
      const int k0 = __ldg(S.ia + i), k1 = __ldg(S.ia + i + 1), kd = __ldg(S.dg + i);
      for (int j = k0; j < kd; ++j) {
        const int jrow = __ldg(S.ja + j);
        const double tl = __dmul_rn(ldcg(l + j), ldcg(l + __ldg(S.dg + jrow)));
        l[j] = tl;
        const int je = __ldg(S.ia + jrow + 1);
        for (int jj = __ldg(S.dg + jrow) + 1; jj < je; ++jj) {
          const int col = __ldg(S.ja + jj);
          // iw(ja(jj)): position of that column in row i, if present
          int lo = k0, hi = k1 - 1, jw = -1;
          while (lo <= hi) {
            int mid = (lo + hi) >> 1, c = __ldg(S.ja + mid);
            if (c == col) { jw = mid; break; }
            if (c < col) lo = mid + 1; else hi = mid - 1;
          }
          if (jw != -1) l[jw] = __dsub_rn(ldcg(l + jw), __dmul_rn(tl, ldcg(l + jj)));
        }
      }
      const double piv = ldcg(l + kd);
      if (piv == 0.0) atomicCAS(A.C.status, 0, FC_ERR_ZERO_PIVOT);
      l[kd] = 1.0 / piv;
    }
    if (!grid_sync(A.C)) return;
  }
  // l(ua(1:n)) = 1/l(ua(1:n))
  for (int i = gt; i < S.n; i += G) {
    const int kd = __ldg(S.dg + i);
    l[kd] = 1.0 / ldcg(l + kd);
  }
}

// lus_cr, linear_solvers.f90:1386-1478: unit lower forward, then upper
// backward with division by the pivot
__global__ void __launch_bounds__(FC_BLOCK) k_lus(IluArgs A) {
  const CsrView<double>& S = A.S;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  const double* l = A.l;
  double* w = A.w;
  for (int i = gt; i < S.n; i += G) w[i] = ldcg(A.r + i);
  if (!grid_sync(A.C)) return;
  for (int lev = 0; lev < S.nlf; ++lev) {
    const int b = __ldg(S.lfp + lev), e = __ldg(S.lfp + lev + 1);
    for (int idx = b + gt; idx < e; idx += G) {
      const int i = __ldg(S.lfr + idx);
      double wi = ldcg(w + i);
      for (int j = __ldg(S.ia + i); j < __ldg(S.dg + i); ++j) wi = __dsub_rn(wi, __dmul_rn(ldcg(l + j), ldcg(w + __ldg(S.ja + j))));
      w[i] = wi;
    }
    if (!grid_sync(A.C)) return;
  }
  for (int lev = 0; lev < S.nlb; ++lev) {
    const int b = __ldg(S.lbp + lev), e = __ldg(S.lbp + lev + 1);
    for (int idx = b + gt; idx < e; idx += G) {
      const int i = __ldg(S.lbr + idx);
      const int kd = __ldg(S.dg + i);
      double wi = ldcg(w + i);
      for (int j = kd + 1; j < __ldg(S.ia + i + 1); ++j) wi = __dsub_rn(wi, __dmul_rn(ldcg(l + j), ldcg(w + __ldg(S.ja + j))));
      w[i] = __ddiv_rn(wi, ldcg(l + kd));
    }
    if (!grid_sync(A.C)) return;
  }
}

__global__ void k_ax(const int* __restrict__ ia, const int* __restrict__ ja, const double* __restrict__ a,
                     const double* __restrict__ x, double* __restrict__ y, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = ia[i]; k < ia[i + 1]; ++k) s = fma(a[k], x[ja[k]], s);
    y[i] = s;
  }
}

// out[slot] = sum_i f(x_i, y_i) in a fixed order: block partials then one
// block sums them (deterministic)
__global__ void k_dot_partial(const double* __restrict__ x, const double* __restrict__ y, int n, int absmode,
                              double* __restrict__ part) {
  __shared__ double sm[FC_BLOCK / 32];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    s += absmode ? fabs(x[i]) : x[i] * y[i];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? sm[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) part[blockIdx.x] = t;
  }
}
__global__ void k_dot_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += 32) s += part[b];
  s = warp_sum(s);
  if (threadIdx.x == 0) *out = s;
}
__global__ void k_axpby(double* __restrict__ y, const double* __restrict__ x, double alpha, double beta, int n) {
  // y = beta*y + alpha*x
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] = beta * y[i] + alpha * x[i];
}
__global__ void k_rsub(double* __restrict__ r, const double* __restrict__ b, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) r[i] = b[i] - r[i];
}

}  // namespace

int gmres_solve(fc_ctx* ctx, CsrSystem* s, const double* a, double* x, const double* b, int itr_max, int mr,
                double tol_abs, double tol_rel, SolveResult* res) {
  const int n = s->n;
  DVec<double> l, V, tmp, part, scal;
  FC_CUDA_TRY(ctx, l.alloc(s->nnz));
  FC_CUDA_TRY(ctx, V.alloc((size_t)n * (mr + 1)));
  FC_CUDA_TRY(ctx, tmp.alloc(n));
  const int nb = std::min(1024, std::max(1, (n + FC_BLOCK - 1) / FC_BLOCK));
  FC_CUDA_TRY(ctx, part.alloc(nb));
  FC_CUDA_TRY(ctx, scal.alloc(1));
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(l.p, a, s->nnz * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  IluArgs A;
  A.S.n = n; A.S.ia = s->ia.p; A.S.ja = s->ja.p; A.S.dg = s->diag.p; A.S.ts = s->tslot.p; A.S.a = a;
  A.S.lfp = s->lf.ptr.p; A.S.lfr = s->lf.rows.p; A.S.nlf = s->lf.nlev;
  A.S.lbp = s->lb.ptr.p; A.S.lbr = s->lb.rows.p; A.S.nlb = s->lb.nlev;
  A.C.bar = s->bar.p; A.C.part = s->part.p; A.C.status = s->status.p; A.C.out = s->out.p;
  A.l = l.p; A.r = nullptr; A.w = nullptr;
  auto coop = [&](const void* fn) -> int {
    int nbk = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbk, fn, FC_BLOCK, 0);
    nbk = std::max(1, std::min(nbk, 2)) * ctx->num_sms;
    nbk = std::max(1, std::min(nbk, (n + FC_BLOCK - 1) / FC_BLOCK));
    cudaMemsetAsync(s->bar.p, 0, 2 * sizeof(unsigned), ctx->stream);
    cudaMemsetAsync(s->status.p, 0, sizeof(int), ctx->stream);
    void* args[1] = {&A};
    cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(nbk), dim3(FC_BLOCK), args, 0, ctx->stream);
    ctx->kernel_launches++;
    if (e != cudaSuccess) return fc_fail(ctx, FC_ERR_CUDA, "cooperative launch (gmres)", e);
    cudaMemcpyAsync(s->h_status, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e2 = cudaStreamSynchronize(ctx->stream);
    if (e2 != cudaSuccess) return fc_fail(ctx, FC_ERR_CUDA, "gmres kernel", e2);
    if (*s->h_status) return fc_fail_msg(ctx, *s->h_status, "gmres: ILU(0) kernel failed (zero pivot or timeout)");
    return FC_OK;
  };
  int st = coop((const void*)k_ilu0);
  if (st) return st;
  const int eb = std::min(4096, std::max(1, (n + 255) / 256));
  auto ax = [&](const double* xin, double* yout) {
    k_ax<<<eb, 256, 0, ctx->stream>>>(s->ia.p, s->ja.p, a, xin, yout, n);
    ctx->kernel_launches++;
  };
  auto lus = [&](const double* rin, double* wout) -> int {
    A.r = rin; A.w = wout;
    return coop((const void*)k_lus);
  };
  auto dot = [&](const double* xa, const double* yb, int absmode) -> double {
    k_dot_partial<<<nb, FC_BLOCK, 0, ctx->stream>>>(xa, yb, n, absmode, part.p);
    k_dot_final<<<1, 32, 0, ctx->stream>>>(part.p, nb, scal.p);
    ctx->kernel_launches += 2;
    double h = 0.0;
    cudaMemcpyAsync(&h, scal.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    return h;
  };
  auto axpby = [&](double* y, const double* xx, double alpha, double beta) {
    k_axpby<<<eb, 256, 0, ctx->stream>>>(y, xx, alpha, beta, n);
    ctx->kernel_launches++;
  };
  auto Vc = [&](int k) { return V.p + (size_t)(k - 1) * n; };  // column k (1-based)
  const double delta = 1.0e-03;
  std::vector<double> c(mr + 2), sv(mr + 2), g(mr + 2), y(mr + 2), h((size_t)(mr + 2) * (mr + 1), 0.0);
  auto H = [&](int i, int j) -> double& { return h[(size_t)j * (mr + 2) + i]; };
  auto givens = [&](double cc, double ss, int k, double* gg) {
    double g1 = cc * gg[k] - ss * gg[k + 1];
    double g2 = ss * gg[k] + cc * gg[k + 1];
    gg[k] = g1; gg[k + 1] = g2;
  };
  double resor = 0.0, rho_tol = 0.0, resl = 0.0;
  int itr_used = 0, k_copy = 0;
  double* r = s->r.p;
  for (int itr = 1; itr <= itr_max; ++itr) {
    ax(x, r);
    k_rsub<<<eb, 256, 0, ctx->stream>>>(r, b, n);
    ctx->kernel_launches++;
    if (itr == 1) {
      resor = dot(r, r, 1);
      rho_tol = resor * tol_rel;
    }
    double rho = std::sqrt(dot(r, r, 0));
    if ((st = lus(r, tmp.p))) return st;
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(Vc(1), tmp.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    axpby(Vc(1), Vc(1), 0.0, 1.0 / rho);
    g[1] = rho;
    for (int i = 2; i <= mr + 1; ++i) g[i] = 0.0;
    std::fill(h.begin(), h.end(), 0.0);
    int k;
    for (k = 1; k <= mr; ++k) {
      k_copy = k;
      ax(Vc(k), tmp.p);
      if ((st = lus(tmp.p, Vc(k + 1)))) return st;
      double av = std::sqrt(dot(Vc(k + 1), Vc(k + 1), 0));
      for (int j = 1; j <= k; ++j) {
        H(j, k) = dot(Vc(k + 1), Vc(j), 0);
        axpby(Vc(k + 1), Vc(j), -H(j, k), 1.0);
      }
      H(k + 1, k) = std::sqrt(dot(Vc(k + 1), Vc(k + 1), 0));
      if ((av + delta * H(k + 1, k)) == av) {
        for (int j = 1; j <= k; ++j) {
          double htmp = dot(Vc(k + 1), Vc(j), 0);
          H(j, k) = H(j, k) + htmp;
          axpby(Vc(k + 1), Vc(j), -htmp, 1.0);
        }
        H(k + 1, k) = std::sqrt(dot(Vc(k + 1), Vc(k + 1), 0));
      }
      if (H(k + 1, k) != 0.0) axpby(Vc(k + 1), Vc(k + 1), 0.0, 1.0 / H(k + 1, k));
      if (1 < k) {
        for (int i = 1; i <= k + 1; ++i) y[i] = H(i, k);
        for (int j = 1; j <= k - 1; ++j) givens(c[j], sv[j], j, y.data());
        for (int i = 1; i <= k + 1; ++i) H(i, k) = y[i];
      }
      double mu = std::sqrt(H(k, k) * H(k, k) + H(k + 1, k) * H(k + 1, k));
      c[k] = H(k, k) / mu;
      sv[k] = -H(k + 1, k) / mu;
      H(k, k) = c[k] * H(k, k) - sv[k] * H(k + 1, k);
      H(k + 1, k) = 0.0;
      givens(c[k], sv[k], k, g.data());
      resl = std::fabs(g[k + 1]);
      ++itr_used;
      if (resl / resor <= rho_tol || resl <= tol_abs) break;
    }
    k = k_copy - 1;
    y[k + 1] = g[k + 1] / H(k + 1, k + 1);
    for (int i = k; i >= 1; --i) {
      double sdot = 0.0;
      for (int q = i + 1; q <= k + 1; ++q) sdot += H(i, q) * y[q];
      y[i] = (g[i] - sdot) / H(i, i);
    }
    for (int q = 1; q <= k + 1; ++q) axpby(x, Vc(q), y[q], 1.0);
    if (resl / resor <= rho_tol || resl <= tol_abs) break;
  }
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  res->res0 = resor;
  res->resor = resor;
  res->resl = resl;
  res->itr_used = itr_used;
  res->factor = 0.0;
  if (!std::isfinite(resl)) res->status = FC_ERR_NAN;
  return FC_OK;
}

namespace {
// w = A^T x as a gather over the column-major view: row j of A^T visits the
// entries (i, j) in ascending i, the order in which atx_cr
// (linear_solvers.f90:1079-1171) scatters into w(j)
__global__ void k_atx(const int* __restrict__ tptr, const int* __restrict__ tsrc, const int* __restrict__ trow,
                      const double* __restrict__ a, const double* __restrict__ x, double* __restrict__ y, int n) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int q = tptr[j]; q < tptr[j + 1]; ++q) s = __dadd_rn(s, __dmul_rn(a[tsrc[q]], x[trow[q]]));
    y[j] = s;
  }
}
}  // namespace

static int build_transpose(fc_ctx* ctx, CsrSystem* s) {
  if (s->tptr.p) return FC_OK;
  const int n = s->n, nnz = s->nnz;
  std::vector<int> ptr(n + 1, 0), src(nnz), row(nnz);
  for (int k = 0; k < nnz; ++k) ptr[s->h_ja[k] + 1]++;
  for (int j = 0; j < n; ++j) ptr[j + 1] += ptr[j];
  std::vector<int> pos(ptr.begin(), ptr.end() - 1);
  for (int i = 0; i < n; ++i)
    for (int k = s->h_ia[i]; k < s->h_ia[i + 1]; ++k) {
      int q = pos[s->h_ja[k]]++;
      src[q] = k;
      row[q] = i;
    }
  FC_CUDA_TRY(ctx, s->tptr.alloc(n + 1));
  FC_CUDA_TRY(ctx, s->tsrc.alloc(nnz));
  FC_CUDA_TRY(ctx, s->trow.alloc(nnz));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->tptr.p, ptr.data(), (n + 1) * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->tsrc.p, src.data(), nnz * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->trow.p, row.data(), nnz * sizeof(int)));
  return FC_OK;
}

// y = A x (ax_cr) or y = A^T x (atx_cr)
int sys_spmv(fc_ctx* ctx, CsrSystem* s, const double* a, const double* x, double* y, int transpose) {
  const int n = s->n;
  const int eb = std::min(8192, std::max(1, (n + 255) / 256));
  if (transpose) {
    int st = build_transpose(ctx, s);
    if (st) return st;
    k_atx<<<eb, 256, 0, ctx->stream>>>(s->tptr.p, s->tsrc.p, s->trow.p, a, x, y, n);
  } else {
    k_ax<<<eb, 256, 0, ctx->stream>>>(s->ia.p, s->ja.p, a, x, y, n);
  }
  ctx->kernel_launches++;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

// ILU(0) factors of ilu_cr into l_out (host or device, nnz values)
int sys_ilu0(fc_ctx* ctx, CsrSystem* s, double* l_out) {
  const int n = s->n;
  DVec<double> l;
  FC_CUDA_TRY(ctx, l.alloc(s->nnz));
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(l.p, s->a.p, s->nnz * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  IluArgs A;
  A.S.n = n; A.S.ia = s->ia.p; A.S.ja = s->ja.p; A.S.dg = s->diag.p; A.S.ts = s->tslot.p; A.S.a = s->a.p;
  A.S.lfp = s->lf.ptr.p; A.S.lfr = s->lf.rows.p; A.S.nlf = s->lf.nlev;
  A.S.lbp = s->lb.ptr.p; A.S.lbr = s->lb.rows.p; A.S.nlb = s->lb.nlev;
  A.C.bar = s->bar.p; A.C.part = s->part.p; A.C.status = s->status.p; A.C.out = s->out.p;
  A.l = l.p; A.r = nullptr; A.w = nullptr;
  int nbk = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nbk, (const void*)k_ilu0, FC_BLOCK, 0);
  nbk = std::max(1, std::min(nbk, 2)) * ctx->num_sms;
  nbk = std::max(1, std::min(nbk, (n + FC_BLOCK - 1) / FC_BLOCK));
  FC_CUDA_TRY(ctx, cudaMemsetAsync(s->bar.p, 0, 2 * sizeof(unsigned), ctx->stream));
  FC_CUDA_TRY(ctx, cudaMemsetAsync(s->status.p, 0, sizeof(int), ctx->stream));
  void* args[1] = {&A};
  FC_CUDA_TRY(ctx, cudaLaunchCooperativeKernel((const void*)k_ilu0, dim3(nbk), dim3(FC_BLOCK), args, 0, ctx->stream));
  ctx->kernel_launches++;
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_status, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(l_out, l.p, s->nnz * sizeof(double),
                                   is_device_ptr(l_out) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (*s->h_status) return fc_fail_msg(ctx, *s->h_status, "ILU(0) failed (zero pivot)");
  return FC_OK;
}
