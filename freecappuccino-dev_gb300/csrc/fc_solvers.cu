// Built-in sparse solvers of freeCappuccino on sm_103a (replaces
// src/linearSolvers/linear_solvers.f90).  Every solve is ONE cooperative,
// persistent kernel: the residual, the preconditioner setup, the Krylov loop
// and its stopping test all run on the device, so the host never waits inside
// an iteration.  Sequential recurrences of the reference (DIC/DILU setup,
// triangular sweeps, Gauss-Seidel) run as level-scheduled sweeps with a grid
// barrier per level and exact (non-contracted) FP64 arithmetic, so the
// preconditioner is the reference's bit for bit.  Dots and norms use a
// deterministic tree and are accumulated in FP64 for every precision.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "fc_internal.hpp"
#include "fc_krylov.cuh"
#include "fc_schedule.hpp"

using namespace fcdev;

extern __shared__ __align__(16) unsigned char fc_smem[];

namespace {

template <class T>
struct KArgs {
  CsrView<T> S;
  GridCtl C;
  T* x;
  const T* b;
  T* r;
  T* r0;
  T* p;
  T* u;
  T* z;
  T* v;
  T* d;
  T* w;
  int itr_max;
  double tol_abs;
  double tol_rel;
  int skip_setup;
  unsigned long long* trace;  // traced instantiation only: phase cycles and step stamps
  int trace_cap;              // step stamps kept per tile and sweep
};

// phases of the ICCG kernel for the optional cycle trace
enum { TR_SETUP = 0, TR_FWD, TR_MID, TR_BWD, TR_DOT, TR_PUPD, TR_SPMV, TR_UPD, FC_TRACE_N = 8 };

// Cycle tracer of the traced ICCG instantiation: per block SM cycles per
// phase (thread 0's clock), and for the first two sweeps after the DIC setup
// (the forward and backward sweep of iteration 1) a stamp (clock64,
// globaltimer) at the start of every step of the tile and after its last.
// trace layout: [blocks][FC_TRACE_N] phase cycles, then
// [2 sweeps][blocks][tl_cap][2] step stamps.
struct Tracer {
  unsigned long long* out;
  int tl_cap, nsweep;
  unsigned long long acc[FC_TRACE_N];
  long long t;
  __device__ Tracer(unsigned long long* o, int cap) : out(o), tl_cap(cap), nsweep(0) {
    for (int k = 0; k < FC_TRACE_N; ++k) acc[k] = 0;
    t = clock64();
  }
  __device__ __forceinline__ void mark(int phase) {
    const long long now = clock64();
    acc[phase] += (unsigned long long)(now - t);
    t = now;
  }
  __device__ __forceinline__ void sweep() { ++nsweep; }
  __device__ __forceinline__ void step(int k) {
    if (threadIdx.x != 0 || nsweep > 2 || k >= tl_cap) return;
    unsigned long long gt;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(gt));
    unsigned long long* q = out + (size_t)gridDim.x * FC_TRACE_N +
                            (((size_t)(nsweep - 1) * gridDim.x + blockIdx.x) * tl_cap + k) * 2;
    q[0] = (unsigned long long)clock64();
    q[1] = gt;
  }
  __device__ void flush() {
    if (threadIdx.x == 0)
      for (int k = 0; k < FC_TRACE_N; ++k) out[(size_t)blockIdx.x * FC_TRACE_N + k] = acc[k];
  }
};

struct NoTracer : NoTrace {
  __device__ NoTracer(unsigned long long*, int) {}
  __device__ void flush() {}
};

template <class T>
__device__ void write_out(const KArgs<T>& A, double res0, double resl, double factor, double resor, int itr, int early) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    A.C.out[FC_OUT_RES0] = res0;
    A.C.out[FC_OUT_RESL] = resl;
    A.C.out[FC_OUT_FACTOR] = factor;
    A.C.out[FC_OUT_RESOR] = resor;
    A.C.out[FC_OUT_ITR] = itr;
    A.C.out[FC_OUT_EARLY] = early;
    if (!isfinite(resl) || !isfinite(res0)) atomicCAS(A.C.status, 0, FC_ERR_NAN);
  }
}

// r = b - A x over all rows; returns L1(r) (identical in every block)
template <class T>
__device__ bool residual_l1(const KArgs<T>& A, int& ph, double& l1out) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  double s[1] = {0.0};
  for (int i = gt; i < A.S.n; i += G) {
    T ri = row_residual(A.S, A.x, ldcg(A.b + i), i);
    A.r[i] = ri;
    s[0] += fabs((double)ri);
  }
  if (!grid_reduce<1>(A.C, ph, s)) return false;
  l1out = s[0];
  return true;
}

// ------------------------------------------------------------------ ICCG
// iccg, linear_solvers.f90:364-545
template <class T, bool TRACE = false>
__global__ void __launch_bounds__(FC_BLOCK, 1) k_iccg(KArgs<T> A) {
  const CsrView<T>& S = A.S;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x, n = S.n;
  int ph = 0;
  SweepCtx X = sweep_ctx(S, fc_smem);
  T *x = A.x, *r = A.r, *p = A.p, *z = A.z, *d = A.d, *yf = A.u;
  const T SENT = Sentinel<T>::value();
  for (int i = gt; i < n; i += G) { p[i] = T(0); z[i] = T(0); yf[i] = SENT; }
  typename std::conditional<TRACE, Tracer, NoTracer>::type tr(A.trace, A.trace_cap);
  double res0;
  if (!residual_l1(A, ph, res0)) return;
  if (res0 < A.tol_abs) { write_out(A, res0, res0, 0.0, 0.0, 0, 1); return; }
  if (!A.skip_setup)
    if (!precond_setup<T, false>(A.C, S, X, d)) return;
  tr.mark(TR_SETUP);
  double s0 = FC_S0, resl = 0.0, factor = 0.0, resor = 0.0;
  int itr_used = 0;
  for (int l = 1; l <= A.itr_max; ++l) {
    double rz[1] = {0.0};
    auto pre = [&](int i) { return ldcg(r + i); };
    auto post = [&](int i, T zi) { rz[0] += (double)ldcg(r + i) * (double)zi; };
    if (!precond_apply(A.C, S, X, d, yf, z, pre, post, false, &tr)) return;
    if (!grid_reduce<1>(A.C, ph, rz)) return;
    tr.mark(TR_DOT);
    const double sk = rz[0];
    const T bet = (T)(sk / s0);
    for (int i = gt; i < n; i += G) p[i] = ldcg(z + i) + bet * ldcg(p + i);
    if (!grid_sync(A.C)) return;
    tr.mark(TR_PUPD);
    double pap[1] = {0.0};
    for (int i = gt; i < n; i += G) {
      T zi = row_dot(S, p, i);
      z[i] = zi;
      pap[0] += (double)ldcg(p + i) * (double)zi;
    }
    if (!grid_reduce<1>(A.C, ph, pap)) return;
    tr.mark(TR_SPMV);
    const T alf = (T)(sk / pap[0]);
    double red[2] = {0.0, 0.0};
    for (int i = gt; i < n; i += G) {
      T xi = ldcg(x + i) + alf * ldcg(p + i);
      x[i] = xi;
      T ri = ldcg(r + i) - alf * ldcg(z + i);
      r[i] = ri;
      yf[i] = SENT;
      red[0] += fabs((double)ri);
      if (l == 1) red[1] += fabs((double)__ldg(S.a + __ldg(S.dg + i)) * (double)xi);
    }
    if (!grid_reduce<2>(A.C, ph, red)) return;
    tr.mark(TR_UPD);
    resl = red[0];
    s0 = sk;
    ++itr_used;
    if (l == 1) { factor = red[1] + FC_SMALL; resor = res0 / factor; }
    const double rsm = resl / (res0 + FC_SMALL);
    if (!(rsm == rsm)) { if (gt == 0) atomicCAS(A.C.status, 0, FC_ERR_NAN); break; }
    if (rsm < A.tol_rel || resl < A.tol_abs) break;
  }
  tr.flush();
  write_out(A, res0, resl, factor, resor, itr_used, 0);
}

// ------------------------------------------------------------- BiCGStab
// bicgstab, linear_solvers.f90:548-786.  The pk update is fused into the
// first forward sweep, and the fi/res updates into the second one (each row
// is updated by the thread that owns it in the sweep).
template <class T>
__global__ void __launch_bounds__(FC_BLOCK, 1) k_bicgstab(KArgs<T> A) {
  const CsrView<T>& S = A.S;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x, n = S.n;
  int ph = 0;
  SweepCtx X = sweep_ctx(S, fc_smem);
  T *x = A.x, *r = A.r, *r0 = A.r0, *p = A.p, *u = A.u, *z = A.z, *v = A.v, *d = A.d, *yf = A.w;
  const T SENT = Sentinel<T>::value();
  double res0;
  if (!residual_l1(A, ph, res0)) return;
  if (res0 < A.tol_abs) { write_out(A, res0, res0, 0.0, 0.0, 0, 1); return; }
  if (!A.skip_setup)
    if (!precond_setup<T, true>(A.C, S, X, d)) return;
  double bb[1] = {0.0};
  for (int i = gt; i < n; i += G) {
    T ri = ldcg(r + i);
    r0[i] = ri; p[i] = T(0); u[i] = T(0); z[i] = T(0); v[i] = T(0); yf[i] = SENT;
    bb[0] += (double)ri * (double)ri;
  }
  if (!grid_reduce<1>(A.C, ph, bb)) return;
  double betn = bb[0];
  double alf = 1.0, beto = 1.0, gam = 1.0, resl = 0.0, factor = 0.0, resor = 0.0;
  int itr_used = 0;
  for (int l = 1; l <= A.itr_max; ++l) {
    const double bet = betn;
    const double om = bet * gam / (alf * beto + FC_SMALL);
    beto = bet;
    const T omT = (T)om, alfT = (T)alf;
    auto pre1 = [&](int i) {
      T pi = ldcg(r + i) + omT * (ldcg(p + i) - alfT * ldcg(u + i));
      p[i] = pi;
      return pi;
    };
    auto nopost = [&](int, T) {};
    if (!precond_apply(A.C, S, X, d, yf, z, pre1, nopost, true)) return;
    double ur[1] = {0.0};
    for (int i = gt; i < n; i += G) {
      T ui = row_dot(S, z, i);
      u[i] = ui;
      yf[i] = SENT;
      ur[0] += (double)ui * (double)ldcg(r0 + i);
    }
    if (!grid_reduce<1>(A.C, ph, ur)) return;
    gam = bet / ur[0];
    const T gamT = (T)gam;
    auto pre2 = [&](int i) {
      x[i] = ldcg(x + i) + gamT * ldcg(z + i);
      T ri = ldcg(r + i) - gamT * ldcg(u + i);
      r[i] = ri;
      return ri;
    };
    if (!precond_apply(A.C, S, X, d, yf, z, pre2, nopost, true)) return;
    double vr[2] = {0.0, 0.0};
    for (int i = gt; i < n; i += G) {
      T vi = row_dot(S, z, i);
      v[i] = vi;
      yf[i] = SENT;
      vr[0] += (double)vi * (double)ldcg(r + i);
      vr[1] += (double)vi * (double)vi;
    }
    if (!grid_reduce<2>(A.C, ph, vr)) return;
    alf = vr[0] / (vr[1] + FC_SMALL);
    const T alT = (T)alf;
    double red[3] = {0.0, 0.0, 0.0};
    for (int i = gt; i < n; i += G) {
      T xi = ldcg(x + i) + alT * ldcg(z + i);
      x[i] = xi;
      T ri = ldcg(r + i) - alT * ldcg(v + i);
      r[i] = ri;
      red[0] += fabs((double)ri);
      red[1] += (double)ri * (double)ldcg(r0 + i);
      if (l == 1) red[2] += fabs((double)__ldg(S.a + __ldg(S.dg + i)) * (double)xi);
    }
    if (!grid_reduce<3>(A.C, ph, red)) return;
    resl = red[0];
    betn = red[1];
    ++itr_used;
    if (l == 1) { factor = red[2] + FC_SMALL; resor = res0 / factor; }
    const double rsm = resl / (res0 + FC_SMALL);
    if (!(rsm == rsm)) { if (gt == 0) atomicCAS(A.C.status, 0, FC_ERR_NAN); break; }
    if (rsm < A.tol_rel || resl < A.tol_abs) break;
  }
  write_out(A, res0, resl, factor, resor, itr_used, 0);
}

// ------------------------------------------------------------------ DPCG
// dpcg, linear_solvers.f90:206-359
template <class T>
__global__ void __launch_bounds__(FC_BLOCK, 1) k_dpcg(KArgs<T> A) {
  const CsrView<T>& S = A.S;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x, n = S.n;
  int ph = 0;
  T *x = A.x, *r = A.r, *p = A.p, *z = A.z;
  for (int i = gt; i < n; i += G) { p[i] = T(0); z[i] = T(0); }
  double res0;
  if (!residual_l1(A, ph, res0)) return;
  if (res0 < A.tol_abs) { write_out(A, res0, res0, 0.0, 0.0, 0, 1); return; }
  double s0 = FC_S0, resl = 0.0, factor = 0.0, resor = 0.0;
  int itr_used = 0;
  for (int l = 1; l <= A.itr_max; ++l) {
    double rz[1] = {0.0};
    for (int i = gt; i < n; i += G) {
      T ri = ldcg(r + i);
      T zi = ri / __ldg(S.a + __ldg(S.dg + i));
      z[i] = zi;
      rz[0] += (double)ri * (double)zi;
    }
    if (!grid_reduce<1>(A.C, ph, rz)) return;
    const double sk = rz[0];
    const T bet = (T)(sk / s0);
    for (int i = gt; i < n; i += G) p[i] = ldcg(z + i) + bet * ldcg(p + i);
    if (!grid_sync(A.C)) return;
    double pap[1] = {0.0};
    for (int i = gt; i < n; i += G) {
      T zi = row_dot(S, p, i);
      z[i] = zi;
      pap[0] += (double)ldcg(p + i) * (double)zi;
    }
    if (!grid_reduce<1>(A.C, ph, pap)) return;
    const T alf = (T)(sk / pap[0]);
    double red[2] = {0.0, 0.0};
    for (int i = gt; i < n; i += G) {
      T xi = ldcg(x + i) + alf * ldcg(p + i);
      x[i] = xi;
      T ri = ldcg(r + i) - alf * ldcg(z + i);
      r[i] = ri;
      red[0] += fabs((double)ri);
      if (l == 1) red[1] += fabs((double)__ldg(S.a + __ldg(S.dg + i)) * (double)xi);
    }
    if (!grid_reduce<2>(A.C, ph, red)) return;
    resl = red[0];
    s0 = sk;
    ++itr_used;
    if (l == 1) { factor = red[1] + FC_SMALL; resor = res0 / factor; }
    const double rsm = resl / (res0 + FC_SMALL);
    if (!(rsm == rsm)) { if (gt == 0) atomicCAS(A.C.status, 0, FC_ERR_NAN); break; }
    if (rsm < A.tol_rel || resl < A.tol_abs) break;
  }
  write_out(A, res0, resl, factor, resor, itr_used, 0);
}

// ---------------------------------------------------------- Gauss-Seidel
// GaussSeidel, linear_solvers.f90:96-201: in-place sweep as a forward
// level-scheduled sweep; entries left of the diagonal read this sweep's
// values (xb), the others the previous sweep's (xa).
__global__ void __launch_bounds__(FC_BLOCK, 1) k_gauss_seidel(KArgs<double> A) {
  const CsrView<double>& S = A.S;
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x, n = S.n;
  int ph = 0;
  SweepCtx X = sweep_ctx(S, fc_smem);
  double* ring = (double*)X.ring;
  double* xa = A.x;
  double* xb = A.w;
  double res0 = 0.0, resl = 0.0, factor = 0.0, resor = 0.0;
  int itr_used = 0, early = 0;
  for (int l = 1; l <= A.itr_max; ++l) {
    double red[2] = {0.0, 0.0};
    for (int i = gt; i < n; i += G) xb[i] = Sentinel<double>::value();
    if (!grid_sync(A.C)) return;
    auto gpre = [&](RowIn<double>& r) { r.q = ldcg(A.b + r.i); };
    auto rowf = [&](const RowIn<double>& r) {
      const int i = r.i;
      const int kd = r.kb + row_entries(r, S.ia, S.dg, true), k1 = __ldg(S.ia + i + 1);
      double s = r.q;
      for (int k = r.kb; k < k1; ++k) {
        const double xj = k < kd ? entry_value(r, k - r.kb, S.code, (const double*)ring, (const double*)xb,
                                               X.abort_flag, A.C)
                                 : ldcg(xa + __ldg(S.ja + k));
        s = __dsub_rn(s, __dmul_rn(__ldg(S.a + k), xj));
      }
      const double aii = __ldg(S.a + kd);
      const double xi = __dadd_rn(ldcg(xa + i), __ddiv_rn(s, __dadd_rn(aii, FC_SMALL)));
      red[0] += fabs(s);
      red[1] += fabs(aii * xi);
      return xi;
    };
    if (!tile_sweep(A.C, S.F, S.a, S.code, (const double*)xb, ring, X.abort_flag, xb, gpre, rowf)) return;
    if (!grid_reduce<2>(A.C, ph, red)) return;
    double* t = xa; xa = xb; xb = t;
    if (l == 1) {
      res0 = red[0];
      if (res0 < A.tol_abs) { early = 1; resl = res0; itr_used = 0; break; }
    }
    resl = red[0];
    ++itr_used;
    if (l == 1) { factor = red[1] + FC_SMALL; resor = res0 / factor; }
    const double rsm = resl / (res0 + FC_SMALL);
    if (!(rsm == rsm)) { if (gt == 0) atomicCAS(A.C.status, 0, FC_ERR_NAN); break; }
    if (rsm < A.tol_rel || resl < A.tol_abs) break;
  }
  if (xa != A.x)
    for (int i = gt; i < n; i += G) A.x[i] = ldcg(xa + i);
  write_out(A, res0, resl, factor, resor, itr_used, early);
}

// preconditioner only: d (DIC or DILU) and optionally z = M^-1 q
template <class T, bool DILU>
__global__ void __launch_bounds__(FC_BLOCK, 1) k_precond(KArgs<T> A, int apply) {
  SweepCtx X = sweep_ctx(A.S, fc_smem);
  if (!A.skip_setup)
    if (!precond_setup<T, DILU>(A.C, A.S, X, A.d)) return;
  if (!apply) return;
  const T* q = A.b;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < A.S.n; i += gridDim.x * blockDim.x)
    A.u[i] = Sentinel<T>::value();
  if (!grid_sync(A.C)) return;
  auto pre = [&](int i) { return ldcg(q + i); };
  auto nopost = [&](int, T) {};
  precond_apply(A.C, A.S, X, A.d, A.u, A.z, pre, nopost, false);
}

// r = b - A x in FP64 with L1 norm (refinement step of the mixed solve)
__global__ void __launch_bounds__(FC_BLOCK, 1) k_residual64(KArgs<double> A) {
  int ph = 0;
  double l1;
  if (!residual_l1(A, ph, l1)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) A.C.out[FC_OUT_RESL] = l1;
  // sum |a_ii x_i| for the reference's normalisation factor
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  double f[1] = {0.0};
  for (int i = gt; i < A.S.n; i += G) f[0] += fabs(__ldg(A.S.a + __ldg(A.S.dg + i)) * ldcg(A.x + i));
  if (!grid_reduce<1>(A.C, ph, f)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) A.C.out[FC_OUT_FACTOR] = f[0];
}

__global__ void k_to_float(const double* __restrict__ s, float* __restrict__ d, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = (float)s[i];
}
__global__ void k_zero_float(float* __restrict__ d, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) d[i] = 0.0f;
}
__global__ void k_add_float(double* __restrict__ x, const float* __restrict__ dx, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) x[i] += (double)dx[i];
}

}  // namespace

// ======================================================================== host

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) { cudaGetLastError(); return false; }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

CsrSystem::~CsrSystem() {
  if (h_out) cudaFreeHost(h_out);
  if (h_status) cudaFreeHost(h_status);
}

static void build_levels(int n, const std::vector<int>& ia, const std::vector<int>& ja, const std::vector<int>& dg,
                         bool lower, LevelSchedule& L, std::vector<int>& lev) {
  lev.assign(n, 0);
  int nlev = 0;
  if (lower) {
    for (int i = 0; i < n; ++i) {
      int m = -1;
      for (int k = ia[i]; k < dg[i]; ++k) m = std::max(m, lev[ja[k]]);
      lev[i] = m + 1;
      nlev = std::max(nlev, lev[i] + 1);
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int m = -1;
      for (int k = dg[i] + 1; k < ia[i + 1]; ++k) m = std::max(m, lev[ja[k]]);
      lev[i] = m + 1;
      nlev = std::max(nlev, lev[i] + 1);
    }
  }
  L.nlev = nlev;
  L.h_ptr.assign(nlev + 1, 0);
  for (int i = 0; i < n; ++i) L.h_ptr[lev[i] + 1]++;
  L.max_width = 0;
  for (int l = 0; l < nlev; ++l) {
    L.max_width = std::max(L.max_width, L.h_ptr[l + 1]);
    L.h_ptr[l + 1] += L.h_ptr[l];
  }
  L.h_rows.assign(n, 0);
  std::vector<int> pos(L.h_ptr.begin(), L.h_ptr.end() - 1);
  for (int i = 0; i < n; ++i) L.h_rows[pos[lev[i]]++] = i;  // ascending row order inside a level
}

static int upload_sweep(fc_ctx* ctx, const SweepSchedule& S, DevSweep& D) {
  D.ntiles = S.ntiles; D.nlev = S.nlev; D.R = S.R; D.max_slots = S.max_slots;
  D.cross = S.cross_tile_entries; D.ring = S.ring_entries; D.global_same = S.global_same_tile_entries;
  auto put = [&](DVec<int>& d, const std::vector<int>& h) -> int {
    FC_CUDA_TRY(ctx, d.alloc(std::max<size_t>(1, h.size())));
    if (!h.empty()) FC_CUDA_TRY(ctx, cudaMemcpy(d.p, h.data(), h.size() * sizeof(int), cudaMemcpyHostToDevice));
    return FC_OK;
  };
  int st;
  if ((st = put(D.tile_step_ptr, S.tile_step_ptr)) || (st = put(D.step_level, S.step_level)) ||
      (st = put(D.tile_slots, S.tile_slots)) || (st = put(D.step_row_ptr, S.step_row_ptr)) ||
      (st = put(D.rows, S.rows)) || (st = put(D.kbne, S.kbne)))
    return st;
  return FC_OK;
}

// step cost and cross-tile latency used to compare tile counts (measured on
// GB300: a step of ~100 FP64 rows takes a few tenths of a microsecond, a flag
// published by one SM is seen by another about a microsecond later)
#define FC_SWEEP_TAU0_US 0.08
#define FC_SWEEP_ROW_US 0.002
#define FC_SWEEP_HOP_US 1.0

int sys_set_pattern(fc_ctx* ctx, CsrSystem* s, int n, int nnz, const int* ia1, const int* ja1, const int* diag1,
                    const double* xyz) {
  if (n <= 0 || nnz < n) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "csr pattern: n <= 0 or nnz < n");
  if (nnz >= (1 << 27)) return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "csr pattern: nnz >= 2^27");
  std::vector<int> ia(n + 1), ja(nnz), dg(n);
  // the caller's arrays may live on the host or the device
  auto fetch = [&](const int* src, int* dst, size_t cnt) -> int {
    if (is_device_ptr(src)) {
      cudaError_t e = cudaMemcpy(dst, src, cnt * sizeof(int), cudaMemcpyDeviceToHost);
      if (e != cudaSuccess) return fc_fail(ctx, FC_ERR_CUDA, "pattern copy", e);
    } else {
      std::memcpy(dst, src, cnt * sizeof(int));
    }
    return FC_OK;
  };
  int st;
  if ((st = fetch(ia1, ia.data(), n + 1)) || (st = fetch(ja1, ja.data(), nnz)) || (st = fetch(diag1, dg.data(), n)))
    return st;
  for (auto& v : ia) v -= 1;
  for (auto& v : ja) v -= 1;
  for (auto& v : dg) v -= 1;
  if (ia[0] != 0 || ia[n] != nnz) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "csr pattern: ia(1) != 1 or ia(n+1) != nnz+1");
  for (int i = 0; i < n; ++i) {
    if (ia[i + 1] <= ia[i]) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "csr pattern: empty or decreasing row");
    for (int k = ia[i]; k < ia[i + 1]; ++k) {
      if (ja[k] < 0 || ja[k] >= n) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "csr pattern: column index out of range");
      if (k > ia[i] && ja[k] <= ja[k - 1])
        return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "csr pattern: columns not strictly increasing in a row");
    }
    if (dg[i] < ia[i] || dg[i] >= ia[i + 1] || ja[dg[i]] != i)
      return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "csr pattern: diag does not point at the diagonal");
  }
  // transpose slots: the reference's search for (j,i) starting at diag(j)
  // (linear_solvers.f90:616-620); it ends one past row j when (j,i) is absent
  std::vector<int> ts(nnz, 0);
  bool oob = false;
  for (int i = 0; i < n; ++i)
    for (int k = ia[i]; k < dg[i]; ++k) {
      int j = ja[k], l;
      for (l = dg[j]; l < ia[j + 1]; ++l)
        if (ja[l] == i) break;
      if (l >= nnz) { oob = true; l = nnz - 1; }
      ts[k] = l;
    }
  s->n = n;
  s->nnz = nnz;
  s->tslot_oob = oob;
  std::vector<int> levf, levb;
  build_levels(n, ia, ja, dg, true, s->lf, levf);
  build_levels(n, ia, ja, dg, false, s->lb, levb);
  // tiled pipeline schedules: at most one tile per SM; the tile count is
  // chosen among a few candidates by the critical-path estimate
  std::vector<int> code(nnz, 0);
  SweepSchedule SF, SB;
  const int sms = std::max(1, ctx->num_sms);
  int tiles = sms;
  {
    double best = 1e300;
    const int cand[4] = {sms, (3 * sms) / 4, sms / 2, sms / 4};
    std::vector<int> scratch(nnz, 0);
    for (int ci = 0; ci < 4; ++ci) {
      if (cand[ci] < 1 || (ci > 0 && cand[ci] == cand[ci - 1])) continue;
      SweepSchedule trial;
      build_sweep_schedule(n, ia.data(), ja.data(), dg.data(), levf, s->lf.nlev, true, cand[ci], xyz, trial, scratch);
      const double est = estimate_sweep_us(trial, FC_SWEEP_TAU0_US, FC_SWEEP_ROW_US, FC_SWEEP_HOP_US);
      if (est < best) { best = est; tiles = cand[ci]; }
    }
    s->est_sweep_us = best;
  }
  build_sweep_schedule(n, ia.data(), ja.data(), dg.data(), levf, s->lf.nlev, true, tiles, xyz, SF, code);
  build_sweep_schedule(n, ia.data(), ja.data(), dg.data(), levb, s->lb.nlev, false, tiles, xyz, SB, code);
  int st2;
  if ((st2 = upload_sweep(ctx, SF, s->sf)) || (st2 = upload_sweep(ctx, SB, s->sb))) return st2;
  FC_CUDA_TRY(ctx, s->code.alloc(nnz));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->code.p, code.data(), nnz * sizeof(int), cudaMemcpyHostToDevice));
  FC_CUDA_TRY(ctx, s->ia.alloc(n + 1));
  FC_CUDA_TRY(ctx, s->ja.alloc(nnz));
  FC_CUDA_TRY(ctx, s->diag.alloc(n));
  FC_CUDA_TRY(ctx, s->tslot.alloc(nnz));
  FC_CUDA_TRY(ctx, s->lf.ptr.alloc(s->lf.nlev + 1));
  FC_CUDA_TRY(ctx, s->lf.rows.alloc(n));
  FC_CUDA_TRY(ctx, s->lb.ptr.alloc(s->lb.nlev + 1));
  FC_CUDA_TRY(ctx, s->lb.rows.alloc(n));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->ia.p, ia.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->ja.p, ja.data(), nnz * sizeof(int), cudaMemcpyHostToDevice));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->diag.p, dg.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->tslot.p, ts.data(), nnz * sizeof(int), cudaMemcpyHostToDevice));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->lf.ptr.p, s->lf.h_ptr.data(), (s->lf.nlev + 1) * sizeof(int), cudaMemcpyHostToDevice));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->lf.rows.p, s->lf.h_rows.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->lb.ptr.p, s->lb.h_ptr.data(), (s->lb.nlev + 1) * sizeof(int), cudaMemcpyHostToDevice));
  FC_CUDA_TRY(ctx, cudaMemcpy(s->lb.rows.p, s->lb.h_rows.data(), n * sizeof(int), cudaMemcpyHostToDevice));
  s->h_ia.swap(ia);
  s->h_ja.swap(ja);
  s->h_diag.swap(dg);
  return sys_alloc_work(ctx, s);
}

int sys_alloc_work(fc_ctx* ctx, CsrSystem* s) {
  const int n = s->n;
  FC_CUDA_TRY(ctx, s->a.alloc(s->nnz));
  DVec<double>* v64[] = {&s->x, &s->b, &s->r, &s->r0, &s->p, &s->u, &s->z, &s->v, &s->d, &s->w};
  for (auto* v : v64) FC_CUDA_TRY(ctx, v->alloc(n));
  const int maxblocks = std::max(1, ctx->num_sms * 8);
  FC_CUDA_TRY(ctx, s->part.alloc((size_t)2 * FC_NPART * maxblocks));
  FC_CUDA_TRY(ctx, s->out.alloc(FC_OUT_N));
  FC_CUDA_TRY(ctx, s->bar.alloc(2));
  FC_CUDA_TRY(ctx, s->status.alloc(1));
  FC_CUDA_TRY(ctx, cudaMemset(s->bar.p, 0, 2 * sizeof(unsigned)));
  if (!s->h_out) FC_CUDA_TRY(ctx, cudaMallocHost(&s->h_out, FC_OUT_N * sizeof(double)));
  if (!s->h_status) FC_CUDA_TRY(ctx, cudaMallocHost(&s->h_status, sizeof(int)));
  return FC_OK;
}

static int alloc_work32(fc_ctx* ctx, CsrSystem* s) {
  const int n = s->n;
  FC_CUDA_TRY(ctx, s->a32.alloc(s->nnz));
  DVec<float>* v32[] = {&s->fr, &s->fr0, &s->fp, &s->fu, &s->fz, &s->fv, &s->fd, &s->fx, &s->fy, &s->fw};
  for (auto* v : v32) FC_CUDA_TRY(ctx, v->alloc(n));
  return FC_OK;
}

int sys_upload_values(fc_ctx* ctx, CsrSystem* s, const double* a, bool a_on_device) {
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->a.p, a, (size_t)s->nnz * sizeof(double),
                                   a_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  return FC_OK;
}

static TileSched tsched_of(DevSweep& D) {
  TileSched t;
  t.ntiles = D.ntiles; t.nlev = D.nlev; t.R = D.R; t.max_slots = D.max_slots;
  t.tile_step_ptr = D.tile_step_ptr.p; t.step_level = D.step_level.p; t.tile_slots = D.tile_slots.p;
  t.step_row_ptr = D.step_row_ptr.p; t.rows = D.rows.p; t.kbne = D.kbne.p;
  return t;
}

template <class T>
static CsrView<T> view_of(CsrSystem* s, const T* a) {
  CsrView<T> v;
  v.n = s->n;
  v.ia = s->ia.p; v.ja = s->ja.p; v.dg = s->diag.p; v.ts = s->tslot.p; v.a = a;
  v.code = s->code.p;
  v.F = tsched_of(s->sf);
  v.B = tsched_of(s->sb);
  v.lfp = s->lf.ptr.p; v.lfr = s->lf.rows.p; v.nlf = s->lf.nlev;
  v.lbp = s->lb.ptr.p; v.lbr = s->lb.rows.p; v.nlb = s->lb.nlev;
  return v;
}

// grid size of a cooperative launch: co-resident blocks, capped so the
// barrier stays cheap, and no more than the rows need
static int coop_blocks(fc_ctx* ctx, const void* fn, int n, int per_sm_cap) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, FC_BLOCK, 0);
  nb = std::max(1, std::min(nb, per_sm_cap));
  int blocks = nb * ctx->num_sms;
  int need = (n + FC_BLOCK - 1) / FC_BLOCK;
  return std::max(1, std::min(blocks, need));
}

template <class T>
static int launch_coop(fc_ctx* ctx, CsrSystem* s, const void* fn, KArgs<T>& A, void** extra, int nextra) {
  // one block per tile of the sweep schedules (every tile must be resident)
  const size_t smem = sweep_smem_bytes<T>(s->sf.R, s->sf.max_slots, s->sb.R, s->sb.max_slots);
  if (smem > 48 * 1024)
    FC_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int nb = 0;
  FC_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, FC_BLOCK, smem));
  const int blocks = std::max(1, std::max(s->sf.ntiles, s->sb.ntiles));
  if (nb * ctx->num_sms < blocks)
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "sweep schedule needs more resident blocks than the GPU holds");
  FC_CUDA_TRY(ctx, cudaMemsetAsync(s->bar.p, 0, 2 * sizeof(unsigned), ctx->stream));
  FC_CUDA_TRY(ctx, cudaMemsetAsync(s->status.p, 0, sizeof(int), ctx->stream));
  void* args[4] = {&A, nullptr, nullptr, nullptr};
  for (int i = 0; i < nextra; ++i) args[1 + i] = extra[i];
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(FC_BLOCK), args, smem, ctx->stream);
  if (e != cudaSuccess) return fc_fail(ctx, FC_ERR_CUDA, "cooperative launch", e);
  ctx->kernel_launches++;
  return FC_OK;
}

template <class T>
static KArgs<T> make_args(CsrSystem* s, const T* a, T* x, const T* b, T* r, T* r0, T* p, T* u, T* z, T* v, T* d,
                          T* w, int itr_max, double tol_abs, double tol_rel) {
  KArgs<T> A;
  A.S = view_of<T>(s, a);
  A.C.bar = s->bar.p; A.C.part = s->part.p; A.C.status = s->status.p; A.C.out = s->out.p;
  A.x = x; A.b = b; A.r = r; A.r0 = r0; A.p = p; A.u = u; A.z = z; A.v = v; A.d = d; A.w = w;
  A.itr_max = itr_max; A.tol_abs = tol_abs; A.tol_rel = tol_rel; A.skip_setup = 0;
  A.trace = nullptr;
  A.trace_cap = 0;
  return A;
}

static int fetch_out(fc_ctx* ctx, CsrSystem* s, SolveResult* res) {
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_out, s->out.p, FC_OUT_N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_status, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  res->res0 = s->h_out[FC_OUT_RES0];
  res->resl = s->h_out[FC_OUT_RESL];
  res->factor = s->h_out[FC_OUT_FACTOR];
  res->resor = s->h_out[FC_OUT_RESOR];
  res->itr_used = (int)s->h_out[FC_OUT_ITR];
  res->early = (int)s->h_out[FC_OUT_EARLY];
  res->status = *s->h_status;
  return FC_OK;
}

static int solve_fp64(fc_ctx* ctx, CsrSystem* s, const std::string& solver, const double* a, double* x,
                      const double* b, int itr_max, double tol_abs, double tol_rel, SolveResult* res) {
  KArgs<double> A = make_args<double>(s, a, x, b, s->r.p, s->r0.p, s->p.p, s->u.p, s->z.p, s->v.p, s->d.p,
                                      s->w.p, itr_max, tol_abs, tol_rel);
  const bool traced = ctx->tracing && solver == "iccg";
  if (traced) {
    const int nb = std::max(1, max(s->sf.ntiles, s->sb.ntiles));
    const int cap = max(s->sf.nlev, s->sb.nlev) + 1;
    FC_CUDA_TRY(ctx, ctx->trace.alloc((size_t)nb * FC_TRACE_N + (size_t)2 * nb * cap * 2));
    FC_CUDA_TRY(ctx, cudaMemsetAsync(ctx->trace.p, 0, ctx->trace.bytes(), ctx->stream));
    A.trace = ctx->trace.p;
    A.trace_cap = cap;
    ctx->trace_blocks = nb;
    ctx->trace_cap = cap;
  }
  FC_CUDA_TRY(ctx, cudaMemsetAsync(s->out.p, 0, FC_OUT_N * sizeof(double), ctx->stream));
  int st;
  if (solver == "iccg")
    st = launch_coop(ctx, s, traced ? (const void*)k_iccg<double, true> : (const void*)k_iccg<double>, A, nullptr,
                     0);
  else if (solver == "bicgstab") {
    if (s->tslot_oob) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "bicgstab: pattern is not structurally symmetric");
    st = launch_coop(ctx, s, (const void*)k_bicgstab<double>, A, nullptr, 0);
  } else if (solver == "dpcg") st = launch_coop(ctx, s, (const void*)k_dpcg<double>, A, nullptr, 0);
  else if (solver == "gauss-seidel") st = launch_coop(ctx, s, (const void*)k_gauss_seidel, A, nullptr, 0);
  else return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "unknown solver '" + solver + "'");
  if (st) return st;
  return fetch_out(ctx, s, res);
}

// Mixed precision: FP32 matrix, preconditioner and Krylov vectors inside an
// FP64 iterative-refinement loop; the outer residual b - A x, the update and
// every norm/dot accumulation are FP64.  Stops on the reference's criterion
// resl/(res0+small) < tol_rel or resl < tol_abs (L1 norms).
static int solve_mixed(fc_ctx* ctx, CsrSystem* s, const std::string& solver, const double* a, double* x,
                       const double* b, int itr_max, double tol_abs, double tol_rel, SolveResult* res) {
  if (solver != "iccg" && solver != "bicgstab" && solver != "dpcg")
    return solve_fp64(ctx, s, solver, a, x, b, itr_max, tol_abs, tol_rel, res);
  if (solver == "bicgstab" && s->tslot_oob)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "bicgstab: pattern is not structurally symmetric");
  int st = alloc_work32(ctx, s);
  if (st) return st;
  const int n = s->n;
  const int eb = std::min(4096, (n + 255) / 256);
  k_to_float<<<std::min(8192, (s->nnz + 255) / 256), 256, 0, ctx->stream>>>(a, s->a32.p, s->nnz);
  ctx->kernel_launches++;
  KArgs<double> R = make_args<double>(s, a, x, b, s->r.p, s->r0.p, s->p.p, s->u.p, s->z.p, s->v.p, s->d.p,
                                      s->w.p, 0, tol_abs, tol_rel);
  const double inner_tol = ctx->inner_tol > 0 ? ctx->inner_tol : 1e-4;
  const int inner_itmax = ctx->inner_itmax > 0 ? ctx->inner_itmax : std::max(itr_max, 1);
  double res0 = 0, resl = 0, factor = 0;
  int total_itr = 0, outer = 0;
  bool first = true;
  const int max_outer = 64;
  for (;;) {
    if ((st = launch_coop(ctx, s, (const void*)k_residual64, R, nullptr, 0))) return st;
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_out, s->out.p, FC_OUT_N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_status, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (*s->h_status) { res->status = *s->h_status; return FC_OK; }
    resl = s->h_out[FC_OUT_RESL];
    if (first) {
      res0 = resl;
      if (res0 < tol_abs) { res->res0 = res0; res->resl = res0; res->early = 1; res->itr_used = 0; return FC_OK; }
      first = false;
    } else if (outer == 1) {
      factor = s->h_out[FC_OUT_FACTOR] + FC_SMALL;
    }
    if (!std::isfinite(resl)) { res->status = FC_ERR_NAN; break; }
    if (!first && outer > 0) {
      double rsm = resl / (res0 + FC_SMALL);
      if (rsm < tol_rel || resl < tol_abs) break;
    }
    if (outer >= max_outer || total_itr >= itr_max) { res->status = FC_WARN_MAXITER; break; }
    // inner FP32 solve of A dx = r from dx = 0
    k_to_float<<<eb, 256, 0, ctx->stream>>>(s->r.p, s->fr0.p, n);
    k_zero_float<<<eb, 256, 0, ctx->stream>>>(s->fx.p, n);
    ctx->kernel_launches += 2;
    KArgs<float> F = make_args<float>(s, s->a32.p, s->fx.p, s->fr0.p, s->fr.p, s->fy.p /*r0*/, s->fp.p, s->fu.p,
                                      s->fz.p, s->fv.p, s->fd.p, s->fw.p, std::min(inner_itmax, itr_max - total_itr),
                                      0.0, inner_tol);
    F.skip_setup = outer > 0 ? 1 : 0;
    const void* fn = solver == "iccg" ? (const void*)k_iccg<float>
                     : solver == "bicgstab" ? (const void*)k_bicgstab<float> : (const void*)k_dpcg<float>;
    if ((st = launch_coop(ctx, s, fn, F, nullptr, 0))) return st;
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_out, s->out.p, FC_OUT_N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_status, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (*s->h_status) { res->status = *s->h_status; return FC_OK; }
    total_itr += (int)s->h_out[FC_OUT_ITR];
    k_add_float<<<eb, 256, 0, ctx->stream>>>(x, s->fx.p, n);
    ctx->kernel_launches++;
    ++outer;
  }
  res->res0 = res0;
  res->resl = resl;
  res->factor = factor;
  res->resor = factor > 0 ? res0 / factor : 0.0;
  res->itr_used = total_itr;
  res->outer = outer;
  return FC_OK;
}

int sys_solve(fc_ctx* ctx, CsrSystem* s, const char* solver_c, const double* a, double* x, const double* b,
              int itr_max, double tol_abs, double tol_rel, SolveResult* res) {
  if (!a) a = s->a.p;
  std::string solver(solver_c ? solver_c : "");
  *res = SolveResult();
  FC_CUDA_TRY(ctx, cudaEventRecord(ctx->sev0, ctx->stream));
  int st;
  if (solver == "pmgmres") {
    st = gmres_solve(ctx, s, a, x, b, itr_max, 4, tol_abs, tol_rel, res);
  } else if (ctx->precision == 1) {
    st = solve_mixed(ctx, s, solver, a, x, b, itr_max, tol_abs, tol_rel, res);
  } else {
    st = solve_fp64(ctx, s, solver, a, x, b, itr_max, tol_abs, tol_rel, res);
  }
  if (st) return st;
  FC_CUDA_TRY(ctx, cudaEventRecord(ctx->sev1, ctx->stream));
  FC_CUDA_TRY(ctx, cudaEventSynchronize(ctx->sev1));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->sev0, ctx->sev1);
  res->ms = ms;
  if (res->status == FC_ERR_TIMEOUT) return fc_fail_msg(ctx, FC_ERR_TIMEOUT, "solver grid barrier timed out");
  if (res->status < 0) return fc_fail_msg(ctx, res->status, "solver reported an error (NaN/Inf or breakdown)");
  if (res->status == 0 && !res->early && res->itr_used >= itr_max && itr_max > 0 &&
      !(res->resl / (res->res0 + FC_SMALL) < tol_rel || res->resl < tol_abs))
    res->status = FC_WARN_MAXITER;
  return FC_OK;
}

// ------------------------------------------------- preconditioner entry points
int sys_precond(fc_ctx* ctx, CsrSystem* s, int dilu, const double* q, double* z_out, double* d_out, int apply) {
  KArgs<double> A = make_args<double>(s, s->a.p, s->x.p, q, s->r.p, s->r0.p, s->p.p, s->u.p, s->z.p, s->v.p, s->d.p,
                                      s->w.p, 0, 0.0, 0.0);
  void* extra[1] = {&apply};
  int st = dilu ? launch_coop(ctx, s, (const void*)k_precond<double, true>, A, extra, 1)
                : launch_coop(ctx, s, (const void*)k_precond<double, false>, A, extra, 1);
  if (st) return st;
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_status, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (d_out) FC_CUDA_TRY(ctx, cudaMemcpyAsync(d_out, s->d.p, s->n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  if (z_out && apply)
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(z_out, s->z.p, s->n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (*s->h_status) return fc_fail_msg(ctx, *s->h_status, "preconditioner kernel failed");
  return FC_OK;
}

// Trace of the last FP64 ICCG solve run with fc_set_tracing on.
// out[0..FC_TRACE_N) = cycles summed over the blocks that ran, per phase;
// out[FC_TRACE_N] = those blocks; out[FC_TRACE_N+1] = blocks of the launch
// (B); out[FC_TRACE_N+2] = stamps per tile and sweep (K); with timeline
// non-null it receives the stamps as [2][B][K][2] (clock64, globaltimer).
extern "C" int fc_trace_get(fc_ctx* ctx, double* out, unsigned long long* timeline) {
  if (!ctx || !out) return FC_ERR_BAD_INPUT;
  if (!ctx->trace.p) return fc_fail_msg(ctx, FC_ERR_STATE, "no trace recorded");
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const int nb = ctx->trace_blocks, cap = ctx->trace_cap;
  std::vector<unsigned long long> h(ctx->trace.n);
  FC_CUDA_TRY(ctx, cudaMemcpy(h.data(), ctx->trace.p, h.size() * sizeof(unsigned long long), cudaMemcpyDeviceToHost));
  int used = 0;
  for (int k = 0; k < FC_TRACE_N; ++k) out[k] = 0.0;
  for (int b = 0; b < nb; ++b) {
    bool any = false;
    for (int k = 0; k < FC_TRACE_N; ++k) {
      out[k] += (double)h[(size_t)b * FC_TRACE_N + k];
      any |= h[(size_t)b * FC_TRACE_N + k] != 0;
    }
    used += any;
  }
  out[FC_TRACE_N] = used;
  out[FC_TRACE_N + 1] = nb;
  out[FC_TRACE_N + 2] = cap;
  if (timeline)
    std::copy(h.begin() + (size_t)nb * FC_TRACE_N, h.end(), timeline);
  return FC_OK;
}

extern "C" int fc_set_tracing(fc_ctx* ctx, int on) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  ctx->tracing = on;
  return FC_OK;
}

// ------------------------------------------------ DPCG without allocation
// fc_dpcg_noalloc: the Jacobi-PCG kernel (k_dpcg, dpcg of
// linear_solvers.f90:206-359) run on a fixed scratch area in static device
// memory instead of a CsrSystem workspace, so the call allocates nothing
// (no cudaMalloc/cudaFree, no event or stream creation, no host heap).
//
// Scratch (one per device, this translation unit): r, p, z (FC_NOALLOC_MAX_N
// doubles each), the grid reduction partials (two sets of FC_NPART per
// block), and the control block (barrier counters, status, results), which
// is cleared before every launch.  The first call on a device resolves the
// scratch address with cudaGetSymbolAddress while that device is current.
namespace {
constexpr int NA_MAX_BLOCKS = 1024;
constexpr size_t NA_VEC = (size_t)FC_NOALLOC_MAX_N * sizeof(double);
constexpr size_t NA_PART = (size_t)2 * FC_NPART * NA_MAX_BLOCKS * sizeof(double);
constexpr size_t NA_OUT = (size_t)FC_OUT_N * sizeof(double);
constexpr size_t NA_CTL = 256;  // bar[2] + status, padded
constexpr size_t NA_BYTES = 3 * NA_VEC + NA_PART + NA_OUT + NA_CTL;
static_assert(NA_VEC % 256 == 0 && NA_PART % 256 == 0, "scratch sections stay 256-byte aligned");
}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[NA_BYTES];

namespace {
constexpr int NA_MAX_DEVICES = 64;
std::mutex g_na_mutex;
unsigned char* g_na_base[NA_MAX_DEVICES] = {};

int na_fail(char* errmsg, int errlen, int code, const char* msg) {
  if (errmsg && errlen > 0) std::snprintf(errmsg, (size_t)errlen, "fc_dpcg_noalloc: %s", msg);
  return code;
}
}  // namespace

extern "C" int fc_dpcg_noalloc(void* stream, int n, int nnz, const int* ia, const int* ja, const double* a,
                               const int* diag, double* x, const double* b, int itr_max, double tol_abs,
                               double tol_rel, fc_solve_info* info, char* errmsg, int errlen) {
  if (errmsg && errlen > 0) errmsg[0] = '\0';
  if (n <= 0 || nnz < n || !ia || !ja || !a || !diag || !x || !b || itr_max < 0)
    return na_fail(errmsg, errlen, FC_ERR_BAD_INPUT, "bad arguments (n > 0, nnz >= n, non-null device arrays)");
  if (n > FC_NOALLOC_MAX_N)
    return na_fail(errmsg, errlen, FC_ERR_BAD_INPUT, "n exceeds FC_NOALLOC_MAX_N (1048576 rows)");
  for (const void* ptr : {(const void*)ia, (const void*)ja, (const void*)a, (const void*)diag, (const void*)x,
                          (const void*)b})
    if (!is_device_ptr(ptr)) return na_fail(errmsg, errlen, FC_ERR_BAD_INPUT, "arrays must be device memory");
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NA_MAX_DEVICES)
    return na_fail(errmsg, errlen, FC_ERR_CUDA, "no current CUDA device");
  unsigned char* base;
  {
    std::lock_guard<std::mutex> lock(g_na_mutex);
    if (!g_na_base[dev]) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess || !p) return na_fail(errmsg, errlen, FC_ERR_CUDA, "cudaGetSymbolAddress of the scratch failed");
      g_na_base[dev] = (unsigned char*)p;
    }
    base = g_na_base[dev];
  }
  int sms = 0, coop = 0, occ = 0;
  const void* fn = (const void*)k_dpcg<double>;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, FC_BLOCK, 0) != cudaSuccess || occ < 1)
    return na_fail(errmsg, errlen, FC_ERR_UNSUPPORTED, "cooperative launch not available");
  const int blocks = std::min(NA_MAX_BLOCKS, sms * occ);

  double* r = (double*)base;
  double* p = (double*)(base + NA_VEC);
  double* z = (double*)(base + 2 * NA_VEC);
  double* part = (double*)(base + 3 * NA_VEC);
  unsigned char* zero_from = base + 3 * NA_VEC + NA_PART;  // out, then bar/status
  double* out = (double*)zero_from;
  unsigned* bar = (unsigned*)(zero_from + NA_OUT);
  int* status = (int*)(zero_from + NA_OUT + 2 * sizeof(unsigned));

  KArgs<double> A;
  std::memset(&A, 0, sizeof(A));
  A.S.n = n;
  A.S.ia = ia; A.S.ja = ja; A.S.dg = diag; A.S.a = a;
  A.C.bar = bar; A.C.part = part; A.C.status = status; A.C.out = out;
  A.x = x; A.b = b; A.r = r; A.p = p; A.z = z;
  A.itr_max = itr_max; A.tol_abs = tol_abs; A.tol_rel = tol_rel;

  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemsetAsync(zero_from, 0, NA_OUT + NA_CTL, st) != cudaSuccess)
    return na_fail(errmsg, errlen, FC_ERR_CUDA, "clearing the control block failed");
  void* args[1] = {&A};
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(FC_BLOCK), args, 0, st);
  if (e != cudaSuccess) return na_fail(errmsg, errlen, FC_ERR_CUDA, "cooperative launch failed");
  double h_out[FC_OUT_N];
  int h_status = 0;
  if (cudaMemcpyAsync(h_out, out, sizeof(h_out), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaMemcpyAsync(&h_status, status, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess)
    return na_fail(errmsg, errlen, FC_ERR_CUDA, "reading the results failed");
  fc_solve_info I;
  std::memset(&I, 0, sizeof(I));
  I.res0_l1 = h_out[FC_OUT_RES0];
  I.resl = h_out[FC_OUT_RESL];
  I.factor = h_out[FC_OUT_FACTOR];
  I.resor = h_out[FC_OUT_RESOR];
  I.itr_used = (int)h_out[FC_OUT_ITR];
  I.early_exit = (int)h_out[FC_OUT_EARLY];
  I.status = h_status;
  if (I.status == 0 && !I.early_exit && I.itr_used >= itr_max && itr_max > 0 &&
      !(I.resl / (I.res0_l1 + FC_SMALL) < tol_rel || I.resl < tol_abs))
    I.status = FC_WARN_MAXITER;
  if (info) *info = I;
  if (h_status == FC_ERR_TIMEOUT) return na_fail(errmsg, errlen, FC_ERR_TIMEOUT, "grid barrier timed out");
  if (h_status < 0) return na_fail(errmsg, errlen, h_status, "solver reported an error (NaN/Inf or breakdown)");
  return I.status;
}
