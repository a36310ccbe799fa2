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
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "fc_internal.hpp"
#include "fc_krylov.cuh"
#include "fc_schedule.hpp"
#include "fc_sweep.cuh"

using namespace fcdev;

extern __shared__ __align__(16) unsigned char fc_smem[];

namespace {

template <class T>
struct KArgs {
  CsrView<T> S;      // original numbering: values a (the caller's), pattern
  OrdView O;         // schedule-ordered structure (iccg, bicgstab, gauss-seidel, precond)
  OrdVals<T> V;      // per-solve values in the new numbering
  int nnz;
  GridCtl C;
  T* x;              // caller's solution (original numbering, in/out)
  const T* b;        // caller's right-hand side (original numbering)
  T* xo;             // x and b in the new numbering
  T* bo;
  T* r;              // work vectors (new numbering for the ordered kernels)
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
  // > 0 (FP32 inner solves of the mixed modes): stop once the L1 residual
  // has gone stall_window iterations without falling below half of its
  // last recorded value; the FP64 refinement around it decides convergence
  int stall_window;
  unsigned long long* trace;  // traced instantiation only: phase cycles and step stamps
  int trace_cap;              // step stamps kept per tile and sweep
};

// phases of the ICCG kernel for the optional cycle trace
enum { TR_SETUP = 0, TR_FWD, TR_MID, TR_BWD, TR_DOT, TR_PUPD, TR_SPMV, TR_UPD, FC_TRACE_N = 8 };
#define FC_TRACE_STAMPS 8

// Cycle tracer of the traced ICCG instantiation: per block SM cycles per
// phase (thread 0's clock), and for the first two sweeps after the DIC setup
// (the forward and backward sweep of iteration 1) FC_TRACE_STAMPS stamps per
// step of the tile: [0] the compute warps' start of the step (clock64), [1]
// the moment its stage buffer had landed, [2] the staging thread's start of
// the step's copies, [3] the start of the step on the global timer (ns),
// and thread 0's progress through its row: [4] the next step's loads
// issued, [5] the row's dependency values in registers, [6] its value
// computed, [7] its stores issued; the stamps after the last step close the
// sweep.  trace layout: [blocks][FC_TRACE_N] phase cycles, then
// [2 sweeps][blocks][tl_cap][FC_TRACE_STAMPS] step stamps.
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
  __device__ __forceinline__ unsigned long long* slot(int k) {
    return out + (size_t)gridDim.x * FC_TRACE_N +
           (((size_t)(nsweep - 1) * gridDim.x + blockIdx.x) * tl_cap + k) * FC_TRACE_STAMPS;
  }
  // stamp idx of step k, taken once dep is available (thread 0)
  template <class V>
  __device__ __forceinline__ void at(int k, int idx, V dep) {
    if (threadIdx.x != 0 || nsweep > 2 || k >= tl_cap) return;
    unsigned long long c;
    asm volatile("mov.u64 %0, %%clock64;" : "=l"(c) : "l"((unsigned long long)(long long)dep) : "memory");
    slot(k)[idx] = c;
  }
  __device__ __forceinline__ void step(int k) {
    if (threadIdx.x != 0 || nsweep > 2 || k >= tl_cap) return;
    unsigned long long gt;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(gt));
    unsigned long long* q = slot(k);
    q[0] = (unsigned long long)clock64();
    q[3] = gt;
  }
  __device__ __forceinline__ void waited(int k) {
    if (threadIdx.x != 0 || nsweep > 2 || k >= tl_cap) return;
    slot(k)[1] = (unsigned long long)clock64();
  }
  // called by the staging thread only
  __device__ __forceinline__ void staged(int k) {
    if (nsweep > 2 || k >= tl_cap) return;
    slot(k)[2] = (unsigned long long)clock64();
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
  if (vg_bid(A.C) == 0 && threadIdx.x == 0) {
    A.C.out[FC_OUT_RES0] = res0;
    A.C.out[FC_OUT_RESL] = resl;
    A.C.out[FC_OUT_FACTOR] = factor;
    A.C.out[FC_OUT_RESOR] = resor;
    A.C.out[FC_OUT_ITR] = itr;
    A.C.out[FC_OUT_EARLY] = early;
    if (!isfinite(resl) || !isfinite(res0)) atomicCAS(A.C.status, 0, FC_ERR_NAN);
  }
}

// r = b - A x over all rows in the original numbering (DPCG, refinement);
// returns L1(r) (identical in every block)
template <class T>
__device__ bool residual_l1(const KArgs<T>& A, int& ph, double& l1out) {
  const int gt = vg_gt(A.C), G = vg_G(A.C);
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

// First phase of the ordered kernels: matrix values into the new numbering,
// exchange arrays to the sentinel, b (and x) gathered; ends with a barrier.
template <class T>
__device__ bool ord_prologue(const KArgs<T>& A, bool dilu, bool with_x) {
  ord_gather_values(A.C, A.O, A.V, A.S.a, A.nnz, dilu);
  ord_gather_vec(A.C, A.O, A.b, A.bo);
  if (with_x) ord_gather_vec(A.C, A.O, (const T*)A.x, A.xo);
  return grid_sync(A.C);
}

// r = b - A x in the new numbering; returns L1(r) (identical in every block)
template <class T>
__device__ bool ord_residual_l1(const KArgs<T>& A, int& ph, double& l1out) {
  const int gt = vg_gt(A.C), G = vg_G(A.C);
  double s[1] = {0.0};
  for (int q = gt; q < A.O.n; q += G) {
    T rq = ord_row_residual(A.O, (const T*)A.V.ap, A.xo, ldcg(A.bo + q), q);
    A.r[q] = rq;
    s[0] += fabs((double)rq);
  }
  if (!grid_reduce<1>(A.C, ph, s)) return false;
  l1out = s[0];
  return true;
}

// z = M^-1 q with the DIC/DILU factors d: forward sweep into yf, barrier,
// backward sweep into z (linear_solvers.f90:458-475); dot (optional) gets
// sum e_i z_i of the rows this thread finished.  No barrier at the end.
template <class T, bool WIDE, class TracerT>
__device__ __forceinline__ bool precond_apply(const KArgs<T>& A, OsCtx& X, const T* q, T* yf, T* z, const T* e, double* dot,
                              TracerT* tr) {
  const OsIO<T> f{q, nullptr, yf};
  if (!osweep<T, OS_FWD, WIDE>(A.C, A.O, A.V, f, X, nullptr, tr)) return false;
  tr->mark(TR_FWD);
  if (!grid_sync(A.C)) return false;
  tr->mark(TR_MID);
  const OsIO<T> g{yf, e, z};
  if (dot) {
    if (!osweep<T, OS_BWD_DOT, WIDE>(A.C, A.O, A.V, g, X, dot, tr)) return false;
  } else {
    if (!osweep<T, OS_BWD, WIDE>(A.C, A.O, A.V, g, X, nullptr, tr)) return false;
  }
  tr->mark(TR_BWD);
  return true;
}

// DIC (DILU) factors d_i, inverted as in the reference
// (linear_solvers.f90:439-445, :613-624); ends with a barrier
template <class T, bool DILU, bool WIDE>
__device__ __forceinline__ bool precond_setup(const KArgs<T>& A, OsCtx& X) {
  const OsIO<T> io{nullptr, nullptr, A.d};
  if (!osweep<T, DILU ? OS_SETUP_DILU : OS_SETUP_DIC, WIDE>(A.C, A.O, A.V, io, X, nullptr)) return false;
  return grid_sync(A.C);
}

// ------------------------------------------------------------------ ICCG
// iccg, linear_solvers.f90:364-545, in the schedule-ordered numbering
template <class T, bool TRACE = false, bool WIDE = false>
__global__ void __launch_bounds__(FC_SWEEP_BLOCK, 1) k_iccg(KArgs<T> A) {
  const int gt = vg_gt(A.C), G = vg_G(A.C), n = A.O.n;
  int ph = 0;
  OsCtx X = osweep_ctx<T>(A.O, fc_smem, vg_bid(A.C));
  T *x = A.xo, *r = A.r, *p = A.p, *z = A.z, *yf = A.u;
  typename std::conditional<TRACE, Tracer, NoTracer>::type tr(A.trace, A.trace_cap);
  for (int i = gt; i < n; i += G) p[i] = T(0);
  if (!ord_prologue(A, false, true)) return;
  double res0;
  if (!ord_residual_l1(A, ph, res0)) return;
  if (res0 < A.tol_abs) { write_out(A, res0, res0, 0.0, 0.0, 0, 1); return; }
  if (!A.skip_setup)
    if (!precond_setup<T, false, WIDE>(A, X)) return;
  tr.mark(TR_SETUP);
  double s0 = FC_S0, resl = 0.0, factor = 0.0, resor = 0.0;
  int itr_used = 0;
  for (int l = 1; l <= A.itr_max; ++l) {
    double rz[1] = {0.0};
    if (!precond_apply<T, WIDE>(A, X, (const T*)r, yf, z, (const T*)r, rz, &tr)) return;
    if (!grid_reduce<1>(A.C, ph, rz)) return;
    tr.mark(TR_DOT);
    const double sk = rz[0];
    const T bet = (T)(sk / s0);
    for (int i = gt; i < n; i += G) p[i] = ldcg(z + i) + bet * ldcg(p + i);
    if (!grid_sync(A.C)) return;
    tr.mark(TR_PUPD);
    double pap[1] = {0.0};
    for (int i = gt; i < n; i += G) {
      T zi = ord_row_dot(A.O, (const T*)A.V.ap, p, i);
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
      red[0] += fabs((double)ri);
      if (l == 1) red[1] += fabs((double)ldcg(A.V.adiag + i) * (double)xi);
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
  ord_scatter_vec(A.C, A.O, (const T*)x, A.x);
  tr.flush();
  write_out(A, res0, resl, factor, resor, itr_used, 0);
}

// ------------------------------------------------------------- BiCGStab
// bicgstab, linear_solvers.f90:548-786, in the schedule-ordered numbering.
// Runs on the blocks A.C names (the launch grid, or one problem's group of a
// batched launch).
template <class T, bool WIDE>
__device__ __forceinline__ void bicgstab_body(const KArgs<T>& A) {
  const int gt = vg_gt(A.C), G = vg_G(A.C), n = A.O.n;
  int ph = 0;
  OsCtx X = osweep_ctx<T>(A.O, fc_smem, vg_bid(A.C));
  T *x = A.xo, *r = A.r, *r0 = A.r0, *p = A.p, *u = A.u, *z = A.z, *v = A.v, *yf = A.w;
  NoTracer tr(nullptr, 0);
  if (!ord_prologue(A, true, true)) return;
  double res0;
  if (!ord_residual_l1(A, ph, res0)) return;
  if (res0 < A.tol_abs) { write_out(A, res0, res0, 0.0, 0.0, 0, 1); return; }
  if (!A.skip_setup)
    if (!precond_setup<T, true, WIDE>(A, X)) return;
  double bb[1] = {0.0};
  for (int i = gt; i < n; i += G) {
    T ri = ldcg(r + i);
    r0[i] = ri; p[i] = T(0); u[i] = T(0); z[i] = T(0); v[i] = T(0);
    bb[0] += (double)ri * (double)ri;
  }
  if (!grid_reduce<1>(A.C, ph, bb)) return;
  double betn = bb[0];
  double alf = 1.0, beto = 1.0, gam = 1.0, resl = 0.0, factor = 0.0, resor = 0.0;
  int itr_used = 0;
  double stall_ref = res0;
  int stall_at = 0;
  for (int l = 1; l <= A.itr_max; ++l) {
    const double bet = betn;
    const double om = bet * gam / (alf * beto + FC_SMALL);
    beto = bet;
    const T omT = (T)om, alfT = (T)alf;
    for (int i = gt; i < n; i += G) p[i] = ldcg(r + i) + omT * (ldcg(p + i) - alfT * ldcg(u + i));
    if (!grid_sync(A.C)) return;
    if (!precond_apply<T, WIDE>(A, X, (const T*)p, yf, z, (const T*)nullptr, nullptr, &tr)) return;
    if (!grid_sync(A.C)) return;
    double ur[1] = {0.0};
    for (int i = gt; i < n; i += G) {
      T ui = ord_row_dot(A.O, (const T*)A.V.ap, z, i);
      u[i] = ui;
      ur[0] += (double)ui * (double)ldcg(r0 + i);
    }
    if (!grid_reduce<1>(A.C, ph, ur)) return;
    gam = bet / ur[0];
    const T gamT = (T)gam;
    for (int i = gt; i < n; i += G) {
      x[i] = ldcg(x + i) + gamT * ldcg(z + i);
      r[i] = ldcg(r + i) - gamT * ldcg(u + i);
    }
    if (!grid_sync(A.C)) return;
    if (!precond_apply<T, WIDE>(A, X, (const T*)r, yf, z, (const T*)nullptr, nullptr, &tr)) return;
    if (!grid_sync(A.C)) return;
    double vr[2] = {0.0, 0.0};
    for (int i = gt; i < n; i += G) {
      T vi = ord_row_dot(A.O, (const T*)A.V.ap, z, i);
      v[i] = vi;
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
      if (l == 1) red[2] += fabs((double)ldcg(A.V.adiag + i) * (double)xi);
    }
    if (!grid_reduce<3>(A.C, ph, red)) return;
    resl = red[0];
    betn = red[1];
    ++itr_used;
    if (l == 1) { factor = red[2] + FC_SMALL; resor = res0 / factor; }
    const double rsm = resl / (res0 + FC_SMALL);
    if (!(rsm == rsm)) { if (gt == 0) atomicCAS(A.C.status, 0, FC_ERR_NAN); break; }
    if (rsm < A.tol_rel || resl < A.tol_abs) break;
    if (A.stall_window > 0) {
      if (resl < 0.5 * stall_ref) { stall_ref = resl; stall_at = l; }
      else if (l - stall_at >= A.stall_window) break;
    }
  }
  ord_scatter_vec(A.C, A.O, (const T*)x, A.x);
  write_out(A, res0, resl, factor, resor, itr_used, 0);
}

template <class T, bool WIDE = false>
__global__ void __launch_bounds__(FC_SWEEP_BLOCK, 1) k_bicgstab(KArgs<T> A) {
  bicgstab_body<T, WIDE>(A);
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
// GaussSeidel, linear_solvers.f90:96-201: the in-place sweep as an ordered
// forward sweep; entries left of the diagonal take this sweep's values
// (xb), the diagonal and the entries right of it the previous sweep's (xa).
template <bool WIDE = false>
__global__ void __launch_bounds__(FC_SWEEP_BLOCK, 1) k_gauss_seidel(KArgs<double> A) {
  const int gt = vg_gt(A.C);
  int ph = 0;
  OsCtx X = osweep_ctx<double>(A.O, fc_smem, vg_bid(A.C));
  if (!ord_prologue(A, false, true)) return;
  double* xa = A.xo;
  double* xb = A.w;
  double res0 = 0.0, resl = 0.0, factor = 0.0, resor = 0.0;
  int itr_used = 0, early = 0;
  for (int l = 1; l <= A.itr_max; ++l) {
    double red[2] = {0.0, 0.0};
    const OsIO<double> io{A.bo, xa, xb};
    if (!osweep<double, OS_GS, WIDE>(A.C, A.O, A.V, io, X, red)) return;
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
  ord_scatter_vec(A.C, A.O, (const double*)xa, A.x);
  write_out(A, res0, resl, factor, resor, itr_used, early);
}

// preconditioner only: d (DIC or DILU) and optionally z = M^-1 q, q = A.b;
// results in the original numbering: d into A.v, z into A.z
template <class T, bool DILU, bool WIDE = false>
__global__ void __launch_bounds__(FC_SWEEP_BLOCK, 1) k_precond(KArgs<T> A, int apply) {
  OsCtx X = osweep_ctx<T>(A.O, fc_smem, vg_bid(A.C));
  NoTracer tr(nullptr, 0);
  if (!ord_prologue(A, DILU, false)) return;
  if (!precond_setup<T, DILU, WIDE>(A, X)) return;
  ord_scatter_vec(A.C, A.O, (const T*)A.d, A.v);
  if (!apply) return;
  if (!precond_apply<T, WIDE>(A, X, (const T*)A.bo, A.u, A.w, (const T*)nullptr, nullptr, &tr)) return;
  if (!grid_sync(A.C)) return;
  ord_scatter_vec(A.C, A.O, (const T*)A.w, A.z);
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

// ------------------------------------------------------- batched launches
// The launch grid is split into groups of consecutive blocks; bprob[b] is
// the problem of block b.  A group copies its problem's KArgs (whose GridCtl
// names the group: base block, block count, its own barrier, partial sums,
// status and out slots) into shared memory and runs the single-problem code
// on it.  Groups never wait on each other.
struct BatchCtl {
  int active;      // 0: the group leaves at once
  int skip_setup;  // inner solves after the first keep the DILU factors
  int itr_max;
  int add_dx;      // refinement: x += dx of the previous inner solve first
  int conv_a;      // refinement: a32 = (float)a as well
  int pad[3];
};
// FP32 work arrays of a problem in the mixed modes (original numbering)
struct BatchMix {
  float* fx;    // inner solution dx
  float* fr0;   // inner right-hand side (the FP64 residual, rounded)
  float* a32;   // FP32 matrix values
  int nnz;
  int pad;
};

__device__ __forceinline__ unsigned long long globaltimer_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

template <class T>
__device__ __forceinline__ KArgs<T>& batch_args(const KArgs<T>* __restrict__ args, int p, unsigned char* raw) {
  static_assert(sizeof(KArgs<T>) % 4 == 0, "KArgs is copied as 32-bit words");
  const int* src = reinterpret_cast<const int*>(args + p);
  int* dst = reinterpret_cast<int*>(raw);
  for (int i = threadIdx.x; i < (int)(sizeof(KArgs<T>) / 4); i += blockDim.x) dst[i] = __ldg(src + i);
  return *reinterpret_cast<KArgs<T>*>(raw);
}

template <class T, bool WIDE = false>
__global__ void __launch_bounds__(FC_SWEEP_BLOCK, 1)
    k_bicgstab_batch(const KArgs<T>* __restrict__ args, const int* __restrict__ bprob, const BatchCtl* __restrict__ ctl) {
  __shared__ __align__(16) unsigned char raw[sizeof(KArgs<T>)];
  const int p = __ldg(bprob + blockIdx.x);
  if (p < 0 || !ctl[p].active) return;
  const unsigned long long t0 = globaltimer_ns();
  KArgs<T>& A = batch_args(args, p, raw);
  __syncthreads();
  if (threadIdx.x == 0) { A.skip_setup = ctl[p].skip_setup; A.itr_max = ctl[p].itr_max; }
  __syncthreads();
  bicgstab_body<T, WIDE>(A);
  if (vg_bid(A.C) == 0 && threadIdx.x == 0) A.C.out[FC_OUT_GT] = (double)(globaltimer_ns() - t0);
}

// Refinement step of the mixed batched solve, per group: x += dx of the
// previous inner solve (add_dx), a32 = a (conv_a), barrier, r = b - A x in
// FP64 with L1(r) and sum |a_ii x_i| (the reference's normalisation), the
// inner right-hand side fr0 = (float)r and dx = 0.  The arithmetic of
// k_residual64, k_to_float, k_zero_float and k_add_float in one pass.
__global__ void __launch_bounds__(FC_SWEEP_BLOCK, 1)
    k_refine_batch(const KArgs<double>* __restrict__ args, const int* __restrict__ bprob,
                   const BatchCtl* __restrict__ ctl, const BatchMix* __restrict__ mix) {
  __shared__ __align__(16) unsigned char raw[sizeof(KArgs<double>)];
  const int p = __ldg(bprob + blockIdx.x);
  if (p < 0 || !ctl[p].active) return;
  const unsigned long long t0 = globaltimer_ns();
  const KArgs<double>& A = batch_args(args, p, raw);
  __syncthreads();
  const BatchCtl c = ctl[p];
  const BatchMix m = mix[p];
  const int gt = vg_gt(A.C), G = vg_G(A.C), n = A.S.n;
  if (c.add_dx)
    for (int i = gt; i < n; i += G) A.x[i] = A.x[i] + (double)m.fx[i];
  if (c.conv_a)
    for (int k = gt; k < m.nnz; k += G) m.a32[k] = (float)__ldg(A.S.a + k);
  if (!grid_sync(A.C)) return;
  int ph = 0;
  double s[1] = {0.0};
  for (int i = gt; i < n; i += G) {
    const double ri = row_residual(A.S, (const double*)A.x, ldcg(A.b + i), i);
    A.r[i] = ri;
    m.fr0[i] = (float)ri;
    m.fx[i] = 0.0f;
    s[0] += fabs(ri);
  }
  if (!grid_reduce<1>(A.C, ph, s)) return;
  double f[1] = {0.0};
  for (int i = gt; i < n; i += G) f[0] += fabs(__ldg(A.S.a + __ldg(A.S.dg + i)) * ldcg(A.x + i));
  if (!grid_reduce<1>(A.C, ph, f)) return;
  if (vg_bid(A.C) == 0 && threadIdx.x == 0) {
    A.C.out[FC_OUT_RESL] = s[0];
    A.C.out[FC_OUT_FACTOR] = f[0];
    A.C.out[FC_OUT_GT] = (double)(globaltimer_ns() - t0);
  }
}

}  // namespace

// ======================================================================== host
// Critical-path model of a sweep schedule used to pick the tile count:
// per step cost, per row cost and the delay of a value pushed to another
// tile (its transfer plus the stage lead of the consumer), microseconds.
#define FC_SWEEP_TAU0_US 0.15
#define FC_SWEEP_ROW_US 0.001
#define FC_SWEEP_HOP_US 1.5
#define FC_RING 4                    // ring depth (steps) of the ordered sweeps
// FP32 inner BiCGStab of the mixed modes: iterations without halving the
// residual after which the inner solve ends (the longest such run in the
// converging solves of the batched convection-diffusion set is 22)
#define FC_INNER_STALL_WINDOW 32
#define FC_SWEEP_SMEM (200 * 1024)   // dynamic shared memory budget of a sweep kernel

bool is_device_ptr(const void* p) {
  if (!p) return false;
  cudaPointerAttributes at;
  cudaError_t e = cudaPointerGetAttributes(&at, p);
  if (e != cudaSuccess) { cudaGetLastError(); return false; }
  return at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
}

CsrSystem::~CsrSystem() {
  mc_release(mc);
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

template <class V>
static cudaError_t upload_vec(cudaStream_t s, DVec<int>& d, const V& h) {
  cudaError_t e = d.alloc(std::max<size_t>(1, h.size()));
  if (e != cudaSuccess) return e;
  if (h.empty()) return fc_zero(s, d.p, sizeof(int));
  return fc_h2d(s, d.p, h.data(), h.size() * sizeof(int));
}

// the stage area of the ordered sweeps: the shared memory the fixed parts
// leave (the sweep modes cut it into as many buffers as fit, at most
// FC_MAX_STAGES); 0 when nothing is left
static size_t ordered_stage_area(int R, int maxW, int max_tile_steps) {
  const size_t fixed = osweep_fixed_bytes<double>(R, maxW, max_tile_steps);
  return fixed >= (size_t)FC_SWEEP_SMEM ? 0 : ((size_t)FC_SWEEP_SMEM - fixed) & ~(size_t)15;
}

// stage buffers of the sweep modes up to last_mode at width maxW (the widest
// tile); the smallest over the modes is the depth the schedule is checked
// against.  The Gauss-Seidel mode (OS_GS, the last) stages the most per row.
static int ordered_min_stages(size_t area, int maxW, int xmax, int pmax, int last_mode = OS_GS) {
  int kmin = FC_MAX_STAGES;
  for (int m = OS_SETUP_DIC; m <= last_mode; ++m) {
    StageLayout L;
    L.init_for<double>(maxW, xmax, pmax, m);
    kmin = std::min(kmin, (size_t)L.bytes <= area ? stages_in(area, L.bytes) : 0);
  }
  return kmin;
}

// largest exchange and push blocks of a step (both directions)
static void ordered_blocks(const OrderedSweep& O, int& xmax, int& pmax) {
  xmax = pmax = 4;
  for (int d = 0; d < 2; ++d)
    for (int gs = 0; gs < O.nsteps; ++gs) {
      xmax = std::max(xmax, O.dir[d].xv_ptr[gs + 1] - O.dir[d].xv_ptr[gs]);
      pmax = std::max(pmax, O.dir[d].push_ptr[gs + 1] - O.dir[d].push_ptr[gs]);
    }
}

// The staging a structure needs: two stage buffers for every sweep mode the
// solves use (the factor setups, the applications, Gauss-Seidel when
// with_gs) and FC_APPLY_STAGES for the applications, which run every
// iteration: with fewer the staging thread cannot run far enough ahead to
// hide its copies (measured on 6M tetrahedra: steps of 616 rows with two
// application stages took 222 ms per SIMPLE iteration, steps of 364 rows
// with four 179 ms, despite 2,512 levels against 4,088).
#define FC_APPLY_STAGES 4
// fewest staged rows of a step for which wide levels are kept whole (below,
// they are split into narrower steps)
#define FC_MIN_STAGED_ROWS 64
static int last_mode_of(bool with_gs) { return with_gs ? OS_GS : OS_BWD_DOT; }
static bool staging_ok(size_t area, int maxW, int xmax, int pmax, bool with_gs) {
  if (ordered_min_stages(area, maxW, xmax, pmax, last_mode_of(with_gs)) < 2) return false;
  for (int m = OS_FWD; m <= OS_BWD_DOT; ++m) {
    StageLayout L;
    L.init_for<double>(maxW, xmax, pmax, m);
    if ((size_t)L.bytes > area || stages_in(area, L.bytes) < FC_APPLY_STAGES) return false;
  }
  return true;
}
static bool ordered_fits(const OrderedSweep& O, bool with_gs) {
  int xmax, pmax;
  ordered_blocks(O, xmax, pmax);
  return staging_ok(ordered_stage_area(O.R, O.maxW, O.max_tile_steps), O.maxW, xmax, pmax, with_gs);
}

// The widest step (a multiple of 32 rows, at most maxW) whose staging
// would be enough with exchange and push blocks of three entries per row, the
// most a capped step of the meshes measured needed, and the tile step
// tables grown in proportion to the split; 0 if none.  The first cap tried
// when a schedule does not fit, instead of halving the width.
static int estimated_step_cap(int R, int maxW, int max_tile_steps, bool with_gs) {
  for (int w = maxW & ~31; w >= 32; w -= 32) {
    const int steps = (int)std::min<long long>(1LL << 24, (long long)max_tile_steps * ((maxW + w - 1) / w));
    if (staging_ok(ordered_stage_area(R, w, steps), w, 3 * w, 3 * w, with_gs)) return w;
  }
  return 0;
}

// largest push block of the steps of at most w rows (the blocks that are staged)
static int staged_push_max(const OrderedSweep& O, int w) {
  int pmax = 4;
  for (int d = 0; d < 2; ++d)
    for (int gs = 0; gs < O.nsteps; ++gs)
      if (O.step_ptr[gs + 1] - O.step_ptr[gs] <= w)
        pmax = std::max(pmax, O.dir[d].push_ptr[gs + 1] - O.dir[d].push_ptr[gs]);
  return pmax;
}

// The rows of a step the stage buffers hold when a wider step reads its
// further rows, and its push block, from global memory: the largest multiple
// of 32 (below maxW) whose staging is enough, with the ring at the full
// width; 0 if none.
static int staged_rows_fit(const OrderedSweep& O, bool with_gs) {
  int xmax, pmax;
  ordered_blocks(O, xmax, pmax);
  const size_t area = ordered_stage_area(O.R, O.maxW, O.max_tile_steps);
  for (int w = (O.maxW - 1) & ~31; w >= 32; w -= 32)
    if (staging_ok(area, w, xmax, staged_push_max(O, w), with_gs)) return w;
  return 0;
}

// Wc > 0: a step stages its first Wc rows (fewer than the widest step)
static int upload_ordered(fc_ctx* ctx, const OrderedSweep& O, DevOrdered& D, bool with_gs, int Wc) {
  D.n = O.n; D.nE = O.nE; D.ntiles = O.ntiles; D.nsteps = O.nsteps; D.nlev = O.nlev; D.R = O.R; D.maxW = O.maxW;
  D.max_tile_steps = O.max_tile_steps;
  ordered_blocks(O, D.xmax, D.pmax);
  D.Wc = Wc > 0 && Wc < D.maxW ? Wc : 0;
  const int Ws = D.Wc > 0 ? D.Wc : D.maxW;
  if (D.Wc > 0) D.pmax = staged_push_max(O, D.Wc);  // the push blocks the stage buffers hold
  D.stage_area = ordered_stage_area(D.R, D.maxW, D.max_tile_steps);
  if (ordered_min_stages(D.stage_area, Ws, D.xmax, D.pmax, last_mode_of(with_gs)) < 2)
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "sweep tiles too wide for shared memory");
  D.gs_ok = ordered_min_stages(D.stage_area, Ws, D.xmax, D.pmax, OS_GS) >= 2;
  {
    // stages of the preconditioner application (sweep statistics)
    StageLayout L;
    L.init_for<double>(Ws, D.xmax, D.pmax, OS_FWD);
    D.K = stages_in(D.stage_area, L.bytes);
  }
  D.ring_entries = D.pushed_entries = D.cross_tile_entries = 0;
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.tile_step_ptr, O.tile_step_ptr));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.step_ptr, O.step_ptr));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.tile_W, O.tile_W));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.perm, O.perm));
  for (int d = 0; d < 2; ++d) {
    const OrderedDir& H = O.dir[d];
    D.novf[d] = H.ovf_ptr.empty() ? 0 : H.ovf_ptr.back();
    D.nxv[d] = H.xv_ptr.back();
    D.ring_entries += H.ring_entries;
    D.pushed_entries += H.pushed_entries;
    D.cross_tile_entries += H.cross_tile_entries;
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.srec[d], H.srec));
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.xv_ptr[d], H.xv_ptr));
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.push_ptr[d], H.push_ptr));
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.push[d], H.push));
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.slot[d], H.slot));
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.ovf_ptr[d], H.ovf_ptr));
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.ovf_code[d], H.ovf_code));
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.ovf_col[d], H.ovf_col));
    FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.ovf_slot[d], H.ovf_slot));
  }
  // columns of the upper entries, 4 per row (Gauss-Seidel)
  std::vector<int> ucol((size_t)4 * O.nE, 0);
  for (int q = 0; q < O.n; ++q)
    for (int e = 0; e < FC_ELL; ++e) ucol[4 * (size_t)q + e] = O.dir[1].col[(size_t)e * O.nE + q];
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.ucol, ucol));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.lo_tslot, O.lo_tslot));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.lo_ovf_tslot, O.lo_ovf_tslot));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.dslot, O.dslot));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.p_ptr, O.p_ptr));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.p_col, O.p_col));
  FC_CUDA_TRY(ctx, upload_vec(ctx->stream, D.p_slot, O.p_slot));
  return FC_OK;
}

int sys_set_pattern(fc_ctx* ctx, CsrSystem* s, int n, int nnz, const int* ia1, const int* ja1, const int* diag1,
                    const double* xyz, int tiles_req, bool with_gs) {
  if (n <= 0 || nnz < n) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "csr pattern: n <= 0 or nnz < n");
  if (nnz >= (1 << 27)) return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "csr pattern: nnz >= 2^27");
  mc_release(s->mc);  // the multicolour layout belongs to the previous pattern
  s->mc = nullptr;
  std::vector<int> ia(n + 1), ja(nnz), dg(n);
  // the caller's arrays may live on the host or the device
  auto fetch = [&](const int* src, int* dst, size_t cnt) -> int {
    if (is_device_ptr(src)) {
      cudaError_t e = fc_d2h(ctx->stream, dst, src, cnt * sizeof(int));
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
  // schedule-ordered sweeps: at most one tile per SM; the tile count is
  // chosen among a few candidates by the critical-path estimate
  const int sms = std::max(1, ctx->num_sms);
  int tiles = sms;
  auto t0 = std::chrono::steady_clock::now();
  auto since = [](std::chrono::steady_clock::time_point a) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - a).count();
  };
  // systems whose tiles the caller plans (the batched solves) split wide
  // levels into steps, as their tile planner assumes; the others keep them
  // whole with staged rows (below)
  const bool planned_tiles = tiles_req > 0;
  if (tiles_req <= 0 && ctx->sweep_tiles > 0) tiles_req = ctx->sweep_tiles;
  if (tiles_req > 0) {
    tiles = std::min(tiles_req, sms);
    s->est_sweep_us = 0.0;
  } else {
    const std::vector<int> cand = {sms, (3 * sms) / 4, sms / 2, sms / 4};
    tiles = pick_sweep_tiles(n, ia.data(), ja.data(), dg.data(), xyz, cand, FC_SWEEP_TAU0_US, FC_SWEEP_ROW_US,
                             FC_SWEEP_HOP_US, &s->est_sweep_us);
  }
  s->t_tiling = since(t0);
  t0 = std::chrono::steady_clock::now();
  OrderedSweep O;
  SweepSchedule S;
  std::string err;
  // the widest step must fit the shared-memory staging of the modes the
  // solves use (Gauss-Seidel only when with_gs; a Gauss-Seidel solve on a
  // structure without it analyses the pattern again): if it does not, wide
  // levels are split into narrower steps (more, shorter steps), first at the
  // estimated widest cap that fits, then at 7/8 of the previous cap, until
  // it does
  int wmax = ctx->sweep_cap > 0 ? ctx->sweep_cap : 0;
  int wc = 0;  // rows a step stages when its further rows stay in global memory
  for (;;) {
    if (!build_ordered_sweep(n, ia.data(), ja.data(), dg.data(), ts.data(), tiles, xyz, FC_RING, O, S, err, wmax))
      return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, err);
    if (ctx->stage_rows > 0 && ctx->stage_rows < O.maxW) {
      // forced (tuning, tests), where every mode the solves use still gets
      // two stage buffers
      int xmax, pmax;
      ordered_blocks(O, xmax, pmax);
      const int w = ctx->stage_rows;
      if (ordered_min_stages(ordered_stage_area(O.R, O.maxW, O.max_tile_steps), w, xmax, staged_push_max(O, w),
                             last_mode_of(with_gs)) >= 2) {
        wc = w;
        break;
      }
    }
    if (ordered_fits(O, with_gs)) break;
    if (wmax == 0 && !planned_tiles) {
      // wide levels kept whole: the stage buffers hold the first rows of a
      // step, the others are read from global memory
      wc = staged_rows_fit(O, with_gs);
      if (wc >= FC_MIN_STAGED_ROWS) break;
      wc = 0;
    }
    const int est = wmax ? 0 : estimated_step_cap(FC_RING, O.maxW, O.max_tile_steps, with_gs);
    wmax = est > 0 ? est : (wmax ? (wmax * 7 / 8) & ~7 : std::max(32, O.maxW / 2));
    if (wmax < 32) return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "sweep steps too wide for shared memory");
  }
  s->t_schedule = since(t0);
  s->xyz_src = xyz;
  int st2 = upload_ordered(ctx, O, s->ord, with_gs, wc);
  if (st2) return st2;
  FC_CUDA_TRY(ctx, s->ia.alloc(n + 1));
  FC_CUDA_TRY(ctx, s->ja.alloc(nnz));
  FC_CUDA_TRY(ctx, s->diag.alloc(n));
  FC_CUDA_TRY(ctx, s->tslot.alloc(nnz));
  FC_CUDA_TRY(ctx, s->lf.ptr.alloc(s->lf.nlev + 1));
  FC_CUDA_TRY(ctx, s->lf.rows.alloc(n));
  FC_CUDA_TRY(ctx, s->lb.ptr.alloc(s->lb.nlev + 1));
  FC_CUDA_TRY(ctx, s->lb.rows.alloc(n));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->ia.p, ia.data(), (n + 1) * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->ja.p, ja.data(), nnz * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->diag.p, dg.data(), n * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->tslot.p, ts.data(), nnz * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->lf.ptr.p, s->lf.h_ptr.data(), (s->lf.nlev + 1) * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->lf.rows.p, s->lf.h_rows.data(), n * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->lb.ptr.p, s->lb.h_ptr.data(), (s->lb.nlev + 1) * sizeof(int)));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, s->lb.rows.p, s->lb.h_rows.data(), n * sizeof(int)));
  s->h_ia.swap(ia);
  s->h_ja.swap(ja);
  s->h_diag.swap(dg);
  return sys_alloc_work(ctx, s);
}

template <class T>
static int alloc_ordered(fc_ctx* ctx, CsrSystem* s, OrdStore<T>& V) {
  const DevOrdered& D = s->ord;
  const size_t nE = D.nE, rec = (size_t)Rec<T>::V * nE;
  FC_CUDA_TRY(ctx, V.vrec0.alloc(rec));
  FC_CUDA_TRY(ctx, V.vrec1.alloc(rec));
  FC_CUDA_TRY(ctx, V.sx.alloc(rec));
  FC_CUDA_TRY(ctx, V.aovf0.alloc(std::max(1, D.novf[0])));
  FC_CUDA_TRY(ctx, V.aovf1.alloc(std::max(1, D.novf[1])));
  FC_CUDA_TRY(ctx, V.tovf.alloc(std::max(1, D.novf[0])));
  FC_CUDA_TRY(ctx, V.xv0.alloc(std::max(4, D.nxv[0])));
  FC_CUDA_TRY(ctx, V.xv1.alloc(std::max(4, D.nxv[1])));
  FC_CUDA_TRY(ctx, V.adiag.alloc(nE));
  FC_CUDA_TRY(ctx, V.ap.alloc(s->nnz));
  FC_CUDA_TRY(ctx, V.xo.alloc(nE));
  FC_CUDA_TRY(ctx, V.bo.alloc(nE));
  // padding rows of the record arrays are read by the staging and never used
  FC_CUDA_TRY(ctx, fc_zero(ctx->stream, V.vrec0.p, V.vrec0.bytes()));
  FC_CUDA_TRY(ctx, fc_zero(ctx->stream, V.vrec1.p, V.vrec1.bytes()));
  FC_CUDA_TRY(ctx, fc_zero(ctx->stream, V.sx.p, V.sx.bytes()));
  return FC_OK;
}

int sys_alloc_work(fc_ctx* ctx, CsrSystem* s) {
  const int n = s->ord.nE;  // padded: the sweeps stage whole 16-byte windows
  FC_CUDA_TRY(ctx, s->a.alloc(s->nnz));
  DVec<double>* v64[] = {&s->x, &s->b, &s->r, &s->r0, &s->p, &s->u, &s->z, &s->v, &s->d, &s->w};
  for (auto* v : v64) FC_CUDA_TRY(ctx, v->alloc(n));
  const int maxblocks = std::max(1, ctx->num_sms * 8);
  FC_CUDA_TRY(ctx, s->part.alloc((size_t)2 * FC_NPART * maxblocks));
  FC_CUDA_TRY(ctx, s->out.alloc(FC_OUT_N));
  FC_CUDA_TRY(ctx, s->bar.alloc(2));
  FC_CUDA_TRY(ctx, s->status.alloc(1));
  FC_CUDA_TRY(ctx, fc_zero(ctx->stream, s->bar.p, 2 * sizeof(unsigned)));
  if (!s->h_out) FC_CUDA_TRY(ctx, cudaMallocHost(&s->h_out, FC_OUT_N * sizeof(double)));
  if (!s->h_status) FC_CUDA_TRY(ctx, cudaMallocHost(&s->h_status, sizeof(int)));
  return alloc_ordered(ctx, s, s->o64);
}

static int alloc_work32(fc_ctx* ctx, CsrSystem* s) {
  const int n = s->ord.nE;
  FC_CUDA_TRY(ctx, s->a32.alloc(s->nnz));
  DVec<float>* v32[] = {&s->fr, &s->fr0, &s->fp, &s->fu, &s->fz, &s->fv, &s->fd, &s->fx, &s->fy, &s->fw};
  for (auto* v : v32) FC_CUDA_TRY(ctx, v->alloc(n));
  return alloc_ordered(ctx, s, s->o32);
}

int sys_upload_values(fc_ctx* ctx, CsrSystem* s, const double* a, bool a_on_device) {
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->a.p, a, (size_t)s->nnz * sizeof(double),
                                   a_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  return FC_OK;
}

template <class T>
static CsrView<T> view_of(CsrSystem* s, const T* a) {
  CsrView<T> v;
  v.n = s->n;
  v.ia = s->ia.p; v.ja = s->ja.p; v.dg = s->diag.p; v.ts = s->tslot.p; v.a = a;
  v.lfp = s->lf.ptr.p; v.lfr = s->lf.rows.p; v.nlf = s->lf.nlev;
  v.lbp = s->lb.ptr.p; v.lbr = s->lb.rows.p; v.nlb = s->lb.nlev;
  return v;
}

static OrdView ord_view_of(CsrSystem* s) {
  DevOrdered& D = s->ord;
  OrdView O;
  O.n = D.n; O.nE = D.nE; O.ntiles = D.ntiles; O.R = D.R; O.stage_area = (int)D.stage_area;
  O.novf0 = D.novf[0]; O.novf1 = D.novf[1];
  O.nsteps = D.nsteps; O.maxW = D.maxW; O.xmax = D.xmax; O.pmax = D.pmax; O.Wc = D.Wc;
  O.tile_step_ptr = D.tile_step_ptr.p; O.step_ptr = D.step_ptr.p; O.tile_W = D.tile_W.p; O.perm = D.perm.p;
  for (int d = 0; d < 2; ++d) {
    O.srec[d] = (const int4*)D.srec[d].p; O.xv_ptr[d] = D.xv_ptr[d].p; O.push_ptr[d] = D.push_ptr[d].p;
    O.push[d] = D.push[d].p; O.slot[d] = D.slot[d].p;
    O.ovf_ptr[d] = D.ovf_ptr[d].p; O.ovf_code[d] = D.ovf_code[d].p; O.ovf_col[d] = D.ovf_col[d].p;
    O.ovf_slot[d] = D.ovf_slot[d].p;
  }
  O.ucol = (const int4*)D.ucol.p;
  O.lo_tslot = D.lo_tslot.p; O.lo_ovf_tslot = D.lo_ovf_tslot.p; O.dslot = D.dslot.p;
  O.p_ptr = D.p_ptr.p; O.p_col = D.p_col.p; O.p_slot = D.p_slot.p;
  return O;
}

template <class T>
static OrdVals<T> vals_of(OrdStore<T>& S) {
  OrdVals<T> V;
  V.vrec[0] = S.vrec0.p; V.vrec[1] = S.vrec1.p; V.sx = S.sx.p; V.aovf[0] = S.aovf0.p; V.aovf[1] = S.aovf1.p;
  V.tovf = S.tovf.p; V.adiag = S.adiag.p; V.ap = S.ap.p; V.xv[0] = S.xv0.p; V.xv[1] = S.xv1.p;
  return V;
}

// Cooperative launch of a persistent solver kernel: one block per SM (the
// ordered sweeps need one resident block per tile, tiles <= SMs).
template <class T>
static int launch_coop(fc_ctx* ctx, CsrSystem* s, const void* fn, KArgs<T>& A, void** extra, int nextra,
                       int block = FC_SWEEP_BLOCK) {
  const DevOrdered& D = s->ord;
  const size_t smem = osweep_smem_bytes<T>(D.R, D.stage_area, D.maxW, D.max_tile_steps);
  if (smem > 48 * 1024)
    FC_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int nb = 0;
  FC_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, block, smem));
  const int blocks = std::max(1, ctx->num_sms);
  if (nb < 1 || D.ntiles > blocks)
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "sweep schedule needs more resident blocks than the GPU holds");
  FC_CUDA_TRY(ctx, cudaMemsetAsync(s->bar.p, 0, 2 * sizeof(unsigned), ctx->stream));
  FC_CUDA_TRY(ctx, cudaMemsetAsync(s->status.p, 0, sizeof(int), ctx->stream));
  void* args[4] = {&A, nullptr, nullptr, nullptr};
  for (int i = 0; i < nextra; ++i) args[1 + i] = extra[i];
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(blocks), dim3(block), args, smem, ctx->stream);
  if (e != cudaSuccess) return fc_fail(ctx, FC_ERR_CUDA, "cooperative launch", e);
  ctx->kernel_launches++;
  return FC_OK;
}

template <class T> static OrdStore<T>& store_of(CsrSystem* s);
template <> OrdStore<double>& store_of<double>(CsrSystem* s) { return s->o64; }
template <> OrdStore<float>& store_of<float>(CsrSystem* s) { return s->o32; }

template <class T>
static KArgs<T> make_args(CsrSystem* s, const T* a, T* x, const T* b, T* r, T* r0, T* p, T* u, T* z, T* v, T* d,
                          T* w, int itr_max, double tol_abs, double tol_rel) {
  KArgs<T> A;
  A.S = view_of<T>(s, a);
  A.O = ord_view_of(s);
  OrdStore<T>& st = store_of<T>(s);
  A.V = vals_of<T>(st);
  A.nnz = s->nnz;
  A.C.bar = s->bar.p; A.C.part = s->part.p; A.C.status = s->status.p; A.C.out = s->out.p;
  A.x = x; A.b = b; A.xo = st.xo.p; A.bo = st.bo.p;
  A.r = r; A.r0 = r0; A.p = p; A.u = u; A.z = z; A.v = v; A.d = d; A.w = w;
  A.itr_max = itr_max; A.tol_abs = tol_abs; A.tol_rel = tol_rel; A.skip_setup = 0;
  A.stall_window = 0;
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

// A Gauss-Seidel solve on a structure whose steps are too wide for the
// Gauss-Seidel staging: the pattern is analysed again with that mode in the
// fit (narrower steps), on the same tiles and row coordinates.  The matrix
// values and work vectors of the system stay in place.
static int sys_reanalyse_for_gs(fc_ctx* ctx, CsrSystem* s) {
  std::vector<int> ia1(s->h_ia), ja1(s->h_ja), dg1(s->h_diag);
  for (auto& v : ia1) ++v;
  for (auto& v : ja1) ++v;
  for (auto& v : dg1) ++v;
  const double* xyz = s->xyz_src;
  if (xyz && !(ctx->has_mesh && xyz == ctx->mesh.h_xyz.data())) xyz = nullptr;  // the mesh it came from is gone
  return sys_set_pattern(ctx, s, s->n, s->nnz, ia1.data(), ja1.data(), dg1.data(), xyz, s->ord.ntiles, true);
}

static int solve_fp64(fc_ctx* ctx, CsrSystem* s, const std::string& solver, const double* a, double* x,
                      const double* b, int itr_max, double tol_abs, double tol_rel, SolveResult* res) {
  if (solver == "gauss-seidel" && !s->ord.gs_ok) {
    const int st = sys_reanalyse_for_gs(ctx, s);
    if (st) return st;
  }
  KArgs<double> A = make_args<double>(s, a, x, b, s->r.p, s->r0.p, s->p.p, s->u.p, s->z.p, s->v.p, s->d.p,
                                      s->w.p, itr_max, tol_abs, tol_rel);
  const bool traced = ctx->tracing && solver == "iccg";
  const bool wide = s->ord.Wc > 0;  // steps wider than the stage buffers hold
  if (traced) {
    const int nb = std::max(1, ctx->num_sms);
    const int cap = s->ord.max_tile_steps + 1;
    FC_CUDA_TRY(ctx, ctx->trace.alloc((size_t)nb * FC_TRACE_N + (size_t)2 * nb * cap * FC_TRACE_STAMPS));
    FC_CUDA_TRY(ctx, cudaMemsetAsync(ctx->trace.p, 0, ctx->trace.bytes(), ctx->stream));
    A.trace = ctx->trace.p;
    A.trace_cap = cap;
    ctx->trace_blocks = nb;
    ctx->trace_cap = cap;
  }
  FC_CUDA_TRY(ctx, cudaMemsetAsync(s->out.p, 0, FC_OUT_N * sizeof(double), ctx->stream));
  int st;
  if (solver == "iccg")
    st = launch_coop(ctx, s,
                     traced ? (wide ? (const void*)k_iccg<double, true, true> : (const void*)k_iccg<double, true>)
                            : wide ? (const void*)k_iccg<double, false, true> : (const void*)k_iccg<double>,
                     A, nullptr,
                     0);
  else if (solver == "bicgstab") {
    if (s->tslot_oob) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "bicgstab: pattern is not structurally symmetric");
    st = launch_coop(ctx, s, wide ? (const void*)k_bicgstab<double, true> : (const void*)k_bicgstab<double>, A,
                     nullptr, 0);
  } else if (solver == "dpcg") st = launch_coop(ctx, s, (const void*)k_dpcg<double>, A, nullptr, 0, FC_BLOCK);
  else if (solver == "gauss-seidel")
    st = launch_coop(ctx, s, wide ? (const void*)k_gauss_seidel<true> : (const void*)k_gauss_seidel<false>, A,
                     nullptr, 0);
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
  // the coloured modes change the ICCG solves only; the others stay FP64
  const bool coloured = ctx->precision == FC_PREC_MIXED_COLOURED || ctx->precision == FC_PREC_COLOURED_FP64;
  if (coloured && solver != "iccg") return solve_fp64(ctx, s, solver, a, x, b, itr_max, tol_abs, tol_rel, res);
  if (solver == "bicgstab" && s->tslot_oob)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "bicgstab: pattern is not structurally symmetric");
  // the coloured modes: the ICCG inner solve runs on the multicolour
  // ordering (fc_mc.cu), in FP32 or, as a diagnostic, in FP64
  int st = alloc_work32(ctx, s);
  if (st) return st;
  const int n = s->n;
  const int eb = std::min(4096, (n + 255) / 256);
  if (!coloured) {
    k_to_float<<<std::min(8192, (s->nnz + 255) / 256), 256, 0, ctx->stream>>>(a, s->a32.p, s->nnz);
    ctx->kernel_launches++;
  }
  KArgs<double> R = make_args<double>(s, a, x, b, s->r.p, s->r0.p, s->p.p, s->u.p, s->z.p, s->v.p, s->d.p,
                                      s->w.p, 0, tol_abs, tol_rel);
  const double inner_tol = ctx->inner_tol > 0 ? ctx->inner_tol : 1e-4;
  const int inner_itmax = ctx->inner_itmax > 0 ? ctx->inner_itmax : std::max(itr_max, 1);
  double res0 = 0, resl = 0, factor = 0;
  int total_itr = 0, outer = 0;
  bool first = true;
  const int max_outer = 64;
  for (;;) {
    if ((st = launch_coop(ctx, s, (const void*)k_residual64, R, nullptr, 0, FC_BLOCK))) return st;
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
    if (coloured) {
      // the last refinement step only needs the reduction that is left to
      // the stopping test (with a factor 4 of margin)
      const double left = 0.25 * tol_rel * (res0 + FC_SMALL) / resl;
      const double tol_k = std::min(1e-1, std::max(inner_tol, left));
      int itr = 0, stat = 0;
      st = mc_inner_solve(ctx, s, a, s->r.p, x, tol_k, std::min(inner_itmax, itr_max - total_itr), outer == 0,
                          ctx->precision == FC_PREC_COLOURED_FP64, &itr, &stat);
      if (st) return st;
      if (stat) { res->status = stat; return FC_OK; }
      total_itr += itr;
      ++outer;
      continue;
    }
    // inner FP32 solve of A dx = r from dx = 0
    k_to_float<<<eb, 256, 0, ctx->stream>>>(s->r.p, s->fr0.p, n);
    k_zero_float<<<eb, 256, 0, ctx->stream>>>(s->fx.p, n);
    ctx->kernel_launches += 2;
    KArgs<float> F = make_args<float>(s, s->a32.p, s->fx.p, s->fr0.p, s->fr.p, s->fy.p /*r0*/, s->fp.p, s->fu.p,
                                      s->fz.p, s->fv.p, s->fd.p, s->fw.p, std::min(inner_itmax, itr_max - total_itr),
                                      0.0, inner_tol);
    F.skip_setup = outer > 0 ? 1 : 0;
    if (solver == "bicgstab") F.stall_window = FC_INNER_STALL_WINDOW;
    const bool wide = s->ord.Wc > 0;
    const void* fn = solver == "iccg" ? (wide ? (const void*)k_iccg<float, false, true> : (const void*)k_iccg<float>)
                     : solver == "bicgstab" ? (wide ? (const void*)k_bicgstab<float, true> : (const void*)k_bicgstab<float>)
                                            : (const void*)k_dpcg<float>;
    if ((st = launch_coop(ctx, s, fn, F, nullptr, 0, solver == "dpcg" ? FC_BLOCK : FC_SWEEP_BLOCK))) return st;
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
  } else if (ctx->precision != FC_PREC_FP64) {
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

// ------------------------------------------------------------- batched solves
struct BatchDev {
  int np = 0, nblocks = 0;
  DVec<KArgs<double>> a64, ar;
  DVec<KArgs<float>> af;
  DVec<BatchMix> mix;
  DVec<BatchCtl> ctl;
  DVec<int> bprob;
  DVec<double> out;       // [np][FC_OUT_N]
  DVec<int> status;       // [np]
  DVec<unsigned> bar;     // [np][2]
  double* h_out = nullptr;
  int* h_status = nullptr;
  BatchCtl* h_ctl = nullptr;
  ~BatchDev() {
    if (h_out) cudaFreeHost(h_out);
    if (h_status) cudaFreeHost(h_status);
    if (h_ctl) cudaFreeHost(h_ctl);
  }
};

void batch_dev_release(BatchDev* d) { delete d; }

int batch_block_budget(fc_ctx* ctx, int* budget) {
  *budget = std::max(1, ctx->num_sms);
  return FC_OK;
}

static int batch_prepare(fc_ctx* ctx, BatchDev& B, const std::vector<BatchItem>& items) {
  const int np = (int)items.size();
  std::vector<int> bprob;
  for (int p = 0; p < np; ++p)
    for (int k = 0; k < items[p].s->ord.ntiles; ++k) bprob.push_back(p);
  if ((int)bprob.size() > std::max(1, ctx->num_sms))
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "batch: the groups need more blocks than the GPU holds resident");
  if (B.np != np) {
    if (B.h_out) cudaFreeHost(B.h_out);
    if (B.h_status) cudaFreeHost(B.h_status);
    if (B.h_ctl) cudaFreeHost(B.h_ctl);
    B.h_out = nullptr; B.h_status = nullptr; B.h_ctl = nullptr;
    FC_CUDA_TRY(ctx, cudaMallocHost(&B.h_out, (size_t)np * FC_OUT_N * sizeof(double)));
    FC_CUDA_TRY(ctx, cudaMallocHost(&B.h_status, (size_t)np * sizeof(int)));
    FC_CUDA_TRY(ctx, cudaMallocHost(&B.h_ctl, (size_t)np * sizeof(BatchCtl)));
    FC_CUDA_TRY(ctx, B.a64.alloc(np));
    FC_CUDA_TRY(ctx, B.ar.alloc(np));
    FC_CUDA_TRY(ctx, B.af.alloc(np));
    FC_CUDA_TRY(ctx, B.mix.alloc(np));
    FC_CUDA_TRY(ctx, B.ctl.alloc(np));
    FC_CUDA_TRY(ctx, B.out.alloc((size_t)np * FC_OUT_N));
    FC_CUDA_TRY(ctx, B.status.alloc(np));
    FC_CUDA_TRY(ctx, B.bar.alloc((size_t)2 * np));
    B.np = np;
  }
  FC_CUDA_TRY(ctx, B.bprob.alloc(bprob.size()));
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(B.bprob.p, bprob.data(), bprob.size() * sizeof(int), cudaMemcpyHostToDevice,
                                   ctx->stream));
  B.nblocks = (int)bprob.size();
  return FC_OK;
}

// GridCtl of problem p: its group of blocks, its slots of the batch arrays
template <class T>
static void batch_ctl(KArgs<T>& A, BatchDev& B, int p, int base, int nb) {
  A.C.out = B.out.p + (size_t)p * FC_OUT_N;
  A.C.status = B.status.p + p;
  A.C.bar = B.bar.p + 2 * p;
  A.C.base = base;
  A.C.nb = nb;
}

static int batch_launch(fc_ctx* ctx, BatchDev& B, const void* fn, void** args, size_t smem) {
  if (smem > 48 * 1024)
    FC_CUDA_TRY(ctx, cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int nb = 0;
  FC_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, FC_SWEEP_BLOCK, smem));
  if (nb < 1 || B.nblocks > nb * std::max(1, ctx->num_sms))
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "batch: the groups need more blocks than the GPU holds resident");
  FC_CUDA_TRY(ctx, cudaMemsetAsync(B.bar.p, 0, B.bar.bytes(), ctx->stream));
  FC_CUDA_TRY(ctx, cudaMemsetAsync(B.status.p, 0, B.status.bytes(), ctx->stream));
  cudaError_t e = cudaLaunchCooperativeKernel(fn, dim3(B.nblocks), dim3(FC_SWEEP_BLOCK), args, smem, ctx->stream);
  if (e != cudaSuccess) return fc_fail(ctx, FC_ERR_CUDA, "batched cooperative launch", e);
  ctx->kernel_launches++;
  return FC_OK;
}

static int batch_fetch(fc_ctx* ctx, BatchDev& B) {
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(B.h_out, B.out.p, B.out.bytes(), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(B.h_status, B.status.p, B.status.bytes(), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FC_OK;
}

static int batch_put_ctl(fc_ctx* ctx, BatchDev& B) {
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(B.ctl.p, B.h_ctl, B.ctl.bytes(), cudaMemcpyHostToDevice, ctx->stream));
  return FC_OK;
}

template <class T>
static size_t batch_smem(const std::vector<BatchItem>& items) {
  size_t m = 0;
  for (const BatchItem& it : items) {
    const DevOrdered& D = it.s->ord;
    m = std::max(m, osweep_smem_bytes<T>(D.R, D.stage_area, D.maxW, D.max_tile_steps));
  }
  return m;
}

// some problem of the batch has steps wider than its stage buffers hold
static bool batch_wide(const std::vector<BatchItem>& items) {
  for (const BatchItem& it : items)
    if (it.s->ord.Wc > 0) return true;
  return false;
}

int batch_solve(fc_ctx* ctx, BatchDev*& dev, std::vector<BatchItem>& items, const char* solver_c, int itr_max,
                double tol_abs, double tol_rel) {
  const std::string solver(solver_c ? solver_c : "");
  if (solver != "bicgstab") return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "batch: solver must be bicgstab");
  const int np = (int)items.size();
  if (np == 0) return FC_OK;
  for (BatchItem& it : items) {
    it.res = SolveResult();
    it.dev_ms = 0.0;
    if (it.s->tslot_oob) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "bicgstab: pattern is not structurally symmetric");
  }
  if (!dev) dev = new BatchDev();
  BatchDev& B = *dev;
  int st = batch_prepare(ctx, B, items);
  if (st) return st;
  std::vector<int> base(np), nbk(np);
  for (int p = 0, acc = 0; p < np; ++p) { base[p] = acc; nbk[p] = items[p].s->ord.ntiles; acc += nbk[p]; }
  const bool mixed = ctx->precision == FC_PREC_MIXED;
  FC_CUDA_TRY(ctx, cudaMemsetAsync(B.out.p, 0, B.out.bytes(), ctx->stream));

  if (!mixed) {
    std::vector<KArgs<double>> h(np);
    for (int p = 0; p < np; ++p) {
      CsrSystem* s = items[p].s;
      h[p] = make_args<double>(s, items[p].a, items[p].x, items[p].b, s->r.p, s->r0.p, s->p.p, s->u.p, s->z.p, s->v.p,
                               s->d.p, s->w.p, itr_max, tol_abs, tol_rel);
      batch_ctl(h[p], B, p, base[p], nbk[p]);
      B.h_ctl[p] = BatchCtl{1, 0, itr_max, 0, 0, {0, 0, 0}};
    }
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(B.a64.p, h.data(), np * sizeof(KArgs<double>), cudaMemcpyHostToDevice, ctx->stream));
    if ((st = batch_put_ctl(ctx, B))) return st;
    KArgs<double>* pa = B.a64.p;
    int* pb = B.bprob.p;
    BatchCtl* pc = B.ctl.p;
    void* args[3] = {&pa, &pb, &pc};
    const void* fn64 = batch_wide(items) ? (const void*)k_bicgstab_batch<double, true>
                                         : (const void*)k_bicgstab_batch<double>;
    if ((st = batch_launch(ctx, B, fn64, args, batch_smem<double>(items)))) return st;
    if ((st = batch_fetch(ctx, B))) return st;
    for (int p = 0; p < np; ++p) {
      const double* o = B.h_out + (size_t)p * FC_OUT_N;
      SolveResult& r = items[p].res;
      r.res0 = o[FC_OUT_RES0]; r.resl = o[FC_OUT_RESL]; r.factor = o[FC_OUT_FACTOR]; r.resor = o[FC_OUT_RESOR];
      r.itr_used = (int)o[FC_OUT_ITR]; r.early = (int)o[FC_OUT_EARLY]; r.status = B.h_status[p];
      items[p].dev_ms = o[FC_OUT_GT] * 1e-6;
    }
  } else {
    // FP32 inner solves inside FP64 refinement, the arithmetic of
    // solve_mixed per problem; the refinement steps of all problems that
    // still run are one launch, their inner solves the next
    std::vector<KArgs<double>> hr(np);
    std::vector<KArgs<float>> hf(np);
    std::vector<BatchMix> hm(np);
    const double inner_tol = ctx->inner_tol > 0 ? ctx->inner_tol : 1e-4;
    const int inner_itmax = ctx->inner_itmax > 0 ? ctx->inner_itmax : std::max(itr_max, 1);
    for (int p = 0; p < np; ++p) {
      CsrSystem* s = items[p].s;
      if ((st = alloc_work32(ctx, s))) return st;
      hr[p] = make_args<double>(s, items[p].a, items[p].x, items[p].b, s->r.p, s->r0.p, s->p.p, s->u.p, s->z.p,
                                s->v.p, s->d.p, s->w.p, 0, tol_abs, tol_rel);
      batch_ctl(hr[p], B, p, base[p], nbk[p]);
      hf[p] = make_args<float>(s, s->a32.p, s->fx.p, s->fr0.p, s->fr.p, s->fy.p, s->fp.p, s->fu.p, s->fz.p, s->fv.p,
                               s->fd.p, s->fw.p, 0, 0.0, inner_tol);
      hf[p].stall_window = FC_INNER_STALL_WINDOW;
      batch_ctl(hf[p], B, p, base[p], nbk[p]);
      hm[p] = BatchMix{s->fx.p, s->fr0.p, s->a32.p, s->nnz, 0};
    }
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(B.ar.p, hr.data(), np * sizeof(KArgs<double>), cudaMemcpyHostToDevice, ctx->stream));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(B.af.p, hf.data(), np * sizeof(KArgs<float>), cudaMemcpyHostToDevice, ctx->stream));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(B.mix.p, hm.data(), np * sizeof(BatchMix), cudaMemcpyHostToDevice, ctx->stream));
    struct PState { bool first = true, done = false, inner = false; int outer = 0, total = 0; double res0 = 0, resl = 0, factor = 0; };
    std::vector<PState> ps(np);
    const int max_outer = 64;
    const size_t smemf = batch_smem<float>(items);
    KArgs<double>* pr = B.ar.p;
    KArgs<float>* pf = B.af.p;
    int* pb = B.bprob.p;
    BatchCtl* pc = B.ctl.p;
    BatchMix* pm = B.mix.p;
    for (;;) {
      // refinement step of every problem that is not done
      int nact = 0;
      for (int p = 0; p < np; ++p) {
        const PState& q = ps[p];
        B.h_ctl[p] = BatchCtl{q.done ? 0 : 1, 0, 0, q.outer > 0 ? 1 : 0, q.first ? 1 : 0, {0, 0, 0}};
        nact += q.done ? 0 : 1;
      }
      if (!nact) break;
      if ((st = batch_put_ctl(ctx, B))) return st;
      void* ra[4] = {&pr, &pb, &pc, &pm};
      if ((st = batch_launch(ctx, B, (const void*)k_refine_batch, ra, 0))) return st;
      if ((st = batch_fetch(ctx, B))) return st;
      int ninner = 0;
      for (int p = 0; p < np; ++p) {
        PState& q = ps[p];
        q.inner = false;
        if (q.done) continue;
        SolveResult& r = items[p].res;
        const double* o = B.h_out + (size_t)p * FC_OUT_N;
        items[p].dev_ms += o[FC_OUT_GT] * 1e-6;
        if (B.h_status[p]) { r.status = B.h_status[p]; q.done = true; continue; }
        q.resl = o[FC_OUT_RESL];
        if (q.first) {
          q.res0 = q.resl;
          q.first = false;
          if (q.res0 < tol_abs) { r.res0 = q.res0; r.resl = q.res0; r.early = 1; r.itr_used = 0; q.done = true; continue; }
        } else if (q.outer == 1) {
          q.factor = o[FC_OUT_FACTOR] + FC_SMALL;
        }
        bool stop = false;
        if (!std::isfinite(q.resl)) { r.status = FC_ERR_NAN; stop = true; }
        else if (q.outer > 0 && (q.resl / (q.res0 + FC_SMALL) < tol_rel || q.resl < tol_abs)) stop = true;
        else if (q.outer >= max_outer || q.total >= itr_max) { r.status = FC_WARN_MAXITER; stop = true; }
        if (stop) {
          q.done = true;
          r.res0 = q.res0; r.resl = q.resl; r.factor = q.factor; r.resor = q.factor > 0 ? q.res0 / q.factor : 0.0;
          r.itr_used = q.total; r.outer = q.outer;
          continue;
        }
        q.inner = true;
        ++ninner;
      }
      if (!ninner) break;
      // inner FP32 solves of A dx = r from dx = 0
      for (int p = 0; p < np; ++p) {
        const PState& q = ps[p];
        B.h_ctl[p] = BatchCtl{q.inner ? 1 : 0, q.outer > 0 ? 1 : 0, std::min(inner_itmax, itr_max - q.total), 0, 0,
                              {0, 0, 0}};
      }
      if ((st = batch_put_ctl(ctx, B))) return st;
      void* fa[3] = {&pf, &pb, &pc};
      const void* fn32 = batch_wide(items) ? (const void*)k_bicgstab_batch<float, true>
                                           : (const void*)k_bicgstab_batch<float>;
      if ((st = batch_launch(ctx, B, fn32, fa, smemf))) return st;
      if ((st = batch_fetch(ctx, B))) return st;
      for (int p = 0; p < np; ++p) {
        PState& q = ps[p];
        if (!q.inner) continue;
        const double* o = B.h_out + (size_t)p * FC_OUT_N;
        items[p].dev_ms += o[FC_OUT_GT] * 1e-6;
        if (B.h_status[p]) { items[p].res.status = B.h_status[p]; q.done = true; continue; }
        q.total += (int)o[FC_OUT_ITR];
        ++q.outer;
      }
    }
  }
  for (BatchItem& it : items) {
    SolveResult& r = it.res;
    if (r.status == 0 && !r.early && r.itr_used >= itr_max && itr_max > 0 &&
        !(r.resl / (r.res0 + FC_SMALL) < tol_rel || r.resl < tol_abs))
      r.status = FC_WARN_MAXITER;
  }
  return FC_OK;
}

// ------------------------------------------------- preconditioner entry points
int sys_precond(fc_ctx* ctx, CsrSystem* s, int dilu, const double* q, double* z_out, double* d_out, int apply) {
  KArgs<double> A = make_args<double>(s, s->a.p, s->x.p, q, s->r.p, s->r0.p, s->p.p, s->u.p, s->z.p, s->v.p, s->d.p,
                                      s->w.p, 0, 0.0, 0.0);
  void* extra[1] = {&apply};
  const bool wide = s->ord.Wc > 0;
  const void* fn = dilu ? (wide ? (const void*)k_precond<double, true, true> : (const void*)k_precond<double, true>)
                        : (wide ? (const void*)k_precond<double, false, true> : (const void*)k_precond<double, false>);
  int st = launch_coop(ctx, s, fn, A, extra, 1);
  if (st) return st;
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->h_status, s->status.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  if (d_out) FC_CUDA_TRY(ctx, cudaMemcpyAsync(d_out, s->v.p, s->n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
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
// non-null it receives the stamps as [2][B][K][FC_TRACE_STAMPS] (see Tracer).
extern "C" int fc_trace_get(fc_ctx* ctx, double* out, unsigned long long* timeline) {
  if (!ctx || !out) return FC_ERR_BAD_INPUT;
  if (!ctx->trace.p) return fc_fail_msg(ctx, FC_ERR_STATE, "no trace recorded");
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const int nb = ctx->trace_blocks, cap = ctx->trace_cap;
  std::vector<unsigned long long> h(ctx->trace.n);
  FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, h.data(), ctx->trace.p, h.size() * sizeof(unsigned long long)));
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
// (no cudaMalloc/cudaFree, no event or stream creation, no host heap).  It
// launches one block per SM as launch_coop does for fc_csrsolve("dpcg"), so
// the grid reductions, and with them the iterates, are the same.
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
  cudaStream_t st = (cudaStream_t)stream;
  if (st) {
    int sdev = -1;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess)
      return na_fail(errmsg, errlen, FC_ERR_BAD_INPUT, "stream is not a valid CUDA stream");
    if (sdev != dev)
      return na_fail(errmsg, errlen, FC_ERR_BAD_INPUT,
                     "stream belongs to another device than the current one (make its device current)");
  }
  for (const void* ptr : {(const void*)ia, (const void*)ja, (const void*)a, (const void*)diag, (const void*)x,
                          (const void*)b}) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, ptr) != cudaSuccess) { cudaGetLastError(); continue; }
    if (at.type == cudaMemoryTypeDevice && at.device != dev)
      return na_fail(errmsg, errlen, FC_ERR_BAD_INPUT, "arrays must be memory of the current device");
  }
  {
    int ends[2] = {-1, -1};
    if (cudaMemcpyAsync(ends, ia, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(ends + 1, ia + n, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
      return na_fail(errmsg, errlen, FC_ERR_CUDA, "reading ia[0] and ia[n] failed");
    if (ends[0] != 0 || ends[1] != nnz)
      return na_fail(errmsg, errlen, FC_ERR_BAD_INPUT, "ia must be 0-based with ia[0] == 0 and ia[n] == nnz");
  }
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
  // one block per SM, the grid of fc_csrsolve's launch
  const int blocks = std::max(1, std::min(NA_MAX_BLOCKS, sms));

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
