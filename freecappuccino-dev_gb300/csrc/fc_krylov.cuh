// Device building blocks of the persistent Krylov kernels: a bounded grid
// barrier, deterministic grid reductions, level-scheduled DIC/DILU setup and
// triangular sweeps (linear_solvers.f90:439-475, :613-683) and CSR row
// products.  Kernels using these are launched cooperatively (one grid of
// co-resident blocks), so the barrier cannot deadlock; every wait is still
// bounded and reports FC_ERR_TIMEOUT instead of hanging.
//
// Memory rule inside these kernels: immutable inputs (ia, ja, a, level
// lists) go through the read-only path; vectors written during the kernel by
// other blocks are read with ld.global.cg (L2, coherent across SMs).
#pragma once
#include <cuda_runtime.h>

#include "fc_internal.hpp"

#define FC_BLOCK 256
#define FC_SPIN_LIMIT (1u << 24)

namespace fcdev {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acqrel_u32(unsigned* p, unsigned v) {
  unsigned old;
  asm volatile("atom.add.acq_rel.gpu.global.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
  return old;
}

template <class T> __device__ __forceinline__ T ldcg(const T* p) { return __ldcg(p); }

// Generation barrier over all blocks of the (cooperative) grid.  Returns
// false if the wait ran out or another block already failed; the caller then
// leaves the kernel.
__device__ __forceinline__ bool grid_sync(const GridCtl& C) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    __threadfence();
    unsigned gen = ld_acquire_u32(C.bar + 1);
    unsigned arrived = atom_add_acqrel_u32(C.bar, 1u);
    if (arrived == gridDim.x - 1) {
      atomicExch(C.bar, 0u);
      st_release_u32(C.bar + 1, gen + 1u);
    } else {
      unsigned spins = 0;
      while (ld_acquire_u32(C.bar + 1) == gen) {
        if (++spins > FC_SPIN_LIMIT || *((volatile int*)C.status) != 0) {
          atomicCAS(C.status, 0, FC_ERR_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(32);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum NV values over the grid.  Deterministic: each block reduces in a fixed
// tree and writes one partial per value; after the barrier every block sums
// the partials in the same fixed order, so all blocks hold identical totals.
// Partials alternate between two slot sets (ph), so a block still reading
// the previous reduction never sees slots of the next one being rewritten.
template <int NV>
__device__ __forceinline__ bool grid_reduce(const GridCtl& C, int& ph, double (&v)[NV]) {
  __shared__ double sm[NV][FC_BLOCK / 32];
  __shared__ double tot[NV];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double* part = C.part + (size_t)(ph & 1) * FC_NPART * gridDim.x;
  ++ph;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double s = warp_sum(v[j]);
    if (lane == 0) sm[j][wid] = s;
  }
  __syncthreads();
  if (wid == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = lane < nw ? sm[j][lane] : 0.0;
      s = warp_sum(s);
      if (lane == 0) part[j * gridDim.x + blockIdx.x] = s;
    }
  }
  if (!grid_sync(C)) return false;
  if (wid == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0.0;
      for (int b = lane; b < (int)gridDim.x; b += 32) s += __ldcg(part + j * gridDim.x + b);
      s = warp_sum(s);
      if (lane == 0) tot[j] = s;
    }
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) v[j] = tot[j];
  return true;
}

// exact-rounding arithmetic for the recurrences (no FMA contraction), so the
// DIC/DILU factors and sweeps reproduce the reference bit for bit in FP64
template <class T> __device__ __forceinline__ T mul_rn(T a, T b);
template <class T> __device__ __forceinline__ T sub_rn(T a, T b);
template <class T> __device__ __forceinline__ T add_rn(T a, T b);
template <class T> __device__ __forceinline__ T div_rn(T a, T b);
template <> __device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ double sub_rn(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }
template <> __device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }

template <class T>
struct CsrView {
  int n;
  const int* __restrict__ ia;
  const int* __restrict__ ja;
  const int* __restrict__ dg;
  const int* __restrict__ ts;  // transpose slot (DILU)
  const T* __restrict__ a;
  const int* __restrict__ lfp;  // forward level pointers / rows
  const int* __restrict__ lfr;
  int nlf;
  const int* __restrict__ lbp;  // backward level pointers / rows
  const int* __restrict__ lbr;
  int nlb;
};

// d_i = a_ii - sum_{k<diag} a_k^2 d_j ; d_i = 1/d_i   (linear_solvers.f90:439-445)
// dilu: d_i = a_ii - sum_{k<diag} a_k d_j a_(j,i) ; d_i = 1/d_i   (:613-624)
template <class T, bool DILU>
__device__ bool precond_setup(const GridCtl& C, const CsrView<T>& S, T* d) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  for (int l = 0; l < S.nlf; ++l) {
    const int b = __ldg(S.lfp + l), e = __ldg(S.lfp + l + 1);
    for (int idx = b + gt; idx < e; idx += G) {
      const int i = __ldg(S.lfr + idx);
      const int k0 = __ldg(S.ia + i), kd = __ldg(S.dg + i);
      T di = __ldg(S.a + kd);
      for (int k = k0; k < kd; ++k) {
        const int j = __ldg(S.ja + k);
        const T ak = __ldg(S.a + k);
        if (DILU) di = sub_rn(di, mul_rn(mul_rn(ak, ldcg(d + j)), __ldg(S.a + __ldg(S.ts + k))));
        else di = sub_rn(di, mul_rn(mul_rn(ak, ak), ldcg(d + j)));
      }
      d[i] = div_rn(T(1), di);
    }
    if (!grid_sync(C)) return false;
  }
  return true;
}

// ILU-type application z = M^-1 q with M = (D'+L) D'^-1 (D'+U), D' = 1/d:
//   forward  z_i = (q_i - sum_{k<diag} a_k z_j) * d_i
//   scale    z_i = z_i / (d_i + small)
//   backward z_i = (z_i - sum_{k>diag} a_k z_j) * d_i
// pre(i) runs on the thread that owns row i in its forward level and returns
// q_i (callers fuse their vector update for row i there); post(i, z_i) runs
// after the final backward value of row i is stored.  The last backward
// level ends with a barrier only if last_sync.
template <class T, class PreF, class PostF>
__device__ bool precond_apply(const GridCtl& C, const CsrView<T>& S, const T* d, T* z, PreF pre, PostF post,
                              bool last_sync) {
  const int gt = blockIdx.x * blockDim.x + threadIdx.x, G = gridDim.x * blockDim.x;
  const T small = T(FC_SMALL);
  for (int l = 0; l < S.nlf; ++l) {
    const int b = __ldg(S.lfp + l), e = __ldg(S.lfp + l + 1);
    for (int idx = b + gt; idx < e; idx += G) {
      const int i = __ldg(S.lfr + idx);
      const int k0 = __ldg(S.ia + i), kd = __ldg(S.dg + i);
      T zi = pre(i);
      for (int k = k0; k < kd; ++k) zi = sub_rn(zi, mul_rn(__ldg(S.a + k), ldcg(z + __ldg(S.ja + k))));
      z[i] = mul_rn(zi, ldcg(d + i));
    }
    if (!grid_sync(C)) return false;
  }
  for (int l = 0; l < S.nlb; ++l) {
    const int b = __ldg(S.lbp + l), e = __ldg(S.lbp + l + 1);
    for (int idx = b + gt; idx < e; idx += G) {
      const int i = __ldg(S.lbr + idx);
      const int kd = __ldg(S.dg + i), k1 = __ldg(S.ia + i + 1);
      const T di = ldcg(d + i);
      T zi = div_rn(ldcg(z + i), add_rn(di, small));
      for (int k = kd + 1; k < k1; ++k) zi = sub_rn(zi, mul_rn(__ldg(S.a + k), ldcg(z + __ldg(S.ja + k))));
      zi = mul_rn(zi, di);
      z[i] = zi;
      post(i, zi);
    }
    if (l + 1 < S.nlb || last_sync)
      if (!grid_sync(C)) return false;
  }
  return true;
}

// sum_k a_k x_j over row i (FMA accumulation, CSR order)
template <class T>
__device__ __forceinline__ T row_dot(const CsrView<T>& S, const T* x, int i) {
  const int k0 = __ldg(S.ia + i), k1 = __ldg(S.ia + i + 1);
  T s = T(0);
  for (int k = k0; k < k1; ++k) s = fma(__ldg(S.a + k), ldcg(x + __ldg(S.ja + k)), s);
  return s;
}

// rhs_i - sum_k a_k x_j over row i (the reference's residual loop order)
template <class T>
__device__ __forceinline__ T row_residual(const CsrView<T>& S, const T* x, T bi, int i) {
  const int k0 = __ldg(S.ia + i), k1 = __ldg(S.ia + i + 1);
  T s = bi;
  for (int k = k0; k < k1; ++k) s = fma(-__ldg(S.a + k), ldcg(x + __ldg(S.ja + k)), s);
  return s;
}

}  // namespace fcdev
