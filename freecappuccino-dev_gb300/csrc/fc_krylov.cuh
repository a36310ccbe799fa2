// Device building blocks of the persistent Krylov kernels: a bounded grid
// barrier, deterministic grid reductions, exact-rounding arithmetic, the
// sentinel used by the sweeps' value exchange and CSR row products.  The
// triangular sweeps themselves are in fc_sweep.cuh.  Kernels using these are launched cooperatively (one grid of
// co-resident blocks), so the barrier cannot deadlock; every wait is still
// bounded and reports FC_ERR_TIMEOUT instead of hanging.
//
// Memory rule inside these kernels: immutable inputs (ia, ja, a, level
// lists) go through the read-only path; vectors written during the kernel by
// other blocks are read with ld.global.cg (L2, coherent across SMs).
#pragma once
#include <cuda_runtime.h>

#include "fc_internal.hpp"

#define FC_BLOCK 512
// block of the kernels with ordered sweeps: 15 compute warps + 1 staging warp
#define FC_SWEEP_BLOCK 512
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

// Block index, block count and grid-stride start/step within the group of
// blocks the kernel runs on (the launch grid unless GridCtl names a group).
__device__ __forceinline__ int vg_bid(const GridCtl& C) { return (int)blockIdx.x - C.base; }
__device__ __forceinline__ int vg_nb(const GridCtl& C) { return C.nb > 0 ? C.nb : (int)gridDim.x; }
__device__ __forceinline__ int vg_gt(const GridCtl& C) { return vg_bid(C) * (int)blockDim.x + (int)threadIdx.x; }
__device__ __forceinline__ int vg_G(const GridCtl& C) { return vg_nb(C) * (int)blockDim.x; }

// Generation barrier over all blocks of the (cooperative) grid or group.  Returns
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
    if (arrived == (unsigned)vg_nb(C) - 1u) {
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
  const int nb = vg_nb(C), bid = vg_bid(C);
  double* part = C.part + (size_t)(ph & 1) * FC_NPART * nb;
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
      if (lane == 0) part[j * nb + bid] = s;
    }
  }
  if (!grid_sync(C)) return false;
  if (wid == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double s = 0.0;
      for (int b = lane; b < nb; b += 32) s += __ldcg(part + j * nb + b);
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

// Original-order CSR view (DPCG, residuals, the ILU(0) kernels of GMRES)
template <class T>
struct CsrView {
  int n;
  const int* __restrict__ ia;
  const int* __restrict__ ja;
  const int* __restrict__ dg;
  const int* __restrict__ ts;    // transpose slot (DILU)
  const T* __restrict__ a;
  const int* __restrict__ lfp;   // level sets (used by the ILU(0) kernels)
  const int* __restrict__ lfr;
  int nlf;
  const int* __restrict__ lbp;
  const int* __restrict__ lbr;
  int nlb;
};

// Exchange slots of the sweeps start filled with a sentinel NaN (a payload no
// arithmetic produces); a value pushed by another tile is read by polling the
// slot until the sentinel is gone.  A 64-bit (32-bit) store is single-copy
// atomic, so the reader sees either the sentinel or the final value and no
// fence or progress flag is needed between tiles.
template <class T> struct Sentinel;
template <> struct Sentinel<double> {
  static __device__ __forceinline__ double value() { return __longlong_as_double(0x7FF4DEADBEEF0001LL); }
  static __device__ __forceinline__ bool is(double v) { return __double_as_longlong(v) == 0x7FF4DEADBEEF0001LL; }
  static __device__ __forceinline__ double poll(const double* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return __longlong_as_double((long long)v);
  }
};
template <> struct Sentinel<float> {
  static __device__ __forceinline__ float value() { return __int_as_float(0x7FA5DEAD); }
  static __device__ __forceinline__ bool is(float v) { return __float_as_int(v) == 0x7FA5DEAD; }
  static __device__ __forceinline__ float poll(const float* p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return __int_as_float((int)v);
  }
};

// Cycle tracing hooks (no-ops unless a kernel is instantiated with a real
// tracer): mark(phase) closes a phase, sweep() opens a sweep, step(k) stamps
// the start of the tile's k-th step.
struct NoTrace {
  __device__ __forceinline__ void mark(int) {}
  __device__ __forceinline__ void sweep() {}
  __device__ __forceinline__ void step(int) {}
  __device__ __forceinline__ void waited(int) {}
  __device__ __forceinline__ void staged(int) {}
  template <class V> __device__ __forceinline__ void at(int, int, V) {}
};

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
