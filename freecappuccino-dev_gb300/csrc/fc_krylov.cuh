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

#define FC_BLOCK 512
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

// Device view of a tiled sweep schedule (fc_schedule.hpp): tile t = block t
// walks its steps (levels) in order.
struct TileSched {
  int ntiles, nlev, R, max_slots;
  const int* __restrict__ tile_step_ptr;
  const int* __restrict__ step_level;
  const int* __restrict__ tile_slots;
  const int* __restrict__ step_row_ptr;
  const int* __restrict__ rows;
  const int* __restrict__ kbne;   // per slot: first swept CSR entry << 4 | entries (15 = 15 or more)
};

// Row data of one slot of a step, loaded a step ahead: the row, its swept
// entries' coefficients and dependency codes (the first FC_PF of them).
#define FC_PF 4
// 1: also read the dependency values produced in other tiles a step early
#define FC_PF_DEPS 1
template <class T>
struct RowIn {
  int i, kb, ne;
  T a[FC_PF];
  int c[FC_PF];
  T g[FC_PF];  // global dependency values read a step early (sentinel if not yet produced)
  T q, d;      // row scalars prepared by the sweep's prefetch functor
};

template <class T>
struct CsrView {
  int n;
  const int* __restrict__ ia;
  const int* __restrict__ ja;
  const int* __restrict__ dg;
  const int* __restrict__ ts;    // transpose slot (DILU)
  const int* __restrict__ code;  // per entry: ring index or -(row)-2 (see fc_schedule.hpp)
  const T* __restrict__ a;
  TileSched F, B;                // forward (lower) and backward (upper) sweeps
  const int* __restrict__ lfp;   // level sets (used by the ILU(0) kernels)
  const int* __restrict__ lfr;
  int nlf;
  const int* __restrict__ lbp;
  const int* __restrict__ lbr;
  int nlb;
};

// Shared-memory context of the sweeps of one kernel: the value ring and a
// block-wide abort flag (set when a bounded wait ran out).
struct SweepCtx {
  void* ring;
  int* abort_flag;
};

// carve the dynamic shared memory of a sweep kernel and clear it
template <class T>
__device__ __forceinline__ SweepCtx sweep_ctx(const CsrView<T>& S, unsigned char* smem) {
  SweepCtx X;
  const int rmax = max(S.F.R * S.F.max_slots, S.B.R * S.B.max_slots);
  size_t off = ((size_t)rmax * sizeof(T) + 15) & ~(size_t)15;
  X.ring = smem;
  X.abort_flag = (int*)(smem + off);
  if (threadIdx.x == 0) *X.abort_flag = 0;
  __syncthreads();
  return X;
}

template <class T>
size_t sweep_smem_bytes(int F_R, int F_slots, int B_R, int B_slots) {
  const int rmax = F_R * F_slots > B_R * B_slots ? F_R * F_slots : B_R * B_slots;
  return (((size_t)rmax * sizeof(T) + 15) & ~(size_t)15) + 16;
}

// Sweep outputs start filled with a sentinel NaN (a payload no arithmetic
// produces); a row published by another tile is read by polling its value
// until the sentinel is gone.  A 64-bit (32-bit) store is single-copy atomic,
// so the reader sees either the sentinel or the final value and no fence or
// progress flag is needed between tiles.
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
};

// value of the dependency of CSR entry k: from the ring when it was produced
// in this tile within the last R steps, else from global memory, polled until
// its producer has stored it (bounded; on timeout the kernel reports
// FC_ERR_TIMEOUT and the sweep is abandoned)
template <class T>
__device__ __forceinline__ T dep_value(const int* __restrict__ code, int k, const T* ring, const T* z, int* abort_flag,
                                       const GridCtl& C) {
  const int c = __ldg(code + k);
  if (c >= 0) return ring[c];
  const T* p = z + (-c - 2);
  T v = Sentinel<T>::poll(p);
  if (Sentinel<T>::is(v)) {
    unsigned spins = 0;
    do {
      if (++spins > FC_SPIN_LIMIT || *((volatile int*)C.status) != 0) {
        atomicCAS(C.status, 0, FC_ERR_TIMEOUT);
        *abort_flag = 1;
        return T(0);
      }
      __nanosleep(16);
      v = Sentinel<T>::poll(p);
    } while (Sentinel<T>::is(v));
  }
  return v;
}

template <class T>
__device__ __forceinline__ void load_row(RowIn<T>& r, const TileSched& TS, const T* __restrict__ aval,
                                         const int* __restrict__ code, const T* z, int q) {
  r.i = __ldg(TS.rows + q);
  const int pk = __ldg(TS.kbne + q);
  r.kb = pk >> 4;
  r.ne = pk & 15;
#pragma unroll
  for (int e = 0; e < FC_PF; ++e) {
    if (e < r.ne) {
      r.a[e] = __ldg(aval + r.kb + e);
      r.c[e] = __ldg(code + r.kb + e);
      r.g[e] = (FC_PF_DEPS && r.c[e] < 0) ? Sentinel<T>::poll(z + (-r.c[e] - 2)) : Sentinel<T>::value();
    } else {
      r.a[e] = T(0); r.c[e] = 0; r.g[e] = T(0);
    }
  }
}

// entry count of a row with more than 14 swept entries (rare; only then is
// the CSR row end read)
template <class T>
__device__ __forceinline__ int row_entries(const RowIn<T>& r, const int* __restrict__ ia, const int* __restrict__ dg,
                                           bool lower) {
  if (r.ne < 15) return r.ne;
  return lower ? __ldg(dg + r.i) - r.kb : __ldg(ia + r.i + 1) - r.kb;
}

// One sweep over a tiled schedule: the block of tile t walks the tile's
// steps (levels) in order.  Software pipelined: while step s computes, the
// rows of step s+1 are loaded (coefficients, dependency codes, dependency
// values produced in other tiles if already there) and pre(row) prepares
// the row's own scalars (row.q, row.d) -- pre may also update vectors at
// the row, since only the row's own thread touches them.  rowf(row) then
// needs only shared-memory ring values, the prefetched values and, for a
// dependency not yet produced, a bounded poll.  The value goes to out[i] and
// to the ring; a block barrier separates steps.  out[] (and the dependency
// array) must hold the sentinel where not yet produced.
template <class T, class PreF, class RowF, class TracerT = NoTrace>
__device__ bool tile_sweep(const GridCtl& C, const TileSched& TS, const T* __restrict__ aval,
                           const int* __restrict__ code, const T* zdep, T* ring, int* abort_flag, T* out, PreF pre,
                           RowF rowf, TracerT* tr = nullptr) {
  if (tr) tr->sweep();
  const int tile = blockIdx.x;
  if (tile >= TS.ntiles) return true;
  const int s0 = __ldg(TS.tile_step_ptr + tile), s1 = __ldg(TS.tile_step_ptr + tile + 1);
  if (s0 >= s1) return true;
  const int slots = __ldg(TS.tile_slots + tile);
  const int qbase = __ldg(TS.step_row_ptr + s0);
  if (slots <= (int)blockDim.x) {
    // one slot per thread
    const int sl = threadIdx.x;
    const bool act = sl < slots;
    RowIn<T> nxt;
    nxt.i = -1;
    if (act) {
      load_row(nxt, TS, aval, code, zdep, qbase + sl);
      if (nxt.i >= 0) pre(nxt);
    }
    for (int gs = s0; gs < s1; ++gs) {
      if (tr) tr->step(gs - s0);
      const RowIn<T> cur = nxt;
      if (act && gs + 1 < s1) {
        load_row(nxt, TS, aval, code, zdep, qbase + (gs + 1 - s0) * slots + sl);
        if (nxt.i >= 0) pre(nxt);
      }
      if (act && cur.i >= 0) {
        const T v = rowf(cur);
        out[cur.i] = v;
        ring[((gs - s0) % TS.R) * slots + sl] = v;
      }
      __syncthreads();
      if (*((volatile int*)abort_flag)) return false;
    }
    if (tr) tr->step(s1 - s0);
  } else {
    for (int gs = s0; gs < s1; ++gs) {
      T* ring_cur = ring + ((gs - s0) % TS.R) * slots;
      for (int sl = threadIdx.x; sl < slots; sl += blockDim.x) {
        RowIn<T> cur;
        load_row(cur, TS, aval, code, zdep, qbase + (gs - s0) * slots + sl);
        if (cur.i >= 0) {
          pre(cur);
          const T v = rowf(cur);
          out[cur.i] = v;
          ring_cur[sl] = v;
        }
      }
      __syncthreads();
      if (*((volatile int*)abort_flag)) return false;
    }
  }
  return true;
}

// value of the e-th swept entry's dependency: ring, prefetched global value,
// or (not produced when prefetched) a bounded poll
template <class T>
__device__ __forceinline__ T entry_value(const RowIn<T>& r, int e, const int* __restrict__ code, const T* ring,
                                         const T* z, int* abort_flag, const GridCtl& C) {
  if (e < FC_PF) {
    const int c = r.c[e];
    if (c >= 0) return ring[c];
    if (!Sentinel<T>::is(r.g[e])) return r.g[e];
  }
  return dep_value(code, r.kb + e, ring, z, abort_flag, C);
}

// sum over the swept entries of a row of coefficient x dependency value,
// subtracted from acc (FMA), for the apply sweeps
template <class T>
__device__ __forceinline__ T sweep_dot(const RowIn<T>& r, int ne, const int* __restrict__ code,
                                       const T* __restrict__ aval, const T* ring, const T* z, int* abort_flag,
                                       const GridCtl& C, T acc) {
#pragma unroll
  for (int e = 0; e < FC_PF; ++e)
    if (e < ne) acc = fma(-r.a[e], entry_value(r, e, code, ring, z, abort_flag, C), acc);
  for (int e = FC_PF; e < ne; ++e)
    acc = fma(-__ldg(aval + r.kb + e), dep_value(code, r.kb + e, ring, z, abort_flag, C), acc);
  return acc;
}

// d_i = a_ii - sum_{k<diag} a_k^2 d_j ; d_i = 1/d_i   (linear_solvers.f90:439-445)
// dilu: d_i = a_ii - sum_{k<diag} a_k d_j a_(j,i) ; d_i = 1/d_i   (:613-624)
// exact rounding, ends with a grid barrier
template <class T, bool DILU>
__device__ bool precond_setup(const GridCtl& C, const CsrView<T>& S, SweepCtx& X, T* d) {
  T* ring = (T*)X.ring;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x) d[i] = Sentinel<T>::value();
  if (!grid_sync(C)) return false;
  auto pre = [&](RowIn<T>& r) { r.q = __ldg(S.a + r.kb + row_entries(r, S.ia, S.dg, true)); };  // a_ii
  auto rowf = [&](const RowIn<T>& r) {
    const int ne = row_entries(r, S.ia, S.dg, true);
    T di = r.q;
    for (int e = 0; e < ne; ++e) {
      const int k = r.kb + e;
      const T ak = e < FC_PF ? r.a[e] : __ldg(S.a + k);
      const T dj = entry_value(r, e, S.code, ring, (const T*)d, X.abort_flag, C);
      if (DILU) di = sub_rn(di, mul_rn(mul_rn(ak, dj), __ldg(S.a + __ldg(S.ts + k))));
      else di = sub_rn(di, mul_rn(mul_rn(ak, ak), dj));
    }
    return div_rn(T(1), di);
  };
  if (!tile_sweep(C, S.F, S.a, S.code, (const T*)d, ring, X.abort_flag, d, pre, rowf)) return false;
  return grid_sync(C);
}

// ILU-type application z = M^-1 q with M = (D'+L) D'^-1 (D'+U), D' = 1/d:
//   forward  y_i = (q_i - sum_{k<diag} a_k y_j) * d_i          (into yf)
//   scale    y_i = y_i / (d_i + small)
//   backward z_i = (y_i - sum_{k>diag} a_k z_j) * d_i          (into z)
// (linear_solvers.f90:458-475).  yf must hold the sentinel on entry (the
// forward sweep refills z with it row by row); on return yf holds the
// sentinel-free forward values and z the result.  pre(i) runs on the thread
// that owns row i in the forward sweep and returns q_i (callers fuse their
// vector update for row i there); post(i, z_i) runs after the final value.
// Grid barrier between the sweeps, and after the backward one if last_sync.
template <class T, class PreF, class PostF, class TracerT = NoTrace>
__device__ bool precond_apply(const GridCtl& C, const CsrView<T>& S, SweepCtx& X, const T* d, T* yf, T* z, PreF pre,
                              PostF post, bool last_sync, TracerT* tr = nullptr) {
  T* ring = (T*)X.ring;
  auto fpre = [&](RowIn<T>& r) {
    r.d = ldcg(d + r.i);
    r.q = pre(r.i);
    z[r.i] = Sentinel<T>::value();
  };
  auto fwd = [&](const RowIn<T>& r) {
    const T zi = sweep_dot(r, row_entries(r, S.ia, S.dg, true), S.code, S.a, ring, (const T*)yf, X.abort_flag, C, r.q);
    return zi * r.d;
  };
  if (!tile_sweep(C, S.F, S.a, S.code, (const T*)yf, ring, X.abort_flag, yf, fpre, fwd, tr)) return false;
  if (tr) tr->mark(1);
  if (!grid_sync(C)) return false;
  if (tr) tr->mark(2);
  const T small = T(FC_SMALL);
  auto bpre = [&](RowIn<T>& r) {
    r.d = ldcg(d + r.i);
    r.q = ldcg(yf + r.i) / (r.d + small);
  };
  auto bwd = [&](const RowIn<T>& r) {
    T zi = sweep_dot(r, row_entries(r, S.ia, S.dg, false), S.code, S.a, ring, (const T*)z, X.abort_flag, C, r.q);
    zi = zi * r.d;
    post(r.i, zi);
    return zi;
  };
  if (!tile_sweep(C, S.B, S.a, S.code, (const T*)z, ring, X.abort_flag, z, bpre, bwd, tr)) return false;
  if (tr) tr->mark(3);
  if (last_sync) return grid_sync(C);
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
