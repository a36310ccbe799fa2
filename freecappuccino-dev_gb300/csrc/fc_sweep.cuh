// Schedule-ordered triangular sweeps of the DIC/DILU preconditioners
// (linear_solvers.f90:439-475, :613-683) and of Gauss-Seidel (:96-201).
//
// The system is renumbered in schedule order (fc_schedule.hpp): tile t is
// block t, and every step of a tile is a contiguous range of new rows.  The
// block is warp-specialised: the last warp stages, the others compute.
//
//  - stager (one thread): for each step, a handful of bulk asynchronous
//    copies (cp.async.bulk, the TMA engine) bring the step's packed row
//    records (16 bytes per row: entry count, push count, offsets, ring
//    codes), its coefficient records (coefficients, d_i, 1/(d_i + small)),
//    the right-hand-side window and the step's exchange and push blocks into
//    a K-deep shared-memory ring of stage buffers, up to K-1 steps ahead.
//    Buffer b is handed over with two mbarriers: full[b] (copies landed) and
//    empty[b] (the compute warps are done with it).
//  - compute warps (one row per thread): wait full[b], read the step from
//    shared memory, take dependencies from the value ring (produced in this
//    tile within the last R-1 steps) or from the exchange block, run the
//    short FMA chain, store the value (vector, ring, pushes to consumers in
//    other tiles or far behind in this one), then a named barrier among the
//    compute warps and release of buffer b.
//
// Exchange: a value a row needs from another tile (or from more than R-1
// steps back) is pushed by its producer into the consumer's slot of the
// exchange array xv, whose slots start every sweep at a sentinel NaN.  The
// static data of a step is staged many steps ahead, but exchanged values
// are not: a copy taken that early is stale, and every stale value costs
// the consumer an L2 round trip on its critical path and, through the lag
// it builds up, delays every tile downstream.  Instead each compute thread
// loads the exchanged values of its row of the next step from global memory
// while it works on the current one (relaxed loads through L2); a value
// that still reads as the sentinel is polled (bounded) until the producer's
// store arrives.  The consumer puts the sentinel back after use.  Bulk
// copies read through L2, so staged data is never an SM's stale L1 line.
#pragma once
#include <type_traits>
#include "fc_krylov.cuh"
#include "fc_schedule.hpp"

namespace fcdev {

// ------------------------------------------------- bulk copies, mbarriers
__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long* mb, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mb)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(unsigned long long* mb, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mb)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* mb, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(mb)), "r"(parity)
      : "memory");
  return ok != 0;
}
// global -> shared bulk copy of bytes (multiple of 16, both addresses
// 16-byte aligned), completion reported to mbarrier mb
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* mb) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(mb))
               : "memory");
}
#define FC_MAX_STAGES 16
#define FC_SMEM_HDR (2 * FC_MAX_STAGES * 8)  // full and empty mbarriers at the start of the dynamic area
#define FC_MBAR_SPIN_LIMIT (1u << 22)
__device__ __forceinline__ void mbar_arrive(unsigned long long* mb) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(mb)) : "memory");
}
// bounded wait for the completion of phase `parity`; false if it ran out.
// backoff_ns > 0 sleeps between polls (a thread that is expected to wait
// long, so that it does not load the shared-memory pipe of the workers)
__device__ __forceinline__ bool mbar_wait(unsigned long long* mb, unsigned parity, unsigned backoff_ns = 0) {
  unsigned spins = 0;
  while (!mbar_try_wait(mb, parity)) {
    if (++spins > FC_MBAR_SPIN_LIMIT) return false;
    if (backoff_ns) __nanosleep(backoff_ns);
  }
  return true;
}
// a hint to bring the line holding p into L2 (prefetch.global.L2)
__device__ __forceinline__ void l2_prefetch(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// barrier among the first nthreads threads (the compute warps)
__device__ __forceinline__ void bar_compute(int nthreads) {
  asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}
// record strides (elements of T) of the per-solve row records
template <class T> struct Rec { static constexpr int V = sizeof(T) == 8 ? 6 : 8; };

// ------------------------------------------------------------------ views
// device copy of an OrderedSweep (fc_schedule.hpp)
struct OrdView {
  int n, nE, ntiles, R, novf0, novf1, nsteps, maxW, xmax, pmax;
  int stage_area;                        // bytes of the stage area (multiple of 16)
  // rows of a step that are staged in shared memory: the rows of a wider
  // step past the first Wc read their records from global memory, and the
  // step's push block is read from global memory too (0: every step fits)
  int Wc;
  const int* __restrict__ tile_step_ptr;
  const int* __restrict__ step_ptr;
  const int* __restrict__ tile_W;
  const int* __restrict__ perm;
  const int4* __restrict__ srec[2];
  const int* __restrict__ xv_ptr[2];
  const int* __restrict__ push_ptr[2];
  const int* __restrict__ push[2];
  const int* __restrict__ slot[2];
  const int4* __restrict__ ucol;      // columns of the upper entries, 4 per row (Gauss-Seidel)
  const int* __restrict__ ovf_ptr[2];
  const int* __restrict__ ovf_code[2];
  const int* __restrict__ ovf_col[2];
  const int* __restrict__ ovf_slot[2];
  const int* __restrict__ lo_tslot;
  const int* __restrict__ lo_ovf_tslot;
  const int* __restrict__ dslot;
  const int* __restrict__ p_ptr;
  const int* __restrict__ p_col;
  const int* __restrict__ p_slot;
};

// per-solve values in the new numbering (gathered by the kernel from the
// caller's CSR values) and the exchange arrays; every vector of n rows is
// allocated with nE entries (the padding is read by the staging windows and
// never used)
template <class T>
struct OrdVals {
  T* vrec[2];  // [nE][Rec::V]: a_0..a_3 of the triangle, d_i, 1/(d_i + small)
  T* sx;       // [nE][Rec::V]: a_ii, then the DILU transposes a_(j,i) of entries 0..3
  T* aovf[2];  // coefficients of the overflow entries
  T* tovf;     // DILU transposes of the lower overflow entries
  T* adiag;    // [nE]
  T* ap;       // [nnz] matrix values in new row order (original entry order)
  T* xv[2];    // exchange arrays (per-step blocks)
};

// ------------------------------------------------------------------ modes
enum { OS_SETUP_DIC = 0, OS_SETUP_DILU, OS_FWD, OS_BWD, OS_BWD_DOT, OS_GS };

// ----------------------------------------------------------- staging area
// One stage buffer: the step's row records, coefficient records, setup
// records (a_ii and transposes), the Gauss-Seidel upper columns and
// coefficients, the q and e windows (rows widened to 16-byte bounds) and
// the exchange and push blocks.  init() lays out every area (the size the
// host reserves per stage); init_for() only the areas one sweep mode reads,
// so that the preconditioner applications, which need about 40% of a full
// buffer, fit more stages into the same shared memory.
struct StageLayout {
  int W, Wp;
  int oS, oV, oX2, oU, oV2, oQ, oE, oXV, oP, bytes;
  template <class T>
  __host__ __device__ void init(int w, int xmax, int pmax) { init_for<T>(w, xmax, pmax, -1); }
  template <class T>
  __host__ __device__ void init_for(int w, int xmax, int pmax, int mode) {
    const bool all = mode < 0;
    const bool setup = all || mode == OS_SETUP_DIC || mode == OS_SETUP_DILU;
    const bool gs = all || mode == OS_GS;
    const bool kq = all || !(mode == OS_SETUP_DIC || mode == OS_SETUP_DILU);
    const bool ke = all || mode == OS_BWD_DOT || mode == OS_GS;
    W = w;
    Wp = ((w + 3) & ~3) + 8;
    int o = 0;
    auto take = [&](bool used, int b) { const int r = o; if (used) o += (b + 15) & ~15; return r; };
    oS = take(true, 16 * W);
    oV = take(true, (int)sizeof(T) * Rec<T>::V * W);
    oX2 = take(setup || gs, (int)sizeof(T) * Rec<T>::V * W);
    oU = take(gs, 16 * W);
    oV2 = take(gs, (int)sizeof(T) * Rec<T>::V * W);
    oQ = take(kq, (int)sizeof(T) * Wp);
    oE = take(ke, (int)sizeof(T) * Wp);
    oXV = take(false, (int)sizeof(T) * xmax);  // exchanged values are not staged (see the file header)
    oP = take(true, 4 * pmax);
    bytes = o;
  }
};

// stage buffers of one mode within a stage area of `area` bytes: the largest
// power of two (at most FC_MAX_STAGES) whose buffers fit
__host__ __device__ inline int stages_in(size_t area, int buffer_bytes) {
  int K = 1;
  while (2 * K <= FC_MAX_STAGES && (size_t)(2 * K) * (size_t)buffer_bytes <= area) K *= 2;
  return K;
}

// dynamic shared memory of an ordered-sweep kernel: 2 FC_MAX_STAGES
// mbarriers, ring, the stage area (cut by every sweep mode into its own
// buffers), the tile's step tables (rows, exchange and push offsets of both
// directions) and the abort flag
template <class T>
inline size_t osweep_fixed_bytes(int R, int maxW, int max_tile_steps) {
  size_t ring = ((size_t)R * maxW * sizeof(T) + 15) & ~(size_t)15;
  size_t tab = ((size_t)5 * (max_tile_steps + 1) * 4 + 15) & ~(size_t)15;
  return FC_SMEM_HDR + ring + tab + 16;
}
template <class T>
inline size_t osweep_smem_bytes(int R, size_t stage_area, int maxW, int max_tile_steps) {
  return osweep_fixed_bytes<T>(R, maxW, max_tile_steps) + stage_area;
}

struct OsCtx {
  unsigned long long* full;   // [FC_MAX_STAGES]
  unsigned long long* empty;  // [FC_MAX_STAGES]
  unsigned char* ring;
  unsigned char* stage;       // the stage area, cut by each sweep mode into its buffers
  size_t stage_area;
  int* sp;                    // [ns+1] first row of each local step (ascending levels)
  int* xp[2];                 // [ns+1] exchange block offsets per direction
  int* pp[2];                 // [ns+1] push block offsets per direction
  int* abort_flag;
  // stage buffer b: bit b of `parity` = parity of its next fill/completion,
  // bit b of `used` = it has been filled before (registers, no runtime-
  // indexed arrays, so the context never goes to local memory)
  unsigned parity, used;
  StageLayout L;
};

template <class T>
__device__ __forceinline__ OsCtx osweep_ctx(const OrdView& O, unsigned char* smem, int t) {
  OsCtx X;
  const int W = t < O.ntiles ? __ldg(O.tile_W + t) : 1;
  X.L.template init<T>(W, O.xmax, O.pmax);
  // carve with this tile's width; the host sized the area for the widest
  X.full = (unsigned long long*)smem;
  X.empty = X.full + FC_MAX_STAGES;
  size_t off = FC_SMEM_HDR;
  X.ring = smem + off;
  off += ((size_t)O.R * W * sizeof(T) + 15) & ~(size_t)15;
  X.stage = smem + off;
  X.stage_area = (size_t)O.stage_area;
  off += X.stage_area;
  const int ns = t < O.ntiles ? __ldg(O.tile_step_ptr + t + 1) - __ldg(O.tile_step_ptr + t) : 0;
  int* tab = (int*)(smem + off);
  X.sp = tab;
  X.xp[0] = tab + (ns + 1);
  X.xp[1] = tab + 2 * (ns + 1);
  X.pp[0] = tab + 3 * (ns + 1);
  X.pp[1] = tab + 4 * (ns + 1);
  off += ((size_t)5 * (ns + 1) * 4 + 15) & ~(size_t)15;
  X.abort_flag = (int*)(smem + off);
  X.parity = 0;
  X.used = 0;
  if (t < O.ntiles) {
    const int s0 = __ldg(O.tile_step_ptr + t);
    for (int k = threadIdx.x; k <= ns; k += blockDim.x) {
      X.sp[k] = __ldg(O.step_ptr + s0 + k);
      X.xp[0][k] = __ldg(O.xv_ptr[0] + s0 + k);
      X.xp[1][k] = __ldg(O.xv_ptr[1] + s0 + k);
      X.pp[0][k] = __ldg(O.push_ptr[0] + s0 + k);
      X.pp[1][k] = __ldg(O.push_ptr[1] + s0 + k);
    }
  }
  if (threadIdx.x == 0) {
    *X.abort_flag = 0;
    for (int b = 0; b < FC_MAX_STAGES; ++b) {
      mbar_init(X.full + b, 1);
      mbar_init(X.empty + b, 1);
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  return X;
}


// Row sources of a sweep.  q: the right-hand side (forward, backward,
// Gauss-Seidel), e: an extra row value (the dot partner of OS_BWD_DOT, the
// previous iterate of Gauss-Seidel), out: where the row values go (the
// setups write d_i there and into the coefficient records).
template <class T>
struct OsIO {
  const T* q;
  const T* e;
  T* out;
};

// bounded poll of an exchange slot; on timeout the kernel's status becomes
// FC_ERR_TIMEOUT and the block's abort flag is raised
template <class T>
__device__ __noinline__ T xv_wait(const GridCtl& C, const T* p, int* abort_flag) {
  unsigned spins = 0;
  T v = Sentinel<T>::poll(p);
  while (Sentinel<T>::is(v)) {
    if (++spins > FC_SPIN_LIMIT || *((volatile int*)C.status) != 0) {
      atomicCAS(C.status, 0, FC_ERR_TIMEOUT);
      *((volatile int*)abort_flag) = 1;
      return T(0);
    }
    v = Sentinel<T>::poll(p);
  }
  return v;
}

// One ordered sweep of tile vg_bid(C).  WIDE: the structure has steps wider
// than the stage buffers hold (OrdView::Wc > 0), whose further rows read
// their records from global memory; without it the staged path is all there is.  dirn 0: forward over the lower
// triangle, 1: backward over the upper one.  red (MODE OS_BWD_DOT: red[0] +=
// e*value; OS_GS: red[0] += |residual|, red[1] += |a_ii x_i|) accumulates
// per thread.  Every thread of the block calls it; it ends with a block
// barrier but no grid barrier, and returns false if a wait ran out.
template <class T, int MODE, bool WIDE = false, class TracerT = NoTrace>
__device__ __forceinline__ bool osweep(const GridCtl& C, const OrdView& O, const OrdVals<T>& V, const OsIO<T>& io, OsCtx& X,
                       double* red, TracerT* tr = nullptr) {
  constexpr int dirn = (MODE == OS_BWD || MODE == OS_BWD_DOT) ? 1 : 0;
  constexpr bool kSetup = MODE == OS_SETUP_DIC || MODE == OS_SETUP_DILU;
  constexpr bool kQ = !kSetup;
  constexpr bool kE = MODE == OS_BWD_DOT || MODE == OS_GS;
  constexpr bool kGS = MODE == OS_GS;
  constexpr int VR = Rec<T>::V;
  if (tr) tr->sweep();
  const int t = vg_bid(C);
  if (t >= O.ntiles) return true;
  const int ns = __ldg(O.tile_step_ptr + t + 1) - __ldg(O.tile_step_ptr + t);
  // the areas this mode reads, as many stage buffers as the area holds
  // W: the tile's widest step (ring stride, compute threads); Ws: the rows of
  // a step the stage buffers hold
  const int W = X.L.W, Ws = WIDE && O.Wc > 0 ? min(W, O.Wc) : W;
  StageLayout L;
  L.template init_for<T>(Ws, O.xmax, O.pmax, MODE);
  const int K = stages_in(X.stage_area, L.bytes), R = O.R;
  const int nct = (int)blockDim.x - 32;  // threads before the staging warp
  // compute threads of this tile: whole warps covering its widest step
  const int ncg = min(nct, (W + 31) & ~31);
  T* ring = (T*)X.ring;
  T* xv = V.xv[dirn];
  const int* sp = X.sp;
  const int* xp = X.xp[dirn];
  const int* pp = X.pp[dirn];
  auto step_of = [&](int k) { return dirn ? ns - 1 - k : k; };

  if ((int)threadIdx.x >= nct) {
    // ------------------------------------------------------------ stager
    if (threadIdx.x == (unsigned)nct) {
      bool ok = true;
      for (int k = 0; k < ns && ok; ++k) {
        if (*((volatile int*)X.abort_flag)) break;
        const int b = k & (K - 1);
        // a timeout here only records the status: the compute warps then run
        // out of their own bounded wait and raise the abort flag themselves,
        // so that they all see it after the same named barrier
        // release of the previous fill of b: its completion had parity
        // (parity bit ^ 1)
        if (((X.used >> b) & 1u) && !mbar_wait(X.empty + b, ((X.parity >> b) & 1u) ^ 1u, 64)) {
          atomicCAS(C.status, 0, FC_ERR_TIMEOUT);
          ok = false;
          break;
        }
        if (tr) tr->staged(k);
        const int ls = step_of(k);
        const int base = sp[ls], cnt = WIDE ? min(sp[ls + 1] - base, Ws) : sp[ls + 1] - base;  // the staged rows
        const int b0 = base & ~3, nw = ((base + cnt + 3) & ~3) - b0;
        const int p0 = pp[ls], np = !WIDE || sp[ls + 1] - base <= Ws ? pp[ls + 1] - p0 : 0;
        unsigned char* B = X.stage + (size_t)b * L.bytes;
        unsigned long long* mb = X.full + b;
        const unsigned vb = (unsigned)(sizeof(T) * VR) * cnt;
        unsigned bytes = 16u * cnt + vb + 4u * np;
        if (kSetup || kGS) bytes += vb;
        if (kGS) bytes += 16u * cnt + vb;
        if (kQ) bytes += (unsigned)sizeof(T) * nw;
        if (kE) bytes += (unsigned)sizeof(T) * nw;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_tx(mb, bytes);
        bulk_g2s(B + L.oS, O.srec[dirn] + base, 16u * cnt, mb);
        bulk_g2s(B + L.oV, V.vrec[dirn] + (size_t)base * VR, vb, mb);
        if (kSetup || kGS) bulk_g2s(B + L.oX2, V.sx + (size_t)base * VR, vb, mb);
        if (kGS) {
          bulk_g2s(B + L.oU, O.ucol + base, 16u * cnt, mb);
          bulk_g2s(B + L.oV2, V.vrec[1] + (size_t)base * VR, vb, mb);
        }
        if (kQ) bulk_g2s(B + L.oQ, io.q + b0, (unsigned)sizeof(T) * nw, mb);
        if (kE) bulk_g2s(B + L.oE, io.e + b0, (unsigned)sizeof(T) * nw, mb);
        if (np) bulk_g2s(B + L.oP, O.push[dirn] + p0, 4u * np, mb);
        X.parity ^= 1u << b;
        X.used |= 1u << b;
      }
    }
  } else if ((int)threadIdx.x < ncg) {
    // ------------------------------------------------------------ compute
    // Only the ceil(W/32) warps that a step of this tile can occupy take
    // part; the others skip the sweep, so they add no shared-memory traffic
    // and no barrier arrivals to the steps.
    const int kmask = K - 1;  // K and R are powers of two
    // the exchanged values of this thread's first row of step k, loaded
    // during step k-1 (pf_ok), and whether step k's buffer was waited for then
    T pf[FC_ELL];
    bool pf_ok = false, pre_waited = false;
#pragma unroll
    for (int e = 0; e < FC_ELL; ++e) pf[e] = T(0);
    // wait for step kk's buffer (warps with rows in it) and load the
    // exchanged values of row threadIdx.x of that step into pf
    auto prefetch = [&](int kk) {
      const int lsk = step_of(kk);
      const int bk = kk & kmask, basek = sp[lsk], cntk = sp[lsk + 1] - basek;
      pf_ok = false;
      pre_waited = false;
      if ((int)(threadIdx.x & ~31u) >= cntk) return;
      if (!mbar_wait(X.full + bk, (X.parity >> bk) & 1u)) {
        atomicCAS(C.status, 0, FC_ERR_TIMEOUT);
        *((volatile int*)X.abort_flag) = 1;
      }
      pre_waited = true;
      if ((int)threadIdx.x >= cntk) return;
      const int4 sr = !WIDE || (int)threadIdx.x < Ws
                          ? ((const int4*)(X.stage + (size_t)bk * L.bytes + L.oS))[threadIdx.x]
                          : __ldg(O.srec[dirn] + basek + threadIdx.x);
      const int ne = sr.x & 255, xoff = (int)((unsigned)sr.x >> 16);
      const unsigned cw[2] = {(unsigned)sr.z, (unsigned)sr.w};
      const T* src = xv + xp[lsk] + xoff;
      int m = 0;
#pragma unroll
      for (int e = 0; e < FC_ELL; ++e) {
        const bool ex = ((cw[e >> 1] >> (16 * (e & 1))) & 0xFFFFu) == 0 && e < ne;
        pf[e] = ex ? Sentinel<T>::poll(src + m) : T(0);
        m += ex ? 1 : 0;
      }
      pf_ok = true;
    };
    if (ns > 0) prefetch(0);
    for (int k = 0; k < ns; ++k) {
      if (tr) tr->step(k);
      const int b = k & kmask;
      const int ls = step_of(k);
      const int base = sp[ls], cnt = sp[ls + 1] - base, woff = base - (base & ~3);
      // only warps with rows in this step read the buffer, so only they wait
      // for it (an mbarrier poll by every warp would serialise on its word)
      if (!pre_waited && (int)(threadIdx.x & ~31u) < cnt && !mbar_wait(X.full + b, (X.parity >> b) & 1u)) {
        atomicCAS(C.status, 0, FC_ERR_TIMEOUT);
        *((volatile int*)X.abort_flag) = 1;
      }
      if (tr) tr->waited(k);
      const bool have_pf = pf_ok;
      T pfk[FC_ELL];
#pragma unroll
      for (int e = 0; e < FC_ELL; ++e) pfk[e] = pf[e];
      // the next step's exchanged values are loaded while this one runs
      if (k + 1 < ns) prefetch(k + 1);
      else { pf_ok = false; pre_waited = false; }
      if constexpr (WIDE) {
        // the records of this thread's unstaged rows of the next step are
        // brought into L2 while this step runs (they are read through L2)
        if (k + 1 < ns) {
          const int lsn = step_of(k + 1), basen = sp[lsn], cntn = sp[lsn + 1] - basen;
          for (int sl = threadIdx.x; sl < cntn; sl += ncg) {
            if (sl < Ws) continue;
            const int qn = basen + sl;
            l2_prefetch(O.srec[dirn] + qn);
            l2_prefetch(V.vrec[dirn] + (size_t)qn * VR);
            l2_prefetch(V.vrec[dirn] + (size_t)qn * VR + VR - 1);
            if (kQ) l2_prefetch(io.q + qn);
            if (kE) l2_prefetch(io.e + qn);
          }
          // a wide step's push block, read from global memory, line by line
          if (cntn > Ws) {
            const int* pb = O.push[dirn] + pp[lsn];
            const int npn = pp[lsn + 1] - pp[lsn];
            for (int o = (int)threadIdx.x * 32; o < npn; o += ncg * 32) l2_prefetch(pb + o);
          }
        }
      }
      if (tr) tr->at(k, 4, (int)pf_ok);
      const int xbase = xp[ls];
      const unsigned char* B = X.stage + (size_t)b * L.bytes;
      const int4* S4 = (const int4*)(B + L.oS);
      const T* VRc = (const T*)(B + L.oV);
      // the push block: staged for a step the stage buffer holds whole, else
      // read from global memory
      const int* PS = !WIDE || cnt <= Ws ? (const int*)(B + L.oP) : O.push[dirn] + pp[ls];
      T* ring_out = ring + (k & (R - 1)) * W;
      // one row of the step; STG: its records are in the stage buffer, else
      // (the rows of a wider step past the staged ones) in global memory
      auto row = [&](const int sl, auto stg_tag) {
        constexpr bool STG = decltype(stg_tag)::value;
        const int q = base + sl;
        const int4 sr = STG ? S4[sl] : __ldg(O.srec[dirn] + q);
        const int ne = sr.x & 255, np = (sr.x >> 8) & 255, xoff = (int)((unsigned)sr.x >> 16), poff = sr.y;
        T vl[VR];  // an unstaged row's coefficient record
        if constexpr (!STG)
#pragma unroll
          for (int e = 0; e < VR; ++e) vl[e] = ldcg(V.vrec[dirn] + (size_t)q * VR + e);
        const T* vr = STG ? VRc + sl * VR : vl;
        // dependency values of entries 0..3 without branches: entries past
        // ne have code 0 and coefficient 0, so they contribute an exact
        // zero; ring (code > 0) or exchanged value (code 0) by select.  The
        // thread's first row takes its exchanged values from the loads of
        // the previous step, every other row polls them below.
        const unsigned cw[2] = {(unsigned)sr.z, (unsigned)sr.w};
        const bool mine = have_pf && sl == (int)threadIdx.x;
        T dv[FC_ELL];
        unsigned xmask = 0;  // entries that come through the exchange array
        int m = 0;
#pragma unroll
        for (int e = 0; e < FC_ELL; ++e) {
          const int c1 = (int)((cw[e >> 1] >> (16 * (e & 1))) & 0xFFFFu);  // code + 1
          const bool ex = c1 == 0 && e < ne;
          const T rv = ring[c1 > 0 ? c1 - 1 : 0];
          const T xv_ = mine ? pfk[e] : Sentinel<T>::value();
          dv[e] = c1 > 0 ? rv : (ex ? xv_ : T(0));
          xmask |= (ex ? 1u : 0u) << e;
          m += ex ? 1 : 0;
        }
        if (xmask) {
          // exchanged values: poll the slot if the early load came before
          // the producer's store, and put the sentinel back
          int mm = 0;
#pragma unroll
          for (int e = 0; e < FC_ELL; ++e)
            if ((xmask >> e) & 1u) {
              T v = dv[e];
              if (Sentinel<T>::is(v)) v = xv_wait<T>(C, xv + xbase + xoff + mm, X.abort_flag);
              xv[xbase + xoff + mm] = Sentinel<T>::value();
              dv[e] = v;
              ++mm;
            }
        }
        if (tr && sl == 0) tr->at(k, 5, __double_as_longlong((double)dv[0] + (double)dv[1] + (double)dv[2]));
        // overflow entry e >= FC_ELL: its value and coefficient
        auto dep_ovf = [&](int e, T& a) -> T {
          const int o = __ldg(O.ovf_ptr[dirn] + q) + e - FC_ELL;
          a = __ldg(V.aovf[dirn] + o);
          const int c = __ldg(O.ovf_code[dirn] + o);
          if (c >= 0) return ring[c];
          const T v = xv_wait<T>(C, xv + xbase + xoff + m, X.abort_flag);
          xv[xbase + xoff + m] = Sentinel<T>::value();
          ++m;
          return v;
        };
        T val;
        if (kSetup) {
          // d_i = a_ii - sum a_k^2 d_j (DIC) or a_k d_j a_(j,i) (DILU), then 1/d_i
          // (the recurrence is exact, so entries past ne are skipped)
          T sl_x[VR];
          if constexpr (!STG)
#pragma unroll
            for (int e = 0; e < VR; ++e) sl_x[e] = ldcg(V.sx + (size_t)q * VR + e);
          const T* sx = STG ? (const T*)(B + L.oX2) + sl * VR : sl_x;
          T di = sx[0];
#pragma unroll
          for (int e = 0; e < FC_ELL; ++e)
            if (e < ne) {
              const T a = vr[e];
              di = MODE == OS_SETUP_DILU ? sub_rn(di, mul_rn(mul_rn(a, dv[e]), sx[1 + e]))
                                         : sub_rn(di, mul_rn(mul_rn(a, a), dv[e]));
            }
          for (int e = FC_ELL; e < ne; ++e) {
            T a;
            const T dj = dep_ovf(e, a);
            const T at = MODE == OS_SETUP_DILU ? __ldg(V.tovf + __ldg(O.ovf_ptr[0] + q) + e - FC_ELL) : a;
            di = MODE == OS_SETUP_DILU ? sub_rn(di, mul_rn(mul_rn(a, dj), at)) : sub_rn(di, mul_rn(mul_rn(a, a), dj));
          }
          val = div_rn(T(1), di);
          const T f = T(1) / (val + (T)FC_SMALL);
          V.vrec[0][(size_t)q * VR + 4] = val;
          V.vrec[0][(size_t)q * VR + 5] = f;
          V.vrec[1][(size_t)q * VR + 4] = val;
          V.vrec[1][(size_t)q * VR + 5] = f;
        } else if (kGS) {
          // s = b - sum_{k<kd} a x_new - a_ii x_old_i - sum_{k>kd} a x_old;
          // x_i = x_old_i + s / (a_ii + small)   (exact arithmetic)
          T s = STG ? ((const T*)(B + L.oQ))[woff + sl] : ldcg(io.q + q);
#pragma unroll
          for (int e = 0; e < FC_ELL; ++e)
            if (e < ne) s = sub_rn(s, mul_rn(vr[e], dv[e]));
          for (int e = FC_ELL; e < ne; ++e) {
            T a;
            const T xj = dep_ovf(e, a);
            s = sub_rn(s, mul_rn(a, xj));
          }
          const T aii = STG ? ((const T*)(B + L.oX2))[sl * VR] : ldcg(V.sx + (size_t)q * VR);
          const T xo = STG ? ((const T*)(B + L.oE))[woff + sl] : ldcg(io.e + q);
          s = sub_rn(s, mul_rn(aii, xo));
          const int nu = __ldg(&O.srec[1][q].x) & 255;
          T v2l[VR];
          if constexpr (!STG)
#pragma unroll
            for (int e = 0; e < VR; ++e) v2l[e] = ldcg(V.vrec[1] + (size_t)q * VR + e);
          const T* v2 = STG ? (const T*)(B + L.oV2) + sl * VR : v2l;
          const int4 uc = STG ? ((const int4*)(B + L.oU))[sl] : __ldg(O.ucol + q);
#pragma unroll
          for (int e = 0; e < FC_ELL; ++e)
            if (e < nu) {
              const int cj = e == 0 ? uc.x : e == 1 ? uc.y : e == 2 ? uc.z : uc.w;
              s = sub_rn(s, mul_rn(v2[e], ldcg(io.e + cj)));
            }
          for (int e = FC_ELL; e < nu; ++e) {
            const int o = __ldg(O.ovf_ptr[1] + q) + e - FC_ELL;
            s = sub_rn(s, mul_rn(__ldg(V.aovf[1] + o), ldcg(io.e + __ldg(O.ovf_col[1] + o))));
          }
          val = add_rn(xo, div_rn(s, add_rn(aii, (T)FC_SMALL)));
          red[0] += fabs((double)s);
          red[1] += fabs((double)aii * (double)val);
        } else {
          // forward: y_i = (q_i - sum a y_j) d_i;
          // backward: z_i = (y_i / (d_i + small) - sum a z_j) d_i, the division
          // taken as a product with 1/(d_i + small) from the setup.  Entries
          // 0..2 unconditionally (padding adds exactly zero), entry 3 when
          // present.
          const T di = vr[4];
          T acc = STG ? ((const T*)(B + L.oQ))[woff + sl] : ldcg(io.q + q);
          if (dirn) acc = acc * vr[5];
          acc = fma(-vr[0], dv[0], acc);
          acc = fma(-vr[1], dv[1], acc);
          acc = fma(-vr[2], dv[2], acc);
          if (ne > 3) acc = fma(-vr[3], dv[3], acc);
          for (int e = FC_ELL; e < ne; ++e) {
            T a;
            const T v = dep_ovf(e, a);
            acc = fma(-a, v, acc);
          }
          val = acc * di;
          if (MODE == OS_BWD_DOT)
            red[0] += (double)(STG ? ((const T*)(B + L.oE))[woff + sl] : ldcg(io.e + q)) * (double)val;
        }
        if (tr && sl == 0) tr->at(k, 6, __double_as_longlong((double)val));
        io.out[q] = val;
        ring_out[sl] = val;
        // plain stores: an aligned 8-byte (4-byte) store is single-copy
        // atomic, so a consumer polling the slot sees the sentinel or the value
        for (int mm = 0; mm < np; ++mm) xv[PS[poff + mm]] = val;
        if (tr && sl == 0) tr->at(k, 7, np);
      };
      for (int sl = threadIdx.x; sl < cnt; sl += ncg) {
        if constexpr (WIDE) {
          if (sl < Ws) row(sl, std::true_type{});
          else row(sl, std::false_type{});
        } else {
          row(sl, std::true_type{});
        }
      }
      bar_compute(ncg);
      if (threadIdx.x == 0) mbar_arrive(X.empty + b);
      X.parity ^= 1u << b;
      X.used |= 1u << b;
      if (*((volatile int*)X.abort_flag)) break;
    }
  }
  __syncthreads();
  if (*((volatile int*)X.abort_flag)) {
    // after an abort, let the copies of fills that were never consumed land
    // (bounded) before the block leaves
    if (threadIdx.x == (unsigned)nct)
      for (int b = 0; b < K; ++b)
        if ((X.used >> b) & 1u) mbar_wait(X.full + b, ((X.parity >> b) & 1u) ^ 1u);
    __syncthreads();
    return false;
  }
  if (tr) tr->step(ns);
  return true;
}

// ------------------------------------------------------ gather / scatter
// Per-solve values in the new numbering from the caller's CSR values a
// (original entry slots), exchange arrays filled with the sentinel.  Grid-
// stride; the caller ends the phase with a grid barrier.
template <class T>
__device__ void ord_gather_values(const GridCtl& C, const OrdView& O, const OrdVals<T>& V, const T* __restrict__ a,
                                  int nnz, bool dilu) {
  const int gt = vg_gt(C), G = vg_G(C), n = O.n, nE = O.nE;
  constexpr int VR = Rec<T>::V;
  const T SENT = Sentinel<T>::value();
  for (int q = gt; q < n; q += G) {
    const T aii = __ldg(a + __ldg(O.dslot + q));
    V.adiag[q] = aii;
    T* sx = V.sx + (size_t)q * VR;
    sx[0] = aii;
    for (int d = 0; d < 2; ++d) {
      T* vr = V.vrec[d] + (size_t)q * VR;
#pragma unroll
      for (int e = 0; e < FC_ELL; ++e) {
        const int s = __ldg(O.slot[d] + (size_t)e * nE + q);
        vr[e] = s >= 0 ? __ldg(a + s) : T(0);
        if (d == 0) sx[1 + e] = (dilu && s >= 0) ? __ldg(a + __ldg(O.lo_tslot + (size_t)e * nE + q)) : T(0);
      }
    }
  }
  for (int d = 0; d < 2; ++d) {
    const int novf = d ? O.novf1 : O.novf0;
    for (int o = gt; o < novf; o += G) {
      V.aovf[d][o] = __ldg(a + __ldg(O.ovf_slot[d] + o));
      if (d == 0 && dilu) V.tovf[o] = __ldg(a + __ldg(O.lo_ovf_tslot + o));
    }
    const int nx = __ldg(O.xv_ptr[d] + O.nsteps);
    for (int p = gt; p < nx; p += G) V.xv[d][p] = SENT;
  }
  for (int k = gt; k < nnz; k += G) V.ap[k] = __ldg(a + __ldg(O.p_slot + k));
}

// y[q] = src[perm[q]] (into the new numbering) / dst[perm[q]] = y[q]
template <class T, class U>
__device__ __forceinline__ void ord_gather_vec(const GridCtl& C, const OrdView& O, const U* __restrict__ src, T* y) {
  for (int q = vg_gt(C); q < O.n; q += vg_G(C))
    y[q] = (T)ldcg(src + __ldg(O.perm + q));
}
template <class T, class U>
__device__ __forceinline__ void ord_scatter_vec(const GridCtl& C, const OrdView& O, const T* y, U* dst) {
  for (int q = vg_gt(C); q < O.n; q += vg_G(C))
    dst[__ldg(O.perm + q)] = (U)ldcg(y + q);
}

// row products in the new numbering (FMA accumulation in the row's original
// entry order, as ax_cr / the residual loops of the reference)
template <class T>
__device__ __forceinline__ T ord_row_dot(const OrdView& O, const T* __restrict__ ap, const T* x, int q) {
  const int k0 = __ldg(O.p_ptr + q), k1 = __ldg(O.p_ptr + q + 1);
  T s = T(0);
  for (int k = k0; k < k1; ++k) s = fma(__ldg(ap + k), ldcg(x + __ldg(O.p_col + k)), s);
  return s;
}
template <class T>
__device__ __forceinline__ T ord_row_residual(const OrdView& O, const T* __restrict__ ap, const T* x, T bq, int q) {
  const int k0 = __ldg(O.p_ptr + q), k1 = __ldg(O.p_ptr + q + 1);
  T s = bq;
  for (int k = k0; k < k1; ++k) s = fma(-__ldg(ap + k), ldcg(x + __ldg(O.p_col + k)), s);
  return s;
}

}  // namespace fcdev
