// Inner solve of the mixed-precision path on a multicolour ordering: FP32
// (FC_PREC_MIXED_COLOURED) and, as a diagnostic of what the precision
// contributes, the same solve in FP64 (FC_PREC_COLOURED_FP64); the kernels
// are templates on the value type.
//
// The FP64 path keeps the reference's natural-order DIC, whose triangular
// sweeps are a long chain of dependent levels: on this GPU the sweep is bound
// by the latency of each level, not by bytes, so running it in FP32 saves
// little.  The coloured inner solve instead colours the rows
// (host/fc_colour.cpp), factors A by DILU in the coloured order (DIC for a
// symmetric matrix) and applies the factors one colour at a time: every pass
// is a data-parallel ELLPACK sweep, bound by HBM bandwidth.  The
// preconditioner is weaker than the natural-order one (more iterations), but
// each iteration is a handful of bandwidth-bound passes.  The refinement loop
// around it (fc_solvers.cu) is unchanged: FP64 residual, the reference's
// stopping test, FP64 accumulation of the corrections.
//
// The inner PCG runs in Eisenstat's form (S. C. Eisenstat, "Efficient
// implementation of a class of preconditioned conjugate gradient methods",
// SIAM J. Sci. Stat. Comput. 2 (1981) 1-4).  With the factor
// M = (D+L) D^-1 (D+U) and A = (D+L) + (D+U) + (A_d - 2D), the operator
// B = (D+L)^-1 A (D+U)^-1 applied to p is t + (D+L)^-1 (p + (A_d - 2D) t) with
// t = (D+U)^-1 p: one backward and one forward sweep, no separate SpMV.  CG on
// B (symmetric for symmetric A) with the diagonal D as preconditioner has the
// iterates of DIC-PCG on A, mapped by x = (D+U)^-1 y and r~ = (D+L)^-1 r, so
// an iteration reads the matrix once instead of twice.  The inner stopping test
// is the relative reduction of the D-norm of r~; the refinement loop checks
// the true residual.
//
// The inner solve is one CUDA graph per system: a prologue (the forward sweep
// on the right-hand side, the first direction), a device-side while loop
// whose body is one kernel per pass, and the final backward sweep x =
// (D+U)^-1 y.  Every kernel runs at full occupancy with one thread per row;
// the scalars of the iteration are finalised in device memory by the last
// block of each reduction, in a fixed order, and the block that decides to
// stop clears the loop's condition.  Dot products and norms are accumulated
// in FP64 in both value types.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>

#include "fc_colour.hpp"
#include "fc_internal.hpp"

#define MCG_BLOCK 512
// the loop-body kernels run grid-stride on at most this many waves of
// resident blocks: the per-block reduction tail (block sum, fence, arrival
// atomic) is then paid once per wave
#define MC_WAVES 1
#define MC_UNROLL 8   // widest block whose loads are issued all at once (hex rows: 6, tets: 4)

// per-colour table in device memory, MC_T entries per field: first row of
// every colour (ncol + 1 values, multiples of 32), first entries of the lower
// and upper blocks, widths of the lower and upper blocks
#define MC_T (FC_MC_MAXCOL + 1)
enum { MC_CR = 0, MC_CEL = MC_T, MC_CEU = 2 * MC_T, MC_CWL = 3 * MC_T, MC_CWU = 4 * MC_T, MC_TAB = 5 * MC_T };

// scalars of one inner solve, in device memory
struct McScal {
  double res0, resl, rz, rzacc, pq, tol;
  double alpha, beta;
  int it, itmax, done, status;
  double rz0;
};

// the buffers of one value type: FP32 (FC_PREC_MIXED_COLOURED) or FP64
// (FC_PREC_COLOURED_FP64) matrix values, DILU diagonal, its reciprocal and
// a_ii - 2 d, the Krylov vectors, and the inner solve's graph
template <class T>
struct McBuf {
  DVec<T> mval, adiag, invd, dvec, kdiag, x, r, p, q, y, t, w;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int wave = 1;  // resident blocks of the widest loop-body kernel on the whole GPU
  bool ready = false;
  ~McBuf() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

struct DevColoured {
  int n = 0, nP = 0, ncol = 0, maxblocks = 1;
  size_t nent = 1;  // ELLPACK entries of the layout
  std::vector<int> crow;
  DVec<int> tab, perm, col, src, tsrc, dslot;
  DVec<double> dset, part;
  DVec<unsigned> cnt;
  DVec<McScal> sc;
  McScal* h_sc = nullptr;
  McBuf<float> f32;
  McBuf<double> f64;
  ~DevColoured() {
    if (h_sc) cudaFreeHost(h_sc);
  }
};

static McBuf<float>& mc_buf(DevColoured& m, float) { return m.f32; }
static McBuf<double>& mc_buf(DevColoured& m, double) { return m.f64; }

void mc_release(DevColoured* m) { delete m; }

namespace {

template <class T>
struct McDevT {
  int nP, ncol, c0end;
  const int* __restrict__ tab;
  const int* __restrict__ col;
  const int* __restrict__ src;
  const int* __restrict__ tsrc;
  const int* __restrict__ dslot;
  const double* __restrict__ a;
  T *mval, *adiag, *invd, *dvec, *kdiag;
  double* dset;
  T *x, *r, *p, *q, *y, *t, *w;
  McScal* sc;
  double* part;     // 2 * blocks of the widest launch
  unsigned* cnt;    // arrival counter of the last-block reductions
  cudaGraphConditionalHandle h;
};

__device__ __forceinline__ double mcg_warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ float mfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double mfma(double a, double b, double c) { return fma(a, b, c); }

// four consecutive values of a vector (16-byte aligned: the padded row count
// is a multiple of 32)
__device__ __forceinline__ void ld4(const float* p, int i4, float (&v)[4]) {
  const float4 t = __ldcg((const float4*)p + i4);
  v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
}
__device__ __forceinline__ void ld4(const double* p, int i4, double (&v)[4]) {
  const double2 a = __ldcg((const double2*)p + 2 * i4), b = __ldcg((const double2*)p + 2 * i4 + 1);
  v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
}
__device__ __forceinline__ void st4(float* p, int i4, const float (&v)[4]) {
  ((float4*)p)[i4] = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void st4(double* p, int i4, const double (&v)[4]) {
  ((double2*)p)[2 * i4] = make_double2(v[0], v[1]);
  ((double2*)p)[2 * i4 + 1] = make_double2(v[2], v[3]);
}

// Sum NV values over the grid of the running kernel, in FP64 throughout: a
// thread's terms (products of FP32 values are exact in FP64), the warp
// tree, the 16 warp sums of a block and the block partials.  Each block
// writes its fixed-order sum; the last block to arrive sums the partials in
// block order, so the totals do not depend on arrival order.  Returns true in
// every thread of that last block, with the totals in tot.
template <int NV, class T>
__device__ __forceinline__ bool mcg_reduce(const McDevT<T>& D, double (&v)[NV], double (&tot)[NV]) {
  __shared__ double sm[NV][MCG_BLOCK / 32];
  __shared__ double s_tot[NV];
  __shared__ int s_last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    const double w = mcg_warp_sum(v[j]);
    if (lane == 0) sm[j][wid] = w;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double t = 0.0;
      for (int w = 0; w < MCG_BLOCK / 32; ++w) t += sm[j][w];
      D.part[j * gridDim.x + blockIdx.x] = t;
    }
    __threadfence();
    s_last = atomicAdd(D.cnt, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  // every thread of the last block sums a strided share of the partials
  // (independent loads in flight), then a fixed tree over the block
#pragma unroll
  for (int j = 0; j < NV; ++j) {
    double t = 0.0;
#pragma unroll 4
    for (int b = threadIdx.x; b < (int)gridDim.x; b += MCG_BLOCK) t += __ldcg(D.part + j * gridDim.x + b);
    t = mcg_warp_sum(t);
    if (lane == 0) sm[j][wid] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int j = 0; j < NV; ++j) {
      double t = 0.0;
      for (int w = 0; w < MCG_BLOCK / 32; ++w) t += sm[j][w];
      s_tot[j] = t;
    }
    *D.cnt = 0;
  }
  __syncthreads();
#pragma unroll
  for (int j = 0; j < NV; ++j) tot[j] = s_tot[j];
  return true;
}

// The scalars a kernel needs, read once per block by thread 0 and broadcast
// through shared memory: every thread reading them from memory would send
// one request per warp to the same L2 line, which serialises on one slice.
struct McBcast {
  int done;
  double alpha, beta;
};
template <class T>
__device__ __forceinline__ McBcast mcg_scalars(const McDevT<T>& D) {
  __shared__ McBcast s;
  if (threadIdx.x == 0) {
    s.done = __ldcg(&D.sc->done);
    s.alpha = __ldcg(&D.sc->alpha);
    s.beta = __ldcg(&D.sc->beta);
  }
  __syncthreads();
  return s;
}

// stop the loop: called by the one thread that decided it
template <class T>
__device__ __forceinline__ void mcg_stop(const McDevT<T>& D, int status) {
  if (status) D.sc->status = status;
  D.sc->done = 1;
  if (D.h) cudaGraphSetConditional(D.h, 0);  // 0 outside the graph (host-launched diagnostic mode)
}

// One row, entry k of a block at e + k * stride, all k < w (padding entries
// hold value 0 and point at the row itself): acc + sum of mval * v[col].
// Blocks up to MC_UNROLL wide (every hex and tet row) issue all index and
// value loads before the gathers, so that they are in flight together; w is
// the same for the whole colour, so no load waits on a per-row count.
template <class T>
__device__ __forceinline__ T ell_sum(const McDevT<T>& D, int e, int stride, int w, const T* v, T acc) {
  if (w <= MC_UNROLL) {
    int c[MC_UNROLL];
    T m[MC_UNROLL];
#pragma unroll
    for (int k = 0; k < MC_UNROLL; ++k)
      if (k < w) {
        c[k] = __ldg(D.col + e + k * stride);
        m[k] = __ldcg(D.mval + e + k * stride);
      }
#pragma unroll
    for (int k = 0; k < MC_UNROLL; ++k)
      if (k < w) acc = mfma(m[k], __ldcg(v + c[k]), acc);
    return acc;
  }
  for (int k = 0; k < w; ++k) acc = mfma(__ldcg(D.mval + e + k * stride), __ldcg(v + __ldg(D.col + e + k * stride)), acc);
  return acc;
}

// r (coloured, value type T) <- r64 (original order); x, p <- 0; scalars reset
template <class T>
__global__ void k_mc_gather(McDevT<T> D, const int* __restrict__ perm, const double* __restrict__ r64, double tol,
                            int itmax) {
  // t, w and q start at zero too: a padding entry of an ELLPACK block (value
  // 0, column = its own row) reads the row's t or w before the iteration has
  // written it, and 0 times uninitialised memory may be NaN
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < D.nP; i += gridDim.x * blockDim.x) {
    const int o = perm[i];
    D.r[i] = o >= 0 ? (T)r64[o] : T(0);
    D.x[i] = T(0);
    D.p[i] = T(0);
    D.t[i] = T(0);
    D.w[i] = T(0);
    D.q[i] = T(0);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    McScal s;
    s.res0 = s.resl = s.rz = s.rzacc = s.pq = s.rz0 = 0.0;
    s.tol = tol;
    s.alpha = s.beta = 0.0;
    s.it = 0; s.itmax = itmax; s.done = 0; s.status = 0;
    *D.sc = s;
  }
}

// x64 (original order) += x (coloured)
template <class T>
__global__ void k_mc_scatter_add(int nP, const int* __restrict__ perm, const T* __restrict__ x, double* x64) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nP; i += gridDim.x * blockDim.x) {
    const int o = perm[i];
    if (o >= 0) x64[o] += (double)x[i];
  }
}

// values and the coloured DILU diagonal of colour c (colours in order):
// d_i = a_ii - sum over lower entries of a_ij a_ji / d_j, in FP64; copies in
// T of d, 1/(d + small) and a_ii - 2 d
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_mcg_setup(McDevT<T> D, int c) {
  const int r0 = __ldg(D.tab + MC_CR + c), r1 = __ldg(D.tab + MC_CR + c + 1), stride = r1 - r0;
  const int cel = __ldg(D.tab + MC_CEL + c), ceu = __ldg(D.tab + MC_CEU + c);
  const int cwl = __ldg(D.tab + MC_CWL + c), cwu = __ldg(D.tab + MC_CWU + c);
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  const int ds = __ldg(D.dslot + i);
  const double aii = ds >= 0 ? __ldg(D.a + ds) : 1.0;
  double d = aii;
  for (int k = 0; k < cwl; ++k) {
    const int e = cel + (i - r0) + k * stride;
    const int sl = __ldg(D.src + e);
    if (sl < 0) continue;
    const double v = __ldg(D.a + sl);
    D.mval[e] = (T)v;
    const int ts = __ldg(D.tsrc + e);
    const double t = ts >= 0 ? __ldg(D.a + ts) : 0.0;
    d -= v * t / __ldcg(D.dset + __ldg(D.col + e));
  }
  for (int k = 0; k < cwu; ++k) {
    const int e = ceu + (i - r0) + k * stride;
    const int sl = __ldg(D.src + e);
    if (sl >= 0) D.mval[e] = (T)__ldg(D.a + sl);
  }
  D.dset[i] = d;
  D.dvec[i] = (T)d;
  D.invd[i] = (T)(1.0 / (d + FC_SMALL));
  D.kdiag[i] = (T)(aii - 2.0 * d);
  D.adiag[i] = ds >= 0 ? (T)aii : T(0);
}

// colour c of (D+L) r~ = b, in place on r (lower colours already hold r~)
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e_fwdb(McDevT<T> D, int c) {
  const int r0 = __ldg(D.tab + MC_CR + c), r1 = __ldg(D.tab + MC_CR + c + 1);
  const int cel = __ldg(D.tab + MC_CEL + c), cwl = __ldg(D.tab + MC_CWL + c);
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  D.r[i] = (__ldcg(D.r + i) - ell_sum(D, cel + (i - r0), r1 - r0, cwl, D.r, T(0))) * __ldcg(D.invd + i);
}

// z = D r~, p = z, t = p / d on the last colour; r~.z starts the iteration
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e_start(McDevT<T> D) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int clast = __ldg(D.tab + MC_CR + D.ncol - 1);
  double v[1] = {0.0};
  if (i < D.nP) {
    const T ri = __ldcg(D.r + i), zi = __ldcg(D.dvec + i) * ri;
    D.y[i] = zi;
    D.p[i] = zi;
    if (i >= clast) D.t[i] = zi * __ldcg(D.invd + i);
    v[0] = (double)ri * (double)zi;
  }
  double tot[1];
  if (!mcg_reduce<1>(D, v, tot) || threadIdx.x != 0) return;
  McScal* S = D.sc;
  S->rz = S->rz0 = S->res0 = S->resl = tot[0];
  S->beta = 0.0;
  if (!(tot[0] == tot[0]) || isinf(tot[0])) mcg_stop(D, FC_ERR_NAN);
  else if (tot[0] == 0.0 || S->itmax <= 0) mcg_stop(D, 0);
}

// backward colour c (1 <= c <= C-2) of (D+U) t = p
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e_bwd(McDevT<T> D, int c) {
  if (mcg_scalars(D).done) return;
  const int r0 = __ldg(D.tab + MC_CR + c), r1 = __ldg(D.tab + MC_CR + c + 1);
  const int ceu = __ldg(D.tab + MC_CEU + c), cwu = __ldg(D.tab + MC_CWU + c);
  for (int i = r0 + blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += gridDim.x * blockDim.x)
    D.t[i] = (__ldcg(D.p + i) - ell_sum(D, ceu + (i - r0), r1 - r0, cwu, D.t, T(0))) * __ldcg(D.invd + i);
}

// colour 0: the last backward colour t = (p - U t) / d and the first forward
// colour w = (p + K t) / d (no lower entries), q = t + w, p.q
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e_bf0(McDevT<T> D) {
  if (mcg_scalars(D).done) return;
  const int r1 = __ldg(D.tab + MC_CR + 1);
  const int ceu = __ldg(D.tab + MC_CEU), cwu = __ldg(D.tab + MC_CWU);
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += gridDim.x * blockDim.x) {
    const T pi = __ldcg(D.p + i), di = __ldcg(D.invd + i), ki = __ldcg(D.kdiag + i);
    const T ti = (pi - ell_sum(D, ceu + i, r1, cwu, D.t, T(0))) * di;
    const T wi = mfma(ki, ti, pi) * di;
    const T qi = ti + wi;
    D.w[i] = wi;
    D.q[i] = qi;
    v[0] += (double)pi * (double)qi;
  }
  double tot[1];
  if (!mcg_reduce<1>(D, v, tot) || threadIdx.x != 0) return;
  McScal* S = D.sc;
  S->pq = tot[0];
  if (D.ncol == 1) {
    const double alpha = S->rz / tot[0];
    if (!(alpha == alpha) || isinf(alpha)) mcg_stop(D, FC_ERR_BREAKDOWN);
    else S->alpha = alpha;
  }
}

// forward colour c >= 1: w = (p + K t - L w) / d, q = t + w, p.q; the last
// colour closes p.q and sets alpha
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e_fwd(McDevT<T> D, int c) {
  if (mcg_scalars(D).done) return;
  const int r0 = __ldg(D.tab + MC_CR + c), r1 = __ldg(D.tab + MC_CR + c + 1);
  const int cel = __ldg(D.tab + MC_CEL + c), cwl = __ldg(D.tab + MC_CWL + c);
  double v[1] = {0.0};
  for (int i = r0 + blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += gridDim.x * blockDim.x) {
    const T pi = __ldcg(D.p + i), di = __ldcg(D.invd + i), ki = __ldcg(D.kdiag + i), ti = __ldcg(D.t + i);
    const T wi = (mfma(ki, ti, pi) - ell_sum(D, cel + (i - r0), r1 - r0, cwl, D.w, T(0))) * di;
    const T qi = ti + wi;
    D.w[i] = wi;
    D.q[i] = qi;
    v[0] += (double)pi * (double)qi;
  }
  double tot[1];
  if (!mcg_reduce<1>(D, v, tot) || threadIdx.x != 0) return;
  McScal* S = D.sc;
  S->pq += tot[0];
  if (c == D.ncol - 1) {
    const double alpha = S->rz / S->pq;
    if (!(alpha == alpha) || isinf(alpha)) mcg_stop(D, FC_ERR_BREAKDOWN);
    else S->alpha = alpha;
  }
}

// y += alpha p, r~ -= alpha q, z = D r~, r~.z; the stopping test on the
// D-norm of r~ (relative to the start) or the iteration limit; beta
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e_upd(McDevT<T> D) {
  const McBcast sc = mcg_scalars(D);
  if (sc.done) return;
  const T alpha = (T)sc.alpha;
  double v[1] = {0.0};
  for (int i4 = blockIdx.x * blockDim.x + threadIdx.x; i4 < (D.nP >> 2); i4 += gridDim.x * blockDim.x) {
    T x4[4], p4[4], q4[4], r4[4], d4[4], zn[4];
    ld4(D.x, i4, x4); ld4(D.p, i4, p4); ld4(D.q, i4, q4); ld4(D.r, i4, r4); ld4(D.dvec, i4, d4);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      r4[k] = mfma(-alpha, q4[k], r4[k]);
      zn[k] = d4[k] * r4[k];
      x4[k] = mfma(alpha, p4[k], x4[k]);
      v[0] += (double)r4[k] * (double)zn[k];
    }
    st4(D.x, i4, x4);
    st4(D.r, i4, r4);
    st4(D.y, i4, zn);
  }
  double tot[1];
  if (!mcg_reduce<1>(D, v, tot) || threadIdx.x != 0) return;
  McScal* S = D.sc;
  S->it += 1;
  S->resl = tot[0];
  if (!(tot[0] == tot[0]) || isinf(tot[0])) { mcg_stop(D, FC_ERR_NAN); return; }
  // r~.z keeps the sign of A (negative for the reference's pressure matrix)
  if (fabs(tot[0]) <= S->tol * S->tol * fabs(S->rz0) || S->it >= S->itmax) { mcg_stop(D, 0); return; }
  S->beta = tot[0] / S->rz;
  S->rz = tot[0];
}

// p = z + beta p; t = p / d on the last colour (the first backward colour)
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e_pupd(McDevT<T> D) {
  const McBcast sc = mcg_scalars(D);
  if (sc.done) return;
  const T beta = (T)sc.beta;
  const int clast = __ldg(D.tab + MC_CR + D.ncol - 1);
  for (int i4 = blockIdx.x * blockDim.x + threadIdx.x; i4 < (D.nP >> 2); i4 += gridDim.x * blockDim.x) {
    T z4[4], p4[4];
    ld4(D.y, i4, z4); ld4(D.p, i4, p4);
#pragma unroll
    for (int k = 0; k < 4; ++k) p4[k] = mfma(beta, p4[k], z4[k]);
    st4(D.p, i4, p4);
    if (4 * i4 >= clast) {  // colour boundaries are multiples of 32 rows
      T d4[4];
      ld4(D.invd, i4, d4);
#pragma unroll
      for (int k = 0; k < 4; ++k) d4[k] = p4[k] * d4[k];
      st4(D.t, i4, d4);
    }
  }
}

// Two colours (red-black): the new direction p = z + beta p is folded into
// the two colour passes, so an iteration is three kernels.  Colour 0 updates
// its own p and gathers t_j = (z_j + beta p_j) / d_j of its colour-1
// neighbours, whose p the colour-1 pass has not yet replaced.
template <class T>
__device__ __forceinline__ T ell_sum_t(const McDevT<T>& D, int e, int stride, int w, T beta, T acc) {
  if (w <= MC_UNROLL) {
    int c[MC_UNROLL];
    T m[MC_UNROLL];
#pragma unroll
    for (int k = 0; k < MC_UNROLL; ++k)
      if (k < w) {
        c[k] = __ldg(D.col + e + k * stride);
        m[k] = __ldcg(D.mval + e + k * stride);
      }
#pragma unroll
    for (int k = 0; k < MC_UNROLL; ++k)
      if (k < w) {
        const T tj = mfma(beta, __ldcg(D.p + c[k]), __ldcg(D.y + c[k])) * __ldcg(D.invd + c[k]);
        acc = mfma(m[k], tj, acc);
      }
    return acc;
  }
  for (int k = 0; k < w; ++k) {
    const int cj = __ldg(D.col + e + k * stride);
    acc = mfma(__ldcg(D.mval + e + k * stride), mfma(beta, __ldcg(D.p + cj), __ldcg(D.y + cj)) * __ldcg(D.invd + cj), acc);
  }
  return acc;
}

// colour 0 of two: p = z + beta p, t = (p - U t)/d, w = (p + K t)/d, q, p.q
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e2_c0(McDevT<T> D) {
  const McBcast sc = mcg_scalars(D);
  if (sc.done) return;
  const T beta = (T)sc.beta;
  const int r1 = __ldg(D.tab + MC_CR + 1);
  const int ceu = __ldg(D.tab + MC_CEU), cwu = __ldg(D.tab + MC_CWU);
  double v[1] = {0.0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += gridDim.x * blockDim.x) {
    const T pi = mfma(beta, __ldcg(D.p + i), __ldcg(D.y + i));
    const T di = __ldcg(D.invd + i), ki = __ldcg(D.kdiag + i);
    const T ti = (pi - ell_sum_t(D, ceu + i, r1, cwu, beta, T(0))) * di;
    const T wi = mfma(ki, ti, pi) * di;
    const T qi = ti + wi;
    D.p[i] = pi;
    D.w[i] = wi;
    D.q[i] = qi;
    v[0] += (double)pi * (double)qi;
  }
  double tot[1];
  if (!mcg_reduce<1>(D, v, tot) || threadIdx.x != 0) return;
  D.sc->pq = tot[0];
}

// colour 1 of two: p = z + beta p, t = p/d, w = (p + K t - L w)/d, q, p.q, alpha
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e2_c1(McDevT<T> D) {
  const McBcast sc = mcg_scalars(D);
  if (sc.done) return;
  const T beta = (T)sc.beta;
  const int r0 = __ldg(D.tab + MC_CR + 1), r1 = __ldg(D.tab + MC_CR + 2);
  const int cel = __ldg(D.tab + MC_CEL + 1), cwl = __ldg(D.tab + MC_CWL + 1);
  double v[1] = {0.0};
  for (int i = r0 + blockIdx.x * blockDim.x + threadIdx.x; i < r1; i += gridDim.x * blockDim.x) {
    const T pi = mfma(beta, __ldcg(D.p + i), __ldcg(D.y + i));
    const T di = __ldcg(D.invd + i), ki = __ldcg(D.kdiag + i);
    const T ti = pi * di;
    const T wi = (mfma(ki, ti, pi) - ell_sum(D, cel + (i - r0), r1 - r0, cwl, D.w, T(0))) * di;
    const T qi = ti + wi;
    D.p[i] = pi;
    D.w[i] = wi;
    D.q[i] = qi;
    v[0] += (double)pi * (double)qi;
  }
  double tot[1];
  if (!mcg_reduce<1>(D, v, tot) || threadIdx.x != 0) return;
  McScal* S = D.sc;
  S->pq += tot[0];
  const double alpha = S->rz / S->pq;
  if (!(alpha == alpha) || isinf(alpha)) mcg_stop(D, FC_ERR_BREAKDOWN);
  else S->alpha = alpha;
}

// colour c of x = (D+U)^-1 y, in place on x (higher colours already hold x)
template <class T>
__global__ void __launch_bounds__(MCG_BLOCK) k_e_xb(McDevT<T> D, int c) {
  const int r0 = __ldg(D.tab + MC_CR + c), r1 = __ldg(D.tab + MC_CR + c + 1);
  const int ceu = __ldg(D.tab + MC_CEU + c), cwu = __ldg(D.tab + MC_CWU + c);
  const int i = r0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= r1) return;
  D.x[i] = (__ldcg(D.x + i) - ell_sum(D, ceu + (i - r0), r1 - r0, cwu, D.x, T(0))) * __ldcg(D.invd + i);
}

}  // namespace

template <class T>
static McDevT<T> mc_dev(DevColoured& m, McBuf<T>& b, const double* a) {
  McDevT<T> D;
  D.nP = m.nP; D.ncol = m.ncol; D.c0end = m.crow[1];
  D.tab = m.tab.p; D.col = m.col.p; D.src = m.src.p; D.tsrc = m.tsrc.p; D.dslot = m.dslot.p; D.a = a;
  D.mval = b.mval.p; D.adiag = b.adiag.p; D.invd = b.invd.p; D.dvec = b.dvec.p; D.kdiag = b.kdiag.p;
  D.dset = m.dset.p;
  D.x = b.x.p; D.r = b.r.p; D.p = b.p.p; D.q = b.q.p; D.y = b.y.p; D.t = b.t.p; D.w = b.w.p;
  D.sc = m.sc.p; D.part = m.part.p; D.cnt = m.cnt.p;
  D.h = 0;
  return D;
}

static inline unsigned mc_blocks(int rows) { return (unsigned)std::max(1, (rows + MCG_BLOCK - 1) / MCG_BLOCK); }

// The inner PCG graph: prologue (init, first preconditioner application) and
// a while node whose body is one iteration.  The kernels' arguments are fixed
// (the system's own buffers); tolerance and iteration limit are read from the
// scalar block, which k_mc_gather resets before every launch.
template <class T>
static int mc_build_graph(fc_ctx* ctx, DevColoured& m, McBuf<T>& b) {
  cudaGraph_t g = nullptr;
  FC_CUDA_TRY(ctx, cudaGraphCreate(&g, 0));
  b.graph = g;
  cudaGraphConditionalHandle h;
  FC_CUDA_TRY(ctx, cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault));
  McDevT<T> D = mc_dev(m, b, nullptr);
  D.h = h;
  const int C = m.ncol;
  // kernel nodes copy their arguments at creation, so the locals below may go
  int cs[FC_MC_MAXCOL];
  for (int c = 0; c < C; ++c) cs[c] = c;
  auto add = [&](cudaGraph_t gr, cudaGraphNode_t& prev, bool have_prev, const void* fn, unsigned blocks,
                 void** args) -> int {
    cudaKernelNodeParams kp = {};
    kp.func = const_cast<void*>(fn);
    kp.gridDim = dim3(blocks);
    kp.blockDim = dim3(MCG_BLOCK);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    kp.extra = nullptr;
    cudaGraphNode_t n;
    FC_CUDA_TRY(ctx, cudaGraphAddKernelNode(&n, gr, have_prev ? &prev : nullptr, have_prev ? 1 : 0, &kp));
    prev = n;
    return FC_OK;
  };
  auto blocks_of = [&](int c) { return mc_blocks(m.crow[c + 1] - m.crow[c]); };
  // loop-body grids: capped at MC_WAVES waves of resident blocks
  auto body_blocks = [&](unsigned nat) { return std::min(nat, (unsigned)(MC_WAVES * b.wave)); };
  int st;
  cudaGraphNode_t prev = nullptr;
  void* a1[1] = {&D};
  // prologue: (D+L) r~ = b colour by colour, then z, p, t and r~.z
  for (int c = 0; c < C; ++c) {
    void* args[2] = {&D, &cs[c]};
    if ((st = add(g, prev, c > 0, (const void*)k_e_fwdb<T>, blocks_of(c), args))) return st;
  }
  if ((st = add(g, prev, true, (const void*)k_e_start<T>, mc_blocks(m.nP), a1))) return st;
  cudaGraphNodeParams cp = {};
  cp.type = cudaGraphNodeTypeConditional;
  cp.conditional.handle = h;
  cp.conditional.type = cudaGraphCondTypeWhile;
  cp.conditional.size = 1;
  cudaGraphNode_t loop;
  FC_CUDA_TRY(ctx, cudaGraphAddNode(&loop, g, &prev, nullptr, 1, &cp));
  // body: backward colours C-2..1, colour 0 (backward + forward), forward
  // colours 1..C-1, the x/r update with the stopping test, the new direction
  cudaGraph_t body = cp.conditional.phGraph_out[0];
  cudaGraphNode_t bp = nullptr;
  bool have = false;
  if (C == 2) {  // red-black: three kernels per iteration
    if ((st = add(body, bp, false, (const void*)k_e2_c0<T>, body_blocks(blocks_of(0)), a1))) return st;
    if ((st = add(body, bp, true, (const void*)k_e2_c1<T>, body_blocks(blocks_of(1)), a1))) return st;
    if ((st = add(body, bp, true, (const void*)k_e_upd<T>, body_blocks(mc_blocks(m.nP / 4)), a1))) return st;
  } else {
    for (int c = C - 2; c >= 1; --c) {
      void* args[2] = {&D, &cs[c]};
      if ((st = add(body, bp, have, (const void*)k_e_bwd<T>, body_blocks(blocks_of(c)), args))) return st;
      have = true;
    }
    if ((st = add(body, bp, have, (const void*)k_e_bf0<T>, body_blocks(blocks_of(0)), a1))) return st;
    for (int c = 1; c < C; ++c) {
      void* args[2] = {&D, &cs[c]};
      if ((st = add(body, bp, true, (const void*)k_e_fwd<T>, body_blocks(blocks_of(c)), args))) return st;
    }
    if ((st = add(body, bp, true, (const void*)k_e_upd<T>, body_blocks(mc_blocks(m.nP / 4)), a1))) return st;
    if ((st = add(body, bp, true, (const void*)k_e_pupd<T>, body_blocks(mc_blocks(m.nP / 4)), a1))) return st;
  }
  // after the loop: x = (D+U)^-1 y, colours C-1..0
  prev = loop;
  for (int c = C - 1; c >= 0; --c) {
    void* args[2] = {&D, &cs[c]};
    if ((st = add(g, prev, true, (const void*)k_e_xb<T>, blocks_of(c), args))) return st;
  }
  FC_CUDA_TRY(ctx, cudaGraphInstantiate(&b.exec, g, 0));
  return FC_OK;
}

static int mc_prepare(fc_ctx* ctx, CsrSystem* s) {
  if (s->mc) return FC_OK;
  ColouredLayout L;
  std::string why;
  if (!build_coloured(s->n, s->h_ia.data(), s->h_ja.data(), s->h_diag.data(), L, &why))
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "multicolour layout: " + why);
  DevColoured* m = new DevColoured();
  m->n = L.n; m->nP = L.nP; m->ncol = L.ncol;
  m->crow.resize(L.ncol + 1);
  for (int c = 0; c <= L.ncol; ++c) m->crow[c] = L.cslice[c] * FC_MC_SLICE;
  std::vector<int> tab(MC_TAB, 0);
  for (int c = 0; c <= FC_MC_MAXCOL; ++c) tab[MC_CR + c] = c <= L.ncol ? m->crow[c] : L.nP;
  for (int c = 0; c < L.ncol; ++c) {
    tab[MC_CEL + c] = (int)L.cel[c];
    tab[MC_CEU + c] = (int)L.ceu[c];
    tab[MC_CWL + c] = L.cwl[c];
    tab[MC_CWU + c] = L.cwu[c];
  }
  auto up = [&](DVec<int>& d, const std::vector<int>& h) -> int {
    FC_CUDA_TRY(ctx, d.alloc(std::max<size_t>(1, h.size())));
    FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, d.p, h.data(), h.size() * sizeof(int)));
    return FC_OK;
  };
  int st = 0;
  if ((st = up(m->tab, tab)) || (st = up(m->perm, L.perm)) || (st = up(m->col, L.col)) || (st = up(m->src, L.src)) ||
      (st = up(m->tsrc, L.tsrc)) || (st = up(m->dslot, L.dslot))) {
    delete m;
    return st;
  }
  const size_t nP = std::max(1, L.nP);
  m->nent = std::max<size_t>(1, (size_t)L.nent);
  m->maxblocks = (int)mc_blocks(L.nP);
  bool ok = m->dset.alloc(nP) == cudaSuccess && m->part.alloc((size_t)2 * m->maxblocks) == cudaSuccess &&
            m->cnt.alloc(1) == cudaSuccess && m->sc.alloc(1) == cudaSuccess &&
            cudaMallocHost(&m->h_sc, sizeof(McScal)) == cudaSuccess;
  if (!ok) {
    delete m;
    return fc_fail_msg(ctx, FC_ERR_NOMEM, "multicolour buffers");
  }
  FC_CUDA_TRY(ctx, fc_zero(ctx->stream, m->cnt.p, sizeof(unsigned)));
  s->mc = m;
  return FC_OK;
}

// the buffers and the graph of value type T, on first use
template <class T>
static int mc_prepare_buf(fc_ctx* ctx, DevColoured& m, McBuf<T>& b) {
  if (b.ready) return FC_OK;
  const size_t nP = std::max(1, m.nP);
  DVec<T>* fv[] = {&b.adiag, &b.invd, &b.dvec, &b.kdiag, &b.x, &b.r, &b.p, &b.q, &b.y, &b.t, &b.w};
  bool ok = true;
  for (auto* v : fv) ok = ok && v->alloc(nP) == cudaSuccess;
  ok = ok && b.mval.alloc(m.nent) == cudaSuccess;
  if (!ok) return fc_fail_msg(ctx, FC_ERR_NOMEM, "multicolour buffers");
  // padding entries keep the value 0 (the setup writes real entries only)
  FC_CUDA_TRY(ctx, fc_zero(ctx->stream, b.mval.p, m.nent * sizeof(T)));
  int nb = 0;  // resident blocks per SM of the widest body kernel
  FC_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_e2_c0<T>, MCG_BLOCK, 0));
  b.wave = std::max(1, ctx->num_sms) * std::max(1, nb);
  int st = mc_build_graph(ctx, m, b);
  if (st) return st;
  b.ready = true;
  return FC_OK;
}

int mc_colours(fc_ctx* ctx, CsrSystem* s, int* ncol) {
  int st = mc_prepare(ctx, s);
  if (st) return st;
  *ncol = s->mc->ncol;
  return FC_OK;
}

// One FP32 inner solve A e = r64 from e = 0 to the relative L1 reduction
// tol, at most itmax iterations; x64 += e.  setup: refresh the FP32 values and
// the DILU diagonal from a (the first inner solve of a refinement loop).
template <class T>
static int mc_inner_solve_t(fc_ctx* ctx, DevColoured& m, const double* a, const double* r64, double* x64, double tol,
                            int itmax, bool setup, int* itr_out, int* status_out) {
  McBuf<T>& b = mc_buf(m, T(0));
  int st = mc_prepare_buf(ctx, m, b);
  if (st) return st;
  McDevT<T> D = mc_dev(m, b, a);
  const unsigned eb = std::min(8192u, mc_blocks(m.nP));
  k_mc_gather<<<eb, MCG_BLOCK, 0, ctx->stream>>>(D, m.perm.p, r64, tol, itmax);
  ctx->kernel_launches++;
  if (setup) {
    for (int c = 0; c < m.ncol; ++c) {
      k_mcg_setup<<<mc_blocks(m.crow[c + 1] - m.crow[c]), MCG_BLOCK, 0, ctx->stream>>>(D, c);
      ctx->kernel_launches++;
    }
  }
  FC_CUDA_TRY(ctx, cudaGetLastError());
  if (!ctx->tracing) {
    FC_CUDA_TRY(ctx, cudaGraphLaunch(b.exec, ctx->stream));
  } else {
    // diagnostic mode (fc_set_tracing): the same kernels launched from the
    // host, so that profilers see every launch; the loop checks the stop
    // flag every 32 iterations (the kernels of later iterations return at once)
    const int C = m.ncol;
    auto blocks_of = [&](int c) { return mc_blocks(m.crow[c + 1] - m.crow[c]); };
    auto body_blocks = [&](unsigned nat) { return std::min(nat, (unsigned)(MC_WAVES * b.wave)); };
    for (int c = 0; c < C; ++c) k_e_fwdb<<<blocks_of(c), MCG_BLOCK, 0, ctx->stream>>>(D, c);
    k_e_start<<<mc_blocks(m.nP), MCG_BLOCK, 0, ctx->stream>>>(D);
    for (int base = 0; base < std::max(itmax, 1); base += 32) {
      for (int k = 0; k < 32; ++k) {
        const unsigned bv = body_blocks(mc_blocks(m.nP / 4));
        if (C == 2) {
          k_e2_c0<<<body_blocks(blocks_of(0)), MCG_BLOCK, 0, ctx->stream>>>(D);
          k_e2_c1<<<body_blocks(blocks_of(1)), MCG_BLOCK, 0, ctx->stream>>>(D);
          k_e_upd<<<bv, MCG_BLOCK, 0, ctx->stream>>>(D);
          continue;
        }
        for (int c = C - 2; c >= 1; --c) k_e_bwd<<<body_blocks(blocks_of(c)), MCG_BLOCK, 0, ctx->stream>>>(D, c);
        k_e_bf0<<<body_blocks(blocks_of(0)), MCG_BLOCK, 0, ctx->stream>>>(D);
        for (int c = 1; c < C; ++c) k_e_fwd<<<body_blocks(blocks_of(c)), MCG_BLOCK, 0, ctx->stream>>>(D, c);
        k_e_upd<<<bv, MCG_BLOCK, 0, ctx->stream>>>(D);
        k_e_pupd<<<bv, MCG_BLOCK, 0, ctx->stream>>>(D);
      }
      FC_CUDA_TRY(ctx, cudaMemcpyAsync(m.h_sc, m.sc.p, sizeof(McScal), cudaMemcpyDeviceToHost, ctx->stream));
      FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      if (m.h_sc->done) break;
    }
    for (int c = C - 1; c >= 0; --c) k_e_xb<<<blocks_of(c), MCG_BLOCK, 0, ctx->stream>>>(D, c);
    FC_CUDA_TRY(ctx, cudaGetLastError());
  }
  k_mc_scatter_add<<<eb, MCG_BLOCK, 0, ctx->stream>>>(m.nP, m.perm.p, b.x.p, x64);
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(m.h_sc, m.sc.p, sizeof(McScal), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  // graph kernels: prologue C + 1, per iteration 2 C (3 for two colours; the
  // last iteration may stop early), the final backward sweep C
  ctx->kernel_launches += 2LL * m.ncol + 1 + (long long)m.h_sc->it * (m.ncol == 2 ? 3 : 2 * m.ncol);
  *itr_out = m.h_sc->it;
  *status_out = m.h_sc->status;
  return FC_OK;
}

int mc_inner_solve(fc_ctx* ctx, CsrSystem* s, const double* a, const double* r64, double* x64, double tol, int itmax,
                   bool setup, bool fp64, int* itr_out, int* status_out) {
  int st = mc_prepare(ctx, s);
  if (st) return st;
  return fp64 ? mc_inner_solve_t<double>(ctx, *s->mc, a, r64, x64, tol, itmax, setup, itr_out, status_out)
              : mc_inner_solve_t<float>(ctx, *s->mc, a, r64, x64, tol, itmax, setup, itr_out, status_out);
}
