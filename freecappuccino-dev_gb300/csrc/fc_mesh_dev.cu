// Mesh on the device: topology upload, geometry (read_mesh_native's geometry
// part, src/mesh/geometry.f90:416-665) computed by face- and cell-parallel
// kernels, and the CSR pattern with its face -> slot maps (create_CSR_matrix,
// src/sparseMatrix/sparse_matrix.f90:86-296).
//
// Deterministic by construction: every cell accumulates its faces in
// ascending face index (the order of the reference's face loops) through a
// cell -> face list, so the geometry sums are those of the reference; the
// geometry uses non-contracted FP64 arithmetic and matches the reference bit
// for bit.  The CSR rows are filled with atomics in arrival order and then
// sorted, which gives the same pattern whatever the order.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "fc_internal.hpp"
#include "fc_mesh.hpp"

namespace {

#define DM __dmul_rn
#define DA __dadd_rn
#define DS __dsub_rn
#define DD __ddiv_rn

// face area vector (triangle fan from node 1) and area-weighted centroid,
// geometry.f90:430-466 and :517-519
__global__ void k_face_geom(int nF, const int* __restrict__ nnodes, const int* __restrict__ nodes,
                            const double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
                            double* arx, double* ary, double* arz, double* xf, double* yf, double* zf) {
  const double third = 1.0 / 3.0;
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nF; f += gridDim.x * blockDim.x) {
    const int* nd = nodes + (size_t)f * FC_NOMAX;
    const int nn = nnodes[f];
    const double x1 = x[nd[0]], y1 = y[nd[0]], z1 = z[nd[0]];
    double ax = 0, ay = 0, az = 0, sx = 0, sy = 0, sz = 0, areasum = 0;
    for (int i = 0; i < nn - 2; ++i) {
      const double x2 = x[nd[i + 1]], y2 = y[nd[i + 1]], z2 = z[nd[i + 1]];
      const double x3 = x[nd[i + 2]], y3 = y[nd[i + 2]], z3 = z[nd[i + 2]];
      const double px = DS(x2, x1), py = DS(y2, y1), pz = DS(z2, z1);
      const double qx = DS(x3, x1), qy = DS(y3, y1), qz = DS(z3, z1);
      const double nx = DM(0.5, DS(DM(py, qz), DM(pz, qy)));
      const double ny = DM(0.5, DS(DM(pz, qx), DM(px, qz)));
      const double nz = DM(0.5, DS(DM(px, qy), DM(py, qx)));
      ax = DA(ax, nx); ay = DA(ay, ny); az = DA(az, nz);
      const double cx = DM(third, DA(DA(x3, x2), x1));
      const double cy = DM(third, DA(DA(y3, y2), y1));
      const double cz = DM(third, DA(DA(z3, z2), z1));
      const double are = __dsqrt_rn(DA(DA(DM(nx, nx), DM(ny, ny)), DM(nz, nz)));
      sx = DA(sx, DM(are, cx)); sy = DA(sy, DM(are, cy)); sz = DA(sz, DM(are, cz));
      areasum = DA(areasum, are);
    }
    arx[f] = ax; ary[f] = ay; arz[f] = az;
    xf[f] = DD(sx, areasum); yf[f] = DD(sy, areasum); zf[f] = DD(sz, areasum);
  }
}

// cell volume and centroid (Wang 1999 divergence formulae), geometry.f90:486-559:
// the cell's faces in ascending index, each face's triangles in order
__global__ void k_cell_geom(int nC, int nI, const int* __restrict__ cf_ptr, const int* __restrict__ cf_face,
                            const int* __restrict__ owner, const int* __restrict__ nnodes,
                            const int* __restrict__ nodes, const double* __restrict__ x,
                            const double* __restrict__ y, const double* __restrict__ z, double* xc, double* yc,
                            double* zc, double* vol) {
  const double third = 1.0 / 3.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += gridDim.x * blockDim.x) {
    double v = 0, X = 0, Y = 0, Z = 0, den = 0;
    for (int q = cf_ptr[c]; q < cf_ptr[c + 1]; ++q) {
      const int f = cf_face[q];
      const bool own = owner[f] == c;
      const int* nd = nodes + (size_t)f * FC_NOMAX;
      const int nn = nnodes[f];
      const double x1 = x[nd[0]], y1 = y[nd[0]], z1 = z[nd[0]];
      for (int i = 0; i < nn - 2; ++i) {
        const double x2 = x[nd[i + 1]], y2 = y[nd[i + 1]], z2 = z[nd[i + 1]];
        const double x3 = x[nd[i + 2]], y3 = y[nd[i + 2]], z3 = z[nd[i + 2]];
        const double px = DS(x2, x1), py = DS(y2, y1), pz = DS(z2, z1);
        const double qx = DS(x3, x1), qy = DS(y3, y1), qz = DS(z3, z1);
        const double nx = DM(0.5, DS(DM(py, qz), DM(pz, qy)));
        const double ny = DM(0.5, DS(DM(pz, qx), DM(px, qz)));
        const double nz = DM(0.5, DS(DM(px, qy), DM(py, qx)));
        const double cx = DM(third, DA(DA(x3, x2), x1));
        const double cy = DM(third, DA(DA(y3, y2), y1));
        const double cz = DM(third, DA(DA(z3, z2), z1));
        double riSi = DA(DA(DM(cx, nx), DM(cy, ny)), DM(cz, nz));
        if (!own) riSi = -riSi;
        v = DA(v, DM(third, riSi));
        X = DA(X, DM(DM(0.75, riSi), cx));
        Y = DA(Y, DM(DM(0.75, riSi), cy));
        Z = DA(Z, DM(DM(0.75, riSi), cz));
        den = DA(den, riSi);
      }
    }
    vol[c] = v;
    xc[c] = DD(X, den); yc[c] = DD(Y, den); zc[c] = DD(Z, den);
  }
  (void)nI;
}

// facint (variant 2, geometry.f90:581-603) and Df (:650-665)
__global__ void k_inner_geom(int nI, const int* __restrict__ owner, const int* __restrict__ neighbour,
                             const double* __restrict__ arx, const double* __restrict__ ary,
                             const double* __restrict__ arz, const double* __restrict__ xf,
                             const double* __restrict__ yf, const double* __restrict__ zf,
                             const double* __restrict__ xc, const double* __restrict__ yc,
                             const double* __restrict__ zc, double* facint, double* Df) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < nI; f += gridDim.x * blockDim.x) {
    const int p = owner[f], n = neighbour[f];
    double xpn = DS(xf[f], xc[p]), ypn = DS(yf[f], yc[p]), zpn = DS(zf[f], zc[p]);
    const double djp = __dsqrt_rn(DA(DA(DM(xpn, xpn), DM(ypn, ypn)), DM(zpn, zpn)));
    xpn = DS(xf[f], xc[n]); ypn = DS(yf[f], yc[n]); zpn = DS(zf[f], zc[n]);
    const double djn = __dsqrt_rn(DA(DA(DM(xpn, xpn), DM(ypn, ypn)), DM(zpn, zpn)));
    facint[f] = DD(djp, DA(djp, djn));
    xpn = DS(xc[n], xc[p]); ypn = DS(yc[n], yc[p]); zpn = DS(zc[n], zc[p]);
    const double ax = arx[f], ay = ary[f], az = arz[f];
    const double are = DA(DA(DM(ax, ax), DM(ay, ay)), DM(az, az));
    Df[f] = DD(are, DA(DA(DM(ax, xpn), DM(ay, ypn)), DM(az, zpn)));
  }
}

// dnw and srdw of the wall faces, geometry.f90:728-748
__global__ void k_wall_geom(int nwal, const int* __restrict__ wall_face, const int* __restrict__ owner,
                            const double* __restrict__ arx, const double* __restrict__ ary,
                            const double* __restrict__ arz, const double* __restrict__ xf,
                            const double* __restrict__ yf, const double* __restrict__ zf,
                            const double* __restrict__ xc, const double* __restrict__ yc,
                            const double* __restrict__ zc, double* srdw, double* dnw_out) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nwal; w += gridDim.x * blockDim.x) {
    const int f = wall_face[w], p = owner[f];
    const double ax = arx[f], ay = ary[f], az = arz[f];
    const double are = __dsqrt_rn(DA(DA(DM(ax, ax), DM(ay, ay)), DM(az, az)));
    const double nxf = DD(ax, are), nyf = DD(ay, are), nzf = DD(az, are);
    const double dnw = DA(DA(DM(DS(xf[f], xc[p]), nxf), DM(DS(yf[f], yc[p]), nyf)), DM(DS(zf[f], zc[p]), nzf));
    srdw[w] = DD(are, dnw);
    dnw_out[w] = dnw;
  }
}

// ------------------------------------------------------------ CSR pattern
// create_CSR_matrix (sparse_matrix.f90:86-296) on the device.  The links of
// the pattern are e = 0..nI-1, the inner faces (owner, neighbour), then
// e = nI..nI+nPer-1, the periodic pairs (owner of the periodic face, owner
// of its twin).  Row i of the pattern is {i} and the cell at the other end of
// every link of i, in ascending column order: the rows the reference gets by
// sorting the (row, column) pairs (sparse_matrix.f90:110-202).
__device__ __forceinline__ void link_cells(int e, int nI, const int* __restrict__ owner,
                                           const int* __restrict__ neighbour, const int* __restrict__ pface,
                                           const int* __restrict__ ptwin, int& i, int& j) {
  if (e < nI) {
    i = owner[e];
    j = neighbour[e];
  } else {
    i = owner[pface[e - nI]];
    j = owner[ptwin[e - nI]];
  }
}

// off-diagonal entries per row
__global__ void k_csr_count(int nL, int nI, const int* __restrict__ owner, const int* __restrict__ neighbour,
                            const int* __restrict__ pface, const int* __restrict__ ptwin, int* cnt) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nL; e += gridDim.x * blockDim.x) {
    int i, j;
    link_cells(e, nI, owner, neighbour, pface, ptwin, i, j);
    atomicAdd(&cnt[i], 1);
    atomicAdd(&cnt[j], 1);
  }
}

// exclusive scan of the row lengths cnt[c] + 1 (c < n) and 0 (c = n) into
// ia[0..n], in three passes: block scans with block totals, a scan of the
// totals, the totals added back
constexpr int SCAN_TB = 1024;

__device__ __forceinline__ int block_exclusive_scan(int v, int* s_w, int& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int w = lane < (int)(blockDim.x >> 5) ? s_w[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    s_w[lane] = w;  // inclusive warp totals
  }
  __syncthreads();
  total = s_w[(blockDim.x >> 5) - 1];
  const int r = x - v + (wid > 0 ? s_w[wid - 1] : 0);
  __syncthreads();
  return r;
}

__global__ void __launch_bounds__(SCAN_TB) k_csr_scan_rows(int n, const int* __restrict__ cnt, int* ia, int* bsum) {
  __shared__ int s_w[32];
  const int c = blockIdx.x * SCAN_TB + threadIdx.x;
  const int v = c < n ? cnt[c] + 1 : 0;
  int total;
  const int r = block_exclusive_scan(v, s_w, total);
  if (c <= n) ia[c] = r;
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

// one block: the block totals scanned in place (exclusive), in chunks
__global__ void __launch_bounds__(SCAN_TB) k_csr_scan_totals(int nb, int* bsum) {
  __shared__ int s_w[32];
  int carry = 0;
  for (int base = 0; base < nb; base += SCAN_TB) {
    const int b = base + threadIdx.x;
    const int v = b < nb ? bsum[b] : 0;
    int total;
    const int r = block_exclusive_scan(v, s_w, total);
    if (b < nb) bsum[b] = carry + r;
    carry += total;
  }
}

__global__ void __launch_bounds__(SCAN_TB) k_csr_scan_add(int n, const int* __restrict__ bsum, int* ia) {
  const int c = blockIdx.x * SCAN_TB + threadIdx.x;
  if (c <= n) ia[c] += bsum[blockIdx.x];
}

// the diagonal first in every row, the other ends of the links after it in
// arrival order (sorted next)
__global__ void k_csr_fill(int nC, int nL, int nI, const int* __restrict__ owner, const int* __restrict__ neighbour,
                           const int* __restrict__ pface, const int* __restrict__ ptwin, const int* __restrict__ ia,
                           int* pos, int* ja) {
  const int stride = gridDim.x * blockDim.x;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += stride) ja[ia[c]] = c;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nL; e += stride) {
    int i, j;
    link_cells(e, nI, owner, neighbour, pface, ptwin, i, j);
    ja[ia[i] + 1 + atomicAdd(&pos[i], 1)] = j;
    ja[ia[j] + 1 + atomicAdd(&pos[j], 1)] = i;
  }
}

// every row sorted (insertion sort: rows hold a cell's neighbours); a column
// repeated in a row (two cells coupled twice) sets bit 0 of *flag; diag[c]
// is the slot of column c in row c
__global__ void k_csr_sort(int nC, const int* __restrict__ ia, int* ja, int* diag, int* flag) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += gridDim.x * blockDim.x) {
    const int b = ia[c], e = ia[c + 1];
    for (int k = b + 1; k < e; ++k) {
      const int v = ja[k];
      int l = k - 1;
      while (l >= b && ja[l] > v) {
        ja[l + 1] = ja[l];
        --l;
      }
      ja[l + 1] = v;
    }
    int d = -1;
    for (int k = b; k < e; ++k) {
      if (k > b && ja[k] == ja[k - 1]) atomicOr(flag, 1);
      if (ja[k] == c) d = k;
    }
    diag[c] = d;
  }
}

// face -> slot maps, csr_to_k (utils.f90:96-147): the first slot of row i
// holding column j, for (owner, neighbour) and (neighbour, owner) of every
// link (sparse_matrix.f90:205-292)
__device__ __forceinline__ int csr_slot(const int* __restrict__ ia, const int* __restrict__ ja, int i, int j) {
  int lo = ia[i], hi = ia[i + 1] - 1;  // columns strictly increasing
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (ja[mid] < j) lo = mid + 1; else hi = mid;
  }
  return ja[lo] == j ? lo : -1;
}

__global__ void k_csr_slots(int nL, int nI, const int* __restrict__ owner, const int* __restrict__ neighbour,
                            const int* __restrict__ pface, const int* __restrict__ ptwin, const int* __restrict__ ia,
                            const int* __restrict__ ja, int* ijk, int* jik) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < nL; e += gridDim.x * blockDim.x) {
    int i, j;
    link_cells(e, nI, owner, neighbour, pface, ptwin, i, j);
    ijk[e] = csr_slot(ia, ja, i, j);
    jik[e] = csr_slot(ia, ja, j, i);
  }
}

}  // namespace

static void free_mesh_dev(MeshDev& m) {
  DVec<double>* dv[] = {&m.x, &m.y, &m.z, &m.arx, &m.ary, &m.arz, &m.xf, &m.yf, &m.zf,
                        &m.xc, &m.yc, &m.zc, &m.vol, &m.facint, &m.Df, &m.srdw, &m.dnw};
  for (auto* v : dv) v->release();
  DVec<int>* iv[] = {&m.nnodes, &m.nodes, &m.owner, &m.neighbour, &m.bface_patch, &m.bface_wall,
                     &m.cf_ptr, &m.cf_face, &m.ijk, &m.jik, &m.wall_face, &m.pface, &m.ptwin,
                     &m.ppos, &m.pflag, &m.bpair, &m.af_ptr, &m.af_ent};
  for (auto* v : iv) v->release();
  m.nPer = 0;
  m.h_owner.clear(); m.h_neighbour.clear(); m.h_xyz.clear();
}

void fc_release_mesh(fc_ctx* ctx) {
  if (!ctx) return;
  free_mesh_dev(ctx->mesh);
  ctx->has_mesh = false;
}

template <class T>
static int up(fc_ctx* ctx, DVec<T>& d, const T* h, size_t n) {
  FC_CUDA_TRY(ctx, d.alloc(n));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, d.p, h, n * sizeof(T)));
  return FC_OK;
}

#define UP(dst, src, cnt) do { int _s = up(ctx, dst, src, cnt); if (_s) return _s; } while (0)

// wall-clock time of the set-up phases: lap() waits for the stream, adds the
// time since the previous lap to the phase and starts the next one
struct PhaseClock {
  fc_ctx* ctx;
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  explicit PhaseClock(fc_ctx* c) : ctx(c) {
    for (double& v : ctx->setup_s) v = 0.0;
  }
  int lap(int phase) {
    FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    const auto now = std::chrono::steady_clock::now();
    ctx->setup_s[phase] += std::chrono::duration<double>(now - t).count();
    t = now;
    return FC_OK;
  }
};
#define FC_TRY(call) do { int _s = (call); if (_s) return _s; } while (0)

// Build everything the path needs from the host mesh.  Host work is the
// one-time topology bookkeeping (cell -> face lists, the periodic face
// mapping) and the sweep schedule of the global matrix; the geometry, the
// CSR pattern and its slot maps are computed on the device.
extern "C" int fc_set_mesh(fc_ctx* ctx, const fc_mesh* hm) {
  FC_RANGE();
  if (!ctx || !hm) return FC_ERR_BAD_INPUT;
  PhaseClock clk(ctx);
  std::string why;
  if (hm->validate(&why, true) != FC_OK) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_set_mesh: " + why);
  cudaSetDevice(ctx->device);
  fc_release_mesh(ctx);
  delete ctx->sys_mesh;
  ctx->sys_mesh = nullptr;
  MeshDev& m = ctx->mesh;
  const int nN = hm->numNodes, nC = hm->numCells, nI = hm->numInnerFaces, nB = hm->numBoundaryFaces;
  const int nF = nI + nB;
  m.numNodes = nN; m.numCells = nC; m.numInnerFaces = nI; m.numBoundaryFaces = nB; m.numFaces = nF;
  m.numTotal = nC + nB;
  m.numBoundaries = (int)hm->bctype.size();
  m.h_bctype = hm->bctype; m.h_nfaces = hm->nfaces; m.h_startFace = hm->startFace;
  // 0-based topology
  std::vector<int> owner(nF), neighbour(nI), nodes((size_t)nF * FC_NOMAX, 0);
  for (int f = 0; f < nF; ++f) {
    owner[f] = hm->owner[f] - 1;
    for (int k = 0; k < hm->nnodes[f]; ++k) nodes[(size_t)f * FC_NOMAX + k] = hm->nodes[(size_t)f * FC_NOMAX + k] - 1;
  }
  for (int f = 0; f < nI; ++f) neighbour[f] = hm->neighbour[f] - 1;
  // cell -> faces, ascending face index
  std::vector<int> cf_ptr, cf_face;
  auto cell_faces = [&]() {
    cf_ptr.assign(nC + 1, 0);
    for (int f = 0; f < nF; ++f) {
      cf_ptr[owner[f] + 1]++;
      if (f < nI) cf_ptr[neighbour[f] + 1]++;
    }
    for (int c = 0; c < nC; ++c) cf_ptr[c + 1] += cf_ptr[c];
    cf_face.assign(cf_ptr[nC], 0);
    std::vector<int> pos(cf_ptr.begin(), cf_ptr.end() - 1);
    for (int f = 0; f < nF; ++f) {  // f ascending -> lists come out sorted
      cf_face[pos[owner[f]]++] = f;
      if (f < nI) cf_face[pos[neighbour[f]]++] = f;
    }
  };
  cell_faces();
  // boundary face -> patch, wall counter
  std::vector<int> bpatch(nB, -1), bwall(nB, -1), wall_face;
  int iwall = 0;
  m.nwal = m.nsym = 0;
  for (int b = 0; b < m.numBoundaries; ++b) {
    for (int i = 0; i < hm->nfaces[b]; ++i) {
      int f = hm->startFace[b] + i - nI;
      bpatch[f] = b;
      if (hm->bctype[b] == FC_BC_WALL) { bwall[f] = iwall++; wall_face.push_back(nI + f); }
    }
    if (hm->bctype[b] == FC_BC_WALL) m.nwal += hm->nfaces[b];
    if (hm->bctype[b] == FC_BC_SYMMETRY) m.nsym += hm->nfaces[b];
  }
  UP(m.x, hm->x.data(), nN); UP(m.y, hm->y.data(), nN); UP(m.z, hm->z.data(), nN);
  UP(m.nnodes, hm->nnodes.data(), nF);
  UP(m.nodes, nodes.data(), nodes.size());
  UP(m.owner, owner.data(), nF);
  UP(m.neighbour, neighbour.data(), nI);
  UP(m.cf_ptr, cf_ptr.data(), cf_ptr.size());
  UP(m.cf_face, cf_face.data(), cf_face.size());
  UP(m.bface_patch, bpatch.data(), nB);
  UP(m.bface_wall, bwall.data(), nB);
  UP(m.wall_face, wall_face.data(), wall_face.size());
  DVec<double>* fv[] = {&m.arx, &m.ary, &m.arz, &m.xf, &m.yf, &m.zf};
  for (auto* v : fv) FC_CUDA_TRY(ctx, v->alloc(nF));
  DVec<double>* cv[] = {&m.xc, &m.yc, &m.zc, &m.vol};
  for (auto* v : cv) FC_CUDA_TRY(ctx, v->alloc(nC));
  FC_CUDA_TRY(ctx, m.facint.alloc(nI));
  FC_CUDA_TRY(ctx, m.Df.alloc(nI));
  FC_TRY(clk.lap(FC_SETUP_TOPOLOGY));
  const int TB = 256;
  auto grid = [&](int n) { return std::max(1, std::min(65535, (n + TB - 1) / TB)); };
  k_face_geom<<<grid(nF), TB, 0, ctx->stream>>>(nF, m.nnodes.p, m.nodes.p, m.x.p, m.y.p, m.z.p, m.arx.p, m.ary.p,
                                                 m.arz.p, m.xf.p, m.yf.p, m.zf.p);
  k_cell_geom<<<grid(nC), TB, 0, ctx->stream>>>(nC, nI, m.cf_ptr.p, m.cf_face.p, m.owner.p, m.nnodes.p, m.nodes.p,
                                                 m.x.p, m.y.p, m.z.p, m.xc.p, m.yc.p, m.zc.p, m.vol.p);
  if (nI > 0)
    k_inner_geom<<<grid(nI), TB, 0, ctx->stream>>>(nI, m.owner.p, m.neighbour.p, m.arx.p, m.ary.p, m.arz.p, m.xf.p,
                                                    m.yf.p, m.zf.p, m.xc.p, m.yc.p, m.zc.p, m.facint.p, m.Df.p);
  ctx->kernel_launches += 3;
  FC_CUDA_TRY(ctx, m.srdw.alloc(m.nwal));
  FC_CUDA_TRY(ctx, m.dnw.alloc(m.nwal));
  if (m.nwal > 0) {
    k_wall_geom<<<grid(m.nwal), TB, 0, ctx->stream>>>(m.nwal, m.wall_face.p, m.owner.p, m.arx.p, m.ary.p, m.arz.p,
                                                      m.xf.p, m.yf.p, m.zf.p, m.xc.p, m.yc.p, m.zc.p, m.srdw.p,
                                                      m.dnw.p);
    ctx->kernel_launches++;
  }
  FC_CUDA_TRY(ctx, cudaGetLastError());
  FC_TRY(clk.lap(FC_SETUP_GEOMETRY));
  m.h_xyz.resize((size_t)3 * nC);
  FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, m.h_xyz.data(), m.xc.p, nC * sizeof(double)));
  FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, m.h_xyz.data() + nC, m.yc.p, nC * sizeof(double)));
  FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, m.h_xyz.data() + 2 * (size_t)nC, m.zc.p, nC * sizeof(double)));
  // periodic pairs, face_mapping (geometry.f90:1848-1997), after the
  // geometry as there: face i of a periodic patch pairs with the twin face
  // whose owner's centre is nearest (L1) to face i's centre, first of equals;
  // the twin faces' owners, centres and area vectors are then reordered so
  // that twin face i belongs to pair i
  std::vector<int> pface, ptwin, ppos, pflag, bpair(nB, -1);
  for (int b = 0; b < m.numBoundaries; ++b) {
    if (hm->bctype[b] != FC_BC_PERIODIC) continue;
    if (pface.empty()) {
      std::vector<double> h((size_t)6 * nF);
      for (int k = 0; k < 6; ++k) FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, h.data() + (size_t)k * nF, fv[k]->p, nF * sizeof(double)));
      m.h_face.swap(h);
    }
    const double* xc = m.h_xyz.data();
    const double *yc = xc + nC, *zc = xc + 2 * (size_t)nC;
    const double *hxf = m.h_face.data() + 3 * (size_t)nF, *hyf = hxf + nF, *hzf = hxf + 2 * (size_t)nF;
    const int n = hm->nfaces[b], sf = hm->startFace[b], tw = hm->twin_of(b);
    int tp = 0;
    while (hm->startFace[tp] != tw) ++tp;  // validated: the twin patch exists
    std::vector<int> tmp(n), itmp(n), hit(n, 0);
    for (int i = 0; i < n; ++i) {
      const int f = sf + i;
      double mindist = (double)1e+30f;
      int best = 0;
      for (int it = 0; it < n; ++it) {
        const int c = owner[tw + it];
        const double dist = std::fabs(hxf[f] - xc[c]) + std::fabs(hyf[f] - yc[c]) + std::fabs(hzf[f] - zc[c]);
        if (dist < mindist) { mindist = dist; best = it; }
      }
      itmp[i] = best;
      tmp[i] = owner[tw + best];
      if (hit[best]++) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_set_mesh: periodic face mapping is not one to one");
    }
    for (int i = 0; i < n; ++i) owner[tw + i] = tmp[i];
    for (int k = 0; k < 6; ++k) {
      double* v = m.h_face.data() + (size_t)k * nF;
      std::vector<double> vt(n);
      for (int i = 0; i < n; ++i) vt[i] = v[tw + itmp[i]];
      for (int i = 0; i < n; ++i) v[tw + i] = vt[i];
    }
    for (int i = 0; i < n; ++i) {
      const int q = (int)pface.size();
      pface.push_back(sf + i);
      ptwin.push_back(tw + i);
      ppos.push_back(i);
      pflag.push_back(tp < b ? 1 : 0);
      bpair[sf + i - nI] = q;
      bpair[tw + i - nI] = q;
      if (owner[sf + i] == owner[tw + i])
        return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "fc_set_mesh: a periodic pair couples a cell with itself");
    }
  }
  const int nPer = (int)pface.size();
  m.nPer = nPer;
  if (nPer > 0) {
    for (int k = 0; k < 6; ++k)
      FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, fv[k]->p, m.h_face.data() + (size_t)k * nF, nF * sizeof(double)));
    m.h_face.clear();
    m.h_face.shrink_to_fit();
    FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, m.owner.p, owner.data(), nF * sizeof(int)));
    cell_faces();  // the twin faces moved to their pairs' cells
    FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, m.cf_ptr.p, cf_ptr.data(), cf_ptr.size() * sizeof(int)));
    FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, m.cf_face.p, cf_face.data(), cf_face.size() * sizeof(int)));
  }
  if (nPer > 0) {
    UP(m.pface, pface.data(), nPer);
    UP(m.ptwin, ptwin.data(), nPer);
  }
  FC_TRY(clk.lap(FC_SETUP_PERIODIC));
  // CSR pattern and slot maps on the device (the kernels above); a cell
  // pair coupled twice (an inner face and a periodic pair, or two faces)
  // would make a repeated column, which is rejected
  const int nL = nI + nPer;
  if (2LL * nL + nC >= (1LL << 31)) return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "fc_set_mesh: nnz >= 2^31");
  const int nnz = 2 * nL + nC;
  const int nb = (nC + 1 + SCAN_TB - 1) / SCAN_TB;
  std::vector<int> ia(nC + 1), ja(nnz), diag(nC);
  {
    DVec<int> cnt, bsum, d_ia, d_ja, d_dg, flag;
    FC_CUDA_TRY(ctx, cnt.alloc(nC));
    FC_CUDA_TRY(ctx, bsum.alloc(nb));
    FC_CUDA_TRY(ctx, d_ia.alloc(nC + 1));
    FC_CUDA_TRY(ctx, d_ja.alloc(nnz));
    FC_CUDA_TRY(ctx, d_dg.alloc(nC));
    FC_CUDA_TRY(ctx, flag.alloc(1));
    FC_CUDA_TRY(ctx, m.ijk.alloc(std::max(1, nL)));
    FC_CUDA_TRY(ctx, m.jik.alloc(std::max(1, nL)));
    FC_CUDA_TRY(ctx, fc_zero(ctx->stream, cnt.p, cnt.bytes()));
    FC_CUDA_TRY(ctx, fc_zero(ctx->stream, flag.p, flag.bytes()));
    const int* pf = nPer ? m.pface.p : nullptr;
    const int* pt = nPer ? m.ptwin.p : nullptr;
    if (nL > 0) k_csr_count<<<grid(nL), TB, 0, ctx->stream>>>(nL, nI, m.owner.p, m.neighbour.p, pf, pt, cnt.p);
    k_csr_scan_rows<<<nb, SCAN_TB, 0, ctx->stream>>>(nC, cnt.p, d_ia.p, bsum.p);
    k_csr_scan_totals<<<1, SCAN_TB, 0, ctx->stream>>>(nb, bsum.p);
    k_csr_scan_add<<<nb, SCAN_TB, 0, ctx->stream>>>(nC, bsum.p, d_ia.p);
    FC_CUDA_TRY(ctx, fc_zero(ctx->stream, cnt.p, cnt.bytes()));
    k_csr_fill<<<grid(std::max(nC, nL)), TB, 0, ctx->stream>>>(nC, nL, nI, m.owner.p, m.neighbour.p, pf, pt, d_ia.p,
                                                               cnt.p, d_ja.p);
    k_csr_sort<<<grid(nC), TB, 0, ctx->stream>>>(nC, d_ia.p, d_ja.p, d_dg.p, flag.p);
    if (nL > 0)
      k_csr_slots<<<grid(nL), TB, 0, ctx->stream>>>(nL, nI, m.owner.p, m.neighbour.p, pf, pt, d_ia.p, d_ja.p,
                                                    m.ijk.p, m.jik.p);
    ctx->kernel_launches += 6 + 2 * (nL > 0);
    FC_CUDA_TRY(ctx, cudaGetLastError());
    int hflag = 0;
    FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, &hflag, flag.p, sizeof(int)));
    if (hflag)
      return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "fc_set_mesh: two cells coupled twice (an inner face and a "
                                                  "periodic pair, or two faces)");
    FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, ia.data(), d_ia.p, ia.size() * sizeof(int)));
    FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, ja.data(), d_ja.p, ja.size() * sizeof(int)));
    FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, diag.data(), d_dg.p, diag.size() * sizeof(int)));
  }
  if (ia[nC] != nnz) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_set_mesh: inconsistent face lists");
  FC_TRY(clk.lap(FC_SETUP_CSR));
  if (nPer > 0) {
    // the assembly lists: a twin face leaves its cell's list, the pair
    // enters the twin-side cell's list at the periodic face's place
    std::vector<int> af_ptr(nC + 1, 0), af_ent;
    af_ent.reserve(cf_face.size());
    std::vector<std::vector<int>> tside(nC);
    for (int q = 0; q < nPer; ++q) tside[owner[ptwin[q]]].push_back(q);
    std::vector<int> row;
    auto key = [&](int e) { return e < nF ? e : pface[e - nF]; };
    for (int c = 0; c < nC; ++c) {
      row.clear();
      for (int q = cf_ptr[c]; q < cf_ptr[c + 1]; ++q) {
        const int f = cf_face[q];
        if (f >= nI && bpair[f - nI] >= 0 && ptwin[bpair[f - nI]] == f) continue;
        row.push_back(f);
      }
      for (int q : tside[c]) row.push_back(nF + q);
      std::stable_sort(row.begin(), row.end(), [&](int a, int b) { return key(a) < key(b); });
      af_ent.insert(af_ent.end(), row.begin(), row.end());
      af_ptr[c + 1] = (int)af_ent.size();
    }
    UP(m.af_ptr, af_ptr.data(), af_ptr.size());
    UP(m.af_ent, af_ent.data(), af_ent.size());
    UP(m.ppos, ppos.data(), nPer);
    UP(m.pflag, pflag.data(), nPer);
  }
  UP(m.bpair, bpair.data(), nB);
  m.h_owner = owner;
  m.h_neighbour = neighbour;
  FC_TRY(clk.lap(FC_SETUP_PERIODIC));
  // the global matrix system of the mesh (module globals ia, ja, a, diag)
  CsrSystem* s = new CsrSystem();
  std::vector<int> ia1(ia), ja1(ja), dg1(diag);
  for (auto& v : ia1) ++v;
  for (auto& v : ja1) ++v;
  for (auto& v : dg1) ++v;
  int st = sys_set_pattern(ctx, s, nC, nnz, ia1.data(), ja1.data(), dg1.data(), m.h_xyz.data());
  if (st) { delete s; return st; }
  FC_CUDA_TRY(ctx, fc_zero(ctx->stream, s->a.p, (size_t)nnz * sizeof(double)));
  ctx->sys_mesh = s;
  ctx->has_mesh = true;
  ctx->mesh_gen++;
  FC_TRY(clk.lap(FC_SETUP_ANALYSIS));
  ctx->setup_s[FC_SETUP_TILING] = s->t_tiling;
  ctx->setup_s[FC_SETUP_SCHEDULE] = s->t_schedule;
  ctx->setup_s[FC_SETUP_ANALYSIS] = std::max(0.0, ctx->setup_s[FC_SETUP_ANALYSIS] - s->t_tiling - s->t_schedule);
  FC_TRY(fc_fields_alloc(ctx));
  return clk.lap(FC_SETUP_FIELDS);
}

extern "C" int fc_get_setup_times(fc_ctx* ctx, double* seconds) {
  if (!ctx || !seconds) return FC_ERR_BAD_INPUT;
  for (int k = 0; k < FC_SETUP_PHASES; ++k) seconds[k] = ctx->setup_s[k];
  return FC_OK;
}

// geometry arrays back to the host (FC_GEO_* selects; length by kind)
extern "C" int fc_get_geometry(fc_ctx* ctx, const char* name, double* out) {
  if (!ctx || !name || !out) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  MeshDev& m = ctx->mesh;
  std::string n(name);
  DVec<double>* v = nullptr;
  if (n == "arx") v = &m.arx; else if (n == "ary") v = &m.ary; else if (n == "arz") v = &m.arz;
  else if (n == "xf") v = &m.xf; else if (n == "yf") v = &m.yf; else if (n == "zf") v = &m.zf;
  else if (n == "xc") v = &m.xc; else if (n == "yc") v = &m.yc; else if (n == "zc") v = &m.zc;
  else if (n == "vol") v = &m.vol; else if (n == "facint") v = &m.facint; else if (n == "Df") v = &m.Df;
  else if (n == "srdw") v = &m.srdw;
  else if (n == "dnw") v = &m.dnw;
  else return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "unknown geometry array '" + n + "'");
  FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, out, v->p, v->bytes()));
  return FC_OK;
}

// CSR pattern and face -> slot maps of the mesh, 1-based as the reference
// stores them (ia(n+1), ja(nnz), diag(n), icell_jcell_csr_index(nI + nPer),
// jcell_icell_csr_index(nI + nPer): the inner faces, then the periodic
// pairs); any pointer may be NULL
extern "C" int fc_get_csr_pattern(fc_ctx* ctx, int* n_out, int* nnz_out, int* ia, int* ja, int* diag, int* ijk,
                                  int* jik) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh || !ctx->sys_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  CsrSystem* s = ctx->sys_mesh;
  if (n_out) *n_out = s->n;
  if (nnz_out) *nnz_out = s->nnz;
  if (ia) for (int i = 0; i <= s->n; ++i) ia[i] = s->h_ia[i] + 1;
  if (ja) for (int k = 0; k < s->nnz; ++k) ja[k] = s->h_ja[k] + 1;
  if (diag) for (int i = 0; i < s->n; ++i) diag[i] = s->h_diag[i] + 1;
  const int nI = ctx->mesh.numInnerFaces + ctx->mesh.nPer;
  if (ijk || jik) {
    std::vector<int> t(nI);
    if (ijk) {
      FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, t.data(), ctx->mesh.ijk.p, nI * sizeof(int)));
      for (int f = 0; f < nI; ++f) ijk[f] = t[f] + 1;
    }
    if (jik) {
      FC_CUDA_TRY(ctx, fc_d2h(ctx->stream, t.data(), ctx->mesh.jik.p, nI * sizeof(int)));
      for (int f = 0; f < nI; ++f) jik[f] = t[f] + 1;
    }
  }
  return FC_OK;
}
