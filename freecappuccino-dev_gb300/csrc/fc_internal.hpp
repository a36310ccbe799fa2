// Internal declarations of the GB300 library: device buffers, the context,
// the CSR system (pattern analysis + solver workspace) and the mesh on device.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "fc_gpu.h"

// Single-precision literals of the reference, promoted to double
// (parameters.f90:6 small = 1e-20, linear_solvers.f90:447 s0 = 1.e20).
constexpr double FC_SMALL = static_cast<double>(1e-20f);
constexpr double FC_S0 = static_cast<double>(1.e20f);

#define FC_CUDA_TRY(ctx, expr)                                                  \
  do {                                                                          \
    cudaError_t _e = (expr);                                                    \
    if (_e != cudaSuccess) return fc_fail((ctx), FC_ERR_CUDA, #expr, _e);       \
  } while (0)

// Copies and fills of the library are ordered on the context's stream.  That
// stream is created non-blocking, so work that cudaMemcpy and cudaMemset put
// on the legacy default stream would not be ordered against the library's
// kernels.  A pageable host source is staged before fc_h2d returns, so it may
// be freed at once; fc_d2h waits for the copy.
inline cudaError_t fc_h2d(cudaStream_t s, void* dst, const void* src, size_t bytes) {
  return bytes ? cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) : cudaSuccess;
}
inline cudaError_t fc_d2h(cudaStream_t s, void* dst, const void* src, size_t bytes) {
  if (!bytes) return cudaSuccess;
  cudaError_t e = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, s);
  return e != cudaSuccess ? e : cudaStreamSynchronize(s);
}
inline cudaError_t fc_zero(cudaStream_t s, void* dst, size_t bytes) {
  return bytes ? cudaMemsetAsync(dst, 0, bytes, s) : cudaSuccess;
}

// Count of the library's device allocations and frees (every device buffer
// goes through DVec), read by fc_device_alloc_count.
void fc_count_device_alloc();
// byte every new device allocation is filled with, or -1 (fc_debug_fill_allocations)
int fc_alloc_fill();

template <class T>
struct DVec {
  T* p = nullptr;
  size_t n = 0;
  DVec() = default;
  DVec(const DVec&) = delete;
  DVec& operator=(const DVec&) = delete;
  ~DVec() { release(); }
  cudaError_t alloc(size_t count) {
    if (count == n && p) return cudaSuccess;
    release();
    if (count == 0) return cudaSuccess;
    fc_count_device_alloc();
    cudaError_t e = cudaMalloc(&p, count * sizeof(T));
    if (e != cudaSuccess) {
      p = nullptr;
      return e;
    }
    n = count;
    const int fill = fc_alloc_fill();
    if (fill >= 0) {
      // synchronous: done before any stream of the library can use the buffer
      e = cudaMemset(p, fill, count * sizeof(T));
      if (e == cudaSuccess) e = cudaDeviceSynchronize();
    }
    return e;
  }
  void release() {
    if (p) { fc_count_device_alloc(); cudaFree(p); }
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Cross-block control block of the persistent solver kernels: a bounded
// generation barrier, per-block partial sums and a sticky status word.
struct GridCtl {
  unsigned* bar = nullptr;     // [0] arrival count, [1] generation
  double* part = nullptr;      // nblocks * FC_NPART partial sums
  int* status = nullptr;       // 0 or a negative FC_* code (first error sticks)
  double* out = nullptr;       // scalar results written by block 0 (FC_OUT_*)
  // the blocks the kernel runs on: [base, base + nb) of the launch grid
  // (nb = 0: the whole grid).  A batched launch gives every problem its own
  // group of blocks, barrier and partial sums.
  int base = 0, nb = 0;
};
#define FC_NPART 4
// FC_OUT_GT: device time of a batched group (ns, written by its first block)
enum { FC_OUT_RES0 = 0, FC_OUT_RESL, FC_OUT_FACTOR, FC_OUT_RESOR, FC_OUT_ITR, FC_OUT_EARLY, FC_OUT_BAD, FC_OUT_GT,
       FC_OUT_N = 16 };

// device copy of a schedule-ordered sweep structure (fc_schedule.hpp)
struct DevOrdered {
  int n = 0, nE = 0, ntiles = 0, nsteps = 0, nlev = 0, R = 4, K = 1, maxW = 0, max_tile_steps = 0;
  size_t stage_area = 0;             // shared memory of the sweeps' stage buffers; K: buffers of an application
  int xmax = 4, pmax = 4;            // largest exchange / push block of a step
  bool gs_ok = false;                // the Gauss-Seidel mode gets two stage buffers
  int Wc = 0;                        // staged rows of a step (0: whole steps are staged)
  int novf[2] = {0, 0}, nxv[2] = {0, 0};
  DVec<int> tile_step_ptr, step_ptr, tile_W, perm;
  DVec<int> srec[2], xv_ptr[2], push_ptr[2], push[2], slot[2], ucol;
  DVec<int> ovf_ptr[2], ovf_code[2], ovf_col[2], ovf_slot[2];
  DVec<int> lo_tslot, lo_ovf_tslot, dslot, p_ptr, p_col, p_slot;
  long long ring_entries = 0, pushed_entries = 0, cross_tile_entries = 0;
};

// per-solve values of an ordered system in one precision (fc_sweep.cuh OrdVals)
template <class T>
struct OrdStore {
  DVec<T> vrec0, vrec1, sx, aovf0, aovf1, tovf, adiag, ap, xv0, xv1, xo, bo;
};

struct LevelSchedule {
  int nlev = 0;
  int max_width = 0;
  std::vector<int> h_ptr, h_rows;
  DVec<int> ptr, rows;
};

// A square CSR system on the device plus everything the solvers need.
struct DevColoured;                  // multicolour layout of the mixed-precision inner solve (fc_mc.cu)
void mc_release(DevColoured* m);

struct CsrSystem {
  int n = 0, nnz = 0;
  DVec<int> ia, ja, diag, tslot;     // 0-based; tslot = transpose slot (DILU search)
  bool tslot_oob = false;            // some DILU search ran past its row (non-symmetric pattern)
  DVec<double> a;
  DVec<float> a32;
  LevelSchedule lf, lb;              // forward (lower) and backward (upper) level sets (ILU(0))
  DevOrdered ord;                    // schedule-ordered sweep structure (DIC/DILU/Gauss-Seidel)
  OrdStore<double> o64;
  OrdStore<float> o32;
  double est_sweep_us = 0.0;         // critical-path estimate of the forward sweep
  double t_tiling = 0.0, t_schedule = 0.0;  // seconds of the tile-count choice and of the ordered sweep build
  const double* xyz_src = nullptr;   // row coordinates the tiles were cut with (the mesh's, or none)
  DevColoured* mc = nullptr;         // built on the first FC_PREC_MIXED_COLOURED solve
  // workspace
  DVec<double> x, b, r, r0, p, u, z, v, d, w;
  DVec<float> fr, fr0, fp, fu, fz, fv, fd, fx, fy, fw;
  DVec<double> part, out;
  DVec<unsigned> bar;
  DVec<int> status;
  double* h_out = nullptr;           // pinned FC_OUT_N doubles
  int* h_status = nullptr;
  // identity of an externally supplied pattern (fc_csrsolve cache)
  const void* key_ia = nullptr; const void* key_ja = nullptr; const void* key_diag = nullptr;
  std::vector<int> h_ia, h_ja, h_diag;  // 0-based host copies
  DVec<int> tptr, tsrc, trow;        // transpose (column-major) view, built on demand
  ~CsrSystem();
};

// Mesh topology and geometry resident on the device (SoA, 0-based).
struct MeshDev {
  int numNodes = 0, numCells = 0, numInnerFaces = 0, numBoundaryFaces = 0, numFaces = 0, numTotal = 0;
  int numBoundaries = 0, nwal = 0, nsym = 0;
  std::vector<int> h_bctype, h_nfaces, h_startFace;  // per patch; startFace 0-based face offset
  DVec<double> x, y, z;
  DVec<int> nnodes, nodes;                 // nodes: numFaces*FC_NOMAX, 0-based node ids
  DVec<int> owner, neighbour;              // 0-based cells
  DVec<int> bface_patch;                   // patch index of every boundary face
  DVec<int> bface_wall;                    // running wall-face counter (iWall-1) or -1
  DVec<int> wall_face;                     // face index of every wall face, in wall-counter order
  DVec<double> srdw;                       // |S| / normal distance per wall face (nwal)
  DVec<double> dnw;                        // normal distance of the owner's centre per wall face (nwal)
  DVec<int> cf_ptr, cf_face;               // cell -> faces (ascending face index)
  DVec<double> arx, ary, arz, xf, yf, zf;  // numFaces
  DVec<double> xc, yc, zc, vol;            // numCells
  DVec<double> facint, Df;                 // numInnerFaces
  DVec<int> ijk, jik;                      // face -> CSR slot (0-based); pairs after the inner faces
  // periodic pairs q = 0..nPer-1 in the order of the reference's pair loops
  // (periodic patches in order, faces in order): the periodic face, its
  // twin face, the face's position in its patch, 1 when the twin patch
  // comes before the periodic one; per boundary face the pair it belongs to
  // (periodic or twin side) or -1
  int nPer = 0;
  DVec<int> pface, ptwin, ppos, pflag, bpair;
  // per cell, the faces the assembly loops visit, in the reference's order:
  // the cell -> face list without twin faces, with nF + q for a cell on the
  // twin side of pair q placed where the periodic face's patch is visited;
  // the cell -> face list itself when the mesh has no periodic pairs
  DVec<int> af_ptr, af_ent;
  std::vector<int> h_owner, h_neighbour;
  std::vector<double> h_xyz;               // cell centroids x..., y..., z... (sweep tiling)
  std::vector<double> h_face;              // face arrays during the periodic face mapping
};

struct FieldStore;
struct SimpleState;
struct AdjState;

// NVTX range over a C-ABI call, named after the function (shown by Nsight
// timelines; a no-op when no tool is attached)
struct FcRange {
  explicit FcRange(const char* name) { nvtxRangePushA(name); }
  ~FcRange() { nvtxRangePop(); }
  FcRange(const FcRange&) = delete;
  FcRange& operator=(const FcRange&) = delete;
};
#define FC_RANGE() FcRange fc_range_guard_(__func__)

struct fc_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;    // the caller's pair (fc_event_record)
  cudaEvent_t sev0 = nullptr, sev1 = nullptr;  // solve timing (fc_solve_info.ms)
  std::string last_error;
  int verbosity = 0;   // 1: print the reference's solver report lines
  int precision = 0;   // FC_PREC_*
  int inner_itmax = 0; double inner_tol = 0.0;
  MeshDev mesh;
  bool has_mesh = false;
  int mesh_gen = 0;    // incremented by every fc_set_mesh
  double setup_s[FC_SETUP_PHASES] = {};  // phase times of the last fc_set_mesh
  CsrSystem* sys_ext = nullptr;    // pattern cache of fc_csrsolve
  CsrSystem* sys_mesh = nullptr;   // global matrix of the mesh (sparse_matrix module)
  std::vector<CsrSystem*> sys_user;
  FieldStore* fields = nullptr;
  SimpleState* simple = nullptr;
  AdjState* adj = nullptr;         // convection-diffusion adjoint (fc_adjoint.cu)
  long long kernel_launches = 0;
  int tracing = 0, trace_blocks = 0, trace_cap = 0;
  int sweep_cap = 0;   // rows per sweep step cap of the next pattern analyses (0: as wide as fits)
  int sweep_tiles = 0; // tile count of the next pattern analyses (0: the estimate's choice)
  int stage_rows = 0;  // staged rows of a step in the next pattern analyses (0: as many as fit; tests)
  std::FILE* solve_log = nullptr;  // JSON line per solve (fc_set_solve_log)
  int grad_limiter = 0;            // FC_LIMITER_* applied by every gradient (fc_set_gradient_limiter)
  DVec<double> limiter_part;       // min/max partials of the limiters
  // node-based Gauss gradients (fc_nodegrad.cu): cell-to-node method and the
  // per-node gather lists built for mesh generation ng_gen
  int node_interp = 0, ng_gen = -1, ng_method = -1;
  DVec<int> ng_ptr, ng_src;
  DVec<double> ng_w, ng_uN;
  DVec<unsigned long long> trace;
};

int fc_fail(fc_ctx* ctx, int code, const char* what, cudaError_t e = cudaSuccess);
int fc_fail_msg(fc_ctx* ctx, int code, const std::string& msg);

// pattern analysis (host) + upload
// xyz: optional row coordinates (3*n, x then y then z) used to cut the sweep tiles
// tiles > 0: that many sweep tiles (at most one per SM) instead of the
// count the critical-path estimate picks
// with_gs: the Gauss-Seidel sweep mode must fit the staging too (else a
// Gauss-Seidel solve analyses the pattern again with it)
int sys_set_pattern(fc_ctx* ctx, CsrSystem* s, int n, int nnz, const int* ia1, const int* ja1, const int* diag1,
                    const double* xyz = nullptr, int tiles = 0, bool with_gs = false);
int sys_upload_values(fc_ctx* ctx, CsrSystem* s, const double* a, bool a_on_device);
int sys_alloc_work(fc_ctx* ctx, CsrSystem* s);

struct SolveResult {
  int status = 0;
  int itr_used = 0;
  double res0 = 0, resl = 0, factor = 0, resor = 0;
  int early = 0;
  double ms = 0;
  int outer = 0;
};

// solve on a system; a (nnz values, NULL = s->a), x and b are device
// vectors (x in/out).  solver: gauss-seidel|dpcg|iccg|bicgstab|pmgmres
// inner solve of FC_PREC_MIXED_COLOURED (FP32) or FC_PREC_COLOURED_FP64
// (fp64) on the multicolour layout of s (fc_mc.cu): A e = r64 from e = 0,
// x64 += e; *itr_out iterations, *status_out a device status (0 or FC_ERR_*)
int mc_inner_solve(fc_ctx* ctx, CsrSystem* s, const double* a, const double* r64, double* x64, double tol, int itmax,
                   bool setup, bool fp64, int* itr_out, int* status_out);
int mc_colours(fc_ctx* ctx, CsrSystem* s, int* ncol);
int sys_solve(fc_ctx* ctx, CsrSystem* s, const char* solver, const double* a, double* x, const double* b,
              int itr_max, double tol_abs, double tol_rel, SolveResult* res);
int sys_precond(fc_ctx* ctx, CsrSystem* s, int dilu, const double* q, double* z_out, double* d_out, int apply);

bool is_device_ptr(const void* p);

// ------------------------------------------------------------ batched solves
// One problem of a batched launch (fc_batch.cu): its system, whose sweep
// schedule has one tile per block of the problem's group, and the device
// arrays of this solve (a: nnz values, x in/out, b: rhs, original numbering).
struct BatchItem {
  CsrSystem* s = nullptr;
  const double* a = nullptr;
  double* x = nullptr;
  const double* b = nullptr;
  SolveResult res;
  double dev_ms = 0.0;   // the group's device time, summed over the launches
};
struct BatchDev;         // device arrays of the batched launches (fc_solvers.cu)
void batch_dev_release(BatchDev* d);
// the reference's solver report line of a solve (when ctx->verbosity is set)
void report_solve(fc_ctx* ctx, const char* solver, const char* chvar, const SolveResult& r);
// one JSON line for the solve in the context's solve log, if one is open
void log_solve(fc_ctx* ctx, const char* api, const char* solver, const char* chvar, int n, const SolveResult& r);
// Resident blocks of the batched BiCGStab kernel (FP64 and FP32 together).
int batch_block_budget(fc_ctx* ctx, int* budget);
// Solves every item: one persistent launch whose block groups are the
// items in order (items[p].s->ord.ntiles blocks each), in FP64; in
// FC_PREC_MIXED FP32 inner launches of the same groups inside FP64
// refinement, each problem with its own stopping test (FC_PREC_MIXED_COLOURED
// mixes ICCG only: these BiCGStab solves stay FP64).  Per-item results in
// items[p].res.
int batch_solve(fc_ctx* ctx, BatchDev*& dev, std::vector<BatchItem>& items, const char* solver, int itr_max,
                double tol_abs, double tol_rel);

// cross-file helpers (C++ linkage)
int solve_global(fc_ctx* ctx, const char* solver, double* x, const double* b, double* res0, int itr_max,
                 double tol_abs, double tol_rel, const char* chvar, fc_solve_info* info);
void launch_soa_to_aos(cudaStream_t st, const double* s, double* a, int n);
int fc_fields_alloc(fc_ctx* ctx);
int gmres_solve(fc_ctx* ctx, CsrSystem* s, const double* a, double* x, const double* b, int itr_max, int mr,
                double tol_abs, double tol_rel, SolveResult* res);
