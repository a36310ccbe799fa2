// C ABI: context management and the drop-in for csrsolve
// (src/linearSolvers/linear_solvers.f90:40-91) plus the standalone
// preconditioner / matrix-vector entry points.
#include <cuda_runtime.h>

#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>

#include "fc_internal.hpp"

static std::atomic<long long> g_device_allocs{0};

void fc_count_device_alloc() { g_device_allocs.fetch_add(1, std::memory_order_relaxed); }

extern "C" long long fc_device_alloc_count(void) { return g_device_allocs.load(std::memory_order_relaxed); }

static std::atomic<int> g_alloc_fill{-1};

int fc_alloc_fill() { return g_alloc_fill.load(std::memory_order_relaxed); }

extern "C" int fc_debug_fill_allocations(int byte) {
  if (byte < -1 || byte > 255) return FC_ERR_BAD_INPUT;
  g_alloc_fill.store(byte, std::memory_order_relaxed);
  return FC_OK;
}

int fc_fail(fc_ctx* ctx, int code, const char* what, cudaError_t e) {
  if (ctx) {
    ctx->last_error = std::string(what ? what : "");
    if (e != cudaSuccess) ctx->last_error += std::string(": ") + cudaGetErrorString(e);
  }
  return code;
}

int fc_fail_msg(fc_ctx* ctx, int code, const std::string& msg) {
  if (ctx) ctx->last_error = msg;
  return code;
}

extern "C" int fc_init(int device, fc_ctx** out) {
  if (!out) return FC_ERR_BAD_INPUT;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) { cudaGetLastError(); return FC_ERR_CUDA; }
  if (device < 0 || device >= ndev) return FC_ERR_BAD_INPUT;
  if (cudaSetDevice(device) != cudaSuccess) return FC_ERR_CUDA;
  fc_ctx* c = new fc_ctx();
  c->device = device;
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device);
  if (!coop) { delete c; return FC_ERR_UNSUPPORTED; }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
      cudaEventCreate(&c->sev0) != cudaSuccess || cudaEventCreate(&c->sev1) != cudaSuccess) {
    delete c;
    return FC_ERR_CUDA;
  }
  *out = c;
  return FC_OK;
}

void fc_release_mesh(fc_ctx* ctx);
void fc_fields_release(fc_ctx* ctx);
void fc_simple_release(fc_ctx* ctx);
void fc_adjoint_release(fc_ctx* ctx);

extern "C" void fc_finalize(fc_ctx* ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  delete ctx->sys_ext;
  delete ctx->sys_mesh;
  for (auto* s : ctx->sys_user) delete s;
  fc_release_mesh(ctx);
  fc_fields_release(ctx);
  fc_simple_release(ctx);
  fc_adjoint_release(ctx);
  cudaEventDestroy(ctx->ev0);
  cudaEventDestroy(ctx->ev1);
  cudaEventDestroy(ctx->sev0);
  cudaEventDestroy(ctx->sev1);
  cudaStreamDestroy(ctx->stream);
  if (ctx->solve_log) std::fclose(ctx->solve_log);
  delete ctx;
}

extern "C" const char* fc_last_error(const fc_ctx* ctx) { return ctx ? ctx->last_error.c_str() : "no context"; }

extern "C" int fc_set_verbosity(fc_ctx* ctx, int level) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  ctx->verbosity = level;
  return FC_OK;
}

extern "C" int fc_set_precision(fc_ctx* ctx, int mode, double inner_tol, int inner_itmax) {
  if (!ctx || (mode != FC_PREC_FP64 && mode != FC_PREC_MIXED && mode != FC_PREC_MIXED_COLOURED &&
               mode != FC_PREC_COLOURED_FP64))
    return FC_ERR_BAD_INPUT;
  ctx->precision = mode;
  ctx->inner_tol = inner_tol;
  ctx->inner_itmax = inner_itmax;
  return FC_OK;
}

extern "C" long long fc_kernel_launches(const fc_ctx* ctx) { return ctx ? ctx->kernel_launches : -1; }

extern "C" int fc_stream_sync(fc_ctx* ctx) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FC_OK;
}

extern "C" void* fc_stream(fc_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

// Get (or build) the cached system for an externally supplied pattern.  The
// pattern arrays are identified by their addresses and sizes, as the
// reference's module globals ia/ja/diag are fixed after create_CSR_matrix;
// fc_csr_pattern_forget() drops the cache after an in-place change.
static int ext_system(fc_ctx* ctx, int n, int nnz, const int* ia, const int* ja, const int* diag, CsrSystem** out) {
  CsrSystem* s = ctx->sys_ext;
  if (s && s->n == n && s->nnz == nnz && s->key_ia == ia && s->key_ja == ja && s->key_diag == diag) {
    *out = s;
    return FC_OK;
  }
  delete ctx->sys_ext;
  ctx->sys_ext = nullptr;
  // a pattern equal to the mesh's CSR gets the cell centroids for its sweep tiling
  const double* xyz = nullptr;
  if (ctx->has_mesh && ctx->sys_mesh && n == ctx->sys_mesh->n && nnz == ctx->sys_mesh->nnz) {
    std::vector<int> hia(n + 1), hja(nnz), hdg(n);
    auto get = [&](const int* src, int* dst, size_t cnt) {
      if (is_device_ptr(src)) return fc_d2h(ctx->stream, dst, src, cnt * sizeof(int)) == cudaSuccess;
      std::memcpy(dst, src, cnt * sizeof(int));
      return true;
    };
    if (get(ia, hia.data(), n + 1) && get(ja, hja.data(), nnz) && get(diag, hdg.data(), n)) {
      const CsrSystem* ms = ctx->sys_mesh;
      bool same = true;
      for (int i = 0; i <= n && same; ++i) same = hia[i] == ms->h_ia[i] + 1;
      for (int k = 0; k < nnz && same; ++k) same = hja[k] == ms->h_ja[k] + 1;
      for (int i = 0; i < n && same; ++i) same = hdg[i] == ms->h_diag[i] + 1;
      if (same) xyz = ctx->mesh.h_xyz.data();
    }
  }
  s = new CsrSystem();
  int st = sys_set_pattern(ctx, s, n, nnz, ia, ja, diag, xyz);
  if (st) { delete s; return st; }
  s->key_ia = ia; s->key_ja = ja; s->key_diag = diag;
  ctx->sys_ext = s;
  *out = s;
  return FC_OK;
}

extern "C" int fc_csr_pattern_forget(fc_ctx* ctx) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  delete ctx->sys_ext;
  ctx->sys_ext = nullptr;
  return FC_OK;
}

static const char* report_name(const std::string& s) {
  if (s == "iccg") return "PCG(IC0)";
  if (s == "bicgstab") return "BiCGStab(ILU(0))";
  if (s == "dpcg") return "PCG(Jacobi)";
  if (s == "gauss-seidel") return "Gauss-Seidel";
  return "PMGMRES_ILU(4)";
}

// The report line of the reference (linear_solvers.f90:540-541 and siblings).
static void print_report(const std::string& solver, const char* chvar, const SolveResult& r) {
  const char* nm = report_name(solver);
  const char* var = chvar ? chvar : "";
  if (r.early) {
    std::printf("  %s:  Solving for %s, Initial residual = %10.3E, Final residual = %10.3E, No Iterations %d\n", nm,
                var, r.res0, r.res0, solver == "gauss-seidel" ? 1 : 0);
  } else if (solver == "pmgmres") {
    std::printf("  %s:  Solving for %s, Initial residual = %10.3E, Final residual = %10.3E, No Iterations %d\n", nm,
                var, r.resor, r.resl, r.itr_used);
  } else {
    std::printf("  %s:  Solving for %s, Initial residual = %10.3E, Final residual = %10.3E, No Iterations %d\n", nm,
                var, r.resor, r.factor != 0 ? r.resl / r.factor : r.resl, r.itr_used);
  }
  std::fflush(stdout);
}

void report_solve(fc_ctx* ctx, const char* solver, const char* chvar, const SolveResult& r) {
  if (ctx->verbosity) print_report(solver ? solver : "", chvar, r);
}

// JSON number (null for NaN/Inf, which JSON cannot hold)
static void json_num(std::string& o, const char* key, double v) {
  char buf[64];
  if (std::isfinite(v)) std::snprintf(buf, sizeof buf, "\"%s\": %.17g", key, v);
  else std::snprintf(buf, sizeof buf, "\"%s\": null", key);
  o += buf;
}

void log_solve(fc_ctx* ctx, const char* api, const char* solver, const char* chvar, int n, const SolveResult& r) {
  if (!ctx->solve_log) return;
  char buf[256];
  std::snprintf(buf, sizeof buf,
                "{\"api\": \"%s\", \"solver\": \"%s\", \"var\": \"%s\", \"n\": %d, \"precision\": %d, "
                "\"status\": %d, \"iterations\": %d, \"outer\": %d, \"early\": %d, ",
                api ? api : "", solver ? solver : "", chvar ? chvar : "", n, ctx->precision, r.status, r.itr_used,
                r.outer, r.early);
  std::string o(buf);
  json_num(o, "res0_l1", r.res0);
  o += ", ";
  json_num(o, "resl", r.resl);
  o += ", ";
  json_num(o, "resor", r.resor);
  o += ", ";
  json_num(o, "factor", r.factor);
  o += ", ";
  json_num(o, "ms", r.ms);
  o += "}\n";
  std::fputs(o.c_str(), ctx->solve_log);
  std::fflush(ctx->solve_log);
}

extern "C" int fc_set_solve_log(fc_ctx* ctx, const char* path) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (ctx->solve_log) std::fclose(ctx->solve_log);
  ctx->solve_log = nullptr;
  if (!path || !*path) return FC_OK;
  ctx->solve_log = std::fopen(path, "a");
  if (!ctx->solve_log) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, std::string("fc_set_solve_log: cannot open ") + path);
  return FC_OK;
}

static void fill_info(fc_solve_info* info, const SolveResult& r) {
  if (!info) return;
  info->status = r.status;
  info->itr_used = r.itr_used;
  info->outer_iterations = r.outer;
  info->early_exit = r.early;
  info->res0_l1 = r.res0;
  info->resor = r.resor;
  info->resl = r.resl;
  info->factor = r.factor;
  info->ms = r.ms;
}

// device staging of an n-vector: in place when the caller passed device
// memory, else copied into dst
static int stage_in(fc_ctx* ctx, const double* src, double* dst, size_t n, const double** use) {
  if (is_device_ptr(src)) { *use = src; return FC_OK; }
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  *use = dst;
  return FC_OK;
}

extern "C" int fc_csrsolve(fc_ctx* ctx, const char* solver, int n, int nnz, const int* ia, const int* ja,
                           const double* a, const int* diag, double* fi, const double* rhs, double* res0,
                           int itr_max, double tol_abs, double tol_rel, const char* chvar, int verbose,
                           fc_solve_info* info) {
  FC_RANGE();
  if (!ctx || !solver || !ia || !ja || !a || !diag || !fi || !rhs || n <= 0 || nnz < n || itr_max < 0)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_csrsolve: bad arguments");
  std::string sv(solver);
  if (sv != "iccg" && sv != "bicgstab" && sv != "dpcg" && sv != "gauss-seidel" && sv != "pmgmres")
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "fc_csrsolve: unknown solver '" + sv + "'");
  cudaSetDevice(ctx->device);
  CsrSystem* s = nullptr;
  int st = ext_system(ctx, n, nnz, ia, ja, diag, &s);
  if (st) return st;
  const double *da, *db;
  if ((st = stage_in(ctx, a, s->a.p, nnz, &da))) return st;
  if ((st = stage_in(ctx, rhs, s->b.p, n, &db))) return st;
  const bool fi_dev = is_device_ptr(fi);
  double* dx = fi_dev ? fi : s->x.p;
  if (!fi_dev) FC_CUDA_TRY(ctx, cudaMemcpyAsync(dx, fi, n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  SolveResult r;
  st = sys_solve(ctx, s, solver, da, dx, db, itr_max, tol_abs, tol_rel, &r);
  if (st) { fill_info(info, r); return st; }
  if (!fi_dev) {
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(fi, dx, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  // res0 is intent(out) = the normalised initial residual; the reference leaves
  // it unset on its early exit, the same happens here
  if (res0 && !r.early) *res0 = r.resor;
  fill_info(info, r);
  if (verbose || ctx->verbosity) print_report(sv, chvar, r);
  log_solve(ctx, "fc_csrsolve", solver, chvar, n, r);
  return r.status;
}

// ------------------------------------------------------------- building blocks
extern "C" int fc_precond_setup(fc_ctx* ctx, const char* kind, int n, int nnz, const int* ia, const int* ja,
                                const double* a, const int* diag, double* d_out) {
  FC_RANGE();
  if (!ctx || !kind || !d_out) return FC_ERR_BAD_INPUT;
  std::string k(kind);
  if (k != "dic" && k != "dilu") return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "kind must be 'dic' or 'dilu'");
  CsrSystem* s = nullptr;
  int st = ext_system(ctx, n, nnz, ia, ja, diag, &s);
  if (st) return st;
  if (k == "dilu" && s->tslot_oob) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "dilu: pattern is not structurally symmetric");
  if ((st = sys_upload_values(ctx, s, a, is_device_ptr(a)))) return st;
  return sys_precond(ctx, s, k == "dilu", s->b.p, nullptr, d_out, 0);
}

extern "C" int fc_precond_apply(fc_ctx* ctx, const char* kind, int n, int nnz, const int* ia, const int* ja,
                                const double* a, const int* diag, const double* q, double* z_out) {
  FC_RANGE();
  if (!ctx || !kind || !q || !z_out) return FC_ERR_BAD_INPUT;
  std::string k(kind);
  if (k != "dic" && k != "dilu") return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "kind must be 'dic' or 'dilu'");
  CsrSystem* s = nullptr;
  int st = ext_system(ctx, n, nnz, ia, ja, diag, &s);
  if (st) return st;
  if (k == "dilu" && s->tslot_oob) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "dilu: pattern is not structurally symmetric");
  if ((st = sys_upload_values(ctx, s, a, is_device_ptr(a)))) return st;
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->b.p, q, n * sizeof(double),
                                   is_device_ptr(q) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  return sys_precond(ctx, s, k == "dilu", s->b.p, z_out, nullptr, 1);
}

int sys_spmv(fc_ctx* ctx, CsrSystem* s, const double* a, const double* x, double* y, int transpose);
int sys_ilu0(fc_ctx* ctx, CsrSystem* s, double* l_out);

extern "C" int fc_spmv(fc_ctx* ctx, int n, int nnz, const int* ia, const int* ja, const double* a,
                           const int* diag, const double* x, double* y, int transpose) {
  FC_RANGE();
  if (!ctx || !x || !y || !a) return FC_ERR_BAD_INPUT;
  CsrSystem* s = nullptr;
  int st = ext_system(ctx, n, nnz, ia, ja, diag, &s);
  if (st) return st;
  // device-resident values and vectors are used in place
  const double *da, *dx;
  if ((st = stage_in(ctx, a, s->a.p, nnz, &da))) return st;
  if ((st = stage_in(ctx, x, s->b.p, n, &dx))) return st;
  const bool ydev = is_device_ptr(y);
  double* dy = ydev ? y : s->w.p;
  if ((st = sys_spmv(ctx, s, da, dx, dy, transpose))) return st;
  if (!ydev) FC_CUDA_TRY(ctx, cudaMemcpyAsync(y, dy, n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FC_OK;
}

extern "C" int fc_ilu0(fc_ctx* ctx, int n, int nnz, const int* ia, const int* ja, const double* a, const int* diag,
                       double* l_out) {
  if (!ctx || !a || !l_out) return FC_ERR_BAD_INPUT;
  CsrSystem* s = nullptr;
  int st = ext_system(ctx, n, nnz, ia, ja, diag, &s);
  if (st) return st;
  if ((st = sys_upload_values(ctx, s, a, is_device_ptr(a)))) return st;
  return sys_ilu0(ctx, s, l_out);
}

// ------------------------------------------------------------------ timing
extern "C" int fc_event_record(fc_ctx* ctx, int which) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  FC_CUDA_TRY(ctx, cudaEventRecord(which ? ctx->ev1 : ctx->ev0, ctx->stream));
  return FC_OK;
}

extern "C" int fc_event_elapsed_ms(fc_ctx* ctx, float* ms) {
  if (!ctx || !ms) return FC_ERR_BAD_INPUT;
  FC_CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
  FC_CUDA_TRY(ctx, cudaEventElapsedTime(ms, ctx->ev0, ctx->ev1));
  return FC_OK;
}

// csrsolve on the mesh's global matrix (module globals of sparse_matrix.f90)
int solve_global(fc_ctx* ctx, const char* solver, double* x, const double* b, double* res0, int itr_max,
                 double tol_abs, double tol_rel, const char* chvar, fc_solve_info* info) {
  std::string sv(solver);
  if (sv != "iccg" && sv != "bicgstab" && sv != "dpcg" && sv != "gauss-seidel" && sv != "pmgmres")
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "unknown solver '" + sv + "'");
  CsrSystem* s = ctx->sys_mesh;
  SolveResult r;
  int st = sys_solve(ctx, s, solver, s->a.p, x, b, itr_max, tol_abs, tol_rel, &r);
  fill_info(info, r);
  if (st) return st;
  if (res0 && !r.early) *res0 = r.resor;
  if (ctx->verbosity) print_report(sv, chvar, r);
  log_solve(ctx, "mesh system", solver, chvar, s->n, r);
  return r.status;
}

// Ordered sweep structure of the mesh system (which = 0) or of the cached
// external pattern (which = 1): out[0..9] = tiles, levels, widest step of a
// tile, ring depth, estimated forward sweep microseconds, ring-served
// entries, pushed entries, cross-tile entries (both triangles), stage depth,
// most steps of a tile.
extern "C" int fc_set_sweep_cap(fc_ctx* ctx, int rows) {
  if (!ctx || rows < 0) return FC_ERR_BAD_INPUT;
  ctx->sweep_cap = rows;
  return FC_OK;
}

extern "C" int fc_set_sweep_tiles(fc_ctx* ctx, int tiles) {
  if (!ctx || tiles < 0) return FC_ERR_BAD_INPUT;
  ctx->sweep_tiles = tiles;
  return FC_OK;
}

extern "C" int fc_mixed_colours(fc_ctx* ctx, int which, int* ncol) {
  if (!ctx || !ncol) return FC_ERR_BAD_INPUT;
  CsrSystem* s = which ? ctx->sys_ext : ctx->sys_mesh;
  if (!s) return fc_fail_msg(ctx, FC_ERR_STATE, "no such system");
  return mc_colours(ctx, s, ncol);
}

extern "C" int fc_sweep_stats(fc_ctx* ctx, int which, double* out) {
  if (!ctx || !out) return FC_ERR_BAD_INPUT;
  CsrSystem* s = which ? ctx->sys_ext : ctx->sys_mesh;
  if (!s) return fc_fail_msg(ctx, FC_ERR_STATE, "no such system");
  const DevOrdered& D = s->ord;
  out[0] = D.ntiles; out[1] = D.nlev; out[2] = D.maxW; out[3] = D.R;
  out[4] = s->est_sweep_us; out[5] = (double)D.ring_entries; out[6] = (double)D.pushed_entries;
  out[7] = (double)D.cross_tile_entries; out[8] = D.K; out[9] = D.max_tile_steps;
  out[10] = D.Wc;
  return FC_OK;
}

extern "C" int fc_set_sweep_stage_rows(fc_ctx* ctx, int rows) {
  if (!ctx || rows < 0) return FC_ERR_BAD_INPUT;
  ctx->stage_rows = rows;
  return FC_OK;
}
