// Batched solves of independent sparse systems: fc_batch_* of fc_gpu.h.
//
// The reference solves such systems one csrsolve call after another
// (linear_solvers.f90:40-91), e.g. the three momentum components of calcuvw
// (velocity.f90:638, :693, :748) or a set of scalar equations.  Here every
// problem keeps its own system (pattern analysis and sweep schedule) and the
// solves of all problems run in one persistent launch whose grid is split
// into one group of blocks per problem (batch_solve, fc_solvers.cu).  The
// group sizes come from the planner (host/fc_batch_plan.cpp): from its cost
// model, or tuned by measured solves (fc_batch_tune) and cached per set of
// problem sizes for the rest of the process.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "fc_batch_plan.hpp"
#include "fc_internal.hpp"
#include "fc_schedule.hpp"

struct fc_batch {
  struct Prob {
    int n = 0, nnz = 0, levels = 0, tiles = 0;   // tiles of the built schedule (0: not built)
    std::vector<int> ia, ja, dg;                 // 1-based, as passed
    std::vector<double> xyz;                     // optional row coordinates (3n)
    CsrSystem* s = nullptr;
  };
  fc_ctx* ctx = nullptr;
  int device = 0;        // the context's device (the batch may outlive the context)
  std::vector<Prob> probs;
  BatchDev* dev = nullptr;
  bool planned = false;
  ~fc_batch() {
    for (Prob& p : probs) delete p.s;
    batch_dev_release(dev);
  }
};

namespace {

std::mutex g_tuned_mu;
std::map<std::vector<long long>, std::vector<int>> g_tuned;  // problem sizes -> tuned tiles

std::vector<long long> size_key(const fc_batch* b) {
  std::vector<long long> k{(long long)b->ctx->num_sms};
  for (const auto& p : b->probs) { k.push_back(p.n); k.push_back(p.nnz); }
  return k;
}

std::vector<BatchCost> costs(const fc_batch* b) {
  std::vector<BatchCost> c(b->probs.size());
  for (size_t p = 0; p < c.size(); ++p) { c[p].rows = b->probs[p].n; c[p].levels = b->probs[p].levels; }
  return c;
}

constexpr int kMinRowsPerTile = 1024;

// (re)build the systems whose tile count changes
int apply_plan(fc_batch* b, const std::vector<int>& tiles) {
  fc_ctx* ctx = b->ctx;
  int budget = 0;
  batch_block_budget(ctx, &budget);
  long long sum = 0;
  for (int t : tiles) {
    if (t < 1) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_batch_plan: tiles < 1");
    sum += t;
  }
  if (tiles.size() != b->probs.size() || sum > budget)
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "fc_batch_plan: the groups need more blocks than the GPU holds resident (" +
                                                    std::to_string(sum) + " > " + std::to_string(budget) + ")");
  for (size_t p = 0; p < tiles.size(); ++p) {
    fc_batch::Prob& q = b->probs[p];
    if (q.s && q.tiles == tiles[p]) continue;
    if (!q.s) q.s = new CsrSystem();
    int st = sys_set_pattern(ctx, q.s, q.n, q.nnz, q.ia.data(), q.ja.data(), q.dg.data(),
                             q.xyz.empty() ? nullptr : q.xyz.data(), tiles[p]);
    if (st) return st;
    q.tiles = tiles[p];
  }
  b->planned = true;
  return FC_OK;
}

std::vector<int> model_plan(fc_batch* b, const std::vector<BatchCost>& c) {
  int budget = 0;
  batch_block_budget(b->ctx, &budget);
  return plan_batch_groups(c, budget, std::max(1, b->ctx->num_sms), kMinRowsPerTile);
}

void fill(fc_solve_info* info, const SolveResult& r, double ms) {
  if (!info) return;
  info->status = r.status;
  info->itr_used = r.itr_used;
  info->outer_iterations = r.outer;
  info->early_exit = r.early;
  info->res0_l1 = r.res0;
  info->resor = r.resor;
  info->resl = r.resl;
  info->factor = r.factor;
  info->ms = ms;
}

// device arrays of problem p for a solve: the caller's when on the device,
// else copies in the system's own staging vectors (x copied back later)
int stage(fc_batch* b, int p, const double* a, double* x, const double* rhs, BatchItem& it, bool& x_host) {
  fc_ctx* ctx = b->ctx;
  CsrSystem* s = b->probs[p].s;
  const int n = b->probs[p].n, nnz = b->probs[p].nnz;
  it.s = s;
  if (!a || !x || !rhs) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_batch_solve: NULL array");
  if (is_device_ptr(a)) it.a = a;
  else { FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->a.p, a, (size_t)nnz * sizeof(double), cudaMemcpyHostToDevice, ctx->stream)); it.a = s->a.p; }
  if (is_device_ptr(rhs)) it.b = rhs;
  else { FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->b.p, rhs, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream)); it.b = s->b.p; }
  x_host = !is_device_ptr(x);
  if (x_host) { FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->x.p, x, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream)); it.x = s->x.p; }
  else it.x = x;
  return FC_OK;
}

// one timed batched solve; ms = device time of the whole call
int run(fc_batch* b, const char* solver, const double* const* a, double* const* x, const double* const* rhs,
        bool x_scratch, int itr_max, double tol_abs, double tol_rel, std::vector<BatchItem>& items, double* ms) {
  fc_ctx* ctx = b->ctx;
  const int np = (int)b->probs.size();
  items.assign(np, BatchItem());
  std::vector<char> xh(np, 0);
  FC_CUDA_TRY(ctx, cudaEventRecord(ctx->sev0, ctx->stream));
  for (int p = 0; p < np; ++p) {
    bool x_host = false;
    int st = stage(b, p, a[p], x_scratch ? b->probs[p].s->x.p : x[p], rhs[p], items[p], x_host);
    if (st) return st;
    if (x_scratch) {
      // tuning: start from the caller's x0 in the system's own vector
      CsrSystem* s = b->probs[p].s;
      const cudaMemcpyKind k = is_device_ptr(x[p]) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
      FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->x.p, x[p], (size_t)b->probs[p].n * sizeof(double), k, ctx->stream));
    }
    xh[p] = x_host ? 1 : 0;
  }
  int st = batch_solve(ctx, b->dev, items, solver, itr_max, tol_abs, tol_rel);
  if (st) return st;
  if (!x_scratch)
    for (int p = 0; p < np; ++p)
      if (xh[p])
        FC_CUDA_TRY(ctx, cudaMemcpyAsync(x[p], items[p].x, (size_t)b->probs[p].n * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaEventRecord(ctx->sev1, ctx->stream));
  FC_CUDA_TRY(ctx, cudaEventSynchronize(ctx->sev1));
  float f = 0;
  cudaEventElapsedTime(&f, ctx->sev0, ctx->sev1);
  *ms = f;
  return FC_OK;
}

int worst_status(fc_batch* b, const std::vector<BatchItem>& items) {
  int warn = FC_OK;
  for (const BatchItem& it : items) {
    if (it.res.status == FC_ERR_TIMEOUT) return fc_fail_msg(b->ctx, FC_ERR_TIMEOUT, "batch: a group barrier timed out");
    if (it.res.status < 0) return fc_fail_msg(b->ctx, it.res.status, "batch: a problem reported an error (NaN/Inf or breakdown)");
    if (it.res.status > 0) warn = it.res.status;
  }
  return warn;
}

}  // namespace

extern "C" int fc_batch_create(fc_ctx* ctx, fc_batch** out) {
  if (!ctx || !out) return FC_ERR_BAD_INPUT;
  fc_batch* b = new fc_batch();
  b->ctx = ctx;
  b->device = ctx->device;
  *out = b;
  return FC_OK;
}

extern "C" int fc_batch_destroy(fc_batch* b) {
  if (!b) return FC_ERR_BAD_INPUT;
  cudaSetDevice(b->device);
  delete b;
  return FC_OK;
}

extern "C" int fc_batch_add(fc_batch* b, int n, int nnz, const int* ia, const int* ja, const int* diag,
                            const double* xyz) {
  if (!b) return FC_ERR_BAD_INPUT;
  fc_ctx* ctx = b->ctx;
  if (!ia || !ja || !diag || n <= 0 || nnz < n) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_batch_add: bad arguments");
  fc_batch::Prob q;
  q.n = n;
  q.nnz = nnz;
  q.ia.resize(n + 1);
  q.ja.resize(nnz);
  q.dg.resize(n);
  auto fetch = [&](const void* src, void* dst, size_t bytes) -> int {
    if (is_device_ptr(src)) {
      cudaError_t e = fc_d2h(ctx->stream, dst, src, bytes);
      if (e != cudaSuccess) return fc_fail(ctx, FC_ERR_CUDA, "fc_batch_add: pattern copy", e);
    } else {
      std::memcpy(dst, src, bytes);
    }
    return FC_OK;
  };
  int st;
  if ((st = fetch(ia, q.ia.data(), (n + 1) * sizeof(int))) || (st = fetch(ja, q.ja.data(), nnz * sizeof(int))) ||
      (st = fetch(diag, q.dg.data(), n * sizeof(int))))
    return st;
  if (xyz) {
    q.xyz.resize((size_t)3 * n);
    if ((st = fetch(xyz, q.xyz.data(), (size_t)3 * n * sizeof(double)))) return st;
  }
  // level-set depth for the planner; the full checks of the pattern are made
  // when its schedule is built
  if (q.ia[0] != 1 || q.ia[n] != nnz + 1) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_batch_add: ia(1) != 1 or ia(n+1) != nnz+1");
  std::vector<int> ia0(n + 1), ja0(nnz), dg0(n), lev;
  for (int i = 0; i <= n; ++i) ia0[i] = q.ia[i] - 1;
  for (int k = 0; k < nnz; ++k) {
    ja0[k] = q.ja[k] - 1;
    if (ja0[k] < 0 || ja0[k] >= n) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_batch_add: column index out of range");
  }
  for (int i = 0; i < n; ++i) {
    dg0[i] = q.dg[i] - 1;
    if (ia0[i + 1] <= ia0[i] || dg0[i] < ia0[i] || dg0[i] >= ia0[i + 1] || ja0[dg0[i]] != i)
      return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_batch_add: diag does not point at the diagonal");
  }
  q.levels = symmetric_levels(n, ia0.data(), ja0.data(), dg0.data(), lev);
  b->probs.push_back(std::move(q));
  b->planned = false;
  return (int)b->probs.size() - 1;
}

extern "C" int fc_batch_plan(fc_batch* b, const int* tiles) {
  FC_RANGE();
  if (!b) return FC_ERR_BAD_INPUT;
  fc_ctx* ctx = b->ctx;
  if (b->probs.empty()) return fc_fail_msg(ctx, FC_ERR_STATE, "fc_batch_plan: no problems");
  cudaSetDevice(ctx->device);
  std::vector<int> t;
  if (tiles) {
    t.assign(tiles, tiles + b->probs.size());
  } else {
    {
      std::lock_guard<std::mutex> lk(g_tuned_mu);
      auto f = g_tuned.find(size_key(b));
      if (f != g_tuned.end()) t = f->second;
    }
    if (t.empty()) t = model_plan(b, costs(b));
    if (t.empty()) return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "fc_batch_plan: more problems than resident blocks");
  }
  return apply_plan(b, t);
}

extern "C" int fc_batch_tiles(fc_batch* b, int* tiles) {
  if (!b || !tiles) return FC_ERR_BAD_INPUT;
  if (!b->planned) return fc_fail_msg(b->ctx, FC_ERR_STATE, "fc_batch_tiles: not planned");
  for (size_t p = 0; p < b->probs.size(); ++p) tiles[p] = b->probs[p].s->ord.ntiles;
  return FC_OK;
}

extern "C" int fc_batch_solve(fc_batch* b, const char* solver, const double* const* a, double* const* x,
                              const double* const* rhs, int itr_max, double tol_abs, double tol_rel,
                              fc_solve_info* info) {
  FC_RANGE();
  if (!b || !solver || !a || !x || !rhs || itr_max < 0) return FC_ERR_BAD_INPUT;
  fc_ctx* ctx = b->ctx;
  cudaSetDevice(ctx->device);
  int st;
  if (!b->planned && (st = fc_batch_plan(b, nullptr))) return st;
  std::vector<BatchItem> items;
  double ms = 0;
  if ((st = run(b, solver, a, x, rhs, false, itr_max, tol_abs, tol_rel, items, &ms))) return st;
  for (size_t p = 0; p < items.size(); ++p) {
    fill(info ? info + p : nullptr, items[p].res, items[p].dev_ms);
    if (ctx->solve_log) {
      SolveResult r = items[p].res;
      r.ms = items[p].dev_ms;
      log_solve(ctx, "fc_batch_solve", solver, ("problem " + std::to_string(p)).c_str(), b->probs[p].n, r);
    }
  }
  return worst_status(b, items);
}

extern "C" int fc_batch_tune(fc_batch* b, const char* solver, const double* const* a, const double* const* x0,
                             const double* const* rhs, int itr_max, double tol_abs, double tol_rel, int rounds,
                             double* best_ms) {
  FC_RANGE();
  if (!b || !solver || !a || !x0 || !rhs || rounds < 1) return FC_ERR_BAD_INPUT;
  fc_ctx* ctx = b->ctx;
  cudaSetDevice(ctx->device);
  if (b->probs.empty()) return fc_fail_msg(ctx, FC_ERR_STATE, "fc_batch_tune: no problems");
  std::vector<BatchCost> c = costs(b);
  std::vector<int> cur = model_plan(b, c);
  if (cur.empty()) return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "fc_batch_tune: more problems than resident blocks");
  std::vector<int> best;
  double best_t = 1e300;
  int st;
  for (int r = 0; r < rounds; ++r) {
    if ((st = apply_plan(b, cur))) return st;
    std::vector<BatchItem> items;
    double ms = 0;
    // the first solve of a plan pays one-off setup (attributes, staging):
    // time the second
    double* const* xs = const_cast<double* const*>(x0);  // read only: the solves run on copies
    if ((st = run(b, solver, a, xs, rhs, true, itr_max, tol_abs, tol_rel, items, &ms))) return st;
    if ((st = run(b, solver, a, xs, rhs, true, itr_max, tol_abs, tol_rel, items, &ms))) return st;
    if ((st = worst_status(b, items)) < 0) return st;
    if (ms < best_t) { best_t = ms; best = cur; }
    // calibrate: measured group time per modelled iteration time
    for (size_t p = 0; p < c.size(); ++p)
      c[p].weight = std::max(1e-9, items[p].dev_ms * 1e3) / batch_iteration_us(c[p], cur[p]);
    std::vector<int> next = model_plan(b, c);
    if (next.empty() || next == cur) break;
    cur = next;
  }
  if ((st = apply_plan(b, best))) return st;
  {
    std::lock_guard<std::mutex> lk(g_tuned_mu);
    g_tuned[size_key(b)] = best;
  }
  if (best_ms) *best_ms = best_t;
  return FC_OK;
}
