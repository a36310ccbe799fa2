// Device-resident fields of the SIMPLE path (the reference's module globals
// of variables.f90 and sparse_matrix.f90) and their host transfers.  Vector
// gradients are stored SoA on the device (three arrays of numTotal) and
// converted to the reference's (3,numTotal) layout at the boundary.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>

#include "fc_fields.hpp"
#include "fc_internal.hpp"

FieldStore& ctx_fields(fc_ctx* ctx) {
  if (!ctx->fields) ctx->fields = new FieldStore();
  return *ctx->fields;
}

void fc_fields_release(fc_ctx* ctx) {
  delete ctx->fields;
  ctx->fields = nullptr;
}

int fc_fields_alloc(fc_ctx* ctx) {
  FieldStore& F = ctx_fields(ctx);
  const MeshDev& m = ctx->mesh;
  const size_t nT = m.numTotal, nC = m.numCells, nF = m.numFaces, nI = m.numInnerFaces;
  const size_t nW = m.nwal > 0 ? m.nwal : 1;
  F.list.clear();
  F.dmat_scheme = 0;  // least-squares cofactors belong to the previous mesh
  auto add = [&](const char* name, DVec<double>* v, size_t n, int kind) {
    FieldSlot s;
    s.name = name; s.vec = v; s.n = n; s.kind = kind;
    F.list.push_back(s);
  };
  add("u", &F.u, nT, 0); add("v", &F.v, nT, 0); add("w", &F.w, nT, 0);
  add("p", &F.p, nT, 0); add("pp", &F.pp, nT, 0);
  add("vis", &F.vis, nT, 0); add("den", &F.den, nT, 0); add("t", &F.t, nT, 0);
  add("flmass", &F.flmass, nF, 0); add("visw", &F.visw, nW, 0);
  add("su", &F.su, nC, 0); add("sv", &F.sv, nC, 0); add("sw", &F.sw, nC, 0);
  add("spu", &F.spu, nC, 0); add("spv", &F.spv, nC, 0); add("sp", &F.sp, nC, 0);
  add("apu", &F.apu, nC, 0); add("apv", &F.apv, nC, 0); add("apw", &F.apw, nC, 0);
  add("dUdxi", &F.gu, 3 * nT, 1); add("dVdxi", &F.gv, 3 * nT, 1); add("dWdxi", &F.gw, 3 * nT, 1);
  add("dPdxi", &F.gp, 3 * nT, 1); add("dTdxi", &F.gt, 3 * nT, 1);
  add("uo", &F.uo, nT, 0); add("vo", &F.vo, nT, 0); add("wo", &F.wo, nT, 0);
  add("uoo", &F.uoo, nT, 0); add("voo", &F.voo, nT, 0); add("woo", &F.woo, nT, 0);
  add("uooo", &F.uooo, nT, 0); add("vooo", &F.vooo, nT, 0); add("wooo", &F.wooo, nT, 0);
  add("rU", &F.rU, nC, 0); add("rV", &F.rV, nC, 0); add("rW", &F.rW, nC, 0);
  add("te", &F.te, nT, 0); add("ed", &F.ed, nT, 0); add("fsst", &F.fsst, nT, 0);
  add("dTEdxi", &F.gte, 3 * nT, 1); add("dEDdxi", &F.ged, 3 * nT, 1);
  add("gen", &F.gen, nC, 0); add("magStrain", &F.mag, nC, 0); add("walldist", &F.wd, nC, 0);
  add("tau", &F.tau, nW, 0); add("ypl", &F.ypl, nW, 0);
  add("fscratch", &F.fscratch, 3 * (nF > 0 ? nF : 1), 2);
  add("cscratch", &F.cscratch, 3 * nC, 2);
  (void)nI;
  for (auto& s : F.list) {
    FC_CUDA_TRY(ctx, s.vec->alloc(s.n));
    FC_CUDA_TRY(ctx, cudaMemsetAsync(s.vec->p, 0, s.n * sizeof(double), ctx->stream));
  }
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FC_OK;
}

FieldSlot* find_field(fc_ctx* ctx, const std::string& name) {
  if (!ctx->fields) return nullptr;
  if (name == "a") return nullptr;
  for (auto& s : ctx->fields->list)
    if (s.name == name) return &s;
  return nullptr;
}

namespace {
// (3,n) column-major <-> SoA [3][n]
__global__ void k_aos_to_soa(const double* __restrict__ a, double* __restrict__ s, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    s[i] = a[3 * (size_t)i];
    s[n + i] = a[3 * (size_t)i + 1];
    s[2 * (size_t)n + i] = a[3 * (size_t)i + 2];
  }
}
__global__ void k_soa_to_aos(const double* __restrict__ s, double* __restrict__ a, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    a[3 * (size_t)i] = s[i];
    a[3 * (size_t)i + 1] = s[n + i];
    a[3 * (size_t)i + 2] = s[2 * (size_t)n + i];
  }
}
__global__ void k_fill(double* __restrict__ d, double v, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) d[i] = v;
}
}  // namespace

void launch_soa_to_aos(cudaStream_t st, const double* s, double* a, int n) {
  k_soa_to_aos<<<std::min(4096, (n + 255) / 256), 256, 0, st>>>(s, a, n);
}

// copy a field in: values (count doubles, host or device).  Gradient fields
// take the (3,numTotal) layout.  "a" sets the global matrix values (nnz).
extern "C" int fc_field_set(fc_ctx* ctx, const char* name, const double* values, long long count) {
  FC_RANGE();
  if (!ctx || !name || !values) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  std::string nm(name);
  const bool dev = is_device_ptr(values);
  const cudaMemcpyKind kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  if (nm == "a") {
    if (count != ctx->sys_mesh->nnz) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "field 'a': count != nnz");
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(ctx->sys_mesh->a.p, values, count * sizeof(double), kind, ctx->stream));
    return FC_OK;
  }
  FieldSlot* s = find_field(ctx, nm);
  if (!s || s->kind == 2) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "unknown field '" + nm + "'");
  if ((size_t)count != s->n) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "field '" + nm + "': wrong count");
  if (s->kind == 1) {
    DVec<double>& tmp = ctx_fields(ctx).cscratch_big;
    FC_CUDA_TRY(ctx, tmp.alloc(s->n));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(tmp.p, values, s->n * sizeof(double), kind, ctx->stream));
    const int n = (int)(s->n / 3);
    k_aos_to_soa<<<std::min(4096, (n + 255) / 256), 256, 0, ctx->stream>>>(tmp.p, s->vec->p, n);
    ctx->kernel_launches++;
  } else {
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(s->vec->p, values, s->n * sizeof(double), kind, ctx->stream));
  }
  return FC_OK;
}

// copies of a field into out, enqueued on the context's stream
static int field_get_async(fc_ctx* ctx, const char* name, double* out, long long count) {
  if (!ctx || !name || !out) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  std::string nm(name);
  const bool dev = is_device_ptr(out);
  const cudaMemcpyKind kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (nm == "a") {
    if (count != ctx->sys_mesh->nnz) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "field 'a': count != nnz");
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(out, ctx->sys_mesh->a.p, count * sizeof(double), kind, ctx->stream));
  } else {
    FieldSlot* s = find_field(ctx, nm);
    if (!s || s->kind == 2) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "unknown field '" + nm + "'");
    if ((size_t)count != s->n) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "field '" + nm + "': wrong count");
    if (s->kind == 1) {
      DVec<double>& tmp = ctx_fields(ctx).cscratch_big;
      FC_CUDA_TRY(ctx, tmp.alloc(s->n));
      const int n = (int)(s->n / 3);
      k_soa_to_aos<<<std::min(4096, (n + 255) / 256), 256, 0, ctx->stream>>>(s->vec->p, tmp.p, n);
      ctx->kernel_launches++;
      FC_CUDA_TRY(ctx, cudaMemcpyAsync(out, tmp.p, s->n * sizeof(double), kind, ctx->stream));
    } else {
      FC_CUDA_TRY(ctx, cudaMemcpyAsync(out, s->vec->p, s->n * sizeof(double), kind, ctx->stream));
    }
  }
  return FC_OK;
}

extern "C" int fc_field_get(fc_ctx* ctx, const char* name, double* out, long long count) {
  FC_RANGE();
  int st = field_get_async(ctx, name, out, count);
  if (st) return st;
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FC_OK;
}

extern "C" int fc_download_fields(fc_ctx* ctx, int nfields, const char* const* names, double* const* out,
                                  const long long* counts) {
  FC_RANGE();
  if (!ctx || nfields < 0 || (nfields && (!names || !out || !counts))) return FC_ERR_BAD_INPUT;
  for (int k = 0; k < nfields; ++k) {
    int st = field_get_async(ctx, names[k], out[k], counts[k]);
    if (st) return st;
  }
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FC_OK;
}

extern "C" int fc_field_fill(fc_ctx* ctx, const char* name, double value) {
  if (!ctx || !name) return FC_ERR_BAD_INPUT;
  std::string nm(name);
  DVec<double>* v;
  if (nm == "a") v = &ctx->sys_mesh->a;
  else {
    FieldSlot* s = find_field(ctx, nm);
    if (!s) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "unknown field '" + nm + "'");
    v = s->vec;
  }
  k_fill<<<std::min<size_t>(4096, (v->n + 255) / 256), 256, 0, ctx->stream>>>(v->p, value, v->n);
  ctx->kernel_launches++;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

// device address of a field (for callers that keep data resident)
extern "C" double* fc_field_ptr(fc_ctx* ctx, const char* name) {
  if (!ctx || !name || !ctx->has_mesh) return nullptr;
  std::string nm(name);
  if (nm == "a") return ctx->sys_mesh->a.p;
  FieldSlot* s = find_field(ctx, nm);
  return s ? s->vec->p : nullptr;
}
