// Finite-volume operators on the device: cell gradients (gradients.f90),
// the implicit Laplacian (laplacian.f90) and csrsolve on the mesh's global
// matrix.  Face loops of the reference that scatter into cells become
// cell-parallel gathers over the cell's faces in ascending face index, so
// every cell sums exactly the terms of the reference in the reference's order
// (bit-identical in FP64, no atomics); face-to-matrix writes go through the
// precomputed face -> CSR slot maps, each slot owned by one face.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "fc_fields.hpp"
#include "fc_fv.cuh"
#include "fc_internal.hpp"

using namespace fcfv;

namespace {

// ------------------------------------------------------------- gradients
// grad_gauss + gradbc, gradients.f90:1607-1715
__global__ void k_grad_gauss(MeshView M, const double* __restrict__ u, double* __restrict__ g) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double gx = 0, gy = 0, gz = 0;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      const double ax = M.arx[f], ay = M.ary[f], az = M.arz[f];
      if (f < M.nI) {
        const int p = M.owner[f], n = M.neighbour[f];
        const double up = u[p], un = u[n];
        const double fie = DA(up, DM(DS(un, up), M.facint[f]));
        const double dx = DM(fie, ax), dy = DM(fie, ay), dz = DM(fie, az);
        if (p == c) { gx = DA(gx, dx); gy = DA(gy, dy); gz = DA(gz, dz); }
        else { gx = DS(gx, dx); gy = DS(gy, dy); gz = DS(gz, dz); }
      } else {
        const double ub = u[M.nC + (f - M.nI)];
        gx = DA(gx, DM(ub, ax)); gy = DA(gy, DM(ub, ay)); gz = DA(gz, DM(ub, az));
      }
    }
    const double volr = DD(1.0, M.vol[c]);
    g[c] = DM(gx, volr);
    g[M.nT + c] = DM(gy, volr);
    g[2 * (size_t)M.nT + c] = DM(gz, volr);
  }
}

// least-squares system matrix (create_matrix_lsq :660-779 / _dm :1157-1328)
// gathered per cell, then the cofactor step
template <bool DM_WEIGHTED>
__global__ void k_lsq_matrix(MeshView M, double* __restrict__ D) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double d11 = 0, d12 = 0, d13 = 0, d22 = 0, d23 = 0, d33 = 0;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      double Dx, Dy, Dz;
      if (f < M.nI) {
        const int p = M.owner[f], n = M.neighbour[f];
        Dx = DS(M.xc[n], M.xc[p]); Dy = DS(M.yc[n], M.yc[p]); Dz = DS(M.zc[n], M.zc[p]);
      } else {
        const int p = M.owner[f];
        Dx = DS(M.xf[f], M.xc[p]); Dy = DS(M.yf[f], M.yc[p]); Dz = DS(M.zf[f], M.zc[p]);
      }
      if (DM_WEIGHTED) {
        const double w = DD(1.0, DA(DA(DM(Dx, Dx), DM(Dy, Dy)), DM(Dz, Dz)));
        d11 = DA(d11, DM(DM(w, Dx), Dx)); d22 = DA(d22, DM(DM(w, Dy), Dy)); d33 = DA(d33, DM(DM(w, Dz), Dz));
        d12 = DA(d12, DM(DM(w, Dx), Dy)); d13 = DA(d13, DM(DM(w, Dx), Dz)); d23 = DA(d23, DM(DM(w, Dy), Dz));
      } else {
        d11 = DA(d11, DM(Dx, Dx)); d22 = DA(d22, DM(Dy, Dy)); d33 = DA(d33, DM(Dz, Dz));
        d12 = DA(d12, DM(Dx, Dy)); d13 = DA(d13, DM(Dx, Dz)); d23 = DA(d23, DM(Dy, Dz));
      }
    }
    const double d21 = d12, d31 = d13, d32 = d23;
    // tmp = 1./(d11*d22*d33 - d11*d23*d32 - d12*d21*d33 + d12*d23*d31 + d13*d21*d32 - d13*d22*d31 + small)
    double det = DM(DM(d11, d22), d33);
    det = DS(det, DM(DM(d11, d23), d32));
    det = DS(det, DM(DM(d12, d21), d33));
    det = DA(det, DM(DM(d12, d23), d31));
    det = DA(det, DM(DM(d13, d21), d32));
    det = DS(det, DM(DM(d13, d22), d31));
    const double tmp = DD(1.0, DA(det, FC_SMALL));
    const size_t n = M.nC;
    D[0 * n + c] = DM(DS(DM(d22, d33), DM(d23, d32)), tmp);
    D[1 * n + c] = DM(DS(DM(d21, d33), DM(d23, d31)), tmp);
    D[2 * n + c] = DM(DS(DM(d21, d32), DM(d22, d31)), tmp);
    D[3 * n + c] = DM(DS(DM(d11, d33), DM(d13, d31)), tmp);
    D[4 * n + c] = DM(DS(DM(d12, d33), DM(d13, d32)), tmp);
    D[5 * n + c] = DM(DS(DM(d11, d32), DM(d12, d31)), tmp);
    D[6 * n + c] = DM(DS(DM(d12, d23), DM(d13, d22)), tmp);
    D[7 * n + c] = DM(DS(DM(d11, d23), DM(d13, d21)), tmp);
    D[8 * n + c] = DM(DS(DM(d11, d22), DM(d12, d21)), tmp);
  }
}

// grad_lsq (:782-893) and grad_lsq_dm (:1334-1486); the y row of the
// cofactor product and the boundary weight of the dm variant (xf at the
// boundary-face counter, :1459) are kept as the reference has them.
// EXACT (FC_GRAD_LSQ_EXACT / FC_GRAD_LSQ_DM_EXACT, no reference
// counterpart): the y row of the adjugate of the symmetric normal matrix,
// -b1 D2 + b2 D4 - b3 D8, and the dm boundary weight at the face's own
// centre, so that the gradient of a linear field is exact
template <bool DM_WEIGHTED, bool EXACT>
__global__ void k_grad_lsq(MeshView M, const double* __restrict__ D, const double* __restrict__ phi,
                           double* __restrict__ g) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double b1 = 0, b2 = 0, b3 = 0;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f < M.nI) {
        const int p = M.owner[f], n = M.neighbour[f];
        const double ddx = DS(M.xc[n], M.xc[p]), ddy = DS(M.yc[n], M.yc[p]), ddz = DS(M.zc[n], M.zc[p]);
        double Dx, Dy, Dz;
        if (DM_WEIGHTED) {
          const double w = DD(DS(phi[n], phi[p]), DA(DA(DM(ddx, ddx), DM(ddy, ddy)), DM(ddz, ddz)));
          Dx = DM(w, ddx); Dy = DM(w, ddy); Dz = DM(w, ddz);
        } else {
          const double delta = DS(phi[n], phi[p]);
          Dx = DM(ddx, delta); Dy = DM(ddy, delta); Dz = DM(ddz, delta);
        }
        b1 = DA(b1, Dx); b2 = DA(b2, Dy); b3 = DA(b3, Dz);
      } else {
        const int p = M.owner[f], bi = f - M.nI;
        const double delta = DS(phi[M.nC + bi], phi[p]);
        const double ddx = DS(M.xf[f], M.xc[p]), ddy = DS(M.yf[f], M.yc[p]), ddz = DS(M.zf[f], M.zc[p]);
        double Dx, Dy, Dz;
        if (DM_WEIGHTED) {
          const int fw = EXACT ? f : bi;
          const double qx = DS(M.xf[fw], M.xc[p]), qy = DS(M.yf[fw], M.yc[p]), qz = DS(M.zf[fw], M.zc[p]);
          const double w = DD(delta, DA(DA(DM(qx, qx), DM(qy, qy)), DM(qz, qz)));
          Dx = DM(w, ddx); Dy = DM(w, ddy); Dz = DM(w, ddz);
        } else {
          Dx = DM(ddx, delta); Dy = DM(ddy, delta); Dz = DM(ddz, delta);
        }
        b1 = DA(b1, Dx); b2 = DA(b2, Dy); b3 = DA(b3, Dz);
      }
    }
    const size_t n = M.nC;
    g[c] = DA(DS(DM(b1, D[0 * n + c]), DM(b2, D[1 * n + c])), DM(b3, D[2 * n + c]));
    if (EXACT) g[M.nT + c] = DS(DS(DM(b2, D[3 * n + c]), DM(b1, D[1 * n + c])), DM(b3, D[7 * n + c]));
    else g[M.nT + c] = DS(DS(DM(b1, D[3 * n + c]), DM(b2, D[4 * n + c])), DM(b3, D[5 * n + c]));
    g[2 * (size_t)M.nT + c] = DA(DS(DM(b1, D[6 * n + c]), DM(b2, D[7 * n + c])), DM(b3, D[8 * n + c]));
  }
}

__global__ void k_zero_bnd_grad(double* __restrict__ g, int nC, int nT) {
  const int nb = nT - nC;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nb; i += gridDim.x * blockDim.x) {
    g[nC + i] = 0.0; g[(size_t)nT + nC + i] = 0.0; g[2 * (size_t)nT + nC + i] = 0.0;
  }
}

// ------------------------------------------------------------- laplacian
// laplacian.f90:40-69 with faceFluxLaplacian :113-151: off-diagonals by face
__global__ void k_lap_face(MeshView M, const double* __restrict__ mu, double* __restrict__ a) {
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < M.nI; f += gridDim.x * blockDim.x) {
    const int p = M.owner[f], n = M.neighbour[f];
    const double fxn = M.facint[f], fxp = DS(1.0, fxn);
    const double xpn = DS(M.xc[n], M.xc[p]), ypn = DS(M.yc[n], M.yc[p]), zpn = DS(M.zc[n], M.zc[p]);
    const double ax = M.arx[f], ay = M.ary[f], az = M.arz[f];
    const double smdpn = DD(DA(DA(DM(ax, ax), DM(ay, ay)), DM(az, az)), DA(DA(DM(ax, xpn), DM(ay, ypn)), DM(az, zpn)));
    const double cap = DM(DA(DM(fxp, mu[p]), DM(fxn, mu[n])), smdpn);
    a[M.ijk[f]] = cap;
    a[M.jik[f]] = cap;
  }
}

// diagonal and Dirichlet boundary terms (laplacian.f90:62-102), per cell in
// face order; dirichlet_mask selects patches (the reference's bctype filter
// at :73 is commented out, i.e. all patches)
__global__ void k_lap_diag(MeshView M, const double* __restrict__ mu, const double* __restrict__ phi,
                           unsigned long long mask, double* __restrict__ a, double* __restrict__ su) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double ad = 0.0, s = su[c];
    bool bnd = false;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f < M.nI) {
        ad = DS(ad, a[M.owner[f] == c ? M.ijk[f] : M.jik[f]]);
      } else {
        const int bi = f - M.nI, patch = M.bpatch[bi];
        if (patch < 64 && !((mask >> patch) & 1ULL)) continue;
        bnd = true;
        const double ax = M.arx[f], ay = M.ary[f], az = M.arz[f];
        const double are = __dsqrt_rn(DA(DA(DM(ax, ax), DM(ay, ay)), DM(az, az)));
        const double nxf = DD(ax, are), nyf = DD(ay, are), nzf = DD(az, are);
        const double dfn = DA(DA(DM(DS(M.xf[f], M.xc[c]), nxf), DM(DS(M.yf[f], M.yc[c]), nyf)), DM(DS(M.zf[f], M.zc[c]), nzf));
        const double dcoef = DD(DM(mu[c], are), dfn);
        ad = DS(ad, dcoef);
        s = DS(s, DM(dcoef, phi[M.nC + bi]));
      }
    }
    a[M.diag[c]] = ad;
    if (bnd) su[c] = s;
  }
}

}  // namespace

MeshView mesh_view(fc_ctx* ctx) {
  MeshDev& m = ctx->mesh;
  MeshView v;
  v.nC = m.numCells; v.nI = m.numInnerFaces; v.nB = m.numBoundaryFaces; v.nF = m.numFaces; v.nT = m.numTotal;
  v.owner = m.owner.p; v.neighbour = m.neighbour.p; v.cf_ptr = m.cf_ptr.p; v.cf_face = m.cf_face.p;
  v.bpatch = m.bface_patch.p; v.bwall = m.bface_wall.p;
  v.srdw = m.srdw.p;
  v.dnw = m.dnw.p;
  v.arx = m.arx.p; v.ary = m.ary.p; v.arz = m.arz.p; v.xf = m.xf.p; v.yf = m.yf.p; v.zf = m.zf.p;
  v.xc = m.xc.p; v.yc = m.yc.p; v.zc = m.zc.p; v.vol = m.vol.p; v.facint = m.facint.p; v.Df = m.Df.p;
  v.ijk = m.ijk.p; v.jik = m.jik.p;
  v.nPer = m.nPer; v.nIP = m.numInnerFaces + m.nPer;
  v.pface = m.pface.p; v.ptwin = m.ptwin.p; v.ppos = m.ppos.p; v.pflag = m.pflag.p; v.bpair = m.bpair.p;
  v.af_ptr = m.nPer ? m.af_ptr.p : m.cf_ptr.p;
  v.af_ent = m.nPer ? m.af_ent.p : m.cf_face.p;
  v.diag = ctx->sys_mesh ? ctx->sys_mesh->diag.p : nullptr;
  v.ia = ctx->sys_mesh ? ctx->sys_mesh->ia.p : nullptr;
  return v;
}

static inline int grid_for(int n) { return std::max(1, std::min(65535, (n + 255) / 256)); }

// gradient of phi (numTotal, device) into g (SoA [3][numTotal], device)
int fv_grad(fc_ctx* ctx, int scheme, const double* phi, double* g) {
  MeshView M = mesh_view(ctx);
  FieldStore& F = ctx_fields(ctx);
  if (scheme == FC_GRAD_GAUSS) {
    k_grad_gauss<<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, phi, g);
    ctx->kernel_launches++;
  } else if (scheme == FC_GRAD_LSQ || scheme == FC_GRAD_LSQ_DM || scheme == FC_GRAD_LSQ_EXACT ||
             scheme == FC_GRAD_LSQ_DM_EXACT) {
    // the matrix of create_matrix_lsq (LSQ, LSQ exact) or _dm (the dm variants)
    const bool dm = scheme == FC_GRAD_LSQ_DM || scheme == FC_GRAD_LSQ_DM_EXACT;
    const int mat = dm ? FC_GRAD_LSQ_DM : FC_GRAD_LSQ;
    if (F.dmat_scheme != mat) {
      FC_CUDA_TRY(ctx, F.dmat.alloc((size_t)9 * M.nC));
      if (!dm) k_lsq_matrix<false><<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, F.dmat.p);
      else k_lsq_matrix<true><<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, F.dmat.p);
      ctx->kernel_launches++;
      F.dmat_scheme = mat;
    }
    if (scheme == FC_GRAD_LSQ) k_grad_lsq<false, false><<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, F.dmat.p, phi, g);
    else if (scheme == FC_GRAD_LSQ_DM)
      k_grad_lsq<true, false><<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, F.dmat.p, phi, g);
    else if (scheme == FC_GRAD_LSQ_EXACT)
      k_grad_lsq<false, true><<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, F.dmat.p, phi, g);
    else k_grad_lsq<true, true><<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, F.dmat.p, phi, g);
    ctx->kernel_launches++;
  } else if (scheme == FC_GRAD_NODE_GAUSS) {
    int st0 = fv_grad_node(ctx, phi, g);
    if (st0) return st0;
  } else {
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "unknown gradient scheme");
  }
  // the limiter of grad_scalar_field (gradients.f90:141-160), cells only
  int st = fv_limit(ctx, phi, g);
  if (st) return st;
  if (M.nT > M.nC) {
    k_zero_bnd_grad<<<grid_for(M.nT - M.nC), 256, 0, ctx->stream>>>(g, M.nC, M.nT);
    ctx->kernel_launches++;
  }
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

// grad_gauss alone (no limiter), boundary entries zeroed: the pressure
// gradient stages of calcp_piso (calcp_piso.f90:369-372)
int fv_grad_gauss(fc_ctx* ctx, const double* phi, double* g) {
  MeshView M = mesh_view(ctx);
  k_grad_gauss<<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, phi, g);
  ctx->kernel_launches++;
  if (M.nT > M.nC) {
    k_zero_bnd_grad<<<grid_for(M.nT - M.nC), 256, 0, ctx->stream>>>(g, M.nC, M.nT);
    ctx->kernel_launches++;
  }
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

// grad(phi, dPhidxi) of the reference (gradients.f90:106-163), with the
// context's limiter
// phi: numTotal values, dphi: (3,numTotal); host or device memory
extern "C" int fc_grad(fc_ctx* ctx, int scheme, const double* phi, double* dphi) {
  FC_RANGE();
  if (!ctx || !phi || !dphi) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  FieldStore& F = ctx_fields(ctx);
  const int nT = ctx->mesh.numTotal;
  FC_CUDA_TRY(ctx, F.cscratch_big.alloc((size_t)4 * nT));
  double* dphi_in = F.cscratch_big.p;
  double* gs = F.cscratch_big.p + nT;
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(dphi_in, phi, nT * sizeof(double),
                                   is_device_ptr(phi) ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, ctx->stream));
  int st = fv_grad(ctx, scheme, dphi_in, gs);
  if (st) return st;
  // SoA -> (3, numTotal)
  DVec<double> aos;
  FC_CUDA_TRY(ctx, aos.alloc((size_t)3 * nT));
  launch_soa_to_aos(ctx->stream, gs, aos.p, nT);
  ctx->kernel_launches++;
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(dphi, aos.p, (size_t)3 * nT * sizeof(double),
                                   is_device_ptr(dphi) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                                   ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return FC_OK;
}

// laplacian(mu, phi) of the reference: a <- -div(mu grad .) coefficients,
// su accumulated with the Dirichlet boundary terms (su is not cleared, as in
// the reference).  mu: numCells, phi: numTotal (host or device).
extern "C" int fc_laplacian(fc_ctx* ctx, const double* mu, const double* phi, unsigned long long dirichlet_mask) {
  FC_RANGE();
  if (!ctx || !mu || !phi) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  MeshView M = mesh_view(ctx);
  FieldStore& F = ctx_fields(ctx);
  FC_CUDA_TRY(ctx, F.cscratch_big.alloc((size_t)M.nC + M.nT));
  const double *dmu = mu, *dphi = phi;
  if (!is_device_ptr(mu)) {
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(F.cscratch_big.p, mu, M.nC * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    dmu = F.cscratch_big.p;
  }
  if (!is_device_ptr(phi)) {
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(F.cscratch_big.p + M.nC, phi, M.nT * sizeof(double), cudaMemcpyHostToDevice,
                                     ctx->stream));
    dphi = F.cscratch_big.p + M.nC;
  }
  double* a = ctx->sys_mesh->a.p;
  if (M.nI > 0) k_lap_face<<<grid_for(M.nI), 256, 0, ctx->stream>>>(M, dmu, a);
  k_lap_diag<<<grid_for(M.nC), 256, 0, ctx->stream>>>(M, dmu, dphi, dirichlet_mask, a, F.su.p);
  ctx->kernel_launches += 2;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

// csrsolve(solver, fi, rhs, res0, itr_max, tol_abs, tol_rel, chvar) on the
// mesh's global matrix with fields named by the reference's variables
// (linear_solvers.f90:40-91): x_field in/out (cells only), rhs_field.
extern "C" int fc_solve_field(fc_ctx* ctx, const char* solver, const char* x_field, const char* rhs_field,
                              double* res0, int itr_max, double tol_abs, double tol_rel, const char* chvar,
                              fc_solve_info* info) {
  FC_RANGE();
  if (!ctx || !solver || !x_field || !rhs_field) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  FieldSlot* xs = find_field(ctx, x_field);
  FieldSlot* bs = find_field(ctx, rhs_field);
  if (!xs || !bs) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "unknown field for fc_solve_field");
  return solve_global(ctx, solver, xs->vec->p, bs->vec->p, res0, itr_max, tol_abs, tol_rel, chvar, info);
}
