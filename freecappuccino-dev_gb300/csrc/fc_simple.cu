// The SIMPLE path on the device: pressure gradient and sources
// (Pressure/nablap.f90, bpres.f90), momentum assembly (Velocity/velocity.f90
// calcuvw, facefluxuvw, facefluxuvw_bnd, updateVelocityAtBoundary), the SIMPLE
// pressure correction (Pressure/calcp_simple.f90 with fluxes/faceflux_mass.f90
// facefluxmass2, fluxmc2, adjustMassFlow and continuityErrors.f90), the
// mass-flux initialisation of init.f90 and the temperature equation
// (ScalarEqns/temperature.f90 with fluxes/scalar_fluxes.f90 facefluxsc and
// boundary/updateBoundary.f90).
//
// This translation unit is compiled with --fmad=false: the expressions below
// are written in the reference's evaluation order and evaluate exactly as the
// reference does in FP64.  Face loops that scatter into cells are split into
// a face-parallel kernel (matrix slots through the face -> CSR maps, per-face
// source terms to scratch) and a cell-parallel gather over the cell's faces
// in ascending face index, which reproduces the reference's summation order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "fc_fields.hpp"
#include "fc_fv.cuh"
#include "fc_batch_plan.hpp"
#include "fc_internal.hpp"

using namespace fcfv;

namespace {

constexpr double SMALL = FC_SMALL;

struct Fld {  // SoA gradient access
  const double* g;
  int nT;
  __device__ double x(int i) const { return g[i]; }
  __device__ double y(int i) const { return g[nT + i]; }
  __device__ double z(int i) const { return g[2 * (size_t)nT + i]; }
};

// ------------------------------------------------------------ interpolation
// face_value_flux_limiter, interpolation.f90:489-650
__device__ double fv_flux_limiter(const MeshView& M, int ijp, int ijn, double lambda, const double* u, Fld g,
                                  int scheme) {
  const double fxp = 1.0 - lambda;
  double psi = 1.0;
  const double xpn = M.xc[ijn] - M.xc[ijp], ypn = M.yc[ijn] - M.yc[ijp], zpn = M.zc[ijn] - M.zc[ijp];
  const double r = (2 * g.x(ijp) * xpn + 2 * g.y(ijp) * ypn + 2 * g.z(ijp) * zpn) /
                       (u[ijn] - u[ijp] + (double)1e-30f) - 1.0;
  const double two3s = (double)(2.0f / 3.0f), one3s = (double)(1.0f / 3.0f);
  const double two3d = 2.0 / 3.0, one3d = 1.0 / 3.0;
  switch (scheme) {
    case FC_SCHEME_MUSCL: psi = fmax(0.0, fmin(fmin(2 * r, 0.5 * r + 0.5), 2.0)); break;
    case FC_SCHEME_UMIST: psi = fmax(0.0, fmin(fmin(fmin(2 * r, 0.75 * r + 0.25), 0.25 * r + 0.75), 2.0)); break;
    case FC_SCHEME_KOREN: psi = fmax(0.0, fmin(fmin(2 * r, two3d * r + one3d), 2.0)); break;
    case FC_SCHEME_SMART: psi = fmax(0.0, fmin(fmin(2 * r, 0.75 * r + 0.25), 4.0)); break;
    case FC_SCHEME_AVLSMART: psi = fmax(0.0, fmin(fmin(1.5 * r, 0.75 * r + 0.25), 2.5)); break;
    case FC_SCHEME_CHARM: psi = fmax(0.0, (r + fabs(r)) * (3 * r + 1.0) / (2 * ((r + 1.0) * (r + 1.0)))); break;
    case FC_SCHEME_VANLEER: psi = fmax(0.0, fmin((r + fabs(r)) / (r + 1.0), 2.0)); break;
    case FC_SCHEME_OSPRE: psi = fmax(0.0, 3 * r * (r + 1.0) / (2 * (r * r + r + 1.0))); break;
    case FC_SCHEME_MINMOD: psi = fmax(0.0, fmin(r, 1.0)); break;
    case FC_SCHEME_BOUNDED_LINEAR_UPWIND: psi = fmax(0.0, fmin(2 * r, 1.0)); break;
    case FC_SCHEME_BOUNDED_LINEAR_UPWIND02: psi = fmax(0.0, fmin(10 * r, 1.0)); break;
    case FC_SCHEME_BOUNDED_CENTRAL: psi = fmax(0.0, fmin(r, 4.0)); break;
    case FC_SCHEME_FROMM: psi = 0.5 * r + 0.5; break;
    case FC_SCHEME_CUI: psi = two3s * r + one3s; break;
    case FC_SCHEME_QUICK: psi = 0.75 * r + 0.25; break;
    case FC_SCHEME_SPL13: psi = fmax(0.0, fmin(fmin(fmin(2 * r, one3s * r + two3s), two3s * r + one3s), 2.0)); break;
    default: psi = 1.0;
  }
  return u[ijp] + fxp * psi * (u[ijn] - u[ijp]);
}

// face_value, interpolation.f90:28-113
__device__ double face_value(const MeshView& M, int ijp, int ijn, double xf, double yf, double zf, double lambda,
                             const double* u, Fld g, int scheme) {
  switch (scheme) {
    case FC_SCHEME_CDS:
      return u[ijp] + (u[ijn] - u[ijp]) * lambda;
    case FC_SCHEME_CENTRAL: {
      const double gr = g.x(ijp) * (xf - M.xc[ijp]) + g.y(ijp) * (yf - M.yc[ijp]) + g.z(ijp) * (zf - M.zc[ijp]) +
                        g.x(ijn) * (xf - M.xc[ijn]) + g.y(ijn) * (yf - M.yc[ijn]) + g.z(ijn) * (zf - M.zc[ijn]);
      return 0.5 * (u[ijp] + u[ijn] + gr);
    }
    case FC_SCHEME_LINEAR_UPWIND: {
      const double gr = g.x(ijp) * (xf - M.xc[ijp]) + g.y(ijp) * (yf - M.yc[ijp]) + g.z(ijp) * (zf - M.zc[ijp]);
      return u[ijp] + gr;
    }
    case FC_SCHEME_KAPPA: {
      const double theta = (double)(2.0f / 3.0f);
      const double g2 = g.x(ijp) * (xf - M.xc[ijp]) + g.y(ijp) * (yf - M.yc[ijp]) + g.z(ijp) * (zf - M.zc[ijp]);
      const double gc = g.x(ijp) * (xf - M.xc[ijp]) + g.y(ijp) * (yf - M.yc[ijp]) + g.z(ijp) * (zf - M.zc[ijp]) +
                        g.x(ijn) * (xf - M.xc[ijn]) + g.y(ijn) * (yf - M.yc[ijn]) + g.z(ijn) * (zf - M.zc[ijn]);
      const double vf2 = (u[ijp] + g2);
      const double vfc = 0.5 * (u[ijp] + u[ijn] + gc);
      return theta * vfc + (1.0 - theta) * vf2;
    }
    default:
      return fv_flux_limiter(M, ijp, ijn, lambda, u, g, scheme);
  }
}

struct Dev {  // per-call device pointers of the fields
  double *u, *v, *w, *p, *pp, *vis, *den, *flmass, *visw, *t;
  double *su, *sv, *sw, *spu, *spv, *sp, *apu, *apv, *apw;
  double *gu, *gv, *gw, *gp, *gt;
  double *uo, *vo, *wo, *uoo, *voo, *woo, *uooo, *vooo, *wooo;  // old time levels
  double *rU, *rV, *rW;  // PISO: explicit momentum terms
  double* a;
  double* fscr;
  const int* ptype;  // FC_BC_* per patch
};

// ------------------------------------------------------- boundary updates
// updateVelocityAtBoundary, velocity.f90:1184-1279 (the symmetry projection
// uses the area vector as written there)
__global__ void k_update_vel_bnd(MeshView M, Dev D) {
  for (int bi = blockIdx.x * blockDim.x + threadIdx.x; bi < M.nB; bi += gridDim.x * blockDim.x) {
    const int t = D.ptype[M.bpatch[bi]];
    const int f = M.nI + bi, p = M.owner[f], b = M.nC + bi;
    if (t == FC_BC_EMPTY || t == FC_BC_PERIODIC) {
      D.u[b] = D.u[p]; D.v[b] = D.v[p]; D.w[b] = D.w[p];
    } else if (t == FC_BC_SYMMETRY) {
      const double Unmag = D.u[p] * M.arx[f] + D.v[p] * M.ary[f] + D.w[p] * M.arz[f];
      D.u[b] = D.u[p] - Unmag * M.arx[f];
      D.v[b] = D.v[p] - Unmag * M.ary[f];
      D.w[b] = D.w[p] - Unmag * M.arz[f];
    }
  }
}

// bpres, bpres.f90:55-180
__global__ void k_bpres(MeshView M, const int* __restrict__ ptype, double* __restrict__ p, Fld g, int stage) {
  for (int bi = blockIdx.x * blockDim.x + threadIdx.x; bi < M.nB; bi += gridDim.x * blockDim.x) {
    const int t = ptype[M.bpatch[bi]];
    const int f = M.nI + bi, c = M.owner[f];
    if (stage == 1) {
      if (t != FC_BC_PRESSURE) p[M.nC + bi] = p[c];
    } else if (t == FC_BC_WALL) {
      const double xpb = M.xf[f] - M.xc[c], ypb = M.yf[f] - M.yc[c], zpb = M.zf[f] - M.zc[c];
      p[M.nC + bi] = p[c] + g.x(c) * xpb + g.y(c) * ypb + g.z(c) * zpb;
    }
  }
}

// -sum_f p_f S_f over inner faces (nablap.f90:52-108), cell gather
__global__ void k_gp_inner(MeshView M, const double* __restrict__ p, Fld gp, const double* __restrict__ apu, int mode,
                           double* __restrict__ su, double* __restrict__ sv, double* __restrict__ sw) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f >= M.nI) break;
      const int ijp = M.owner[f], ijn = M.neighbour[f];
      double pf;
      if (mode == 0) pf = p[ijp] + (p[ijn] - p[ijp]) * M.facint[f];
      else if (mode == 1) pf = face_value(M, ijp, ijn, M.xf[f], M.yf[f], M.zf[f], M.facint[f], p, gp, FC_SCHEME_CENTRAL);
      else pf = (p[ijp] * apu[ijp] + p[ijn] * apu[ijn]) / (apu[ijp] + apu[ijn] + SMALL);
      const double dfxe = pf * M.arx[f], dfye = pf * M.ary[f], dfze = pf * M.arz[f];
      if (ijp == c) { sx = sx - dfxe; sy = sy - dfye; sz = sz - dfze; }
      else { sx = sx + dfxe; sy = sy + dfye; sz = sz + dfze; }
    }
    su[c] = sx; sv[c] = sy; sw[c] = sz;
  }
}

// dPdxi from the accumulated sources plus boundary faces, /vol (nablap.f90:145-172)
__global__ void k_gp_grad(MeshView M, const double* __restrict__ p, const double* __restrict__ su,
                          const double* __restrict__ sv, const double* __restrict__ sw, double* __restrict__ g) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double gx = -su[c], gy = -sv[c], gz = -sw[c];
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f < M.nI) continue;
      const double pb = p[M.nC + (f - M.nI)];
      gx = gx + pb * M.arx[f]; gy = gy + pb * M.ary[f]; gz = gz + pb * M.arz[f];
    }
    const double volr = 1.0 / M.vol[c];
    g[c] = gx * volr;
    g[M.nT + c] = gy * volr;
    g[2 * (size_t)M.nT + c] = gz * volr;
  }
}

// su,sv,sw -= p_b S_b over boundary faces (nablap.f90:176-186)
__global__ void k_gp_final(MeshView M, const double* __restrict__ p, double* __restrict__ su, double* __restrict__ sv,
                           double* __restrict__ sw) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double sx = su[c], sy = sv[c], sz = sw[c];
    bool any = false;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f < M.nI) continue;
      const double pb = p[M.nC + (f - M.nI)];
      sx = sx - pb * M.arx[f]; sy = sy - pb * M.ary[f]; sz = sz - pb * M.arz[f];
      any = true;
    }
    if (any) { su[c] = sx; sv[c] = sy; sw[c] = sz; }
  }
}

// ------------------------------------------------------------- momentum
struct MomParams {
  double gds, viscos;
  int scheme;
  double vis_sym;  // vis(inp) with inp = numCells+1 after the cell loop (velocity.f90:379)
  int tscheme;     // FC_TIME_*: unsteady term of the cell loop (velocity.f90:226-290)
  double timestep;
};

// sngrad (variant 1), gradients.f90:1720-1779
__device__ __forceinline__ void sngrad(const MeshView& M, int i, int ijp, int ijn, double arx, double ary, double arz,
                                       double lambda, const double* Phi, Fld dPhidxi, double& dfixi, double& dfiyi,
                                       double& dfizi, double& dfixii, double& dfiyii, double& dfizii) {
  const double fxn = lambda, fxp = 1.0 - lambda;
  const double xpn = M.xc[ijn] - M.xc[ijp], ypn = M.yc[ijn] - M.yc[ijp], zpn = M.zc[ijn] - M.zc[ijp];
  const double vole = xpn * arx + ypn * ary + zpn * arz;
  dfixi = dPhidxi.x(ijp) * fxp + dPhidxi.x(ijn) * fxn;
  dfiyi = dPhidxi.y(ijp) * fxp + dPhidxi.y(ijn) * fxn;
  dfizi = dPhidxi.z(ijp) * fxp + dPhidxi.z(ijn) * fxn;
  dfixii = dfixi + arx / vole * (Phi[ijn] - Phi[ijp] - dfixi * xpn - dfiyi * ypn - dfizi * zpn);
  dfiyii = dfiyi + ary / vole * (Phi[ijn] - Phi[ijp] - dfixi * xpn - dfiyi * ypn - dfizi * zpn);
  dfizii = dfizi + arz / vole * (Phi[ijn] - Phi[ijp] - dfixi * xpn - dfiyi * ypn - dfizi * zpn);
  dfixi = dfixi * (arx - M.Df[i] * xpn);
  dfiyi = dfiyi * (ary - M.Df[i] * ypn);
  dfizi = dfizi * (arz - M.Df[i] * zpn);
}

// facefluxuvw, velocity.f90:754-878: a(k_ij)=can, a(k_ji)=cap; sources to scratch
__global__ void k_mom_face(MeshView M, Dev D, MomParams P) {
  const int nT = M.nT;
  const Fld gu{D.gu, nT}, gv{D.gv, nT}, gw{D.gw, nT};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double xf = M.xf[i], yf = M.yf[i], zf = M.zf[i];
    const double arx = M.arx[i], ary = M.ary[i], arz = M.arz[i];
    const double flomass = D.flmass[i], lambda = M.facint[i], gam = P.gds;
    const double fxn = lambda, fxp = 1.0 - lambda;
    const double game = D.vis[ijp] + (D.vis[ijn] - D.vis[ijp]) * lambda;
    const double de = game * M.Df[i];
    const double ce = fmin(flomass, 0.0), cp = fmax(flomass, 0.0);
    const double can = -de + ce;
    const double cap = -de - cp;
    double duxi, duyi, duzi, duxii, duyii, duzii, dvxi, dvyi, dvzi, dvxii, dvyii, dvzii, dwxi, dwyi, dwzi, dwxii,
        dwyii, dwzii;
    sngrad(M, i, ijp, ijn, arx, ary, arz, lambda, D.u, gu, duxi, duyi, duzi, duxii, duyii, duzii);
    sngrad(M, i, ijp, ijn, arx, ary, arz, lambda, D.v, gv, dvxi, dvyi, dvzi, dvxii, dvyii, dvzii);
    sngrad(M, i, ijp, ijn, arx, ary, arz, lambda, D.w, gw, dwxi, dwyi, dwzi, dwxii, dwyii, dwzii);
    double fdue = game * (duxii * arx + dvxii * ary + dwxii * arz);
    double fdve = game * (duyii * arx + dvyii * ary + dwyii * arz);
    double fdwe = game * (duzii * arx + dvzii * ary + dwzii * arz);
    const double fdui = game * (duxi + duyi + duzi);
    const double fdvi = game * (dvxi + dvyi + dvzi);
    const double fdwi = game * (dwxi + dwyi + dwzi);
    fdue = fdue + fdui;
    fdve = fdve + fdvi;
    fdwe = fdwe + fdwi;
    const double fuuds = cp * D.u[ijp] + ce * D.u[ijn];
    const double fvuds = cp * D.v[ijp] + ce * D.v[ijn];
    const double fwuds = cp * D.w[ijp] + ce * D.w[ijn];
    double ue, ve, we;
    if (flomass >= 0.0) {
      ue = face_value(M, ijp, ijn, xf, yf, zf, fxp, D.u, gu, P.scheme);
      ve = face_value(M, ijp, ijn, xf, yf, zf, fxp, D.v, gv, P.scheme);
      we = face_value(M, ijp, ijn, xf, yf, zf, fxp, D.w, gw, P.scheme);
    } else {
      ue = face_value(M, ijn, ijp, xf, yf, zf, fxn, D.u, gu, P.scheme);
      ve = face_value(M, ijn, ijp, xf, yf, zf, fxn, D.v, gv, P.scheme);
      we = face_value(M, ijn, ijp, xf, yf, zf, fxn, D.w, gw, P.scheme);
    }
    const double fuhigh = flomass * ue, fvhigh = flomass * ve, fwhigh = flomass * we;
    D.a[M.ijk[i]] = can;
    D.a[M.jik[i]] = cap;
    D.fscr[i] = -(gam * (fuhigh - fuuds)) + fdue;
    D.fscr[M.nIP + i] = -(gam * (fvhigh - fvuds)) + fdve;
    D.fscr[2 * (size_t)M.nIP + i] = -(gam * (fwhigh - fwuds)) + fdwe;
  }
}

// facefluxuvw_periodic, velocity.f90:1038-1179, per periodic pair (the
// periodic branch of calcuvw's boundary loop, :393-430): central weights
// 1/2, the distance vector 2 (xf - xc(ijp)), the full stress tensor of the
// face gradient, cds face values; a(k_ij) = can, a(k_ji) = cap, sources to
// scratch entry nI + q
__global__ void k_mom_pair(MeshView M, Dev D, MomParams P) {
  const int nT = M.nT;
  const Fld gu{D.gu, nT}, gv{D.gv, nT}, gw{D.gw, nT};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < M.nPer; q += gridDim.x * blockDim.x) {
    const int f = M.pface[q], ijp = M.owner[f], ijn = M.owner[M.ptwin[q]];
    const double xf = M.xf[f], yf = M.yf[f], zf = M.zf[f], arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
    const double flomass = D.flmass[f], gam = P.gds;
    const double fxn = 0.5, fxp = fxn;
    const double xpn = 2 * (xf - M.xc[ijp]), ypn = 2 * (yf - M.yc[ijp]), zpn = 2 * (zf - M.zc[ijp]);
    const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    const double are = sqrt(arx * arx + ary * ary + arz * arz);
    const double game = D.vis[ijp] * fxp + D.vis[ijn] * fxn;
    const double de = game * (arx * arx + ary * ary + arz * arz) / (xpn * arx + ypn * ary + zpn * arz);
    const double ce = fmin(flomass, 0.0), cp = fmax(flomass, 0.0);
    const double can = -de + ce;
    const double cap = -de - cp;
    const double duxi = gu.x(ijp) * fxp + gu.x(ijn) * fxn, duyi = gu.y(ijp) * fxp + gu.y(ijn) * fxn,
                 duzi = gu.z(ijp) * fxp + gu.z(ijn) * fxn;
    const double dvxi = gv.x(ijp) * fxp + gv.x(ijn) * fxn, dvyi = gv.y(ijp) * fxp + gv.y(ijn) * fxn,
                 dvzi = gv.z(ijp) * fxp + gv.z(ijn) * fxn;
    const double dwxi = gw.x(ijp) * fxp + gw.x(ijn) * fxn, dwyi = gw.y(ijp) * fxp + gw.y(ijn) * fxn,
                 dwzi = gw.z(ijp) * fxp + gw.z(ijn) * fxn;
    const double fdue = game * ((duxi + duxi) * arx + (duyi + dvxi) * ary + (duzi + dwxi) * arz);
    const double fdve = game * ((duyi + dvxi) * arx + (dvyi + dvyi) * ary + (dvzi + dwyi) * arz);
    const double fdwe = game * ((duzi + dwxi) * arx + (dwyi + dvzi) * ary + (dwzi + dwzi) * arz);
    const double fdui = game * are / dpn * (duxi * xpn + duyi * ypn + duzi * zpn);
    const double fdvi = game * are / dpn * (dvxi * xpn + dvyi * ypn + dvzi * zpn);
    const double fdwi = game * are / dpn * (dwxi * xpn + dwyi * ypn + dwzi * zpn);
    const double fuuds = cp * D.u[ijp] + ce * D.u[ijn];
    const double fvuds = cp * D.v[ijp] + ce * D.v[ijn];
    const double fwuds = cp * D.w[ijp] + ce * D.w[ijn];
    double ue, ve, we;
    if (flomass >= 0.0) {  // face_value_cds, interpolation.f90:116-157
      ue = D.u[ijp] + (D.u[ijn] - D.u[ijp]) * fxp;
      ve = D.v[ijp] + (D.v[ijn] - D.v[ijp]) * fxp;
      we = D.w[ijp] + (D.w[ijn] - D.w[ijp]) * fxp;
    } else {
      ue = D.u[ijn] + (D.u[ijp] - D.u[ijn]) * fxn;
      ve = D.v[ijn] + (D.v[ijp] - D.v[ijn]) * fxn;
      we = D.w[ijn] + (D.w[ijp] - D.w[ijn]) * fxn;
    }
    const double fuhigh = flomass * ue, fvhigh = flomass * ve, fwhigh = flomass * we;
    const int l = M.nI + q;
    D.a[M.ijk[l]] = can;
    D.a[M.jik[l]] = cap;
    D.fscr[l] = -gam * (fuhigh - fuuds) + fdue - fdui;
    D.fscr[M.nIP + l] = -gam * (fvhigh - fvuds) + fdve - fdvi;
    D.fscr[2 * (size_t)M.nIP + l] = -gam * (fwhigh - fwuds) + fdwe - fdwi;
  }
}

// facefluxuvw_bnd, velocity.f90:882-1034
__device__ void facefluxuvw_bnd(const MeshView& M, const Dev& D, int ijp, int ijb, int f, double& cb, double& sup,
                                double& svp, double& swp) {
  const int nT = M.nT;
  const double xf = M.xf[f], yf = M.yf[f], zf = M.zf[f], arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
  const double flomass = D.flmass[f];
  const double xpn = xf - M.xc[ijp], ypn = yf - M.yc[ijp], zpn = zf - M.zc[ijp];
  const double vole = xpn * arx + ypn * ary + zpn * arz;
  const double Dfi = (arx * arx + ary * ary + arz * arz) / vole;
  const double game = D.vis[ijb];
  const double de = game * Dfi;
  cb = -de + fmin(flomass, 0.0);  // 'can' of the reference, returned as cb
  double comp[3][6];
  const double* flds[3] = {D.u, D.v, D.w};
  const double* grads[3] = {D.gu, D.gv, D.gw};
  for (int q = 0; q < 3; ++q) {
    const double* F = flds[q];
    const Fld g{grads[q], nT};
    double dxi = g.x(ijp), dyi = g.y(ijp), dzi = g.z(ijp);
    const double dxii = dxi + arx / vole * (F[ijb] - F[ijp] - dxi * xpn - dyi * ypn - dzi * zpn);
    const double dyii = dyi + ary / vole * (F[ijb] - F[ijp] - dxi * xpn - dyi * ypn - dzi * zpn);
    const double dzii = dzi + arz / vole * (F[ijb] - F[ijp] - dxi * xpn - dyi * ypn - dzi * zpn);
    dxi = dxi * (arx - Dfi * xpn);
    dyi = dyi * (ary - Dfi * ypn);
    dzi = dzi * (arz - Dfi * zpn);
    comp[q][0] = dxi; comp[q][1] = dyi; comp[q][2] = dzi;
    comp[q][3] = dxii; comp[q][4] = dyii; comp[q][5] = dzii;
  }
  const double fdue = game * (comp[0][3] * arx + comp[1][3] * ary + comp[2][3] * arz);
  const double fdve = game * (comp[0][4] * arx + comp[1][4] * ary + comp[2][4] * arz);
  const double fdwe = game * (comp[0][5] * arx + comp[1][5] * ary + comp[2][5] * arz);
  const double fdui = game * (comp[0][0] + comp[0][1] + comp[0][2]);
  const double fdvi = game * (comp[1][0] + comp[1][1] + comp[1][2]);
  const double fdwi = game * (comp[2][0] + comp[2][1] + comp[2][2]);
  sup = fdue + fdui;
  svp = fdve + fdvi;
  swp = fdwe + fdwi;
}

// sources and diagonal contributions per cell: inner-face sources in face
// order (velocity.f90:306-313), then the boundary conditions (:326-562) in
// patch order, the periodic pairs' sources on both of their cells (:393-430)
__global__ void k_mom_cell(MeshView M, Dev D, MomParams P) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double su = D.su[c], sv = D.sv[c], sw = D.sw[c];
    double spu = 0.0, spv = 0.0, sp = 0.0;
    // unsteady term, velocity.f90:226-290 (before the face fluxes)
    if (P.tscheme != FC_TIME_STEADY) {
      const double apotime = D.den[c] * M.vol[c] / P.timestep;
      if (P.tscheme == FC_TIME_BDF) {
        su = su + apotime * D.uo[c];
        sv = sv + apotime * D.vo[c];
        sw = sw + apotime * D.wo[c];
        spu = spu + apotime; spv = spv + apotime; sp = sp + apotime;
      } else if (P.tscheme == FC_TIME_BDF2) {
        su = su + apotime * (2 * D.uo[c] - 0.5 * D.uoo[c]);
        sv = sv + apotime * (2 * D.vo[c] - 0.5 * D.voo[c]);
        sw = sw + apotime * (2 * D.wo[c] - 0.5 * D.woo[c]);
        spu = spu + 1.5 * apotime; spv = spv + 1.5 * apotime; sp = sp + 1.5 * apotime;
      } else {
        su = su + apotime * (3 * D.uo[c] - 1.5 * D.uoo[c] + 1. / 3.0 * D.uooo[c]);
        sv = sv + apotime * (3 * D.vo[c] - 1.5 * D.voo[c] + 1. / 3.0 * D.vooo[c]);
        sw = sw + apotime * (3 * D.wo[c] - 1.5 * D.woo[c] + 1. / 3.0 * D.wooo[c]);
        spu = spu + 11. / 6.0 * apotime; spv = spv + 11. / 6.0 * apotime; sp = sp + 11. / 6.0 * apotime;
      }
    }
    for (int q = M.af_ptr[c]; q < M.af_ptr[c + 1]; ++q) {
      const int f = M.af_ent[q];
      if (f < M.nI || f >= M.nF) {  // inner face, or the twin side of pair f - nF
        const int l = f < M.nI ? f : M.nI + (f - M.nF);
        const double sup = D.fscr[l], svp = D.fscr[M.nIP + l], swp = D.fscr[2 * (size_t)M.nIP + l];
        if (f < M.nI && M.owner[f] == c) { su = su + sup; sv = sv + svp; sw = sw + swp; }
        else { su = su - sup; sv = sv - svp; sw = sw - swp; }
        continue;
      }
      const int bi = f - M.nI, ijb = M.nC + bi, ijp = c;
      const int t = D.ptype[M.bpatch[bi]];
      if (t == FC_BC_PERIODIC) {  // the owner side of pair bpair
        const int l = M.nI + M.bpair[bi];
        su = su + D.fscr[l]; sv = sv + D.fscr[M.nIP + l]; sw = sw + D.fscr[2 * (size_t)M.nIP + l];
      } else if (t == FC_BC_INLET || t == FC_BC_OUTLET || t == FC_BC_PRESSURE) {
        double cb, sup, svp, swp;
        facefluxuvw_bnd(M, D, ijp, ijb, f, cb, sup, svp, swp);
        spu = spu - cb; spv = spv - cb; sp = sp - cb;
        su = su - cb * D.u[ijb] + sup;
        sv = sv - cb * D.v[ijb] + svp;
        sw = sw - cb * D.w[ijb] + swp;
      } else if (t == FC_BC_SYMMETRY) {
        const double are = sqrt(M.arx[f] * M.arx[f] + M.ary[f] * M.ary[f] + M.arz[f] * M.arz[f]);
        const double arer = 1.0 / are;
        const double nxf = M.arx[f] * arer, nyf = M.ary[f] * arer, nzf = M.arz[f] * arer;
        const double dpb = (M.xf[f] - M.xc[ijp]) * nxf + (M.yf[f] - M.yc[ijp]) * nyf + (M.zf[f] - M.zc[ijp]) * nzf;
        const double cf = 2 * P.vis_sym * are / dpb;
        su = su - cf * nxf * (nyf * D.v[ijp] + nzf * D.w[ijp]);
        sv = sv - cf * nyf * (nxf * D.u[ijp] + nzf * D.w[ijp]);
        sw = sw - cf * nzf * (nxf * D.u[ijp] + nyf * D.v[ijp]);
        spu = spu + cf * (nxf * nxf);
        spv = spv + cf * (nyf * nyf);
        sp = sp + cf * (nzf * nzf);
      } else if (t == FC_BC_WALL) {
        const double viss = fmax(P.viscos, D.visw[M.bwall[bi]]);
        const double are = sqrt(M.arx[f] * M.arx[f] + M.ary[f] * M.ary[f] + M.arz[f] * M.arz[f]);
        const double arer = 1.0 / are;
        const double nxf = M.arx[f] * arer, nyf = M.ary[f] * arer, nzf = M.arz[f] * arer;
        const double dpb = (M.xf[f] - M.xc[ijp]) * nxf + (M.yf[f] - M.yc[ijp]) * nyf + (M.zf[f] - M.zc[ijp]) * nzf;
        const double vsol = viss * are / dpb;
        const double upb = D.u[ijp] - D.u[ijb], vpb = D.v[ijp] - D.v[ijb], wpb = D.w[ijp] - D.w[ijb];
        spu = spu + vsol * (1. - nxf * nxf);
        spv = spv + vsol * (1. - nyf * nyf);
        sp = sp + vsol * (1. - nzf * nzf);
        su = su + vsol * (D.u[ijb] * (1. - nxf * nxf) + vpb * nyf * nxf + wpb * nzf * nxf);
        sv = sv + vsol * (upb * nxf * nyf + D.v[ijb] * (1. - nyf * nyf) + wpb * nzf * nyf);
        sw = sw + vsol * (upb * nxf * nzf + vpb * nyf * nzf + D.w[ijb] * (1. - nzf * nzf));
      }
    }
    D.su[c] = su; D.sv[c] = sv; D.sw[c] = sw;
    D.spu[c] = spu; D.spv[c] = spv; D.sp[c] = sp;
  }
}

// main diagonal = sp - sum(off-diagonal row), apx = 1/(a_P + small),
// under-relaxation (velocity.f90:611-635, :667-690, :722-745).  The U pass
// subtracts the diagonal slot as found (the previous matrix's value); V and
// W clear it first.
__global__ void k_mom_diag(int n, const int* __restrict__ ia, const int* __restrict__ diag, double* __restrict__ a,
                           const double* __restrict__ spx, double* __restrict__ apx, const double* __restrict__ src,
                           double* __restrict__ su, const double* __restrict__ fld, double urf, int clear_diag) {
  const double urfr = 1.0 / urf, urfm = 1.0 - urf;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int kd = diag[i];
    const double ad0 = clear_diag ? 0.0 : a[kd];
    double s = 0.0;
    for (int k = ia[i]; k < ia[i + 1]; ++k) s = s + (k == kd ? ad0 : a[k]);
    const double off = s - ad0;
    double ad = spx[i] - off;
    apx[i] = 1. / (ad + SMALL);
    ad = ad * urfr;
    a[kd] = ad;
    su[i] = src[i] + urfm * ad * fld[i];
  }
}

// ------------------------------------------------------------- pressure
// facefluxmass2, faceflux_mass.f90:175-249 (dPdxi weights as written there)
__global__ void k_p_face(MeshView M, Dev D) {
  const Fld gp{D.gp, M.nT};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double lambda = M.facint[i], fxn = lambda, fxp = 1.0 - lambda;
    const double xpn = M.xc[ijn] - M.xc[ijp], ypn = M.yc[ijn] - M.yc[ijp], zpn = M.zc[ijn] - M.zc[ijp];
    const double dene = D.den[ijp] * fxp + D.den[ijn] * fxn;
    const double Kj = M.vol[ijp] * D.apu[ijp] * fxp + M.vol[ijn] * D.apu[ijn] * fxn;
    const double cap = -(dene * Kj * M.Df[i]);
    const double ui = D.u[ijp] + (D.u[ijn] - D.u[ijp]) * lambda;
    const double vi = D.v[ijp] + (D.v[ijn] - D.v[ijp]) * lambda;
    const double wi = D.w[ijp] + (D.w[ijn] - D.w[ijp]) * lambda;
    const double dpxi = (gp.x(ijn) * fxp + gp.x(ijp) * fxn) * xpn;
    const double dpyi = (gp.y(ijn) * fxp + gp.y(ijp) * fxn) * ypn;
    const double dpzi = (gp.z(ijn) * fxp + gp.z(ijp) * fxn) * zpn;
    D.flmass[i] = dene * (ui * M.arx[i] + vi * M.ary[i] + wi * M.arz[i]) +
                  cap * (D.p[ijn] - D.p[ijp] - dpxi - dpyi - dpzi);
    D.a[M.ijk[i]] = cap;
    D.a[M.jik[i]] = cap;
  }
}

// facefluxmassPressBnd, faceflux_mass.f90:765-830, per pressure face:
// boundary velocity, mass flux and the face's coefficient cap of the
// pressure-correction equation (kept in bcap for k_p_cell); pp = 0 at the
// face (calcp_simple.f90:162-183)
__global__ void k_p_press(MeshView M, Dev D, double* __restrict__ bcap) {
  const Fld gp{D.gp, M.nT};
  for (int bi = blockIdx.x * blockDim.x + threadIdx.x; bi < M.nB; bi += gridDim.x * blockDim.x) {
    if (D.ptype[M.bpatch[bi]] != FC_BC_PRESSURE) continue;
    const int f = M.nI + bi, ijp = M.owner[f], ijb = M.nC + bi;
    const double arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
    const double xpn = M.xf[f] - M.xc[ijp], ypn = M.yf[f] - M.yc[ijp], zpn = M.zf[f] - M.zc[ijp];
    const double capp = M.vol[ijp] * D.apu[ijp] / (arx * xpn + ary * ypn + arz * zpn);
    const double dpcor = D.p[ijb] - D.p[ijp] - (gp.x(ijp) * xpn + gp.y(ijp) * ypn + gp.z(ijp) * zpn);
    const double ub = D.u[ijp] - arx * capp * dpcor;
    const double vb = D.v[ijp] - ary * capp * dpcor;
    const double wb = D.w[ijp] - arz * capp * dpcor;
    D.u[ijb] = ub; D.v[ijb] = vb; D.w[ijb] = wb;
    D.flmass[f] = D.den[ijp] * (ub * arx + vb * ary + wb * arz);
    bcap[bi] = -(D.den[ijp] * (arx * arx + ary * ary + arz * arz) * capp);
    D.pp[ijb] = 0.0;
  }
}

// facefluxmassCorrPressBnd, faceflux_mass.f90:699-762, per pressure face
// after a pressure-correction solve (calcp_simple.f90:344-356)
__global__ void k_p_press_corr(MeshView M, Dev D) {
  for (int bi = blockIdx.x * blockDim.x + threadIdx.x; bi < M.nB; bi += gridDim.x * blockDim.x) {
    if (D.ptype[M.bpatch[bi]] != FC_BC_PRESSURE) continue;
    const int f = M.nI + bi, ijp = M.owner[f], ijb = M.nC + bi;
    const double arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
    const double xpn = M.xf[f] - M.xc[ijp], ypn = M.yf[f] - M.yc[ijp], zpn = M.zf[f] - M.zc[ijp];
    const double cap = M.vol[ijp] * D.apu[ijp] / (arx * xpn + ary * ypn + arz * zpn);
    const double dpcor = -D.pp[ijp];
    D.u[ijb] = D.u[ijb] - arx * cap * dpcor;
    D.v[ijb] = D.v[ijb] - ary * cap * dpcor;
    D.w[ijb] = D.w[ijb] - arz * cap * dpcor;
    D.flmass[f] = D.flmass[f] - D.den[ijp] * (arx * arx + ary * ary + arz * arz) * cap * dpcor;
  }
}

// facefluxmass2_periodic, faceflux_mass.f90:313-384, per periodic pair (the
// periodic branch of calcp_simple.f90:185-225 and calcp_piso.f90:248-289):
// the pair's mass flux through its periodic face, cap in both slots.  Df is
// indexed by the face's position within its patch, as the reference writes it.
__global__ void k_p_pair(MeshView M, Dev D) {
  const Fld gp{D.gp, M.nT};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < M.nPer; q += gridDim.x * blockDim.x) {
    const int f = M.pface[q], ijp = M.owner[f], ijn = M.owner[M.ptwin[q]];
    const double arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
    const double lambda = 0.5, fxn = lambda, fxp = 1.0 - lambda;
    const double xpn = 2 * (M.xf[f] - M.xc[ijp]), ypn = 2 * (M.yf[f] - M.yc[ijp]), zpn = 2 * (M.zf[f] - M.zc[ijp]);
    const double dene = D.den[ijp] * fxp + D.den[ijn] * fxn;
    double Kj = M.vol[ijp] * D.apu[ijp] * fxp + M.vol[ijn] * D.apu[ijn] * fxn;
    const double cap = -(dene * Kj * M.Df[M.ppos[q]]);
    Kj = (D.apu[ijp] + D.apu[ijn] + SMALL);
    const double ui = (D.u[ijp] * D.apu[ijn] + D.u[ijn] * D.apu[ijp]) / Kj;
    const double vi = (D.v[ijp] * D.apv[ijn] + D.v[ijn] * D.apv[ijp]) / Kj;
    const double wi = (D.w[ijp] * D.apw[ijn] + D.w[ijn] * D.apw[ijp]) / Kj;
    const double dpxi = (gp.x(ijn) * fxp + gp.x(ijp) * fxn) * xpn;
    const double dpyi = (gp.y(ijn) * fxp + gp.y(ijp) * fxn) * ypn;
    const double dpzi = (gp.z(ijn) * fxp + gp.z(ijp) * fxn) * zpn;
    D.flmass[f] = dene * (ui * arx + vi * ary + wi * arz) + cap * (D.p[ijn] - D.p[ijp] - dpxi - dpyi - dpzi);
    const int l = M.nI + q;
    D.a[M.ijk[l]] = cap;
    D.a[M.jik[l]] = cap;
  }
}

// flux correction of the periodic pairs (calcp_simple.f90:322-342 with
// phi = pp, calcp_piso.f90:437-456 with phi = p): the twin face takes the
// periodic face's corrected mass flux
__global__ void k_flux_correct_pair(MeshView M, Dev D, const double* __restrict__ phi) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < M.nPer; q += gridDim.x * blockDim.x) {
    const int f = M.pface[q], t = M.ptwin[q], ijp = M.owner[f], ijn = M.owner[t];
    const double fm = D.flmass[f] + D.a[M.ijk[M.nI + q]] * (phi[ijn] - phi[ijp]);
    D.flmass[f] = fm;
    D.flmass[t] = fm;
  }
}

// diagonal -sum(cap) and source -/+flmass in face order (calcp_simple.f90:104-117),
// then inlet/outlet mass fluxes, pressure faces and periodic pairs
// (:131-225); a cell's boundary faces follow its inner faces and come in
// patch order, the order of the reference's loops
__global__ void k_p_cell(MeshView M, Dev D, const double* __restrict__ bcap) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double ad = 0.0, s = 0.0;
    for (int q = M.af_ptr[c]; q < M.af_ptr[c + 1]; ++q) {
      const int f = M.af_ent[q];
      if (f < M.nI) {
        ad = ad - D.a[M.ijk[f]];
        if (M.owner[f] == c) s = s - D.flmass[f];
        else s = s + D.flmass[f];
      } else if (f >= M.nF) {  // the twin side of pair f - nF
        const int pq = f - M.nF;
        ad = ad - D.a[M.ijk[M.nI + pq]];
        s = s + D.flmass[M.pface[pq]];
      } else {
        const int t = D.ptype[M.bpatch[f - M.nI]];
        if (t == FC_BC_PERIODIC) {
          ad = ad - D.a[M.ijk[M.nI + M.bpair[f - M.nI]]];
          s = s - D.flmass[f];
        } else if (t == FC_BC_INLET || t == FC_BC_OUTLET) s = s - D.flmass[f];
        else if (t == FC_BC_PRESSURE) {
          ad = ad - bcap[f - M.nI];
          s = s - D.flmass[f];
        }
      }
    }
    D.a[M.diag[c]] = ad;
    D.su[c] = s;
  }
}

// adjustMassFlow, faceflux_mass.f90:833-916: one thread, outlet faces in order
__global__ void k_adjust_mass_flow(MeshView M, Dev D, double flomas) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  double flowo = 0.0;
  for (int bi = 0; bi < M.nB; ++bi) {
    if (D.ptype[M.bpatch[bi]] != FC_BC_OUTLET) continue;
    const int f = M.nI + bi, p = M.owner[f], b = M.nC + bi;
    D.u[b] = D.u[p]; D.v[b] = D.v[p]; D.w[b] = D.w[p];
    D.flmass[f] = D.den[p] * (D.u[b] * M.arx[f] + D.v[b] * M.ary[f] + D.w[b] * M.arz[f]);
    flowo = flowo + D.flmass[f];
  }
  const double fac = flomas / (flowo + SMALL);
  for (int bi = 0; bi < M.nB; ++bi) {
    if (D.ptype[M.bpatch[bi]] != FC_BC_OUTLET) continue;
    const int f = M.nI + bi, b = M.nC + bi;
    D.flmass[f] = D.flmass[f] * fac;
    D.u[b] = D.u[b] * fac; D.v[b] = D.v[b] * fac; D.w[b] = D.w[b] * fac;
  }
}

// flmass += a(k_ij) (pp_N - pp_P)  (calcp_simple.f90:331-341)
__global__ void k_flux_correct(MeshView M, Dev D) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x)
    D.flmass[i] = D.flmass[i] + D.a[M.ijk[i]] * (D.pp[M.neighbour[i]] - D.pp[M.owner[i]]);
}

// u += su*apu, ..., p += urfP (pp - pp(pRefCell))  (calcp_simple.f90:406-419)
__global__ void k_correct_vel_p(int nC, Dev D, double urfP, int pref, int have_pref) {
  const double ppref = have_pref ? D.pp[pref] : 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nC; i += gridDim.x * blockDim.x) {
    D.u[i] = D.u[i] + D.su[i] * D.apu[i];
    D.v[i] = D.v[i] + D.sv[i] * D.apv[i];
    D.w[i] = D.w[i] + D.sw[i] * D.apw[i];
    D.p[i] = D.p[i] + urfP * (D.pp[i] - ppref);
  }
}

// fluxmc2, faceflux_mass.f90:650-696 (non-orthogonal corrector)
__global__ void k_fluxmc2_face(MeshView M, Dev D) {
  const Fld gp{D.gp, M.nT};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double sx = M.arx[i], sy = M.ary[i], sz = M.arz[i];
    const double xpn = M.xc[ijn] - M.xc[ijp], ypn = M.yc[ijn] - M.yc[ijp], zpn = M.zc[ijn] - M.zc[ijp];
    const double s2 = sx * sx + sy * sy + sz * sz;
    const double dn = xpn * sx + ypn * sy + zpn * sz;
    const double rapr = -(0.5 * (D.apu[ijp] * D.den[ijp] + D.apu[ijn] * D.den[ijn]));
    const double dpx = 0.5 * (gp.x(ijn) + gp.x(ijp));
    const double dpy = 0.5 * (gp.y(ijn) + gp.y(ijp));
    const double dpz = 0.5 * (gp.z(ijn) + gp.z(ijp));
    const double fmc = rapr * ((dn * sx - xpn * s2) * dpx + (dn * sy - ypn * s2) * dpy + (dn * sz - zpn * s2) * dpz);
    D.flmass[i] = D.flmass[i] + fmc;
    D.fscr[i] = fmc;
  }
}

__global__ void k_fluxmc2_cell(MeshView M, Dev D) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f >= M.nI) break;
      if (M.owner[f] == c) s = s - D.fscr[f];
      else s = s + D.fscr[f];
    }
    D.su[c] = s;
  }
}

// continuityErrors, continuityErrors.f90:1-77 (flmass indexed by the owner
// cell as written at :26-27): per-block partials of vol*|su*apu|, vol, su
__global__ void k_conterr(MeshView M, Dev D, double* __restrict__ part) {
  __shared__ double sm[3][8];
  double w = 0.0, vs = 0.0, gs = 0.0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f < M.nI) {
        const int ijp = M.owner[f];
        if (ijp == c) s = s - D.flmass[ijp];
        else s = s + D.flmass[ijp];
      } else {
        const int t = D.ptype[M.bpatch[f - M.nI]];
        if (t == FC_BC_INLET || t == FC_BC_OUTLET) s = s - D.flmass[f];
      }
    }
    w += M.vol[c] * fabs(s * D.apu[c]);
    vs += M.vol[c];
    gs += s;
    D.su[c] = 0.0;
  }
  double v3[3] = {w, vs, gs};
  for (int j = 0; j < 3; ++j) {
    double t = v3[j];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if ((threadIdx.x & 31) == 0) sm[j][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x < 3) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sm[threadIdx.x][k];
    part[threadIdx.x * gridDim.x + blockIdx.x] = t;
  }
}

// warp j sums the block partials of quantity j in a fixed order (lane l
// takes blocks l, l+32, ..., then a shuffle tree), so the sum is the same
// on every run; one thread per quantity looping over the partials took a
// thousand dependent loads
__global__ void k_conterr_final(const double* __restrict__ part, int nb, double* __restrict__ out) {
  const int j = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (j >= 3) return;
  double t = 0.0;
  for (int b = lane; b < nb; b += 32) t += part[j * nb + b];
  for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
  if (lane == 0) out[j] = t;
}

// inner-face mass flux from the face-interpolated velocity, init.f90:167-176
__global__ void k_init_flmass(MeshView M, Dev D) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double fxn = M.facint[i], fxp = 1.0 - M.facint[i];
    const double ui = D.u[ijp] * fxp + D.u[ijn] * fxn;
    const double vi = D.v[ijp] * fxp + D.v[ijn] * fxn;
    const double wi = D.w[ijp] * fxp + D.w[ijn] * fxn;
    D.flmass[i] = D.den[ijp] * (M.arx[i] * ui + M.ary[i] * vi + M.arz[i] * wi);
  }
}


// ------------------------------------------------------------ temperature
// ------------------------------------------------------------------- PISO
// su = rU - sum_nb h u_nb per cell, faces in ascending order (calcp_piso.f90:
// 94-117: owner terms through the (P,N) slot, neighbour terms through (N,P))
__global__ void k_piso_h(MeshView M, Dev D, const double* __restrict__ h) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double su = D.rU[c], sv = D.rV[c], sw = D.rW[c];
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f >= M.nI) break;
      double hk;
      int o;
      if (M.owner[f] == c) { hk = h[M.ijk[f]]; o = M.neighbour[f]; }
      else { hk = h[M.jik[f]]; o = M.owner[f]; }
      su = su - hk * D.u[o];
      sv = sv - hk * D.v[o];
      sw = sw - hk * D.w[o];
    }
    D.su[c] = su; D.sv[c] = sv; D.sw[c] = sw;
  }
}

// u = apu su (calcp_piso.f90:120-122)
__global__ void k_piso_u(int nC, Dev D) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nC; i += gridDim.x * blockDim.x) {
    D.u[i] = D.apu[i] * D.su[i];
    D.v[i] = D.apv[i] * D.sv[i];
    D.w[i] = D.apw[i] * D.sw[i];
  }
}

// facefluxmass_piso, faceflux_mass.f90:389-559: a(k_ij) = can, a(k_ji) = cap
__global__ void k_piso_face(MeshView M, Dev D) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double lambda = M.facint[i], fxn = lambda, fxp = 1.0 - lambda;
    const double dene = D.den[ijp] * fxp + D.den[ijn] * fxn;
    const double Kj = M.vol[ijp] * D.apu[ijp] * fxp + M.vol[ijn] * D.apu[ijn] * fxn;
    const double cap = -(dene * Kj * M.Df[i]);
    const double ui = D.u[ijp] + (D.u[ijn] - D.u[ijp]) * lambda;
    const double vi = D.v[ijp] + (D.v[ijn] - D.v[ijp]) * lambda;
    const double wi = D.w[ijp] + (D.w[ijn] - D.w[ijp]) * lambda;
    D.flmass[i] = dene * (ui * M.arx[i] + vi * M.ary[i] + wi * M.arz[i]);
    D.a[M.ijk[i]] = cap;
    D.a[M.jik[i]] = cap;
  }
}

// per-block sums of pp over the cells (pavg, calcp_piso.f90:361)
__global__ void k_sum_cells(const double* __restrict__ x, int nC, double* __restrict__ part) {
  __shared__ double sm[8];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nC; i += gridDim.x * blockDim.x) s += x[i];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += sm[k];
    part[blockIdx.x] = t;
  }
}

// the block sums into part[nb] (one thread, fixed order)
// the block partials summed by one warp in a fixed order (as k_conterr_final)
__global__ void k_sum_final(double* __restrict__ part, int nb) {
  if (blockIdx.x != 0 || threadIdx.x >= 32) return;
  double s = 0.0;
  for (int b = threadIdx.x; b < nb; b += 32) s += part[b];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) part[nb] = s;
}

// p = (1 - urfP) p + urfP (pp - pavg), pavg = sum(pp)/numCells (:361-363)
__global__ void k_piso_p(int nC, Dev D, const double* __restrict__ sum, double urfP) {
  const double pavg = *sum / (double)nC;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nC; i += gridDim.x * blockDim.x)
    D.p[i] = (1.0 - urfP) * D.p[i] + urfP * (D.pp[i] - pavg);
}

// fluxmc, faceflux_mass.f90:564-647 (the projections xpp, xep as written)
__global__ void k_fluxmc_face(MeshView M, Dev D) {
  const Fld gp{D.gp, M.nT};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double fxn = M.facint[i], fxp = 1.0 - M.facint[i];
    const double xf = M.xf[i], yf = M.yf[i], zf = M.zf[i], arx = M.arx[i], ary = M.ary[i], arz = M.arz[i];
    const double xpn = M.xc[ijn] - M.xc[ijp], ypn = M.yc[ijn] - M.yc[ijp], zpn = M.zc[ijn] - M.zc[ijp];
    const double are = sqrt(arx * arx + ary * ary + arz * arz);
    const double nxx = arx / are, nyy = ary / are, nzz = arz / are;
    double xpp = xf - (xf - M.xc[ijp]) * nxx, ypp = yf - (yf - M.yc[ijp]) * nyy, zpp = zf - (zf - M.zc[ijp]) * nzz;
    double xep = xf - (xf - M.xc[ijn]) * nxx, yep = yf - (yf - M.yc[ijn]) * nyy, zep = zf - (zf - M.zc[ijn]) * nzz;
    xpp = xpp - M.xc[ijp]; ypp = ypp - M.yc[ijp]; zpp = zpp - M.zc[ijp];
    xep = xep - M.xc[ijn]; yep = yep - M.yc[ijn]; zep = zep - M.zc[ijn];
    const double rapr = -((D.apu[ijp] * D.den[ijp] * M.vol[ijp] * fxp + D.apu[ijn] * D.den[ijn] * M.vol[ijn] * fxn) *
                          are / (xpn * nxx + ypn * nyy + zpn * nzz));
    D.fscr[i] = rapr * ((gp.x(ijn) * xep - gp.x(ijp) * xpp) + (gp.y(ijn) * yep - gp.y(ijp) * ypp) +
                        (gp.z(ijn) * zep - gp.z(ijp) * zpp));
  }
}

// su -= fmcor at the owner, += at the neighbour, on top of su (:382-392)
__global__ void k_fluxmc_cell(MeshView M, Dev D) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double s = D.su[c];
    for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
      const int f = M.cf_face[q];
      if (f >= M.nI) break;
      if (M.owner[f] == c) s = s - D.fscr[f];
      else s = s + D.fscr[f];
    }
    D.su[c] = s;
  }
}

// flmass += a(k_ij) (p_N - p_P) (:396-401)
__global__ void k_flux_correct_p(MeshView M, Dev D) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x)
    D.flmass[i] = D.flmass[i] + D.a[M.ijk[i]] * (D.p[M.neighbour[i]] - D.p[M.owner[i]]);
}

// u += su apu (:413-415)
__global__ void k_vel_correct(int nC, Dev D) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nC; i += gridDim.x * blockDim.x) {
    D.u[i] = D.u[i] + D.su[i] * D.apu[i];
    D.v[i] = D.v[i] + D.sv[i] * D.apv[i];
    D.w[i] = D.w[i] + D.sw[i] * D.apw[i];
  }
}

struct ScParams {
  double viscos, prl, prtr, sigt, pranl, gam;
  int scheme;
  const int* pkind;   // per patch: SC_* below
  const int* pwall;   // per patch: iWall before its first face (isothermal walls)
  const int* pstart;  // per patch: boundary index of its first face
};
enum { SC_NONE = 0, SC_FLOW = 1, SC_ISOTHERMAL = 2, SC_ADIABATIC = 3 };

// facefluxsc (inner face i), scalar_fluxes.f90:32-141, for a given diffusion
// coefficient: the matrix coefficients and the explicit source suadd
__device__ __forceinline__ void facefluxsc_inner(const MeshView& M, int i, int ijp, int ijn, double fm, double dcoef,
                                                 double gam, int scheme, const double* fi, const Fld& g,
                                                 double& cap, double& can, double& suadd) {
  const double lambda = M.facint[i];
  const double arx = M.arx[i], ary = M.ary[i], arz = M.arz[i];
  const double fxn = lambda, fxp = 1.0 - lambda;
  const double xpn = M.xc[ijn] - M.xc[ijp], ypn = M.yc[ijn] - M.yc[ijp], zpn = M.zc[ijn] - M.zc[ijp];
  const double Df = M.Df[i];
  const double de = dcoef * Df;
  const double ce = fmin(fm, 0.0), cp = fmax(fm, 0.0);
  can = -de + ce;
  cap = -de - cp;
  double dfixi = g.x(ijp) * fxp + g.x(ijn) * fxn;
  double dfiyi = g.y(ijp) * fxp + g.y(ijn) * fxn;
  double dfizi = g.z(ijp) * fxp + g.z(ijn) * fxn;
  dfixi = dfixi * (arx - Df * xpn);
  dfiyi = dfiyi * (ary - Df * ypn);
  dfizi = dfizi * (arz - Df * zpn);
  const double fdfie = dcoef * (dfixi + dfiyi + dfizi);
  double fii;
  if (fm >= 0.0) fii = face_value(M, ijp, ijn, M.xf[i], M.yf[i], M.zf[i], fxp, fi, g, scheme);
  else fii = face_value(M, ijn, ijp, M.xf[i], M.yf[i], M.zf[i], fxn, fi, g, scheme);
  double fcfie = fm * fii;
  const double fcfii = ce * fi[ijn] + cp * fi[ijp];
  fcfie = gam * (fcfie - fcfii);
  suadd = -fcfie + fdfie;
}

// facefluxsc_boundary, scalar_fluxes.f90:256-337, face f of cell ijp: can
// and suadd (cap is not used by the callers)
__device__ __forceinline__ void facefluxsc_bnd(const MeshView& M, int f, int ijp, double fm, double dcoef,
                                               const Fld& g, double& can, double& suadd) {
  const double arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
  const double xpn = M.xf[f] - M.xc[ijp], ypn = M.yf[f] - M.yc[ijp], zpn = M.zf[f] - M.zc[ijp];
  const double Dfi = (arx * arx + ary * ary + arz * arz) / (xpn * arx + ypn * ary + zpn * arz);
  const double de = dcoef * Dfi;
  can = -de + fmin(fm, 0.0);
  double dfixi = g.x(ijp), dfiyi = g.y(ijp), dfizi = g.z(ijp);
  dfixi = dfixi * (arx - Dfi * xpn);
  dfiyi = dfiyi * (ary - Dfi * ypn);
  dfizi = dfizi * (arz - Dfi * zpn);
  suadd = dcoef * (dfixi + dfiyi + dfizi);
}

// facefluxsc_periodic, scalar_fluxes.f90:147-251, pair q, with the pair's
// two cell values fp (owner side) and fn (twin side): central weights 1/2,
// the distance vector 2 (xf - xc(ijp)), Df of the face's position in its
// patch (as written there), cds face value
__device__ __forceinline__ void facefluxsc_pair2(const MeshView& M, int q, int ijp, int ijn, double fm, double dcoef,
                                                 double gam, double fp, double fn, const Fld& g, double& cap,
                                                 double& can, double& suadd) {
  const int f = M.pface[q], i = M.ppos[q];
  const double arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
  const double fxn = 0.5, fxp = fxn;
  const double xpn = 2 * (M.xf[f] - M.xc[ijp]), ypn = 2 * (M.yf[f] - M.yc[ijp]), zpn = 2 * (M.zf[f] - M.zc[ijp]);
  const double Df = M.Df[i];
  const double de = dcoef * Df;
  const double ce = fmin(fm, 0.0), cp = fmax(fm, 0.0);
  can = -de + ce;
  cap = -de - cp;
  double dfixi = g.x(ijp) * fxp + g.x(ijn) * fxn;
  double dfiyi = g.y(ijp) * fxp + g.y(ijn) * fxn;
  double dfizi = g.z(ijp) * fxp + g.z(ijn) * fxn;
  dfixi = dfixi * (arx - Df * xpn);
  dfiyi = dfiyi * (ary - Df * ypn);
  dfizi = dfizi * (arz - Df * zpn);
  const double fdfie = dcoef * (dfixi + dfiyi + dfizi);
  const double fii = fm >= 0.0 ? fp + (fn - fp) * fxp : fn + (fp - fn) * fxn;
  double fcfie = fm * fii;
  const double fcfii = ce * fn + cp * fp;
  fcfie = gam * (fcfie - fcfii);
  suadd = -fcfie + fdfie;
}

// the same with the cell values read from the field fi
__device__ __forceinline__ void facefluxsc_pair(const MeshView& M, int q, int ijp, int ijn, double fm, double dcoef,
                                                double gam, const double* fi, const Fld& g, double& cap, double& can,
                                                double& suadd) {
  facefluxsc_pair2(M, q, ijp, ijn, fm, dcoef, gam, fi[ijp], fi[ijn], g, cap, can, suadd);
}

// facefluxsc (inner face), scalar_fluxes.f90:32-141, with the diffusion
// coefficient of temperature.f90:122: a(k_ij)=can, a(k_ji)=cap, suadd to scratch
__global__ void k_sc_face(MeshView M, Dev D, ScParams P) {
  const Fld g{D.gt, M.nT};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double lambda = M.facint[i];
    const double dcoef =
        P.viscos * P.prl + ((D.vis[ijp] + (D.vis[ijn] - D.vis[ijp]) * lambda) - P.viscos) * P.prtr;
    double cap, can, suadd;
    facefluxsc_inner(M, i, ijp, ijn, D.flmass[i], dcoef, P.gam, P.scheme, D.t, g, cap, can, suadd);
    D.a[M.ijk[i]] = can;
    D.a[M.jik[i]] = cap;
    D.fscr[i] = suadd;
  }
}

// facefluxsc_periodic, scalar_fluxes.f90:147-251, per periodic pair (the
// periodic branch of temperature.f90:262-313): the diffusion coefficient
// with facint, and Df, of the face's position within its patch, as written
// there; central weights 1/2, cds face value; a(k_ij) = can, a(k_ji) = cap,
// suadd to scratch entry nI + q
__global__ void k_sc_pair(MeshView M, Dev D, ScParams P) {
  const Fld g{D.gt, M.nT};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < M.nPer; q += gridDim.x * blockDim.x) {
    const int f = M.pface[q], ijp = M.owner[f], ijn = M.owner[M.ptwin[q]], i = M.ppos[q];
    const double dcoef =
        P.viscos * P.prl + ((D.vis[ijp] + (D.vis[ijn] - D.vis[ijp]) * M.facint[i]) - P.viscos) * P.prtr;
    double cap, can, suadd;
    facefluxsc_pair(M, q, ijp, ijn, D.flmass[f], dcoef, P.gam, D.t, g, cap, can, suadd);
    const int l = M.nI + q;
    D.a[M.ijk[l]] = can;
    D.a[M.jik[l]] = cap;
    D.fscr[l] = suadd;
  }
}

// per cell in face order: the main-diagonal accumulation a(diag) -= can/cap
// and su +/- suadd of the inner faces (temperature.f90:137-155), then the
// boundary conditions of :166-225 (facefluxsc_boundary, scalar_fluxes.f90:256-337)
__global__ void k_sc_cell(MeshView M, Dev D, ScParams P) {
  const Fld g{D.gt, M.nT};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double ad = 0.0, su = 0.0, sp = 0.0;
    for (int q = M.af_ptr[c]; q < M.af_ptr[c + 1]; ++q) {
      const int f = M.af_ent[q];
      if (f < M.nI) {
        if (M.owner[f] == c) { ad = ad - D.a[M.ijk[f]]; su = su + D.fscr[f]; }
        else { ad = ad - D.a[M.jik[f]]; su = su - D.fscr[f]; }
        continue;
      }
      if (f >= M.nF) {  // the twin side of pair f - nF
        const int l = M.nI + (f - M.nF);
        ad = ad - D.a[M.jik[l]];
        su = su - D.fscr[l];
        continue;
      }
      const int bi = f - M.nI, ijb = M.nC + bi, ijp = c, b = M.bpatch[bi];
      if (D.ptype[b] == FC_BC_PERIODIC) {
        const int l = M.nI + M.bpair[bi];
        ad = ad - D.a[M.ijk[l]];
        su = su + D.fscr[l];
        continue;
      }
      const int kind = P.pkind[b];
      if (kind == SC_FLOW) {
        const double dcoef = P.viscos * P.prl + (D.vis[ijp] - P.viscos) / P.sigt;
        double can, suadd;
        facefluxsc_bnd(M, f, ijp, D.flmass[f], dcoef, g, can, suadd);
        sp = sp - can;
        su = su - can * D.t[ijb] + suadd;
      } else if (kind == SC_ISOTHERMAL) {
        const int iwall = P.pwall[b] + (bi - P.pstart[b]);
        double dcoef = P.viscos / P.pranl + (D.vis[ijp] - P.viscos) / P.sigt;
        dcoef = dcoef * M.srdw[iwall];
        sp = sp + dcoef;
        su = su + dcoef * D.t[ijb];
      } else if (kind == SC_ADIABATIC) {
        D.t[ijb] = D.t[ijp];
      }
    }
    D.a[M.diag[c]] = ad;
    D.su[c] = su;
    D.sp[c] = sp;
  }
}

// updateBoundary(T), updateBoundary.f90:1-77: outlet, symmetry, pressure
// and empty faces take the owner's value; a periodic face and its twin the
// mean of the pair's cells.  The reference visits the patches in order, so a
// twin face ends with the mean when its patch comes before the periodic one,
// else with its owner's value.
__global__ void k_update_boundary(MeshView M, const int* __restrict__ ptype, double* __restrict__ phi) {
  for (int bi = blockIdx.x * blockDim.x + threadIdx.x; bi < M.nB; bi += gridDim.x * blockDim.x) {
    const int t = ptype[M.bpatch[bi]];
    const int q = M.nPer ? M.bpair[bi] : -1;
    if (t == FC_BC_PERIODIC || (q >= 0 && M.pflag[q])) {
      const int ijp = M.owner[M.pface[q]], ijn = M.owner[M.ptwin[q]];
      phi[M.nC + bi] = 0.5 * (phi[ijp] + phi[ijn]);
    } else if (t == FC_BC_OUTLET || t == FC_BC_SYMMETRY || t == FC_BC_PRESSURE || t == FC_BC_EMPTY) {
      phi[M.nC + bi] = phi[M.owner[M.nI + bi]];
    }
  }
}

// min and max of phi(1:n) per block (temperature.f90:375-376)
__global__ void k_minmax(int n, const double* __restrict__ phi, double* __restrict__ part) {
  __shared__ double smin[32], smax[32];
  double lo = INFINITY, hi = -INFINITY;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    lo = fmin(lo, phi[i]);
    hi = fmax(hi, phi[i]);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if ((threadIdx.x & 31) == 0) { smin[threadIdx.x >> 5] = lo; smax[threadIdx.x >> 5] = hi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) { lo = fmin(lo, smin[w]); hi = fmax(hi, smax[w]); }
    part[blockIdx.x] = lo;
    part[gridDim.x + blockIdx.x] = hi;
  }
}

// T = max(T, small) on the cells when min(T) < 0 (temperature.f90:381);
// every block folds the per-block minima itself
__global__ void k_clip_small(int n, double* __restrict__ phi, const double* __restrict__ part, int nb) {
  // every block reduces the per-block minima itself, all threads sharing the
  // loads (a single thread's serial loop over them dominated the pass)
  __shared__ double s_w[32];
  __shared__ double s_lo;
  double lo = INFINITY;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) lo = fmin(lo, part[b]);
  for (int o = 16; o > 0; o >>= 1) lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
  if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = lo;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = s_w[0];
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmin(m, s_w[w]);
    s_lo = m;
  }
  __syncthreads();
  if (!(s_lo < 0.0)) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    phi[i] = fmax(phi[i], SMALL);
}


// ---------------------------------------------------------------- k-omega SST
// k_omega_SST.f90:21-38 and parameters.f90:15-17
#define SST_BETTAST 0.09
#define SST_SIGMK1 0.85
#define SST_SIGMK2 1.0
#define SST_SIGMOM1 0.5
#define SST_SIGMOM2 0.856
#define SST_BETAI1 0.075
#define SST_BETAI2 0.0828
#define SST_A1 0.31
#define SST_ALPHA2 0.44
#define SST_CAPPA 0.41
#define SST_ELOG 8.432

struct Turb {  // the model's device fields and constants of one call
  double *te, *ed, *fsst, *gte, *ged, *gen, *mag, *wd, *tau, *ypl;
  double viscos, densit, cmu25, alpha1;
};

// calc_strain_and_vorticity.f90:1-60: the strain magnitude sqrt(2 Sij Sij)
__global__ void k_sst_strain(int nC, int nT, const double* __restrict__ gu, const double* __restrict__ gv,
                             const double* __restrict__ gw, double* __restrict__ mag) {
  const Fld u{gu, nT}, v{gv, nT}, w{gw, nT};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += gridDim.x * blockDim.x) {
    const double s11 = u.x(c), s12 = 0.5 * (u.y(c) + v.x(c)), s13 = 0.5 * (u.z(c) + w.x(c));
    const double s22 = v.y(c), s23 = 0.5 * (v.z(c) + w.y(c)), s33 = w.z(c);
    mag[c] = sqrt(2 * (s11 * s11 + s22 * s22 + s33 * s33 + 2 * (s12 * s12 + s13 * s13 + s23 * s23)));
  }
}

// k sources, k_omega_SST.f90:159-219: the production and its limiter, the
// production to su, the destruction beta* omega rho vol to sp
__global__ void k_sst_src_k(MeshView M, Dev D, Turb T) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double gen = fabs(D.vis[c] - T.viscos) * T.mag[c] * T.mag[c];
    gen = fmin(gen, 0.9 * D.den[c] * T.te[c] * T.ed[c]);
    T.gen[c] = gen;
    const double genp = fmax(gen, 0.0), genn = fmin(gen, 0.0);
    D.su[c] = genp * M.vol[c];
    double sp = SST_BETTAST * T.ed[c] * D.den[c] * M.vol[c];
    D.sp[c] = sp - genn * M.vol[c] / (T.te[c] + SMALL);
  }
}

// omega sources, k_omega_SST.f90:300-398: the blending function F1 (fsst),
// production alpha gen / nu_t, cross diffusion, destruction beta rho omega^2
__global__ void k_sst_src_w(MeshView M, Dev D, Turb T) {
  const Fld gk{T.gte, M.nT}, gw{T.ged, M.nT};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    const double wldist = T.wd[c], den = D.den[c], te = T.te[c], ed = T.ed[c];
    const double dot = gk.x(c) * gw.x(c) + gk.y(c) * gw.y(c) + gk.z(c) * gw.z(c);
    const double domegapl = fmax(2 * SST_SIGMOM2 * den / (ed) * dot, SMALL);
    const double ksi = fmin(fmax(sqrt(te) / (SST_BETTAST * wldist * ed + SMALL),
                                 500.0 * T.viscos / den / (wldist * wldist * ed + SMALL)),
                            4.0 * den * te * SST_SIGMOM2 / (domegapl * (wldist * wldist)));
    const double ksi2 = ksi * ksi;
    const double f1 = tanh(ksi2 * ksi2);
    T.fsst[c] = f1;
    const double genp = fmax(T.gen[c], 0.0), genn = fmin(T.gen[c], 0.0);
    const double vist = (D.vis[c] - T.viscos) / T.densit;
    const double alphasst = f1 * T.alpha1 + (1.0 - f1) * SST_ALPHA2;
    double su = alphasst * genp * M.vol[c] / (vist + SMALL);
    double domega = 2 * (1.0 - f1) * den * SST_SIGMOM2 / (ed + SMALL) * dot;
    domega = fmax(domega, 0.0);
    D.su[c] = su + domega * M.vol[c];
    const double bettasst = f1 * SST_BETAI1 + (1.0 - f1) * SST_BETAI2;
    const double sp = bettasst * den * ed * M.vol[c];
    D.sp[c] = sp - alphasst * genn * M.vol[c] / (vist * ed + SMALL);
  }
}

// the blended diffusion coefficient of cell c: sigma1 F1 + sigma2 (1 - F1)
__device__ __forceinline__ double sst_prtr(const Turb& T, int c, int ifi) {
  return ifi == 1 ? T.fsst[c] * SST_SIGMK1 + (1.0 - T.fsst[c]) * SST_SIGMK2
                  : T.fsst[c] * SST_SIGMOM1 + (1.0 - T.fsst[c]) * SST_SIGMOM2;
}

// inner faces of calcsc, k_omega_SST.f90:448-488: the owner's blended sigma
__global__ void k_sst_face(MeshView M, Dev D, Turb T, int ifi, double gam, int scheme) {
  const double* fi = ifi == 1 ? T.te : T.ed;
  const Fld g{ifi == 1 ? T.gte : T.ged, M.nT};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < M.nI; i += gridDim.x * blockDim.x) {
    const int ijp = M.owner[i], ijn = M.neighbour[i];
    const double prtr = sst_prtr(T, ijp, ifi);
    const double viste = (D.vis[ijp] + (D.vis[ijn] - D.vis[ijp]) * M.facint[i]) - T.viscos;
    const double dcoef = T.viscos + viste * prtr;
    double cap, can, suadd;
    facefluxsc_inner(M, i, ijp, ijn, D.flmass[i], dcoef, gam, scheme, fi, g, cap, can, suadd);
    D.a[M.ijk[i]] = can;
    D.a[M.jik[i]] = cap;
    D.fscr[i] = suadd;
  }
}

// omega fixed in a wall cell by its wall face w, k_omega_SST.f90:625-650
__device__ __forceinline__ double sst_wall_omega(const MeshView& M, const Dev& D, const Turb& T, int c, int w) {
  const double dnw = M.dnw[w];
  const double wlog = sqrt(T.te[c]) / (T.cmu25 * SST_CAPPA * dnw);
  const double wvis = 6.0 * (T.viscos / D.den[c]) / (SST_BETAI1 * (dnw * dnw));
  return sqrt(wvis * wvis + wlog * wlog);
}

// omega of cell c as the boundary loop leaves it when it reaches patch pb:
// the wall faces of earlier patches have already fixed it (the last one wins)
__device__ double sst_omega_before(const MeshView& M, const Dev& D, const Turb& T, int c, int pb) {
  double e = T.ed[c];
  for (int q = M.cf_ptr[c]; q < M.cf_ptr[c + 1]; ++q) {
    const int f = M.cf_face[q];
    if (f < M.nI) continue;
    const int bi = f - M.nI, b = M.bpatch[bi];
    if (b < pb && D.ptype[b] == FC_BC_WALL) e = sst_wall_omega(M, D, T, c, M.bwall[bi]);
  }
  return e;
}

// periodic pairs of calcsc, k_omega_SST.f90:521-560: the pair's mean sigma
// and mean viscosity.  In the omega equation the pair sees the omega values
// that the wall patches listed before its periodic patch have fixed.
__global__ void k_sst_pair(MeshView M, Dev D, Turb T, int ifi, double gam) {
  const double* fi = ifi == 1 ? T.te : T.ed;
  const Fld g{ifi == 1 ? T.gte : T.ged, M.nT};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < M.nPer; q += gridDim.x * blockDim.x) {
    const int f = M.pface[q], ijp = M.owner[f], ijn = M.owner[M.ptwin[q]];
    const double prtr = 0.5 * (sst_prtr(T, ijp, ifi) + sst_prtr(T, ijn, ifi));
    const double viste = 0.5 * (D.vis[ijp] + D.vis[ijn]) - T.viscos;
    const double dcoef = T.viscos + viste * prtr;
    double cap, can, suadd;
    if (ifi == 2) {
      const int pb = M.bpatch[f - M.nI];
      facefluxsc_pair2(M, q, ijp, ijn, D.flmass[f], dcoef, gam, sst_omega_before(M, D, T, ijp, pb),
                       sst_omega_before(M, D, T, ijn, pb), g, cap, can, suadd);
    } else {
      facefluxsc_pair(M, q, ijp, ijn, D.flmass[f], dcoef, gam, fi, g, cap, can, suadd);
    }
    const int l = M.nI + q;
    D.a[M.ijk[l]] = can;
    D.a[M.jik[l]] = cap;
    D.fscr[l] = suadd;
  }
}

// per cell, in the reference's order: the face sources, then the boundary
// conditions of k_omega_SST.f90:495-660 patch by patch (flow patches through
// facefluxsc_boundary; walls: the wall-function production of k, omega fixed
// in the wall cell with its matrix row cleared), then the main diagonal and
// the under-relaxation (:712-726)
__global__ void k_sst_cell(MeshView M, Dev D, Turb T, int ifi, double urf) {
  double* fi = ifi == 1 ? T.te : T.ed;
  const Fld g{ifi == 1 ? T.gte : T.ged, M.nT};
  const double urfrs = 1.0 / urf, urfms = 1.0 - urf;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    double su = D.su[c], sp = D.sp[c];
    int cleared_at = -1;  // list position of the last wall face that cleared the row
    for (int q = M.af_ptr[c]; q < M.af_ptr[c + 1]; ++q) {
      const int f = M.af_ent[q];
      if (f < M.nI) {
        if (M.owner[f] == c) su = su + D.fscr[f];
        else su = su - D.fscr[f];
        continue;
      }
      if (f >= M.nF) {  // the twin side of pair f - nF
        su = su - D.fscr[M.nI + (f - M.nF)];
        continue;
      }
      const int bi = f - M.nI, ijb = M.nC + bi;
      const int t = D.ptype[M.bpatch[bi]];
      if (t == FC_BC_PERIODIC) {
        su = su + D.fscr[M.nI + M.bpair[bi]];
      } else if (t == FC_BC_INLET || t == FC_BC_OUTLET || t == FC_BC_PRESSURE) {
        const double viste = D.vis[ijb] - T.viscos;
        const double dcoef = T.viscos + viste * sst_prtr(T, c, ifi);
        double can, suadd;
        facefluxsc_bnd(M, f, c, D.flmass[f], dcoef, g, can, suadd);
        sp = sp - can;
        su = su - can * fi[ijb] + suadd;
      } else if (t == FC_BC_WALL) {
        const int iw = M.bwall[bi];
        const double dnw = M.dnw[iw];
        if (ifi == 1) {
          su = su - T.gen[c] * M.vol[c];
          const double viss = fmax(T.viscos, D.visw[iw]);
          const double arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
          const double are = sqrt(arx * arx + ary * ary + arz * arz);
          const double nxf = arx / are, nyf = ary / are, nzf = arz / are;
          const double Vnp = D.u[c] * nxf + D.v[c] * nyf + D.w[c] * nzf;
          double xtp = D.u[c] - Vnp * nxf, ytp = D.v[c] - Vnp * nyf, ztp = D.w[c] - Vnp * nzf;
          const double Vtp = sqrt(xtp * xtp + ytp * ytp + ztp * ztp);
          xtp = xtp / Vtp;
          ytp = ytp / Vtp;
          ztp = ztp / Vtp;
          const double Ut2 = fabs((D.u[ijb] - D.u[c]) * xtp + (D.v[ijb] - D.v[c]) * ytp + (D.w[ijb] - D.w[c]) * ztp);
          const double tau = viss * Ut2 / dnw;
          T.tau[iw] = tau;
          const double gen = fabs(tau) * T.cmu25 * sqrt(T.te[c]) / (dnw * SST_CAPPA);
          T.gen[c] = gen;
          su = su + gen * M.vol[c];
        } else {
          const double ed = sst_wall_omega(M, D, T, c, iw);
          T.ed[c] = ed;
          su = ed;
          sp = 1.0;
          cleared_at = q;
        }
      }
    }
    const int kd = M.diag[c], k0 = M.ia[c], k1 = M.ia[c + 1];
    if (cleared_at >= 0) {
      // the row is cleared where the wall face comes; periodic pairs of
      // later patches write their slots of this row afterwards, as there
      int kslot[4];
      double kval[4];
      int nk = 0;
      for (int q = cleared_at + 1; q < M.af_ptr[c + 1] && nk < 4; ++q) {
        const int f = M.af_ent[q];
        int slot = -1;
        if (f >= M.nF) slot = M.jik[M.nI + (f - M.nF)];
        else if (f >= M.nI && D.ptype[M.bpatch[f - M.nI]] == FC_BC_PERIODIC) slot = M.ijk[M.nI + M.bpair[f - M.nI]];
        if (slot >= 0) { kslot[nk] = slot; kval[nk] = D.a[slot]; ++nk; }
      }
      for (int k = k0; k < k1; ++k) D.a[k] = 0.0;
      for (int j = 0; j < nk; ++j) D.a[kslot[j]] = kval[j];
    }
    double ad = sp;
    for (int k = k0; k < k1; ++k)
      if (k != kd) ad = ad - D.a[k];
    ad = ad * urfrs;
    D.a[kd] = ad;
    D.su[c] = su + urfms * ad * fi[c];
    D.sp[c] = sp;
  }
}

// modify_mu_eff, k_omega_SST.f90:800-830: the eddy viscosity with the F2
// limiter, under-relaxed
__global__ void k_sst_mu(MeshView M, Dev D, Turb T, double urf) {
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < M.nC; c += gridDim.x * blockDim.x) {
    const double visold = D.vis[c], wldist = T.wd[c], te = T.te[c], ed = T.ed[c], den = D.den[c];
    const double etha = fmax(2 * sqrt(te) / (SST_BETTAST * wldist * ed), (500 * T.viscos / den) / (wldist * wldist * ed));
    const double f2 = tanh(etha * etha);
    double vis = T.viscos + den * SST_A1 * te / (fmax(SST_A1 * ed, T.mag[c] * f2));
    D.vis[c] = urf * vis + (1.0 - urf) * visold;
  }
}

// the wall faces of modify_mu_eff, k_omega_SST.f90:836-955: y+, the wall
// shear stress and the wall viscosity from the blended wall law
__global__ void k_sst_mu_wall(MeshView M, Dev D, Turb T, int nwal, const int* __restrict__ wall_face) {
  for (int w = blockIdx.x * blockDim.x + threadIdx.x; w < nwal; w += gridDim.x * blockDim.x) {
    const int f = wall_face[w], c = M.owner[f], ijb = M.nC + (f - M.nI);
    const double dnw = M.dnw[w], den = D.den[c];
    const double arx = M.arx[f], ary = M.ary[f], arz = M.arz[f];
    const double are = sqrt(arx * arx + ary * ary + arz * arz);
    const double nxf = arx / are, nyf = ary / are, nzf = arz / are;
    const double Vnp = D.u[c] * nxf + D.v[c] * nyf + D.w[c] * nzf;
    const double xtp = D.u[c] - Vnp * nxf, ytp = D.v[c] - Vnp * nyf, ztp = D.w[c] - Vnp * nzf;
    const double Vtp = sqrt(xtp * xtp + ytp * ytp + ztp * ztp);
    const double Utau = sqrt(T.viscos * Vtp / (T.densit * dnw) + T.cmu25 * T.te[c]);
    const double ypl = den * Utau * dnw / T.viscos;
    T.ypl[w] = ypl;
    const double Utauvis = ypl;
    const double Utaulog = 1.0 / SST_CAPPA * log(SST_ELOG * ypl);
    const double uv2 = Utauvis * Utauvis, ul2 = Utaulog * Utaulog;
    const double Upl = sqrt(sqrt(uv2 * uv2 + ul2 * ul2));
    const double viscw = den * Utau * dnw / Upl;
    const double r = Vtp / Upl;
    T.tau[w] = den * (r * r);
    const double visw = fmax(T.viscos, viscw);
    D.visw[w] = visw;
    D.vis[ijb] = visw;
  }
}

// wall_distance.f90: non-wall boundary values of phi from the owners, then
// (after the Gauss gradient) d = -|grad phi| + sqrt(|grad phi|^2 + 2 phi)
__global__ void k_wd_bnd(MeshView M, const int* __restrict__ ptype, double* __restrict__ phi) {
  for (int bi = blockIdx.x * blockDim.x + threadIdx.x; bi < M.nB; bi += gridDim.x * blockDim.x)
    if (ptype[M.bpatch[bi]] != FC_BC_WALL) phi[M.nC + bi] = phi[M.owner[M.nI + bi]];
}
__global__ void k_wd_dist(int nC, int nT, const double* __restrict__ phi, const double* __restrict__ gphi,
                          double* __restrict__ wd) {
  const Fld g{gphi, nT};
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nC; c += gridDim.x * blockDim.x) {
    const double gx = g.x(c), gy = g.y(c), gz = g.z(c);
    wd[c] = -sqrt(gx * gx + gy * gy + gz * gz) + sqrt(gx * gx + gy * gy + gz * gz + 2 * phi[c]);
  }
}
__global__ void k_wd_init(int nC, int nT, const double* __restrict__ vol, double* __restrict__ q,
                          double* __restrict__ mu, double* __restrict__ phi) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nT; i += gridDim.x * blockDim.x) {
    if (i < nC) { q[i] = -vol[i]; mu[i] = 1.0; }
    phi[i] = 0.0;
  }
}

}  // namespace

// ====================================================================== host

struct SimpleState {
  fc_simple_params prm;
  bool have_prm = false;
  DVec<int> ptype;
  int ptype_gen = -1;  // mesh generation the patch types were uploaded for
  DVec<double> part, out;
  double cumulativeContErr = 0.0;
  double resor[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  // temperature equation
  fc_temperature_params tprm;
  bool have_tprm = false;
  int tprm_gen = -1;      // mesh generation the patch tables belong to
  DVec<int> tpatch;       // [kind | iWall start | first boundary index] x numBoundaries
  DVec<double> tpart;     // per-block min/max of T
  // transient momentum and PISO (fc_transient_set_params)
  fc_transient_params trp = {1.0, FC_TIME_STEADY, 0, 1};
  DVec<double> h, ppart;  // calcp_piso: h = a, pavg partials
  // k-omega SST (fc_turbulence_set_params)
  fc_turbulence_params kprm;
  bool have_kprm = false;
  // batched U, V, W solves (fc_simple_set_batched_momentum)
  int batch_mom = 0;
  struct MomBatch* mb = nullptr;
  ~SimpleState();
};

// Three systems on the mesh pattern (one per velocity component, each with a
// third of the resident blocks as the batch planner splits them), the V and
// W matrix values and sources, and the batched launch's device arrays.
struct MomBatch {
  int gen = -1;  // mesh generation the systems were built for
  CsrSystem* sys[3] = {nullptr, nullptr, nullptr};
  DVec<double> av, aw, bv, bw;
  BatchDev* dev = nullptr;
  ~MomBatch() {
    for (CsrSystem* s : sys) delete s;
    batch_dev_release(dev);
  }
};

SimpleState::~SimpleState() { delete mb; }

static SimpleState& sstate(fc_ctx* ctx) {
  if (!ctx->simple) ctx->simple = new SimpleState();
  return *ctx->simple;
}

void fc_simple_release(fc_ctx* ctx) {
  delete ctx->simple;
  ctx->simple = nullptr;
}

static inline int gridn(int n) { return std::max(1, std::min(65535, (n + 255) / 256)); }

static int make_dev(fc_ctx* ctx, Dev& D, bool allow_pressure = true) {
  FieldStore& F = ctx_fields(ctx);
  SimpleState& S = sstate(ctx);
  const MeshDev& m = ctx->mesh;
  if (S.ptype_gen != ctx->mesh_gen) {
    FC_CUDA_TRY(ctx, S.ptype.alloc(std::max(1, m.numBoundaries)));
    S.ptype_gen = ctx->mesh_gen;
    if (m.numBoundaries)
      FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, S.ptype.p, m.h_bctype.data(), m.numBoundaries * sizeof(int)));
  }
  for (int b = 0; b < m.numBoundaries; ++b) {
    if (m.h_bctype[b] == FC_BC_PRESSURE && !allow_pressure)
      return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "pressure boundaries are not supported by the PISO corrector");
  }
  D.u = F.u.p; D.v = F.v.p; D.w = F.w.p; D.p = F.p.p; D.pp = F.pp.p; D.vis = F.vis.p; D.den = F.den.p;
  D.flmass = F.flmass.p; D.visw = F.visw.p;
  D.su = F.su.p; D.sv = F.sv.p; D.sw = F.sw.p; D.spu = F.spu.p; D.spv = F.spv.p; D.sp = F.sp.p;
  D.apu = F.apu.p; D.apv = F.apv.p; D.apw = F.apw.p;
  D.gu = F.gu.p; D.gv = F.gv.p; D.gw = F.gw.p; D.gp = F.gp.p;
  D.t = F.t.p; D.gt = F.gt.p;
  D.uo = F.uo.p; D.vo = F.vo.p; D.wo = F.wo.p; D.uoo = F.uoo.p; D.voo = F.voo.p; D.woo = F.woo.p;
  D.uooo = F.uooo.p; D.vooo = F.vooo.p; D.wooo = F.wooo.p;
  D.rU = F.rU.p; D.rV = F.rV.p; D.rW = F.rW.p;
  D.a = ctx->sys_mesh->a.p;
  D.fscr = F.fscratch.p;
  D.ptype = S.ptype.p;
  return FC_OK;
}

// gradp_and_sources(p), nablap.f90:19-208, p = "p" or "pp"
static int gradp_and_sources(fc_ctx* ctx, const Dev& D, double* p, int pscheme) {
  MeshView M = mesh_view(ctx);
  const int gc = gridn(M.nC), gb = gridn(M.nB);
  const Fld gp{D.gp, M.nT};
  k_gp_inner<<<gc, 256, 0, ctx->stream>>>(M, p, gp, D.apu, pscheme == 2 ? 2 : 0, D.su, D.sv, D.sw);
  for (int stage = 1; stage <= 2; ++stage) {
    if (M.nB) k_bpres<<<gb, 256, 0, ctx->stream>>>(M, D.ptype, p, gp, stage);
    if (stage == 2 && pscheme == 1) k_gp_inner<<<gc, 256, 0, ctx->stream>>>(M, p, gp, D.apu, 1, D.su, D.sv, D.sw);
    k_gp_grad<<<gc, 256, 0, ctx->stream>>>(M, p, D.su, D.sv, D.sw, D.gp);
    ctx->kernel_launches += 2 + (stage == 2 && pscheme == 1);
  }
  k_gp_final<<<gc, 256, 0, ctx->stream>>>(M, p, D.su, D.sv, D.sw);
  ctx->kernel_launches += 2;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

static int update_velocity_at_boundary(fc_ctx* ctx, const Dev& D) {
  MeshView M = mesh_view(ctx);
  if (!M.nB) return FC_OK;
  k_update_vel_bnd<<<gridn(M.nB), 256, 0, ctx->stream>>>(M, D);
  ctx->kernel_launches++;
  return FC_OK;
}

extern "C" int fc_simple_set_params(fc_ctx* ctx, const fc_simple_params* prm) {
  if (!ctx || !prm) return FC_ERR_BAD_INPUT;
  if (prm->urfU[0] <= 0 || prm->urfU[1] <= 0 || prm->urfU[2] <= 0 || prm->npcor < 1)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_simple_set_params: bad under-relaxation or npcor");
  SimpleState& S = sstate(ctx);
  S.prm = *prm;
  S.prm.lSolverU[sizeof(S.prm.lSolverU) - 1] = 0;
  S.prm.lSolverP[sizeof(S.prm.lSolverP) - 1] = 0;
  S.have_prm = true;
  return FC_OK;
}

extern "C" int fc_gradp_and_sources(fc_ctx* ctx, const char* field) {
  FC_RANGE();
  if (!ctx || !field) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  Dev D;
  int st = make_dev(ctx, D);
  if (st) return st;
  std::string f(field);
  double* p = f == "pp" ? D.pp : f == "p" ? D.p : nullptr;
  if (!p) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "field must be 'p' or 'pp'");
  int ps = sstate(ctx).have_prm ? sstate(ctx).prm.pscheme : 0;
  return gradp_and_sources(ctx, D, p, ps);
}

extern "C" int fc_init_flmass(fc_ctx* ctx) {
  FC_RANGE();
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  Dev D;
  int st = make_dev(ctx, D);
  if (st) return st;
  MeshView M = mesh_view(ctx);
  if (M.nI) k_init_flmass<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D);
  ctx->kernel_launches++;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

extern "C" int fc_update_velocity_at_boundary(fc_ctx* ctx) {
  FC_RANGE();
  if (!ctx || !ctx->has_mesh) return FC_ERR_STATE;
  Dev D;
  int st = make_dev(ctx, D);
  if (st) return st;
  return update_velocity_at_boundary(ctx, D);
}

static int mom_batch_prepare(fc_ctx* ctx, SimpleState& S) {
  if (S.mb && S.mb->gen == ctx->mesh_gen) return FC_OK;
  delete S.mb;
  S.mb = new MomBatch();
  MomBatch& mb = *S.mb;
  const CsrSystem* m = ctx->sys_mesh;
  const int n = m->n, nnz = m->nnz;
  std::vector<int> ia1(m->h_ia), ja1(m->h_ja), dg1(m->h_diag);
  for (int& v : ia1) ++v;
  for (int& v : ja1) ++v;
  for (int& v : dg1) ++v;
  int budget = 0;
  batch_block_budget(ctx, &budget);
  std::vector<BatchCost> c(3);
  for (BatchCost& x : c) { x.rows = n; x.levels = m->ord.nlev; }
  const std::vector<int> g = plan_batch_groups(c, budget, budget, 1024);
  if (g.size() != 3) return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED, "batched momentum: fewer than 3 resident blocks");
  for (int k = 0; k < 3; ++k) {
    mb.sys[k] = new CsrSystem();
    int st = sys_set_pattern(ctx, mb.sys[k], n, nnz, ia1.data(), ja1.data(), dg1.data(),
                             ctx->mesh.h_xyz.empty() ? nullptr : ctx->mesh.h_xyz.data(), g[k]);
    if (st) return st;
  }
  FC_CUDA_TRY(ctx, mb.av.alloc(nnz));
  FC_CUDA_TRY(ctx, mb.aw.alloc(nnz));
  FC_CUDA_TRY(ctx, mb.bv.alloc(n));
  FC_CUDA_TRY(ctx, mb.bw.alloc(n));
  mb.gen = ctx->mesh_gen;
  return FC_OK;
}

extern "C" int fc_simple_set_batched_momentum(fc_ctx* ctx, int on) {
  if (!ctx) return FC_ERR_BAD_INPUT;
  sstate(ctx).batch_mom = on ? 1 : 0;
  return FC_OK;
}

static int solve_into(fc_ctx* ctx, const char* solver, double* x, const double* b, double* resor_out, int itr,
                      double tol_abs, double tol_rel, const char* chvar) {
  fc_solve_info info;
  int st = solve_global(ctx, solver, x, b, resor_out, itr, tol_abs, tol_rel, chvar, &info);
  return st;
}

// calcuvw, velocity.f90:50-750 (steady SIMPLE; no buoyancy, MHD, transient
// or periodic terms).  resor[0..2] receive the normalised initial residuals.
extern "C" int fc_calcuvw(fc_ctx* ctx, double* resor) {
  FC_RANGE();
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  SimpleState& S = sstate(ctx);
  if (!S.have_prm) return fc_fail_msg(ctx, FC_ERR_STATE, "fc_simple_set_params not called");
  Dev D;
  int st = make_dev(ctx, D);
  if (st) return st;
  const fc_simple_params& P = S.prm;
  MeshView M = mesh_view(ctx);
  CsrSystem* sys = ctx->sys_mesh;
  update_velocity_at_boundary(ctx, D);
  if ((st = fv_grad(ctx, P.gradScheme, D.u, D.gu))) return st;
  if ((st = fv_grad(ctx, P.gradScheme, D.v, D.gv))) return st;
  if ((st = fv_grad(ctx, P.gradScheme, D.w, D.gw))) return st;
  if ((st = gradp_and_sources(ctx, D, D.p, P.pscheme))) return st;
  MomParams mp;
  mp.gds = P.gdsU;
  mp.viscos = P.viscos;
  mp.scheme = P.cSchemeU;
  mp.vis_sym = 0.0;
  mp.tscheme = S.trp.scheme;
  mp.timestep = S.trp.timestep;
  if (M.nB > 0) FC_CUDA_TRY(ctx, cudaMemcpyAsync(&mp.vis_sym, D.vis + M.nC, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (M.nI) k_mom_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D, mp);
  if (M.nPer) {
    k_mom_pair<<<gridn(M.nPer), 256, 0, ctx->stream>>>(M, D, mp);
    ctx->kernel_launches++;
  }
  k_mom_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, mp);
  ctx->kernel_launches += 2;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  // PISO keeps the explicit convection and diffusion terms (velocity.f90:565-570)
  if (S.trp.piso) {
    const size_t bc = (size_t)M.nC * sizeof(double);
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(D.rU, D.su, bc, cudaMemcpyDeviceToDevice, ctx->stream));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(D.rV, D.sv, bc, cudaMemcpyDeviceToDevice, ctx->stream));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(D.rW, D.sw, bc, cudaMemcpyDeviceToDevice, ctx->stream));
  }
  double r[3] = {0, 0, 0};
  if (S.batch_mom && std::strcmp(P.lSolverU, "bicgstab") == 0) {
    // the three solves in one batched launch: V and W get copies of the
    // matrix (same off-diagonals) with their own diagonal and source
    if ((st = mom_batch_prepare(ctx, S))) return st;
    MomBatch& mb = *S.mb;
    const size_t nnz = (size_t)sys->nnz;
    k_mom_diag<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, sys->ia.p, sys->diag.p, D.a, D.spu, D.apu, D.su, D.su,
                                                     D.u, P.urfU[0], 0);
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(mb.av.p, D.a, nnz * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(mb.aw.p, D.a, nnz * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    k_mom_diag<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, sys->ia.p, sys->diag.p, mb.av.p, D.spv, D.apv, D.sv,
                                                     mb.bv.p, D.v, P.urfU[1], 1);
    k_mom_diag<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, sys->ia.p, sys->diag.p, mb.aw.p, D.sp, D.apw, D.sw,
                                                     mb.bw.p, D.w, P.urfU[2], 1);
    ctx->kernel_launches += 3;
    std::vector<BatchItem> it(3);
    const double* av[3] = {D.a, mb.av.p, mb.aw.p};
    double* xv[3] = {D.u, D.v, D.w};
    const double* bv[3] = {D.su, mb.bv.p, mb.bw.p};
    for (int k = 0; k < 3; ++k) { it[k].s = mb.sys[k]; it[k].a = av[k]; it[k].x = xv[k]; it[k].b = bv[k]; }
    if ((st = batch_solve(ctx, mb.dev, it, "bicgstab", P.maxiterU, P.tolAbsU, P.tolRelU))) return st;
    const char* nm[3] = {"U", "V", "W"};
    for (int k = 0; k < 3; ++k) {
      const SolveResult& rs = it[k].res;
      if (rs.status == FC_ERR_TIMEOUT) return fc_fail_msg(ctx, FC_ERR_TIMEOUT, "solver grid barrier timed out");
      if (rs.status < 0) return fc_fail_msg(ctx, rs.status, "solver reported an error (NaN/Inf or breakdown)");
      if (!rs.early) r[k] = rs.resor;
      report_solve(ctx, "bicgstab", nm[k], rs);
      log_solve(ctx, "mesh system (batched)", "bicgstab", nm[k], M.nC, rs);
    }
    // the matrix and source arrays end as the sequential passes leave them
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(D.a, mb.aw.p, nnz * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(D.su, mb.bw.p, (size_t)M.nC * sizeof(double), cudaMemcpyDeviceToDevice,
                                     ctx->stream));
    for (int k = 0; k < 3; ++k) S.resor[k + 1] = r[k];
    if (resor) for (int k = 0; k < 3; ++k) resor[k] = r[k];
    return FC_OK;
  }
  // U
  k_mom_diag<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, sys->ia.p, sys->diag.p, D.a, D.spu, D.apu, D.su, D.su, D.u,
                                                   P.urfU[0], 0);
  ctx->kernel_launches++;
  st = solve_into(ctx, P.lSolverU, D.u, D.su, &r[0], P.maxiterU, P.tolAbsU, P.tolRelU, "U");
  if (st < 0) return st;
  // V
  k_mom_diag<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, sys->ia.p, sys->diag.p, D.a, D.spv, D.apv, D.sv, D.su, D.v,
                                                   P.urfU[1], 1);
  ctx->kernel_launches++;
  st = solve_into(ctx, P.lSolverU, D.v, D.su, &r[1], P.maxiterU, P.tolAbsU, P.tolRelU, "V");
  if (st < 0) return st;
  // W
  k_mom_diag<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, sys->ia.p, sys->diag.p, D.a, D.sp, D.apw, D.sw, D.su, D.w,
                                                   P.urfU[2], 1);
  ctx->kernel_launches++;
  st = solve_into(ctx, P.lSolverU, D.w, D.su, &r[2], P.maxiterU, P.tolAbsU, P.tolRelU, "W");
  if (st < 0) return st;
  for (int k = 0; k < 3; ++k) S.resor[k + 1] = r[k];
  if (resor) for (int k = 0; k < 3; ++k) resor[k] = r[k];
  return FC_OK;
}

// calcp_simple, calcp_simple.f90:1-470 (incompressible; pressure
// boundaries and periodic pairs).  *resor4 receives resor(4) as
// continuityErrors sets it.
// continuityErrors, continuityErrors.f90:1-77: resor(4) into *resor4
static int continuity_errors(fc_ctx* ctx, const Dev& D, double* resor4) {
  SimpleState& S = sstate(ctx);
  MeshView M = mesh_view(ctx);
  const int nb = std::min(1024, gridn(M.nC));
  FC_CUDA_TRY(ctx, S.part.alloc((size_t)3 * nb));
  FC_CUDA_TRY(ctx, S.out.alloc(3));
  k_conterr<<<nb, 256, 0, ctx->stream>>>(M, D, S.part.p);
  k_conterr_final<<<1, 96, 0, ctx->stream>>>(S.part.p, nb, S.out.p);
  ctx->kernel_launches += 2;
  double h[3];
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(h, S.out.p, 3 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const double wavg = h[0] / h[1];
  S.cumulativeContErr += h[2];
  S.resor[4] = wavg;
  if (resor4) *resor4 = wavg;
  if (ctx->verbosity)
    std::printf("  continuity errors : avg local = %10.3E, global = %10.3E, cumulative = %10.3E\n", wavg, h[2],
                S.cumulativeContErr);
  return FC_OK;
}

extern "C" int fc_calcp_simple(fc_ctx* ctx, double* resor4) {
  FC_RANGE();
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  SimpleState& S = sstate(ctx);
  if (!S.have_prm) return fc_fail_msg(ctx, FC_ERR_STATE, "fc_simple_set_params not called");
  Dev D;
  int st = make_dev(ctx, D, true);
  if (st) return st;
  const fc_simple_params& P = S.prm;
  MeshView M = mesh_view(ctx);
  if (M.nI) k_p_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D);
  if (M.nPer) {
    k_p_pair<<<gridn(M.nPer), 256, 0, ctx->stream>>>(M, D);
    ctx->kernel_launches++;
  }
  bool outlets = false, pressure = false;
  for (int b = 0; b < ctx->mesh.numBoundaries; ++b) {
    outlets |= ctx->mesh.h_bctype[b] == FC_BC_OUTLET;
    pressure |= ctx->mesh.h_bctype[b] == FC_BC_PRESSURE;
  }
  if (outlets) k_adjust_mass_flow<<<1, 32, 0, ctx->stream>>>(M, D, P.flomas);
  // the pressure faces' coefficients, one per boundary face, in the face
  // scratch (free during calcp_simple)
  double* bcap = D.fscr;
  if (pressure) k_p_press<<<gridn(M.nB), 256, 0, ctx->stream>>>(M, D, bcap);
  k_p_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, bcap);
  ctx->kernel_launches += 2 + outlets + pressure;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  double r4 = 0;
  for (int ipcorr = 1; ipcorr <= P.npcor; ++ipcorr) {
    st = solve_into(ctx, P.lSolverP, D.pp, D.su, &r4, P.maxiterP, P.tolAbsP, P.tolRelP, "p");
    if (st < 0) return st;
    if (M.nI) k_flux_correct<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D);
    if (M.nPer) {
      k_flux_correct_pair<<<gridn(M.nPer), 256, 0, ctx->stream>>>(M, D, D.pp);
      ctx->kernel_launches++;
    }
    if (pressure) {
      k_p_press_corr<<<gridn(M.nB), 256, 0, ctx->stream>>>(M, D);
      ctx->kernel_launches++;
    }
    // ppref = pp(pRefCell) before gradp_and_sources(pp), which only touches
    // boundary values of pp; with a pressure boundary the reference p' is 0
    // (calcp_simple.f90:363-369)
    if ((st = gradp_and_sources(ctx, D, D.pp, P.pscheme))) return st;
    const int pref = std::max(0, std::min(M.nC - 1, P.pRefCell - 1));
    k_correct_vel_p<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, D, P.urfP, pref, pressure ? 0 : 1);
    ctx->kernel_launches += 2;
    update_velocity_at_boundary(ctx, D);
    if (ipcorr != P.npcor) {
      if (M.nI) k_fluxmc2_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D);
      k_fluxmc2_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D);
      ctx->kernel_launches += 2;
    }
  }
  return continuity_errors(ctx, D, resor4);
}

// transient parameters (velocity.f90 unsteady term, PISO)
extern "C" int fc_transient_set_params(fc_ctx* ctx, const fc_transient_params* prm) {
  if (!ctx || !prm) return FC_ERR_BAD_INPUT;
  if (prm->scheme < FC_TIME_STEADY || prm->scheme > FC_TIME_BDF3)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_transient_set_params: unknown time scheme");
  if (prm->scheme != FC_TIME_STEADY && !(prm->timestep > 0))
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_transient_set_params: timestep must be > 0");
  if (prm->piso && prm->ncorr < 1) return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_transient_set_params: ncorr < 1");
  if (prm->piso && (prm->scheme == FC_TIME_BDF2 || prm->scheme == FC_TIME_BDF3))
    return fc_fail_msg(ctx, FC_ERR_UNSUPPORTED,
                       "PISO with bdf2/bdf3: the reference extrapolates from old mass fluxes and pressures that "
                       "time_shift never updates");
  sstate(ctx).trp = *prm;
  return FC_OK;
}

// time_shift, time_shift.f90 (velocity levels)
extern "C" int fc_time_shift(fc_ctx* ctx) {
  FC_RANGE();
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  SimpleState& S = sstate(ctx);
  FieldStore& F = ctx_fields(ctx);
  const size_t b = (size_t)ctx->mesh.numTotal * sizeof(double);
  auto cp = [&](DVec<double>& d, const DVec<double>& s) {
    return cudaMemcpyAsync(d.p, s.p, b, cudaMemcpyDeviceToDevice, ctx->stream);
  };
  if (S.trp.scheme == FC_TIME_BDF3) {
    FC_CUDA_TRY(ctx, cp(F.uooo, F.uoo)); FC_CUDA_TRY(ctx, cp(F.vooo, F.voo)); FC_CUDA_TRY(ctx, cp(F.wooo, F.woo));
  }
  if (S.trp.scheme == FC_TIME_BDF3 || S.trp.scheme == FC_TIME_BDF2) {
    FC_CUDA_TRY(ctx, cp(F.uoo, F.uo)); FC_CUDA_TRY(ctx, cp(F.voo, F.vo)); FC_CUDA_TRY(ctx, cp(F.woo, F.wo));
  }
  FC_CUDA_TRY(ctx, cp(F.uo, F.u)); FC_CUDA_TRY(ctx, cp(F.vo, F.v)); FC_CUDA_TRY(ctx, cp(F.wo, F.w));
  return FC_OK;
}

// calcp_piso, calcp_piso.f90:86-489 (incompressible; periodic pairs, no
// pressure boundaries; nipgrad = 2, parameters.f90:62)
extern "C" int fc_calcp_piso(fc_ctx* ctx, double* resor4) {
  FC_RANGE();
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  SimpleState& S = sstate(ctx);
  if (!S.have_prm) return fc_fail_msg(ctx, FC_ERR_STATE, "fc_simple_set_params not called");
  if (!S.trp.piso) return fc_fail_msg(ctx, FC_ERR_STATE, "fc_calcp_piso: PISO not enabled (fc_transient_set_params)");
  Dev D;
  int st = make_dev(ctx, D, false);
  if (st) return st;
  const fc_simple_params& P = S.prm;
  MeshView M = mesh_view(ctx);
  const size_t nnz = (size_t)ctx->sys_mesh->nnz;
  FC_CUDA_TRY(ctx, S.h.alloc(nnz));
  FC_CUDA_TRY(ctx, cudaMemcpyAsync(S.h.p, D.a, nnz * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream));
  const int nbs = std::min(1024, gridn(M.nC));
  FC_CUDA_TRY(ctx, S.ppart.alloc(nbs + 1));
  bool outlets = false;
  for (int b = 0; b < ctx->mesh.numBoundaries; ++b) outlets |= ctx->mesh.h_bctype[b] == FC_BC_OUTLET;
  double r4 = 0, wavg = 0;
  for (int icorr = 1; icorr <= S.trp.ncorr; ++icorr) {
    k_piso_h<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, S.h.p);
    k_piso_u<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, D);
    if (M.nI) k_piso_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D);
    if (M.nPer) {
      k_p_pair<<<gridn(M.nPer), 256, 0, ctx->stream>>>(M, D);
      ctx->kernel_launches++;
    }
    if (outlets) k_adjust_mass_flow<<<1, 32, 0, ctx->stream>>>(M, D, P.flomas);
    k_p_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, D.fscr);
    ctx->kernel_launches += 4 + outlets;
    FC_CUDA_TRY(ctx, cudaGetLastError());
    for (int ipcorr = 1; ipcorr <= P.npcor; ++ipcorr) {
      st = solve_into(ctx, P.lSolverP, D.pp, D.su, &r4, P.maxiterP, P.tolAbsP, P.tolRelP, "p");
      if (st < 0) return st;
      k_sum_cells<<<nbs, 256, 0, ctx->stream>>>(D.pp, M.nC, S.ppart.p);
      k_sum_final<<<1, 32, 0, ctx->stream>>>(S.ppart.p, nbs);
      k_piso_p<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, D, S.ppart.p + nbs, P.urfP);
      ctx->kernel_launches += 3;
      const Fld gp{D.gp, M.nT};
      for (int stage = 1; stage <= 2; ++stage) {
        if (M.nB) {
          k_bpres<<<gridn(M.nB), 256, 0, ctx->stream>>>(M, D.ptype, D.p, gp, stage);
          ctx->kernel_launches++;
        }
        if ((st = fv_grad_gauss(ctx, D.p, D.gp))) return st;
      }
      if (ipcorr != P.npcor) {
        if (M.nI) k_fluxmc_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D);
        k_fluxmc_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D);
        ctx->kernel_launches += 2;
      } else {
        if (M.nI) k_flux_correct_p<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D);
        ctx->kernel_launches++;
        if ((st = continuity_errors(ctx, D, &wavg))) return st;
      }
    }
    if ((st = gradp_and_sources(ctx, D, D.p, P.pscheme))) return st;
    k_vel_correct<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, D);
    ctx->kernel_launches++;
    if (M.nPer) {  // the pairs' flux correction with the last p (calcp_piso.f90:437-456)
      k_flux_correct_pair<<<gridn(M.nPer), 256, 0, ctx->stream>>>(M, D, D.p);
      ctx->kernel_launches++;
    }
    update_velocity_at_boundary(ctx, D);
  }
  FC_CUDA_TRY(ctx, cudaGetLastError());
  if (resor4) *resor4 = wavg;
  return FC_OK;
}

// main.f90:132-267: time steps, iterations, convergence and divergence stops
extern "C" int fc_run(fc_ctx* ctx, const fc_run_params* prm, int* steps, int* iterations, double* resor) {
  FC_RANGE();
  if (!ctx || !prm || prm->numstep < 0 || prm->maxit < 1) return FC_ERR_BAD_INPUT;
  SimpleState& S = sstate(ctx);
  const bool transient = S.trp.scheme != FC_TIME_STEADY;
  int nsteps = 0, niters = 0, st = FC_OK;
  double r[4] = {0, 0, 0, 0};
  bool done = false;
  for (int itime = 1; itime <= prm->numstep && !done; ++itime) {
    if (transient && (st = fc_time_shift(ctx))) return st;
    ++nsteps;
    for (int iter = 1; iter <= prm->maxit; ++iter) {
      if ((st = fc_calcuvw(ctx, r)) < 0) return st;
      if ((st = S.trp.piso ? fc_calcp_piso(ctx, &r[3]) : fc_calcp_simple(ctx, &r[3])) < 0) return st;
      if (prm->temperature) {
        double r7 = 0;
        if ((st = fc_calculate_temperature(ctx, 1, &r7)) < 0) return st;
      }
      ++niters;
      if (steps) *steps = nsteps;
      if (iterations) *iterations = niters;
      if (resor) for (int k = 0; k < 4; ++k) resor[k] = r[k];
      const double source = std::max(r[0], std::max(r[1], r[2]));
      if (!(source <= (double)1e+30f)) return fc_fail_msg(ctx, FC_ERR_NAN, "iterations diverge");
      if (source < prm->tolerance) {
        if (!transient) done = true;
        break;
      }
    }
  }
  if (steps) *steps = nsteps;
  if (iterations) *iterations = niters;
  return FC_OK;
}

// one PISO iteration of main.f90:159-165 (calcuvw + calcp_piso)
extern "C" int fc_piso_iteration(fc_ctx* ctx, double* resor) {
  FC_RANGE();
  double r[4];
  int st = fc_calcuvw(ctx, r);
  if (st < 0) return st;
  st = fc_calcp_piso(ctx, &r[3]);
  if (st < 0) return st;
  if (resor) for (int k = 0; k < 4; ++k) resor[k] = r[k];
  const double source = std::max(r[0], std::max(r[1], r[2]));
  if (!(source <= (double)1e+30f)) return fc_fail_msg(ctx, FC_ERR_NAN, "PISO iterations diverge");
  return FC_OK;
}

// one outer iteration of main.f90:150-267 (calcuvw + calcp_simple)
extern "C" int fc_simple_iteration(fc_ctx* ctx, double* resor) {
  FC_RANGE();
  double r[4];
  int st = fc_calcuvw(ctx, r);
  if (st < 0) return st;
  st = fc_calcp_simple(ctx, &r[3]);
  if (st < 0) return st;
  if (resor) for (int k = 0; k < 4; ++k) resor[k] = r[k];
  // divergence check of main.f90:202-207
  const double source = std::max(r[0], std::max(r[1], r[2]));
  if (!(source <= (double)1e+30f)) return fc_fail_msg(ctx, FC_ERR_NAN, "SIMPLE iterations diverge");
  return FC_OK;
}

// ------------------------------------------------------------ temperature

extern "C" int fc_temperature_set_params(fc_ctx* ctx, const fc_temperature_params* prm, const double* bc_dfraction) {
  if (!ctx || !prm) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  if (!(prm->urfT > 0) || !(prm->pranl > 0) || !(prm->sigt > 0) || prm->maxiterT < 0)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_temperature_set_params: urfT, pranl and sigt must be > 0");
  if (prm->gradScheme < FC_GRAD_GAUSS || prm->gradScheme > FC_GRAD_LSQ_DM_EXACT)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_temperature_set_params: unknown gradient scheme");
  SimpleState& S = sstate(ctx);
  const MeshDev& m = ctx->mesh;
  const int nb = m.numBoundaries;
  // patch tables: the wall counter of temperature.f90:203,236 advances on
  // isothermal walls only, so each isothermal patch starts at the number of
  // isothermal wall faces before it
  std::vector<int> tab((size_t)3 * std::max(1, nb), 0);
  int iwall = 0;
  for (int b = 0; b < nb; ++b) {
    const int t = m.h_bctype[b];
    const double fr = bc_dfraction ? bc_dfraction[b] : 0.0;
    int kind = 0;
    if (t == FC_BC_INLET || t == FC_BC_OUTLET || t == FC_BC_PRESSURE) kind = 1;
    else if (t == FC_BC_WALL && fr == 1.0) kind = 2;
    else if (t == FC_BC_WALL && fr == 0.0) kind = 3;
    tab[b] = kind;
    tab[nb + b] = iwall;
    tab[2 * nb + b] = m.h_startFace[b] - m.numInnerFaces;
    if (kind == 2) iwall += m.h_nfaces[b];
  }
  FC_CUDA_TRY(ctx, S.tpatch.alloc(tab.size()));
  FC_CUDA_TRY(ctx, fc_h2d(ctx->stream, S.tpatch.p, tab.data(), tab.size() * sizeof(int)));
  S.tprm = *prm;
  S.tprm.lSolverT[sizeof(S.tprm.lSolverT) - 1] = 0;
  S.have_tprm = true;
  S.tprm_gen = ctx->mesh_gen;
  return FC_OK;
}

// calculate_temperature, temperature.f90:35-385 (steady; no turbulent heat
// flux, Crank-Nicolson or periodic terms)
extern "C" int fc_calculate_temperature(fc_ctx* ctx, int solve, double* resor7) {
  FC_RANGE();
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  SimpleState& S = sstate(ctx);
  if (!S.have_tprm || S.tprm_gen != ctx->mesh_gen)
    return fc_fail_msg(ctx, FC_ERR_STATE, "fc_temperature_set_params not called for this mesh");
  Dev D;
  int st = make_dev(ctx, D, true);
  if (st) return st;
  const fc_temperature_params& P = S.tprm;
  MeshView M = mesh_view(ctx);
  CsrSystem* sys = ctx->sys_mesh;
  FieldStore& F = ctx_fields(ctx);
  if ((st = fv_grad(ctx, P.gradScheme, D.t, D.gt))) return st;
  ScParams sp;
  sp.viscos = P.viscos;
  sp.prl = 1.0 / P.pranl;
  sp.prtr = 1. / P.sigt;
  sp.sigt = P.sigt;
  sp.pranl = P.pranl;
  sp.gam = P.gdsT;
  sp.scheme = P.cSchemeT;
  const int nb = ctx->mesh.numBoundaries;
  sp.pkind = S.tpatch.p;
  sp.pwall = S.tpatch.p + nb;
  sp.pstart = S.tpatch.p + 2 * nb;
  FC_CUDA_TRY(ctx, cudaMemsetAsync(D.a, 0, (size_t)sys->nnz * sizeof(double), ctx->stream));
  if (M.nI) k_sc_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D, sp);
  if (M.nPer) {
    k_sc_pair<<<gridn(M.nPer), 256, 0, ctx->stream>>>(M, D, sp);
    ctx->kernel_launches++;
  }
  k_sc_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, sp);
  // main diagonal and under-relaxation (:354-365); the apx output of the
  // shared kernel goes to scratch
  k_mom_diag<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, sys->ia.p, sys->diag.p, D.a, D.sp, F.cscratch.p, D.su, D.su,
                                                   D.t, P.urfT, 0);
  ctx->kernel_launches += 2 + (M.nI > 0);
  FC_CUDA_TRY(ctx, cudaGetLastError());
  if (!solve) return FC_OK;
  double r7 = 0.0;
  st = solve_into(ctx, P.lSolverT, D.t, D.su, &r7, P.maxiterT, P.tolAbsT, P.tolRelT, "Temp");
  if (st < 0) return st;
  if (M.nB) {
    k_update_boundary<<<gridn(M.nB), 256, 0, ctx->stream>>>(M, D.ptype, D.t);
    ctx->kernel_launches++;
  }
  const int nbk = std::min(ctx->num_sms > 0 ? 2 * ctx->num_sms : 256, gridn(M.nC));
  FC_CUDA_TRY(ctx, S.tpart.alloc((size_t)2 * nbk));
  k_minmax<<<nbk, 256, 0, ctx->stream>>>(M.nC, D.t, S.tpart.p);
  k_clip_small<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, D.t, S.tpart.p, nbk);
  ctx->kernel_launches += 2;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  if (ctx->verbosity) {
    std::vector<double> h((size_t)2 * nbk);
    FC_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), S.tpart.p, h.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                     ctx->stream));
    FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    double lo = h[0], hi = h[nbk];
    for (int b = 1; b < nbk; ++b) { lo = std::min(lo, h[b]); hi = std::max(hi, h[nbk + b]); }
    std::printf("  %11.4E <= Temperature <= %11.4E\n", lo, hi);
  }
  S.resor[7] = r7;
  if (resor7) *resor7 = r7;
  return FC_OK;
}

// ------------------------------------------------------------ k-omega SST
static bool turb_scalar_ok(const fc_turb_scalar& t) {
  return t.urf > 0 && t.maxiter >= 0 && t.tolRel >= 0 && t.tolAbs >= 0;
}

extern "C" int fc_turbulence_set_params(fc_ctx* ctx, const fc_turbulence_params* prm) {
  if (!ctx || !prm) return FC_ERR_BAD_INPUT;
  if (!turb_scalar_ok(prm->k) || !turb_scalar_ok(prm->omega) || !(prm->urfVis > 0))
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_turbulence_set_params: urf > 0, maxiter >= 0 and tolerances >= 0");
  if (prm->gradScheme < FC_GRAD_GAUSS || prm->gradScheme > FC_GRAD_LSQ_DM_EXACT)
    return fc_fail_msg(ctx, FC_ERR_BAD_INPUT, "fc_turbulence_set_params: unknown gradient scheme");
  SimpleState& S = sstate(ctx);
  S.kprm = *prm;
  S.kprm.k.lSolver[sizeof(S.kprm.k.lSolver) - 1] = 0;
  S.kprm.omega.lSolver[sizeof(S.kprm.omega.lSolver) - 1] = 0;
  S.have_kprm = true;
  return FC_OK;
}

// wall_distance_poisson, wall_distance.f90:29-118
extern "C" int fc_wall_distance(fc_ctx* ctx) {
  FC_RANGE();
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  Dev D;
  int st = make_dev(ctx, D, true);
  if (st) return st;
  MeshView M = mesh_view(ctx);
  FieldStore& F = ctx_fields(ctx);
  DVec<double> q, mu, phi, gphi;
  FC_CUDA_TRY(ctx, q.alloc(M.nC));
  FC_CUDA_TRY(ctx, mu.alloc(M.nC));
  FC_CUDA_TRY(ctx, phi.alloc(M.nT));
  FC_CUDA_TRY(ctx, gphi.alloc(3 * (size_t)M.nT));
  k_wd_init<<<gridn(M.nT), 256, 0, ctx->stream>>>(M.nC, M.nT, M.vol, q.p, mu.p, phi.p);
  ctx->kernel_launches++;
  if ((st = fc_laplacian(ctx, mu.p, phi.p, ~0ULL))) return st;
  double r = 0.0;
  st = solve_into(ctx, "iccg", phi.p, q.p, &r, 500, (double)1e-12f, (double)1e-10f, "Wdis");
  if (st < 0) return st;
  if (M.nB) {
    k_wd_bnd<<<gridn(M.nB), 256, 0, ctx->stream>>>(M, D.ptype, phi.p);
    ctx->kernel_launches++;
  }
  if ((st = fv_grad_gauss(ctx, phi.p, gphi.p))) return st;
  k_wd_dist<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, M.nT, phi.p, gphi.p, F.wd.p);
  ctx->kernel_launches++;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  FC_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));  // the temporaries go out of scope
  return FC_OK;
}

// calcsc, k_omega_SST.f90:91-785, for ifi = 1 (k) or 2 (omega)
static int sst_calcsc(fc_ctx* ctx, const Dev& D, const Turb& T, int ifi, double* resor) {
  SimpleState& S = sstate(ctx);
  const fc_turb_scalar& P = ifi == 1 ? S.kprm.k : S.kprm.omega;
  MeshView M = mesh_view(ctx);
  CsrSystem* sys = ctx->sys_mesh;
  double* fi = ifi == 1 ? T.te : T.ed;
  int st = fv_grad(ctx, S.kprm.gradScheme, fi, ifi == 1 ? T.gte : T.ged);
  if (st) return st;
  FC_CUDA_TRY(ctx, cudaMemsetAsync(D.a, 0, (size_t)sys->nnz * sizeof(double), ctx->stream));
  if (ifi == 1) k_sst_src_k<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, T);
  else k_sst_src_w<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, T);
  if (M.nI) k_sst_face<<<gridn(M.nI), 256, 0, ctx->stream>>>(M, D, T, ifi, P.gds, P.cScheme);
  if (M.nPer) k_sst_pair<<<gridn(M.nPer), 256, 0, ctx->stream>>>(M, D, T, ifi, P.gds);
  k_sst_cell<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, T, ifi, P.urf);
  ctx->kernel_launches += 2 + (M.nI > 0) + (M.nPer > 0);
  FC_CUDA_TRY(ctx, cudaGetLastError());
  st = solve_into(ctx, P.lSolver, fi, D.su, resor, P.maxiter, P.tolAbs, P.tolRel, ifi == 1 ? "k" : "Omega");
  if (st < 0) return st;
  if (M.nB) {
    k_update_boundary<<<gridn(M.nB), 256, 0, ctx->stream>>>(M, D.ptype, fi);
    ctx->kernel_launches++;
  }
  // the clip to small when min(fi) < 0, over all numTotal values (:771-782)
  const int nbk = std::min(ctx->num_sms > 0 ? 2 * ctx->num_sms : 256, gridn(M.nT));
  FC_CUDA_TRY(ctx, S.tpart.alloc((size_t)2 * nbk));
  k_minmax<<<nbk, 256, 0, ctx->stream>>>(M.nT, fi, S.tpart.p);
  k_clip_small<<<gridn(M.nT), 256, 0, ctx->stream>>>(M.nT, fi, S.tpart.p, nbk);
  ctx->kernel_launches += 2;
  FC_CUDA_TRY(ctx, cudaGetLastError());
  return FC_OK;
}

// modify_viscosity_turbulence.f90:25-45 with the k-omega SST model
extern "C" int fc_kw_sst(fc_ctx* ctx, double* resor56) {
  FC_RANGE();
  if (!ctx) return FC_ERR_BAD_INPUT;
  if (!ctx->has_mesh) return fc_fail_msg(ctx, FC_ERR_STATE, "no mesh");
  SimpleState& S = sstate(ctx);
  if (!S.have_prm) return fc_fail_msg(ctx, FC_ERR_STATE, "fc_simple_set_params not called");
  if (!S.have_kprm) return fc_fail_msg(ctx, FC_ERR_STATE, "fc_turbulence_set_params not called");
  Dev D;
  int st = make_dev(ctx, D, true);
  if (st) return st;
  MeshView M = mesh_view(ctx);
  FieldStore& F = ctx_fields(ctx);
  Turb T;
  T.te = F.te.p; T.ed = F.ed.p; T.fsst = F.fsst.p; T.gte = F.gte.p; T.ged = F.ged.p;
  T.gen = F.gen.p; T.mag = F.mag.p; T.wd = F.wd.p; T.tau = F.tau.p; T.ypl = F.ypl.p;
  T.viscos = S.prm.viscos;
  T.densit = S.prm.densit;
  T.cmu25 = std::sqrt(std::sqrt(0.09));
  T.alpha1 = 5. / 9.0;
  if ((st = fv_grad_gauss(ctx, D.u, D.gu))) return st;
  if ((st = fv_grad_gauss(ctx, D.v, D.gv))) return st;
  if ((st = fv_grad_gauss(ctx, D.w, D.gw))) return st;
  k_sst_strain<<<gridn(M.nC), 256, 0, ctx->stream>>>(M.nC, M.nT, D.gu, D.gv, D.gw, T.mag);
  ctx->kernel_launches++;
  double r5 = 0.0, r6 = 0.0;
  if ((st = sst_calcsc(ctx, D, T, 1, &r5))) return st;
  if ((st = sst_calcsc(ctx, D, T, 2, &r6))) return st;
  k_sst_mu<<<gridn(M.nC), 256, 0, ctx->stream>>>(M, D, T, S.kprm.urfVis);
  ctx->kernel_launches++;
  if (M.nB) {
    k_update_boundary<<<gridn(M.nB), 256, 0, ctx->stream>>>(M, D.ptype, D.vis);
    ctx->kernel_launches++;
  }
  const MeshDev& m = ctx->mesh;
  if (m.nwal > 0) {
    k_sst_mu_wall<<<gridn(m.nwal), 256, 0, ctx->stream>>>(M, D, T, m.nwal, m.wall_face.p);
    ctx->kernel_launches++;
  }
  FC_CUDA_TRY(ctx, cudaGetLastError());
  S.resor[5] = r5;
  S.resor[6] = r6;
  if (resor56) { resor56[0] = r5; resor56[1] = r6; }
  return FC_OK;
}
