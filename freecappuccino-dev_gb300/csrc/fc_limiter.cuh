// Slope limiters of the cell gradients (gradients.f90:141-160, applied by
// grad_scalar_field after every gradient when `limiter` is set), written
// once per cell for the CUDA kernels (fc_limiter.cu, built without FMA
// contraction) and for the host replay that checks them against the oracle
// (tests/replay/limiter_replay.cpp, built -ffp-contract=off).  Arrays are
// 0-based; the gradient is SoA: g[c], g[nT + c], g[2 nT + c].
//
//  FC_LIMITER_BJ     Barth-Jespersen        gradients.f90:288-366
//  FC_LIMITER_VENKAT Venkatakrishnan        gradients.f90:373-451
//  FC_LIMITER_R      the 'R3' case, whose active line is the R4 function
//                                           gradients.f90:456-535
//  FC_LIMITER_MD     multidimensional       gradients.f90:541-656
//
// The first three scale a cell's gradient by the smallest limiter value over
// its CSR row (the neighbours), with r = (global max or min of phi over the
// cells - phi_c) / (g_c . (x_n - x_c)) and r = 1 where |g_c . d| < 1.e-6 (a
// default-real literal, compared in double).  The multidimensional limiter
// corrects the gradient face by face, in ascending inner-face order, so one
// thread per cell walking its faces in that order reproduces the reference's
// face loop exactly.
#pragma once

#include <cmath>

#if defined(__CUDACC__)
#define FC_HD __host__ __device__ __forceinline__
#else
#define FC_HD inline
#endif

// the values of fc_gpu.h
#ifndef FC_LIMITER_NONE
#define FC_LIMITER_NONE 0
#define FC_LIMITER_BJ 1
#define FC_LIMITER_VENKAT 2
#define FC_LIMITER_R 3
#define FC_LIMITER_MD 4
#endif

namespace fclim {

// the literal 1.e-6 of the reference's comparison: a single-precision
// constant, promoted to double
constexpr double kTinyDelta = (double)1.e-6f;

FC_HD double dmin(double a, double b) { return b < a ? b : a; }
FC_HD double dmax(double a, double b) { return b > a ? b : a; }

// limiter function of r for the three scaling limiters
template <int KIND>
FC_HD double limiter_fn(double r) {
  if (KIND == FC_LIMITER_BJ) return r;
  if (KIND == FC_LIMITER_VENKAT) return (r * r + 2.0 * r) / (r * r + r + 2.0);
  const double r2 = r * r, r3 = r2 * r, r4 = r2 * r2;
  return (r4 + 2.0 * r3 - 4.0 * r2 + 8.0 * r) / (r4 + r3 + 2.0 * r2 - 4.0 * r + 8.0);
}

// scale factor of cell c's gradient (gx, gy, gz) for KIND in BJ, VENKAT, R;
// fimin/fimax: min/max of phi over all cells
template <int KIND>
FC_HD double limit_factor(int c, const int* ia, const int* ja, const int* dg, const double* xc, const double* yc,
                          const double* zc, const double* phi, double gx, double gy, double gz, double fimin,
                          double fimax) {
  const double deltamax = fimax - phi[c];
  const double deltamin = fimin - phi[c];
  double slopelimit = 1.0;
  const int kd = dg[c];
  for (int k = ia[c]; k < ia[c + 1]; ++k) {
    if (k == kd) continue;
    const int n = ja[k];
    const double delta_face = gx * (xc[n] - xc[c]) + gy * (yc[n] - yc[c]) + gz * (zc[n] - zc[c]);
    double r;
    if ((delta_face < 0.0 ? -delta_face : delta_face) < kTinyDelta) r = 1.0;
    else if (delta_face > 0.0) r = deltamax / delta_face;
    else r = deltamin / delta_face;
    slopelimit = dmin(slopelimit, limiter_fn<KIND>(r));
  }
  return slopelimit;
}

// multidimensional limiter of cell c: its gradient corrected face by face
// over its inner faces in ascending order (cf_face ascending, boundary faces
// f >= nI skipped); phimax/phimin over the cell's CSR row in row order
FC_HD void limit_md(int c, const int* ia, const int* ja, const int* cf_ptr, const int* cf_face, int nI,
                    const double* xf, const double* yf, const double* zf, const double* xc, const double* yc,
                    const double* zc, const double* phi, double& gx, double& gy, double& gz) {
  double phimax = phi[ja[ia[c]]], phimin = phimax;
  for (int k = ia[c] + 1; k < ia[c + 1]; ++k) {
    phimax = dmax(phimax, phi[ja[k]]);
    phimin = dmin(phimin, phi[ja[k]]);
  }
  const double pc = phi[c];
  const double dPhimax = phimax - pc, dPhimin = phimin - pc;
  for (int q = cf_ptr[c]; q < cf_ptr[c + 1]; ++q) {
    const int f = cf_face[q];
    if (f >= nI) continue;
    const double xpn = xf[f] - xc[c], ypn = yf[f] - yc[c], zpn = zf[f] - zc[c];
    const double dpn = sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    const double nx = xpn / dpn, ny = ypn / dpn, nz = zpn / dpn;
    const double gn = gx * nx + gy * ny + gz * nz;
    const double gtx = gx - gn * nx, gty = gy - gn * ny, gtz = gz - gn * nz;
    const double dPhi = gx * xpn + gy * ypn + gz * zpn;
    if (phimax > pc && dPhi > dPhimax) {
      gx = gtx + nx * dPhimax;
      gy = gty + ny * dPhimax;
      gz = gtz + nz * dPhimax;
    }
    if (phimin < pc && dPhi < dPhimin) {
      gx = gtx + nx * dPhimin;
      gy = gty + ny * dPhimin;
      gz = gtz + nz * dPhimin;
    }
  }
}

}  // namespace fclim
