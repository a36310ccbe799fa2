// ORACLE (test infrastructure only) -- the k-omega SST turbulence model of
// the reference, restated in the oracle's conventions (1-based arrays,
// statement order kept, FP64 without contraction):
//   - wall_distance_poisson, mesh/wall_distance.f90:29-118;
//   - calc_strain_and_vorticity (the strain magnitude),
//     fvExplicit/calc_strain_and_vorticity.f90:1-60;
//   - calcsc and modify_mu_eff of TurbulenceModels/k_omega_SST.f90:91-958
//     (high-Re form: LowRe = .false., no buoyancy, steady, no Crank-Nicolson);
//   - the driver order of modify_viscosity_turbulence,
//     TurbulenceModels/modify_viscosity_turbulence.f90:25-45.
// Integer powers are expanded as products, as gfortran expands them.
#include <algorithm>
#include <cmath>

#include "oracle.hpp"

namespace orc {

namespace {
// k_omega_SST.f90:21-38 and parameters.f90:15-17
const double BETTAST = 0.09, SIGMK1 = 0.85, SIGMK2 = 1.0, SIGMOM1 = 0.5, SIGMOM2 = 0.856;
const double BETAI1 = 0.075, BETAI2 = 0.0828, A1 = 0.31, ALPHA1 = 5. / 9.0, ALPHA2 = 0.44;
const double CAPPA = 0.41, ELOG = 8.432;
inline double cmu25() { return std::sqrt(std::sqrt(BETTAST)); }
}  // namespace

// wall_distance_poisson, wall_distance.f90:29-118: the Laplace problem
// lap(phi) = -1 with the reference's laplacian (Dirichlet phi = 0 on every
// patch), ICCG to 1e-10 (500 iterations at most), non-wall boundary values
// taken from the owners, then d = -|grad phi| + sqrt(|grad phi|^2 + 2 phi).
int wall_distance_poisson(Case& c) {
  const int nC = c.numCells, nT = c.numTotal;
  std::vector<double> q(nC + 1), mu(nC + 1, 1.0), phi(nT + 1, 0.0), dpdxi(3 * (size_t)(nT + 1), 0.0);
  for (int i = 1; i <= nC; ++i) q[i] = -c.vol[i];
  laplacian(c, mu, phi, ~0ULL);  // also adds its boundary terms to su, which the solve does not use
  double resn = 0;
  SolveInfo si;
  int st = csrsolve(c, "iccg", phi, q, resn, 500, (double)1e-12f, (double)1e-10f, si);
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] == BC_WALL) continue;
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
      phi[ijb] = phi[ijp];
    }
  }
  grad_gauss(c, phi, dpdxi);
  c.walldist.assign(nC + 1, 0.0);
  for (int i = 1; i <= nC; ++i) {
    double gx = G(dpdxi, 1, i), gy = G(dpdxi, 2, i), gz = G(dpdxi, 3, i);
    c.walldist[i] = -std::sqrt(gx * gx + gy * gy + gz * gz) + std::sqrt(gx * gx + gy * gy + gz * gz + 2 * phi[i]);
  }
  return st;
}

// calc_strain_and_vorticity.f90:1-60: magStrain = sqrt(2 Sij Sij) from the
// velocity gradients
void calc_strain(Case& c) {
  for (int inp = 1; inp <= c.numCells; ++inp) {
    double dudx = G(c.dUdxi, 1, inp), dudy = G(c.dUdxi, 2, inp), dudz = G(c.dUdxi, 3, inp);
    double dvdx = G(c.dVdxi, 1, inp), dvdy = G(c.dVdxi, 2, inp), dvdz = G(c.dVdxi, 3, inp);
    double dwdx = G(c.dWdxi, 1, inp), dwdy = G(c.dWdxi, 2, inp), dwdz = G(c.dWdxi, 3, inp);
    double s11 = dudx, s12 = 0.5 * (dudy + dvdx), s13 = 0.5 * (dudz + dwdx);
    double s22 = dvdy, s23 = 0.5 * (dvdz + dwdy), s33 = dwdz;
    c.magStrain[inp] =
        std::sqrt(2 * (s11 * s11 + s22 * s22 + s33 * s33 + 2 * (s12 * s12 + s13 * s13 + s23 * s23)));
  }
}

// calcsc, k_omega_SST.f90:91-785, ifi = 1 (k, te) or 2 (omega, ed)
int calcsc_sst(Case& c, int ifi) {
  const int nC = c.numCells;
  const TurbScalar& P = ifi == 1 ? c.turbK : c.turbW;
  std::vector<double>& fi = ifi == 1 ? c.te : c.ed;
  std::vector<double>& dfidxi = ifi == 1 ? c.dTEdxi : c.dEDdxi;
  const double gam = P.gds, urf = P.urf;
  const double CMU25 = cmu25();
  grad(c, fi, dfidxi);
  std::fill(c.a.begin(), c.a.end(), 0.0);
  std::fill(c.su.begin(), c.su.end(), 0.0);
  std::fill(c.sp.begin(), c.sp.end(), 0.0);
  if (ifi == 1) {
    // production and its limiter (:159-180), sources (:185-219)
    for (int inp = 1; inp <= nC; ++inp) {
      c.gen[inp] = std::fabs(c.vis[inp] - c.viscos) * c.magStrain[inp] * c.magStrain[inp];
      c.gen[inp] = std::min(c.gen[inp], 0.9 * c.den[inp] * c.te[inp] * c.ed[inp]);
    }
    for (int inp = 1; inp <= nC; ++inp) {
      double genp = std::max(c.gen[inp], 0.0), genn = std::min(c.gen[inp], 0.0);
      c.su[inp] = genp * c.vol[inp];
      c.sp[inp] = BETTAST * c.ed[inp] * c.den[inp] * c.vol[inp];
      c.sp[inp] = c.sp[inp] - genn * c.vol[inp] / (c.te[inp] + kSmall);
    }
  } else {
    // the blending function (:300-330) and the omega sources (:332-398)
    for (int inp = 1; inp <= nC; ++inp) {
      double wldist = c.walldist[inp];
      double dtedx = G(c.dTEdxi, 1, inp), dtedy = G(c.dTEdxi, 2, inp), dtedz = G(c.dTEdxi, 3, inp);
      double deddx = G(c.dEDdxi, 1, inp), deddy = G(c.dEDdxi, 2, inp), deddz = G(c.dEDdxi, 3, inp);
      double domegapl =
          std::max(2 * SIGMOM2 * c.den[inp] / (c.ed[inp]) * (dtedx * deddx + dtedy * deddy + dtedz * deddz), kSmall);
      double ksi = std::min(std::max(std::sqrt(c.te[inp]) / (BETTAST * wldist * c.ed[inp] + kSmall),
                                     500.0 * c.viscos / c.den[inp] / (wldist * wldist * c.ed[inp] + kSmall)),
                            4.0 * c.den[inp] * c.te[inp] * SIGMOM2 / (domegapl * (wldist * wldist)));
      double ksi2 = ksi * ksi;
      c.fsst[inp] = std::tanh(ksi2 * ksi2);
    }
    for (int inp = 1; inp <= nC; ++inp) {
      double genp = std::max(c.gen[inp], 0.0), genn = std::min(c.gen[inp], 0.0);
      double vist = (c.vis[inp] - c.viscos) / c.densit;
      double alphasst = c.fsst[inp] * ALPHA1 + (1.0 - c.fsst[inp]) * ALPHA2;
      c.su[inp] = alphasst * genp * c.vol[inp] / (vist + kSmall);
      double dtedx = G(c.dTEdxi, 1, inp), dtedy = G(c.dTEdxi, 2, inp), dtedz = G(c.dTEdxi, 3, inp);
      double deddx = G(c.dEDdxi, 1, inp), deddy = G(c.dEDdxi, 2, inp), deddz = G(c.dEDdxi, 3, inp);
      double domega = 2 * (1.0 - c.fsst[inp]) * c.den[inp] * SIGMOM2 / (c.ed[inp] + kSmall) *
                      (dtedx * deddx + dtedy * deddy + dtedz * deddz);
      domega = std::max(domega, 0.0);
      c.su[inp] = c.su[inp] + domega * c.vol[inp];
      double bettasst = c.fsst[inp] * BETAI1 + (1.0 - c.fsst[inp]) * BETAI2;
      c.sp[inp] = bettasst * c.den[inp] * c.ed[inp] * c.vol[inp];
      c.sp[inp] = c.sp[inp] - alphasst * genn * c.vol[inp] / (vist * c.ed[inp] + kSmall);
    }
  }
  const double s1 = ifi == 1 ? SIGMK1 : SIGMOM1, s2 = ifi == 1 ? SIGMK2 : SIGMOM2;
  // inner faces (:448-488): the blended sigma of the owner cell
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double prtr = c.fsst[ijp] * s1 + (1.0 - c.fsst[ijp]) * s2;
    double viste = (c.vis[ijp] + (c.vis[ijn] - c.vis[ijp]) * c.facint[i]) - c.viscos;
    double dcoef = c.viscos + viste * prtr;
    double cap, can, suadd;
    facefluxsc(c, i, ijp, ijn, c.xf[i], c.yf[i], c.zf[i], c.arx[i], c.ary[i], c.arz[i], c.flmass[i], c.facint[i],
               gam, P.cScheme, fi, dfidxi, dcoef, cap, can, suadd);
    c.a[c.ijk[i]] = can;
    c.a[c.jik[i]] = cap;
    c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - can;
    c.a[c.diag[ijn]] = c.a[c.diag[ijn]] - cap;
    c.su[ijp] = c.su[ijp] + suadd;
    c.su[ijn] = c.su[ijn] - suadd;
  }
  // boundaries (:495-660)
  int iWall = 0, iPer = 0, l = c.numInnerFaces;
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    int t = c.bctype[ib];
    if (t == BC_INLET || t == BC_OUTLET || t == BC_PRESSURE) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        double prtr = c.fsst[ijp] * s1 + (1.0 - c.fsst[ijp]) * s2;
        double viste = c.vis[ijb] - c.viscos;
        double dcoef = c.viscos + viste * prtr;
        double cap, can, suadd;
        facefluxsc_bnd(c, ijp, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface], c.arz[iface],
                       c.flmass[iface], dfidxi, dcoef, cap, can, suadd);
        c.sp[ijp] = c.sp[ijp] - can;
        c.su[ijp] = c.su[ijp] - can * fi[ijb] + suadd;
      }
    } else if (t == BC_PERIODIC) {
      ++iPer;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface];
        int ijn = c.owner[c.startFaceTwin[iPer] + i];
        double prtr_ijp = c.fsst[ijp] * s1 + (1.0 - c.fsst[ijp]) * s2;
        double prtr_ijn = c.fsst[ijn] * s1 + (1.0 - c.fsst[ijn]) * s2;
        double prtr = 0.5 * (prtr_ijp + prtr_ijn);
        double viste = 0.5 * (c.vis[ijp] + c.vis[ijn]) - c.viscos;
        double dcoef = c.viscos + viste * prtr;
        double cap, can, suadd;
        facefluxsc_periodic(c, i, ijp, ijn, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface],
                            c.arz[iface], c.flmass[iface], gam, fi, dfidxi, dcoef, cap, can, suadd);
        ++l;
        c.a[c.ijk[l]] = can;
        c.a[c.jik[l]] = cap;
        c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - can;
        c.a[c.diag[ijn]] = c.a[c.diag[ijn]] - cap;
        c.su[ijp] = c.su[ijp] + suadd;
        c.su[ijn] = c.su[ijn] - suadd;
      }
    } else if (t == BC_WALL) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        ++iWall;
        if (ifi == 1) {
          // the wall-function production replaces the standard one (:583-620)
          c.su[ijp] = c.su[ijp] - c.gen[ijp] * c.vol[ijp];
          double viss = std::max(c.viscos, c.visw[iWall]);
          double are = std::sqrt(c.arx[iface] * c.arx[iface] + c.ary[iface] * c.ary[iface] +
                                 c.arz[iface] * c.arz[iface]);
          double nxf = c.arx[iface] / are, nyf = c.ary[iface] / are, nzf = c.arz[iface] / are;
          double Vnp = c.u[ijp] * nxf + c.v[ijp] * nyf + c.w[ijp] * nzf;
          double xtp = c.u[ijp] - Vnp * nxf, ytp = c.v[ijp] - Vnp * nyf, ztp = c.w[ijp] - Vnp * nzf;
          double Vtp = std::sqrt(xtp * xtp + ytp * ytp + ztp * ztp);
          xtp = xtp / Vtp;
          ytp = ytp / Vtp;
          ztp = ztp / Vtp;
          double Ut2 = std::fabs((c.u[ijb] - c.u[ijp]) * xtp + (c.v[ijb] - c.v[ijp]) * ytp +
                                 (c.w[ijb] - c.w[ijp]) * ztp);
          c.tau[iWall] = viss * Ut2 / c.dnw[iWall];
          c.gen[ijp] = std::fabs(c.tau[iWall]) * CMU25 * std::sqrt(c.te[ijp]) / (c.dnw[iWall] * CAPPA);
          c.su[ijp] = c.su[ijp] + c.gen[ijp] * c.vol[ijp];
        } else {
          // omega fixed in the wall cell (:625-650)
          double wlog = std::sqrt(c.te[ijp]) / (CMU25 * CAPPA * c.dnw[iWall]);
          double wvis = 6.0 * (c.viscos / c.den[ijp]) / (BETAI1 * (c.dnw[iWall] * c.dnw[iWall]));
          c.ed[ijp] = std::sqrt(wvis * wvis + wlog * wlog);
          c.su[ijp] = c.ed[ijp];
          for (int k = c.ia[ijp]; k <= c.ia[ijp + 1] - 1; ++k) c.a[k] = 0.0;
          c.sp[ijp] = 1.0;
        }
      }
    }
  }
  // main diagonal and under-relaxation (:712-726)
  const double urfrs = 1.0 / urf, urfms = 1.0 - urf;
  for (int inp = 1; inp <= nC; ++inp) {
    int kd = c.diag[inp];
    c.a[kd] = c.sp[inp];
    for (int k = c.ia[inp]; k <= c.ia[inp + 1] - 1; ++k) {
      if (k == kd) continue;
      c.a[kd] = c.a[kd] - c.a[k];
    }
    c.a[kd] = c.a[kd] * urfrs;
    c.su[inp] = c.su[inp] + urfms * c.a[kd] * fi[inp];
  }
  SolveInfo si;
  int st = csrsolve(c, P.lSolver, fi, c.su, c.resor[ifi == 1 ? 5 : 6], P.maxiter, P.tolAbs, P.tolRel, si);
  updateBoundary(c, fi);
  double fimin = fi[1];
  for (int i = 2; i <= c.numTotal; ++i) fimin = std::min(fimin, fi[i]);
  if (fimin < 0.0)
    for (int i = 1; i <= c.numTotal; ++i) fi[i] = std::max(fi[i], kSmall);
  return st;
}

// modify_mu_eff, k_omega_SST.f90:790-958 (high-Re form)
void modify_mu_eff_sst(Case& c) {
  const double urf = c.urfVis, CMU25 = cmu25();
  for (int inp = 1; inp <= c.numCells; ++inp) {
    double visold = c.vis[inp];
    double wldist = c.walldist[inp];
    double etha = std::max(2 * std::sqrt(c.te[inp]) / (BETTAST * wldist * c.ed[inp]),
                           (500 * c.viscos / c.den[inp]) / (wldist * wldist * c.ed[inp]));
    double f2_sst = std::tanh(etha * etha);
    c.vis[inp] = c.viscos + c.den[inp] * A1 * c.te[inp] / (std::max(A1 * c.ed[inp], c.magStrain[inp] * f2_sst));
    c.vis[inp] = urf * c.vis[inp] + (1.0 - urf) * visold;
  }
  updateBoundary(c, c.vis);
  int iWall = 0;
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] != BC_WALL) continue;
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
      ++iWall;
      double are = std::sqrt(c.arx[iface] * c.arx[iface] + c.ary[iface] * c.ary[iface] + c.arz[iface] * c.arz[iface]);
      double nxf = c.arx[iface] / are, nyf = c.ary[iface] / are, nzf = c.arz[iface] / are;
      double Vnp = c.u[ijp] * nxf + c.v[ijp] * nyf + c.w[ijp] * nzf;
      double xtp = c.u[ijp] - Vnp * nxf, ytp = c.v[ijp] - Vnp * nyf, ztp = c.w[ijp] - Vnp * nzf;
      double Vtp = std::sqrt(xtp * xtp + ytp * ytp + ztp * ztp);
      double Utau = std::sqrt(c.viscos * Vtp / (c.densit * c.dnw[iWall]) + CMU25 * c.te[ijp]);
      c.ypl[iWall] = c.den[ijp] * Utau * c.dnw[iWall] / c.viscos;
      double Utauvis = c.ypl[iWall];
      double Utaulog = 1.0 / CAPPA * std::log(ELOG * c.ypl[iWall]);
      double uv2 = Utauvis * Utauvis, ul2 = Utaulog * Utaulog;
      double Upl = std::sqrt(std::sqrt(uv2 * uv2 + ul2 * ul2));
      double viscw = c.den[ijp] * Utau * c.dnw[iWall] / Upl;
      double r = Vtp / Upl;
      c.tau[iWall] = c.den[ijp] * (r * r);
      c.visw[iWall] = std::max(c.viscos, viscw);
      c.vis[ijb] = c.visw[iWall];
    }
  }
}

// modify_viscosity_turbulence.f90:25-45 with TurbModel%name = 'k_omega_sst':
// Gauss velocity gradients, the strain magnitude, the k and omega equations,
// the eddy viscosity
int modify_viscosity_k_omega_sst(Case& c) {
  grad_gauss(c, c.u, c.dUdxi);
  grad_gauss(c, c.v, c.dVdxi);
  grad_gauss(c, c.w, c.dWdxi);
  calc_strain(c);
  int st = calcsc_sst(c, 1);
  st = std::min(st, calcsc_sst(c, 2));
  modify_mu_eff_sst(c);
  return st;
}

}  // namespace orc
