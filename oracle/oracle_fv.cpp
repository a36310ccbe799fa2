// ORACLE (test infrastructure only) -- finite-volume operators of the SIMPLE
// path: gradients (src/finiteVolume/fvExplicit/gradients.f90), face
// interpolation (src/finiteVolume/interpolation/interpolation.f90), implicit
// Laplacian (src/finiteVolume/fvImplicit/laplacian.f90), pressure gradient
// and sources (Pressure/nablap.f90, Pressure/bpres.f90), momentum assembly
// (Velocity/velocity.f90) and SIMPLE pressure correction
// (Pressure/calcp_simple.f90, fluxes/faceflux_mass.f90,
// Pressure/continuityErrors.f90), mass-flux initialisation
// (cappuccino/init.f90:167-176).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <vector>

#include "oracle.hpp"

namespace orc {

// ---------------------------------------------------------------- gradients
// grad_gauss + gradbc, gradients.f90:1607-1715
void grad_gauss(Case& c, const std::vector<double>& u, std::vector<double>& dudxi) {
  std::fill(dudxi.begin(), dudxi.end(), 0.0);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double fie = u[ijp] + (u[ijn] - u[ijp]) * c.facint[i];
    double dfxe = fie * c.arx[i], dfye = fie * c.ary[i], dfze = fie * c.arz[i];
    G(dudxi, 1, ijp) = G(dudxi, 1, ijp) + dfxe;
    G(dudxi, 2, ijp) = G(dudxi, 2, ijp) + dfye;
    G(dudxi, 3, ijp) = G(dudxi, 3, ijp) + dfze;
    G(dudxi, 1, ijn) = G(dudxi, 1, ijn) - dfxe;
    G(dudxi, 2, ijn) = G(dudxi, 2, ijn) - dfye;
    G(dudxi, 3, ijn) = G(dudxi, 3, ijn) - dfze;
  }
  for (int i = 1; i <= c.numBoundaryFaces; ++i) {
    int iface = c.numInnerFaces + i;
    int ijp = c.owner[iface], ijb = c.numCells + i;
    G(dudxi, 1, ijp) = G(dudxi, 1, ijp) + u[ijb] * c.arx[iface];
    G(dudxi, 2, ijp) = G(dudxi, 2, ijp) + u[ijb] * c.ary[iface];
    G(dudxi, 3, ijp) = G(dudxi, 3, ijp) + u[ijb] * c.arz[iface];
  }
  for (int ijp = 1; ijp <= c.numCells; ++ijp) {
    double volr = 1.0 / c.vol[ijp];
    for (int k = 1; k <= 3; ++k) G(dudxi, k, ijp) = G(dudxi, k, ijp) * volr;
  }
}

// shared cofactor step of create_matrix_lsq (:742-777) and _dm (:1292-1326)
static void lsq_invert(Case& c) {
  for (int inp = 1; inp <= c.numCells; ++inp) {
    double* D = &c.Dmat[9 * (size_t)inp];
    double d11 = D[0], d12 = D[1], d13 = D[2], d22 = D[3], d23 = D[4], d33 = D[5];
    double d21 = d12, d31 = d13, d32 = d23;
    double tmp = 1.0 / (d11 * d22 * d33 - d11 * d23 * d32 - d12 * d21 * d33 + d12 * d23 * d31 + d13 * d21 * d32 -
                        d13 * d22 * d31 + kSmall);
    D[0] = (d22 * d33 - d23 * d32) * tmp;
    D[1] = (d21 * d33 - d23 * d31) * tmp;
    D[2] = (d21 * d32 - d22 * d31) * tmp;
    D[3] = (d11 * d33 - d13 * d31) * tmp;
    D[4] = (d12 * d33 - d13 * d32) * tmp;
    D[5] = (d11 * d32 - d12 * d31) * tmp;
    D[6] = (d12 * d23 - d13 * d22) * tmp;
    D[7] = (d11 * d23 - d13 * d21) * tmp;
    D[8] = (d11 * d22 - d12 * d21) * tmp;
  }
}

// create_matrix_lsq, gradients.f90:660-779
void create_matrix_lsq(Case& c) {
  c.Dmat.assign(9 * (size_t)(c.numCells + 1), 0.0);
  c.dmatScheme = 1;
  auto D = [&](int k, int i) -> double& { return c.Dmat[9 * (size_t)i + (k - 1)]; };
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double Dx = c.xc[ijn] - c.xc[ijp], Dy = c.yc[ijn] - c.yc[ijp], Dz = c.zc[ijn] - c.zc[ijp];
    D(1, ijp) = D(1, ijp) + Dx * Dx; D(1, ijn) = D(1, ijn) + Dx * Dx;
    D(4, ijp) = D(4, ijp) + Dy * Dy; D(4, ijn) = D(4, ijn) + Dy * Dy;
    D(6, ijp) = D(6, ijp) + Dz * Dz; D(6, ijn) = D(6, ijn) + Dz * Dz;
    D(2, ijp) = D(2, ijp) + Dx * Dy; D(2, ijn) = D(2, ijn) + Dx * Dy;
    D(3, ijp) = D(3, ijp) + Dx * Dz; D(3, ijn) = D(3, ijn) + Dx * Dz;
    D(5, ijp) = D(5, ijp) + Dy * Dz; D(5, ijn) = D(5, ijn) + Dy * Dz;
  }
  for (int i = 1; i <= c.numBoundaryFaces; ++i) {
    int iface = c.numInnerFaces + i, ijp = c.owner[iface];
    double Dx = c.xf[iface] - c.xc[ijp], Dy = c.yf[iface] - c.yc[ijp], Dz = c.zf[iface] - c.zc[ijp];
    D(1, ijp) = D(1, ijp) + Dx * Dx;
    D(4, ijp) = D(4, ijp) + Dy * Dy;
    D(6, ijp) = D(6, ijp) + Dz * Dz;
    D(2, ijp) = D(2, ijp) + Dx * Dy;
    D(3, ijp) = D(3, ijp) + Dx * Dz;
    D(5, ijp) = D(5, ijp) + Dy * Dz;
  }
  // D(1..6) hold d11 d12 d13 d22 d23 d33 before inversion
  lsq_invert(c);
}

// create_matrix_lsq_dm, gradients.f90:1157-1328
void create_matrix_lsq_dm(Case& c) {
  c.Dmat.assign(9 * (size_t)(c.numCells + 1), 0.0);
  c.dmatScheme = 2;
  auto D = [&](int k, int i) -> double& { return c.Dmat[9 * (size_t)i + (k - 1)]; };
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double ddx = c.xc[ijn] - c.xc[ijp], ddy = c.yc[ijn] - c.yc[ijp], ddz = c.zc[ijn] - c.zc[ijp];
    double w = 1.0 / (ddx * ddx + ddy * ddy + ddz * ddz);
    double Dx = c.xc[ijn] - c.xc[ijp], Dy = c.yc[ijn] - c.yc[ijp], Dz = c.zc[ijn] - c.zc[ijp];
    D(1, ijp) = D(1, ijp) + w * Dx * Dx; D(1, ijn) = D(1, ijn) + w * Dx * Dx;
    D(4, ijp) = D(4, ijp) + w * Dy * Dy; D(4, ijn) = D(4, ijn) + w * Dy * Dy;
    D(6, ijp) = D(6, ijp) + w * Dz * Dz; D(6, ijn) = D(6, ijn) + w * Dz * Dz;
    D(2, ijp) = D(2, ijp) + w * Dx * Dy; D(2, ijn) = D(2, ijn) + w * Dx * Dy;
    D(3, ijp) = D(3, ijp) + w * Dx * Dz; D(3, ijn) = D(3, ijn) + w * Dx * Dz;
    D(5, ijp) = D(5, ijp) + w * Dy * Dz; D(5, ijn) = D(5, ijn) + w * Dy * Dz;
  }
  for (int i = 1; i <= c.numBoundaryFaces; ++i) {
    int iface = c.numInnerFaces + i, ijp = c.owner[iface];
    double ddx = c.xf[iface] - c.xc[ijp], ddy = c.yf[iface] - c.yc[ijp], ddz = c.zf[iface] - c.zc[ijp];
    double w = 1.0 / (ddx * ddx + ddy * ddy + ddz * ddz);
    double Dx = c.xf[iface] - c.xc[ijp], Dy = c.yf[iface] - c.yc[ijp], Dz = c.zf[iface] - c.zc[ijp];
    D(1, ijp) = D(1, ijp) + w * Dx * Dx;
    D(4, ijp) = D(4, ijp) + w * Dy * Dy;
    D(6, ijp) = D(6, ijp) + w * Dz * Dz;
    D(2, ijp) = D(2, ijp) + w * Dx * Dy;
    D(3, ijp) = D(3, ijp) + w * Dx * Dz;
    D(5, ijp) = D(5, ijp) + w * Dy * Dz;
  }
  lsq_invert(c);
}

// cofactor apply of grad_lsq (:883-889) / grad_lsq_dm (:1476-1482),
// including the reference's y-row (b1*D4 - b2*D5 - b3*D6).  exact: the
// y-row of the adjugate of the symmetric normal matrix instead,
// -b1*D2 + b2*D4 - b3*D8, evaluated as (b2*D4 - b1*D2) - b3*D8 (the
// least-squares extension lsq_exact; the other rows are the reference's)
static void lsq_apply(Case& c, std::vector<double>& g, bool exact) {
  for (int inp = 1; inp <= c.numCells; ++inp) {
    const double* D = &c.Dmat[9 * (size_t)inp];
    double b1 = G(g, 1, inp), b2 = G(g, 2, inp), b3 = G(g, 3, inp);
    G(g, 1, inp) = b1 * D[0] - b2 * D[1] + b3 * D[2];
    if (exact) G(g, 2, inp) = (b2 * D[3] - b1 * D[1]) - b3 * D[7];
    else G(g, 2, inp) = b1 * D[3] - b2 * D[4] - b3 * D[5];
    G(g, 3, inp) = b1 * D[6] - b2 * D[7] + b3 * D[8];
  }
}

// grad_lsq, gradients.f90:782-893 (exact: the correct y-row, lsq_apply)
void grad_lsq(Case& c, const std::vector<double>& phi, std::vector<double>& g, bool exact) {
  std::fill(g.begin(), g.end(), 0.0);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double delta = phi[ijn] - phi[ijp];
    double Dx = (c.xc[ijn] - c.xc[ijp]) * delta, Dy = (c.yc[ijn] - c.yc[ijp]) * delta,
           Dz = (c.zc[ijn] - c.zc[ijp]) * delta;
    G(g, 1, ijp) = G(g, 1, ijp) + Dx; G(g, 2, ijp) = G(g, 2, ijp) + Dy; G(g, 3, ijp) = G(g, 3, ijp) + Dz;
    G(g, 1, ijn) = G(g, 1, ijn) + Dx; G(g, 2, ijn) = G(g, 2, ijn) + Dy; G(g, 3, ijn) = G(g, 3, ijn) + Dz;
  }
  for (int i = 1; i <= c.numBoundaryFaces; ++i) {
    int iface = c.numInnerFaces + i, ijp = c.owner[iface], ijn = c.numCells + i;
    double delta = phi[ijn] - phi[ijp];
    double Dx = (c.xf[iface] - c.xc[ijp]) * delta, Dy = (c.yf[iface] - c.yc[ijp]) * delta,
           Dz = (c.zf[iface] - c.zc[ijp]) * delta;
    G(g, 1, ijp) = G(g, 1, ijp) + Dx; G(g, 2, ijp) = G(g, 2, ijp) + Dy; G(g, 3, ijp) = G(g, 3, ijp) + Dz;
  }
  lsq_apply(c, g, exact);
}

// grad_lsq_dm, gradients.f90:1334-1486 (boundary weight reads xf(i)...
// at the boundary-face counter i, as the reference does at :1459; exact:
// the face's own xf(iface)..., the weight create_matrix_lsq_dm uses, and
// the correct y-row)
void grad_lsq_dm(Case& c, const std::vector<double>& phi, std::vector<double>& g, bool exact) {
  std::fill(g.begin(), g.end(), 0.0);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double ddx = c.xc[ijn] - c.xc[ijp], ddy = c.yc[ijn] - c.yc[ijp], ddz = c.zc[ijn] - c.zc[ijp];
    double w = (phi[ijn] - phi[ijp]) / (ddx * ddx + ddy * ddy + ddz * ddz);
    double Dx = w * (c.xc[ijn] - c.xc[ijp]), Dy = w * (c.yc[ijn] - c.yc[ijp]), Dz = w * (c.zc[ijn] - c.zc[ijp]);
    G(g, 1, ijp) = G(g, 1, ijp) + Dx; G(g, 2, ijp) = G(g, 2, ijp) + Dy; G(g, 3, ijp) = G(g, 3, ijp) + Dz;
    G(g, 1, ijn) = G(g, 1, ijn) + Dx; G(g, 2, ijn) = G(g, 2, ijn) + Dy; G(g, 3, ijn) = G(g, 3, ijn) + Dz;
  }
  for (int i = 1; i <= c.numBoundaryFaces; ++i) {
    int iface = c.numInnerFaces + i, ijp = c.owner[iface], ijn = c.numCells + i;
    const int iw = exact ? iface : i;
    double ddx = c.xf[iw] - c.xc[ijp], ddy = c.yf[iw] - c.yc[ijp], ddz = c.zf[iw] - c.zc[ijp];
    double w = (phi[ijn] - phi[ijp]) / (ddx * ddx + ddy * ddy + ddz * ddz);
    double Dx = w * (c.xf[iface] - c.xc[ijp]), Dy = w * (c.yf[iface] - c.yc[ijp]), Dz = w * (c.zf[iface] - c.zc[ijp]);
    G(g, 1, ijp) = G(g, 1, ijp) + Dx; G(g, 2, ijp) = G(g, 2, ijp) + Dy; G(g, 3, ijp) = G(g, 3, ijp) + Dz;
  }
  lsq_apply(c, g, exact);
}

// the least-squares matrix a gradient scheme uses (1: create_matrix_lsq,
// 2: create_matrix_lsq_dm, 0: none), built on first use as the reference
// builds it at initialisation
void prepare_lsq(Case& c, int scheme) {
  const int m = lsq_matrix_of(scheme);
  if (m == 1 && c.dmatScheme != 1) create_matrix_lsq(c);
  if (m == 2 && c.dmatScheme != 2) create_matrix_lsq_dm(c);
}

// one gradient scheme without the limiter: 0 Gauss, 1 LSQ, 2 LSQ_DM, 3 node
// Gauss, 4 LSQ with the correct y-row, 5 LSQ_DM with the correct y-row and
// boundary weight
void grad_scheme(Case& c, int scheme, const std::vector<double>& phi, std::vector<double>& g) {
  prepare_lsq(c, scheme);
  if (scheme == 1 || scheme == 4) grad_lsq(c, phi, g, scheme == 4);
  else if (scheme == 2 || scheme == 5) grad_lsq_dm(c, phi, g, scheme == 5);
  else if (scheme == 3) grad_node_based_gauss(c, phi, g);
  else grad_gauss(c, phi, g);
}

// grad_scalar_field, gradients.f90:106-163: the gradient, then the limiter
void grad(Case& c, const std::vector<double>& phi, std::vector<double>& g) {
  // the least-squares matrices of the scheme (create_matrix_lsq / _dm, built
  // at initialisation in the reference) on first use
  grad_scheme(c, c.gradScheme, phi, g);
  slope_limiter(c, phi, g);
}

// --------------------------------------------------- node interpolation
// node_interpolation.f90: cell-to-node weights in the module's running
// order (inner faces ascending, per face node, owner then neighbour), and
// face-to-node weights of the boundary faces.  tiny is geometry.f90:41's
// default-real 1e-30.
static inline int NODE(const Case& c, int k, int iface) { return c.node[(size_t)iface * 6 + (k - 1)]; }

// weights_inverse_distance, node_interpolation.f90:88-260
static void weights_inverse_distance(Case& c) {
  std::vector<double> dsum(c.numNodes + 1, 0.0);
  auto dist = [&](double xa, double ya, double za, int ino) {
    double dx = xa - c.x[ino], dy = ya - c.y[ino], dz = za - c.z[ino];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
  };
  int cnt = 0;
  for (int iface = 1; iface <= c.numInnerFaces; ++iface) {
    int ijp = c.owner[iface], ijn = c.neighbour[iface];
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      dsum[ino] = dsum[ino] + 1. / dist(c.xc[ijp], c.yc[ijp], c.zc[ijp], ino);
      dsum[ino] = dsum[ino] + 1. / dist(c.xc[ijn], c.yc[ijn], c.zc[ijn], ino);
      cnt += 2;
    }
  }
  c.wCellToNode.assign(cnt + 1, 0.0);
  int i = 0;
  for (int iface = 1; iface <= c.numInnerFaces; ++iface) {
    int ijp = c.owner[iface], ijn = c.neighbour[iface];
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      double dcp = dist(c.xc[ijp], c.yc[ijp], c.zc[ijp], ino);
      c.wCellToNode[++i] = 1. / (dcp * dsum[ino]);
      dcp = dist(c.xc[ijn], c.yc[ijn], c.zc[ijn], ino);
      c.wCellToNode[++i] = 1. / (dcp * dsum[ino]);
    }
  }
  std::fill(dsum.begin(), dsum.end(), 0.0);
  cnt = 0;
  for (int iface = c.numInnerFaces + 1; iface <= c.numFaces; ++iface)
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      dsum[ino] = dsum[ino] + 1. / dist(c.xf[iface], c.yf[iface], c.zf[iface], ino);
      ++cnt;
    }
  c.wFaceToNode.assign(cnt + 1, 0.0);
  i = 0;
  for (int iface = c.numInnerFaces + 1; iface <= c.numFaces; ++iface)
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      double dcp = dist(c.xf[iface], c.yf[iface], c.zf[iface], ino);
      c.wFaceToNode[++i] = 1. / (dcp * dsum[ino]);
    }
}

// pseudo-Laplacian moments of one point about a node
struct PslMoments {
  std::vector<double> rx, ry, rz, ixx, iyy, izz, ixy, ixz, iyz;
  explicit PslMoments(int n)
      : rx(n, 0.0), ry(n, 0.0), rz(n, 0.0), ixx(n, 0.0), iyy(n, 0.0), izz(n, 0.0), ixy(n, 0.0), ixz(n, 0.0),
        iyz(n, 0.0) {}
  void add(int ino, double dx, double dy, double dz) {
    rx[ino] = rx[ino] + dx; ry[ino] = ry[ino] + dy; rz[ino] = rz[ino] + dz;
    ixx[ino] = ixx[ino] + dx * dx; iyy[ino] = iyy[ino] + dy * dy; izz[ino] = izz[ino] + dz * dz;
    ixy[ino] = ixy[ino] + dx * dy; ixz[ino] = ixz[ino] + dx * dz; iyz[ino] = iyz[ino] + dy * dz;
  }
  // min(|1 + lam . d|, 1) with the lambdas as node_interpolation.f90:386-407 writes them
  double weight(int ino, double dx, double dy, double dz) const {
    const double Ixx = ixx[ino], Iyy = iyy[ino], Izz = izz[ino], Ixy = ixy[ino], Ixz = ixz[ino], Iyz = iyz[ino];
    const double Rx = rx[ino], Ry = ry[ino], Rz = rz[ino];
    double D = Ixx * (Iyy * Izz - Iyz * Iyz) - Ixy * (Ixy * Izz - Ixz * Iyz) + Ixz * (Ixy * Iyz - Iyy * Ixz) + kTiny30;
    double lamx = (-(Rx * (Ixx * Izz - Iyz * Iyz)) + Ry * (Ixy * Izz - Ixz * Iyz) - Rz * (Ixy * Iyz - Iyy * Ixz)) / D;
    double lamy = (Rx * (Ixy * Izz - Ixz * Iyz) - Ry * (Ixx * Izz - Ixz * Ixz) + Rz * (Ixx * Iyz - Ixy * Ixz)) / D;
    double lamz = (-(Rx * (Ixy * Iyz - Iyy * Ixz)) + Ry * (Ixx * Iyz - Ixy * Ixz) - Rz * (Ixx * Iyy - Ixy * Ixy)) / D;
    double w = 1.0 + lamx * dx + lamy * dy + lamz * dz;
    return std::min(std::fabs(w), 1.0);
  }
};

// weights_pseudolaplacian, node_interpolation.f90:265-631
static void weights_pseudolaplacian(Case& c) {
  const int nn = c.numNodes + 1;
  {
    PslMoments M(nn);
    int cnt = 0;
    for (int iface = 1; iface <= c.numInnerFaces; ++iface) {
      int ijp = c.owner[iface], ijn = c.neighbour[iface];
      for (int k = 1; k <= c.nnodes[iface]; ++k) {
        int ino = NODE(c, k, iface);
        M.add(ino, c.xc[ijp] - c.x[ino], c.yc[ijp] - c.y[ino], c.zc[ijp] - c.z[ino]);
        M.add(ino, c.xc[ijn] - c.x[ino], c.yc[ijn] - c.y[ino], c.zc[ijn] - c.z[ino]);
        cnt += 2;
      }
    }
    c.wCellToNode.assign(cnt + 1, 0.0);
    int i = 0;
    for (int iface = 1; iface <= c.numInnerFaces; ++iface) {
      int ijp = c.owner[iface], ijn = c.neighbour[iface];
      for (int k = 1; k <= c.nnodes[iface]; ++k) {
        int ino = NODE(c, k, iface);
        c.wCellToNode[++i] = M.weight(ino, c.xc[ijp] - c.x[ino], c.yc[ijp] - c.y[ino], c.zc[ijp] - c.z[ino]);
        c.wCellToNode[++i] = M.weight(ino, c.xc[ijn] - c.x[ino], c.yc[ijn] - c.y[ino], c.zc[ijn] - c.z[ino]);
      }
    }
    std::vector<double> wsum(nn, 0.0);
    i = 0;
    for (int iface = 1; iface <= c.numInnerFaces; ++iface)
      for (int k = 1; k <= c.nnodes[iface]; ++k) {
        int ino = NODE(c, k, iface);
        ++i; wsum[ino] = wsum[ino] + c.wCellToNode[i];
        ++i; wsum[ino] = wsum[ino] + c.wCellToNode[i];
      }
    i = 0;
    for (int iface = 1; iface <= c.numInnerFaces; ++iface)
      for (int k = 1; k <= c.nnodes[iface]; ++k) {
        int ino = NODE(c, k, iface);
        ++i; c.wCellToNode[i] = c.wCellToNode[i] / wsum[ino];
        ++i; c.wCellToNode[i] = c.wCellToNode[i] / wsum[ino];
      }
  }
  PslMoments M(nn);
  int cnt = 0;
  for (int iface = c.numInnerFaces + 1; iface <= c.numFaces; ++iface)
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      M.add(ino, c.xf[iface] - c.x[ino], c.yf[iface] - c.y[ino], c.zf[iface] - c.z[ino]);
      ++cnt;
    }
  c.wFaceToNode.assign(cnt + 1, 0.0);
  int i = 0;
  for (int iface = c.numInnerFaces + 1; iface <= c.numFaces; ++iface)
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      c.wFaceToNode[++i] = M.weight(ino, c.xf[iface] - c.x[ino], c.yf[iface] - c.y[ino], c.zf[iface] - c.z[ino]);
    }
  std::vector<double> wsum(nn, 0.0);
  i = 0;
  for (int iface = c.numInnerFaces + 1; iface <= c.numFaces; ++iface)
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      ++i; wsum[ino] = wsum[ino] + c.wFaceToNode[i];
    }
  i = 0;
  for (int iface = c.numInnerFaces + 1; iface <= c.numFaces; ++iface)
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      ++i; c.wFaceToNode[i] = c.wFaceToNode[i] / wsum[ino];
    }
}

// set_interpolation_weights, node_interpolation.f90:46-84
void set_interpolation_weights(Case& c) {
  if (c.c2n == 1) weights_inverse_distance(c);
  else weights_pseudolaplacian(c);
}

// interpolate_to_nodes, node_interpolation.f90:635-700
void interpolate_to_nodes(Case& c, const std::vector<double>& phiC, std::vector<double>& phiN) {
  phiN.assign(c.numNodes + 1, 0.0);
  int i = 0;
  for (int iface = 1; iface <= c.numInnerFaces; ++iface) {
    int ijp = c.owner[iface], ijn = c.neighbour[iface];
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      ++i; phiN[ino] = phiN[ino] + c.wCellToNode[i] * phiC[ijp];
      ++i; phiN[ino] = phiN[ino] + c.wCellToNode[i] * phiC[ijn];
    }
  }
  for (int iface = c.numInnerFaces + 1; iface <= c.numFaces; ++iface)
    for (int k = 1; k <= c.nnodes[iface]; ++k) phiN[NODE(c, k, iface)] = 0.;
  i = 0;
  for (int iface = c.numInnerFaces + 1; iface <= c.numFaces; ++iface) {
    int ib = c.numCells + (iface - c.numInnerFaces);
    for (int k = 1; k <= c.nnodes[iface]; ++k) {
      int ino = NODE(c, k, iface);
      ++i; phiN[ino] = phiN[ino] + c.wFaceToNode[i] * phiC[ib];
    }
  }
}

// grad_node_based_gauss, gradients.f90:1491-1602
void grad_node_based_gauss(Case& c, const std::vector<double>& u, std::vector<double>& dudxi) {
  if (c.wCellToNode.empty()) set_interpolation_weights(c);
  std::vector<double> uN;
  interpolate_to_nodes(c, u, uN);
  std::fill(dudxi.begin(), dudxi.end(), 0.0);
  for (int iface = 1; iface <= c.numFaces; ++iface) {
    double fie = 0.0;
    for (int k = 1; k <= c.nnodes[iface]; ++k) fie = fie + uN[NODE(c, k, iface)];
    fie = fie / (double)c.nnodes[iface];
    double dfxe = fie * c.arx[iface], dfye = fie * c.ary[iface], dfze = fie * c.arz[iface];
    int ijp = c.owner[iface];
    G(dudxi, 1, ijp) = G(dudxi, 1, ijp) + dfxe;
    G(dudxi, 2, ijp) = G(dudxi, 2, ijp) + dfye;
    G(dudxi, 3, ijp) = G(dudxi, 3, ijp) + dfze;
    if (iface <= c.numInnerFaces) {
      int ijn = c.neighbour[iface];
      G(dudxi, 1, ijn) = G(dudxi, 1, ijn) - dfxe;
      G(dudxi, 2, ijn) = G(dudxi, 2, ijn) - dfye;
      G(dudxi, 3, ijn) = G(dudxi, 3, ijn) - dfze;
    }
  }
  for (int ijp = 1; ijp <= c.numCells; ++ijp) {
    double volr = 1. / c.vol[ijp];
    for (int k = 1; k <= 3; ++k) G(dudxi, k, ijp) = G(dudxi, k, ijp) * volr;
  }
}

// slope_limiter_Barth_Jespersen (:288-366), _Venkatakrishnan (:373-451) and
// _r345 (:456-535, whose active line is the R4 function): the gradient of
// each cell scaled by the smallest limiter value over its CSR row.  phi_min
// of those routines is computed but never used; the deltas use the global
// extremes.  abs(delta_face) < 1.e-6 compares with a default-real literal.
static void limiter_scale(Case& c, const std::vector<double>& phi, std::vector<double>& g) {
  const double tiny = (double)1.e-6f;
  double fimin = phi[1], fimax = phi[1];
  for (int inp = 2; inp <= c.numCells; ++inp) {
    fimin = std::min(fimin, phi[inp]);
    fimax = std::max(fimax, phi[inp]);
  }
  for (int inp = 1; inp <= c.numCells; ++inp) {
    double deltamax = fimax - phi[inp];
    double deltamin = fimin - phi[inp];
    double slopelimit = 1.0;
    for (int k = c.ia[inp]; k <= c.ia[inp + 1] - 1; ++k) {
      if (k == c.diag[inp]) continue;
      int ijp = inp, ijn = c.ja[k];
      double delta_face = G(g, 1, ijp) * (c.xc[ijn] - c.xc[ijp]) + G(g, 2, ijp) * (c.yc[ijn] - c.yc[ijp]) +
                          G(g, 3, ijp) * (c.zc[ijn] - c.zc[ijp]);
      double r;
      if (std::fabs(delta_face) < tiny) r = 1.0;
      else if (delta_face > 0.0) r = deltamax / delta_face;
      else r = deltamin / delta_face;
      double lim;
      if (c.limiter == 1) {
        lim = r;
      } else if (c.limiter == 2) {
        lim = (r * r + 2.0 * r) / (r * r + r + 2.0);
      } else {
        double r2 = r * r, r3 = r2 * r, r4 = r2 * r2;
        lim = (r4 + 2 * r3 - 4 * r2 + 8 * r) / (r4 + r3 + 2 * r2 - 4 * r + 8.0);
      }
      slopelimit = std::min(slopelimit, lim);
    }
    for (int k = 1; k <= 3; ++k) G(g, k, inp) = slopelimit * G(g, k, inp);
  }
}

// slope_limiter_multidimensional, gradients.f90:541-656
static void limiter_multidimensional(Case& c, const std::vector<double>& phi, std::vector<double>& g) {
  std::vector<double> phimax(c.numCells + 1), phimin(c.numCells + 1);
  for (int inp = 1; inp <= c.numCells; ++inp) {
    phimax[inp] = phi[c.ja[c.ia[inp]]];
    phimin[inp] = phi[c.ja[c.ia[inp]]];
    for (int k = c.ia[inp] + 1; k <= c.ia[inp + 1] - 1; ++k) {
      phimax[inp] = std::max(phimax[inp], phi[c.ja[k]]);
      phimin[inp] = std::min(phimin[inp], phi[c.ja[k]]);
    }
  }
  for (int iface = 1; iface <= c.numInnerFaces; ++iface) {
    for (int k = 1; k <= 2; ++k) {
      int ijp = k == 1 ? c.owner[iface] : c.neighbour[iface];
      double gx = G(g, 1, ijp), gy = G(g, 2, ijp), gz = G(g, 3, ijp);
      double xpn = c.xf[iface] - c.xc[ijp], ypn = c.yf[iface] - c.yc[ijp], zpn = c.zf[iface] - c.zc[ijp];
      double dpn = std::sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
      double nx = xpn / dpn, ny = ypn / dpn, nz = zpn / dpn;
      double gn = gx * nx + gy * ny + gz * nz;
      double gtx = gx - gn * nx, gty = gy - gn * ny, gtz = gz - gn * nz;
      double dPhi = gx * xpn + gy * ypn + gz * zpn;
      double dPhimax = phimax[ijp] - phi[ijp];
      double dPhimin = phimin[ijp] - phi[ijp];
      if (phimax[ijp] > phi[ijp] && dPhi > dPhimax) {
        gx = gtx + nx * dPhimax; gy = gty + ny * dPhimax; gz = gtz + nz * dPhimax;
      }
      if (phimin[ijp] < phi[ijp] && dPhi < dPhimin) {
        gx = gtx + nx * dPhimin; gy = gty + ny * dPhimin; gz = gtz + nz * dPhimin;
      }
      G(g, 1, ijp) = gx; G(g, 2, ijp) = gy; G(g, 3, ijp) = gz;
    }
  }
}

// the select case on `limiter` of grad_scalar_field, gradients.f90:141-160
void slope_limiter(Case& c, const std::vector<double>& phi, std::vector<double>& g) {
  if (c.limiter >= 1 && c.limiter <= 3) limiter_scale(c, phi, g);
  else if (c.limiter == 4) limiter_multidimensional(c, phi, g);
}

// ------------------------------------------------------------ interpolation
// Scheme ids shared with the GPU library (fc_gpu.h FC_SCHEME_*).
enum {
  S_CDS = 0, S_CENTRAL = 1, S_LINEARUPWIND = 2, S_KAPPA = 3,
  S_MUSCL = 10, S_UMIST, S_KOREN, S_SMART, S_AVLSMART, S_CHARM, S_VANLEER, S_OSPRE, S_MINMOD,
  S_BLU, S_BLU02, S_BCENTRAL, S_FROMM, S_CUI, S_QUICK, S_SPL13
};

// face_value_flux_limiter, interpolation.f90:489-650
static double face_value_flux_limiter(Case& c, int ijp, int ijn, double lambda, const std::vector<double>& u,
                                      std::vector<double>& dUdxi, int scheme) {
  double fxp = 1.0 - lambda;
  double psi = 1.0;
  double xpn = c.xc[ijn] - c.xc[ijp], ypn = c.yc[ijn] - c.yc[ijp], zpn = c.zc[ijn] - c.zc[ijp];
  double r = (2 * G(dUdxi, 1, ijp) * xpn + 2 * G(dUdxi, 2, ijp) * ypn + 2 * G(dUdxi, 3, ijp) * zpn) /
                 (u[ijn] - u[ijp] + kTiny30) - 1.0;
  const double two3s = (double)(2.0f / 3.0f), one3s = (double)(1.0f / 3.0f);  // 2./3. and 1./3. (single)
  const double two3d = 2.0 / 3.0, one3d = 1.0 / 3.0;                          // 2./3._dp, 1./3.0_dp
  switch (scheme) {
    case S_MUSCL: psi = std::max(0.0, std::min(std::min(2 * r, 0.5 * r + 0.5), 2.0)); break;
    case S_UMIST: psi = std::max(0.0, std::min(std::min(std::min(2 * r, 0.75 * r + 0.25), 0.25 * r + 0.75), 2.0)); break;
    case S_KOREN: psi = std::max(0.0, std::min(std::min(2 * r, two3d * r + one3d), 2.0)); break;
    case S_SMART: psi = std::max(0.0, std::min(std::min(2 * r, 0.75 * r + 0.25), 4.0)); break;
    case S_AVLSMART: psi = std::max(0.0, std::min(std::min(1.5 * r, 0.75 * r + 0.25), 2.5)); break;
    case S_CHARM: psi = std::max(0.0, (r + std::fabs(r)) * (3 * r + 1.0) / (2 * ((r + 1.0) * (r + 1.0)))); break;
    case S_VANLEER: psi = std::max(0.0, std::min((r + std::fabs(r)) / (r + 1.0), 2.0)); break;
    case S_OSPRE: psi = std::max(0.0, 3 * r * (r + 1.0) / (2 * (r * r + r + 1.0))); break;
    case S_MINMOD: psi = std::max(0.0, std::min(r, 1.0)); break;
    case S_BLU: psi = std::max(0.0, std::min(2 * r, 1.0)); break;
    case S_BLU02: psi = std::max(0.0, std::min(10 * r, 1.0)); break;
    case S_BCENTRAL: psi = std::max(0.0, std::min(r, 4.0)); break;
    case S_FROMM: psi = 0.5 * r + 0.5; break;
    case S_CUI: psi = two3s * r + one3s; break;
    case S_QUICK: psi = 0.75 * r + 0.25; break;
    case S_SPL13:
      psi = std::max(0.0, std::min(std::min(std::min(2 * r, one3s * r + two3s), two3s * r + one3s), 2.0));
      break;
    default: psi = 1.0; break;
  }
  return u[ijp] + fxp * psi * (u[ijn] - u[ijp]);
}

// face_value, interpolation.f90:28-113
double face_value(Case& c, int ijp, int ijn, double xf, double yf, double zf, double lambda,
                  const std::vector<double>& u, std::vector<double>& dUdxi, int scheme) {
  switch (scheme) {
    case S_CDS:  // face_value_cds :116-157
      return u[ijp] + (u[ijn] - u[ijp]) * lambda;
    case S_CENTRAL: {  // face_value_central :218-264
      double gradfidr = G(dUdxi, 1, ijp) * (xf - c.xc[ijp]) + G(dUdxi, 2, ijp) * (yf - c.yc[ijp]) +
                        G(dUdxi, 3, ijp) * (zf - c.zc[ijp]) + G(dUdxi, 1, ijn) * (xf - c.xc[ijn]) +
                        G(dUdxi, 2, ijn) * (yf - c.yc[ijn]) + G(dUdxi, 3, ijn) * (zf - c.zc[ijn]);
      return 0.5 * (u[ijp] + u[ijn] + gradfidr);
    }
    case S_LINEARUPWIND: {  // face_value_2nd_upwind :318-356
      double gradfidr = G(dUdxi, 1, ijp) * (xf - c.xc[ijp]) + G(dUdxi, 2, ijp) * (yf - c.yc[ijp]) +
                        G(dUdxi, 3, ijp) * (zf - c.zc[ijp]);
      return u[ijp] + gradfidr;
    }
    case S_KAPPA: {  // face_value_kappa :359-416, theta = 2./3. (single)
      const double theta = (double)(2.0f / 3.0f);
      double g2 = G(dUdxi, 1, ijp) * (xf - c.xc[ijp]) + G(dUdxi, 2, ijp) * (yf - c.yc[ijp]) +
                  G(dUdxi, 3, ijp) * (zf - c.zc[ijp]);
      double gc = G(dUdxi, 1, ijp) * (xf - c.xc[ijp]) + G(dUdxi, 2, ijp) * (yf - c.yc[ijp]) +
                  G(dUdxi, 3, ijp) * (zf - c.zc[ijp]) + G(dUdxi, 1, ijn) * (xf - c.xc[ijn]) +
                  G(dUdxi, 2, ijn) * (yf - c.yc[ijn]) + G(dUdxi, 3, ijn) * (zf - c.zc[ijn]);
      double vf2 = (u[ijp] + g2);
      double vfc = 0.5 * (u[ijp] + u[ijn] + gc);
      return theta * vfc + (1.0 - theta) * vf2;
    }
    default:
      return face_value_flux_limiter(c, ijp, ijn, lambda, u, dUdxi, scheme);
  }
}

// ----------------------------------------------------------------- laplacian
// laplacian + faceFluxLaplacian, laplacian.f90:1-151.  The reference applies
// the boundary term on every patch (its bctype filter is commented out at
// :73); dirichlet_mask selects patches (bit ib-1), all bits = reference.
void laplacian(Case& c, const std::vector<double>& mu, const std::vector<double>& phi,
               unsigned long long dirichlet_mask) {
  std::fill(c.a.begin(), c.a.end(), 0.0);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double fxn = c.facint[i], fxp = 1.0 - c.facint[i];
    double xpn = c.xc[ijn] - c.xc[ijp], ypn = c.yc[ijn] - c.yc[ijp], zpn = c.zc[ijn] - c.zc[ijp];
    double smdpn = (c.arx[i] * c.arx[i] + c.ary[i] * c.ary[i] + c.arz[i] * c.arz[i]) /
                   (c.arx[i] * xpn + c.ary[i] * ypn + c.arz[i] * zpn);
    double cap = (fxp * mu[ijp] + fxn * mu[ijn]) * smdpn;
    double can = cap;
    c.a[c.ijk[i]] = can;
    c.a[c.jik[i]] = cap;
    c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - can;
    c.a[c.diag[ijn]] = c.a[c.diag[ijn]] - cap;
  }
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (ib <= 64 && !((dirichlet_mask >> (ib - 1)) & 1ULL)) continue;
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
      double are = std::sqrt(c.arx[iface] * c.arx[iface] + c.ary[iface] * c.ary[iface] + c.arz[iface] * c.arz[iface]);
      double nxf = c.arx[iface] / are, nyf = c.ary[iface] / are, nzf = c.arz[iface] / are;
      double dfn = (c.xf[iface] - c.xc[ijp]) * nxf + (c.yf[iface] - c.yc[ijp]) * nyf + (c.zf[iface] - c.zc[ijp]) * nzf;
      double dcoef = mu[ijp] * are / dfn;
      c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - dcoef;
      c.su[ijp] = c.su[ijp] - dcoef * phi[ijb];
    }
  }
}

// ------------------------------------------------------ pressure gradient
// bpres, bpres.f90:55-180
void bpres(Case& c, std::vector<double>& p, int istage) {
  if (istage == 1) {
    for (int ib = 1; ib <= c.numBoundaries; ++ib) {
      if (c.bctype[ib] == BC_PRESSURE) continue;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        p[ijb] = p[ijp];
      }
    }
  } else {
    for (int ib = 1; ib <= c.numBoundaries; ++ib) {
      if (c.bctype[ib] != BC_WALL) continue;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        double xpb = c.xf[iface] - c.xc[ijp], ypb = c.yf[iface] - c.yc[ijp], zpb = c.zf[iface] - c.zc[ijp];
        p[ijb] = p[ijp] + G(c.dPdxi, 1, ijp) * xpb + G(c.dPdxi, 2, ijp) * ypb + G(c.dPdxi, 3, ijp) * zpb;
      }
    }
  }
}

// gradp_and_sources, nablap.f90:19-208
void gradp_and_sources(Case& c, std::vector<double>& p) {
  const int nC = c.numCells;
  auto inner_sum = [&](int mode) {
    for (int i = 1; i <= c.numInnerFaces; ++i) {
      int ijp = c.owner[i], ijn = c.neighbour[i];
      double pf;
      if (mode == 0) pf = p[ijp] + (p[ijn] - p[ijp]) * c.facint[i];
      else if (mode == 1) pf = face_value(c, ijp, ijn, c.xf[i], c.yf[i], c.zf[i], c.facint[i], p, c.dPdxi, S_CENTRAL);
      else pf = (p[ijp] * c.apu[ijp] + p[ijn] * c.apu[ijn]) / (c.apu[ijp] + c.apu[ijn] + kSmall);
      double dfxe = pf * c.arx[i], dfye = pf * c.ary[i], dfze = pf * c.arz[i];
      c.su[ijp] = c.su[ijp] - dfxe; c.sv[ijp] = c.sv[ijp] - dfye; c.sw[ijp] = c.sw[ijp] - dfze;
      c.su[ijn] = c.su[ijn] + dfxe; c.sv[ijn] = c.sv[ijn] + dfye; c.sw[ijn] = c.sw[ijn] + dfze;
    }
  };
  std::fill(c.su.begin(), c.su.end(), 0.0);
  std::fill(c.sv.begin(), c.sv.end(), 0.0);
  std::fill(c.sw.begin(), c.sw.end(), 0.0);
  inner_sum(c.pscheme == 2 ? 2 : 0);
  for (int istage = 1; istage <= 2; ++istage) {
    bpres(c, p, istage);
    if (istage == 2 && c.pscheme == 1) {
      std::fill(c.su.begin(), c.su.end(), 0.0);
      std::fill(c.sv.begin(), c.sv.end(), 0.0);
      std::fill(c.sw.begin(), c.sw.end(), 0.0);
      inner_sum(1);
    }
    for (int i = 1; i <= nC; ++i) {
      G(c.dPdxi, 1, i) = -c.su[i];
      G(c.dPdxi, 2, i) = -c.sv[i];
      G(c.dPdxi, 3, i) = -c.sw[i];
    }
    for (int i = 1; i <= c.numBoundaryFaces; ++i) {
      int iface = c.numInnerFaces + i, ijp = c.owner[iface], ijb = nC + i;
      G(c.dPdxi, 1, ijp) = G(c.dPdxi, 1, ijp) + p[ijb] * c.arx[iface];
      G(c.dPdxi, 2, ijp) = G(c.dPdxi, 2, ijp) + p[ijb] * c.ary[iface];
      G(c.dPdxi, 3, ijp) = G(c.dPdxi, 3, ijp) + p[ijb] * c.arz[iface];
    }
    for (int ijp = 1; ijp <= nC; ++ijp) {
      double volr = 1.0 / c.vol[ijp];
      for (int k = 1; k <= 3; ++k) G(c.dPdxi, k, ijp) = G(c.dPdxi, k, ijp) * volr;
    }
  }
  for (int i = 1; i <= c.numBoundaryFaces; ++i) {
    int iface = c.numInnerFaces + i, ijp = c.owner[iface], ijb = nC + i;
    c.su[ijp] = c.su[ijp] - p[ijb] * c.arx[iface];
    c.sv[ijp] = c.sv[ijp] - p[ijb] * c.ary[iface];
    c.sw[ijp] = c.sw[ijp] - p[ijb] * c.arz[iface];
  }
}

// updateVelocityAtBoundary, velocity.f90:1184-1279
void updateVelocityAtBoundary(Case& c) {
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] == BC_EMPTY || c.bctype[ib] == BC_PERIODIC) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        c.u[ijb] = c.u[ijp]; c.v[ijb] = c.v[ijp]; c.w[ijb] = c.w[ijp];
      }
    } else if (c.bctype[ib] == BC_SYMMETRY) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        double Unmag = c.u[ijp] * c.arx[iface] + c.v[ijp] * c.ary[iface] + c.w[ijp] * c.arz[iface];
        c.u[ijb] = c.u[ijp] - Unmag * c.arx[iface];
        c.v[ijb] = c.v[ijp] - Unmag * c.ary[iface];
        c.w[ijb] = c.w[ijp] - Unmag * c.arz[iface];
      }
    }
  }
}

// inner-face mass flux initialisation, init.f90:167-176
void init_flmass(Case& c) {
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double fxn = c.facint[i], fxp = 1.0 - c.facint[i];
    double ui = c.u[ijp] * fxp + c.u[ijn] * fxn;
    double vi = c.v[ijp] * fxp + c.v[ijn] * fxn;
    double wi = c.w[ijp] * fxp + c.w[ijn] * fxn;
    c.flmass[i] = c.den[ijp] * (c.arx[i] * ui + c.ary[i] * vi + c.arz[i] * wi);
  }
}

// --------------------------------------------------------------- momentum
// sngrad (variant 1), gradients.f90:1720-1779
static inline void sngrad(Case& c, int i, int ijp, int ijn, double arx, double ary, double arz, double lambda,
                          const std::vector<double>& Phi, std::vector<double>& dPhidxi, double& dfixi, double& dfiyi,
                          double& dfizi, double& dfixii, double& dfiyii, double& dfizii) {
  double fxn = lambda, fxp = 1.0 - lambda;
  double xpn = c.xc[ijn] - c.xc[ijp], ypn = c.yc[ijn] - c.yc[ijp], zpn = c.zc[ijn] - c.zc[ijp];
  double vole = xpn * arx + ypn * ary + zpn * arz;
  dfixi = G(dPhidxi, 1, ijp) * fxp + G(dPhidxi, 1, ijn) * fxn;
  dfiyi = G(dPhidxi, 2, ijp) * fxp + G(dPhidxi, 2, ijn) * fxn;
  dfizi = G(dPhidxi, 3, ijp) * fxp + G(dPhidxi, 3, ijn) * fxn;
  dfixii = dfixi + arx / vole * (Phi[ijn] - Phi[ijp] - dfixi * xpn - dfiyi * ypn - dfizi * zpn);
  dfiyii = dfiyi + ary / vole * (Phi[ijn] - Phi[ijp] - dfixi * xpn - dfiyi * ypn - dfizi * zpn);
  dfizii = dfizi + arz / vole * (Phi[ijn] - Phi[ijp] - dfixi * xpn - dfiyi * ypn - dfizi * zpn);
  dfixi = dfixi * (arx - c.Df[i] * xpn);
  dfiyi = dfiyi * (ary - c.Df[i] * ypn);
  dfizi = dfizi * (arz - c.Df[i] * zpn);
}

// facefluxuvw, velocity.f90:754-878
static void facefluxuvw(Case& c, int i, int ijp, int ijn, double xf, double yf, double zf, double arx, double ary,
                        double arz, double flomass, double lambda, double gam, double& cap, double& can, double& sup,
                        double& svp, double& swp) {
  double fxn = lambda, fxp = 1.0 - lambda;
  double game = c.vis[ijp] + (c.vis[ijn] - c.vis[ijp]) * lambda;
  double de = game * c.Df[i];
  double ce = std::min(flomass, 0.0), cp = std::max(flomass, 0.0);
  can = -de + ce;
  cap = -de - cp;
  double duxi, duyi, duzi, duxii, duyii, duzii, dvxi, dvyi, dvzi, dvxii, dvyii, dvzii, dwxi, dwyi, dwzi, dwxii,
      dwyii, dwzii;
  sngrad(c, i, ijp, ijn, arx, ary, arz, lambda, c.u, c.dUdxi, duxi, duyi, duzi, duxii, duyii, duzii);
  sngrad(c, i, ijp, ijn, arx, ary, arz, lambda, c.v, c.dVdxi, dvxi, dvyi, dvzi, dvxii, dvyii, dvzii);
  sngrad(c, i, ijp, ijn, arx, ary, arz, lambda, c.w, c.dWdxi, dwxi, dwyi, dwzi, dwxii, dwyii, dwzii);
  double fdue = game * (duxii * arx + dvxii * ary + dwxii * arz);
  double fdve = game * (duyii * arx + dvyii * ary + dwyii * arz);
  double fdwe = game * (duzii * arx + dvzii * ary + dwzii * arz);
  double fdui = game * (duxi + duyi + duzi);
  double fdvi = game * (dvxi + dvyi + dvzi);
  double fdwi = game * (dwxi + dwyi + dwzi);
  fdue = fdue + fdui;
  fdve = fdve + fdvi;
  fdwe = fdwe + fdwi;
  double fuuds = cp * c.u[ijp] + ce * c.u[ijn];
  double fvuds = cp * c.v[ijp] + ce * c.v[ijn];
  double fwuds = cp * c.w[ijp] + ce * c.w[ijn];
  double ue, ve, we;
  if (flomass >= 0.0) {
    ue = face_value(c, ijp, ijn, xf, yf, zf, fxp, c.u, c.dUdxi, c.cSchemeU);
    ve = face_value(c, ijp, ijn, xf, yf, zf, fxp, c.v, c.dVdxi, c.cSchemeU);
    we = face_value(c, ijp, ijn, xf, yf, zf, fxp, c.w, c.dWdxi, c.cSchemeU);
  } else {
    ue = face_value(c, ijn, ijp, xf, yf, zf, fxn, c.u, c.dUdxi, c.cSchemeU);
    ve = face_value(c, ijn, ijp, xf, yf, zf, fxn, c.v, c.dVdxi, c.cSchemeU);
    we = face_value(c, ijn, ijp, xf, yf, zf, fxn, c.w, c.dWdxi, c.cSchemeU);
  }
  double fuhigh = flomass * ue, fvhigh = flomass * ve, fwhigh = flomass * we;
  sup = -gam * (fuhigh - fuuds) + fdue;
  svp = -gam * (fvhigh - fvuds) + fdve;
  swp = -gam * (fwhigh - fwuds) + fdwe;
}

// facefluxuvw_bnd, velocity.f90:882-1034
static void facefluxuvw_bnd(Case& c, int ijp, int ijb, double xf, double yf, double zf, double arx, double ary,
                            double arz, double flomass, double& cap, double& can, double& sup, double& svp,
                            double& swp) {
  double xpn = xf - c.xc[ijp], ypn = yf - c.yc[ijp], zpn = zf - c.zc[ijp];
  double vole = xpn * arx + ypn * ary + zpn * arz;
  double Dfi = (arx * arx + ary * ary + arz * arz) / vole;
  double game = c.vis[ijb];
  double de = game * Dfi;
  can = -de + std::min(flomass, 0.0);
  cap = -de - std::max(flomass, 0.0);
  auto comp = [&](const std::vector<double>& f, std::vector<double>& g, double& dxi, double& dyi, double& dzi,
                  double& dxii, double& dyii, double& dzii) {
    dxi = G(g, 1, ijp); dyi = G(g, 2, ijp); dzi = G(g, 3, ijp);
    dxii = dxi + arx / vole * (f[ijb] - f[ijp] - dxi * xpn - dyi * ypn - dzi * zpn);
    dyii = dyi + ary / vole * (f[ijb] - f[ijp] - dxi * xpn - dyi * ypn - dzi * zpn);
    dzii = dzi + arz / vole * (f[ijb] - f[ijp] - dxi * xpn - dyi * ypn - dzi * zpn);
    dxi = dxi * (arx - Dfi * xpn);
    dyi = dyi * (ary - Dfi * ypn);
    dzi = dzi * (arz - Dfi * zpn);
  };
  double duxi, duyi, duzi, duxii, duyii, duzii, dvxi, dvyi, dvzi, dvxii, dvyii, dvzii, dwxi, dwyi, dwzi, dwxii,
      dwyii, dwzii;
  comp(c.u, c.dUdxi, duxi, duyi, duzi, duxii, duyii, duzii);
  comp(c.v, c.dVdxi, dvxi, dvyi, dvzi, dvxii, dvyii, dvzii);
  comp(c.w, c.dWdxi, dwxi, dwyi, dwzi, dwxii, dwyii, dwzii);
  double fdue = game * (duxii * arx + dvxii * ary + dwxii * arz);
  double fdve = game * (duyii * arx + dvyii * ary + dwyii * arz);
  double fdwe = game * (duzii * arx + dvzii * ary + dwzii * arz);
  double fdui = game * (duxi + duyi + duzi);
  double fdvi = game * (dvxi + dvyi + dvzi);
  double fdwi = game * (dwxi + dwyi + dwzi);
  sup = fdue + fdui;
  svp = fdve + fdvi;
  swp = fdwe + fdwi;
}

// facefluxuvw_periodic, velocity.f90:1038-1179: momentum fluxes through a
// periodic face between ijp and the twin's owner ijn, central weights 1/2,
// the distance vector 2 (xf - xc(ijp)), the full stress tensor of the face
// gradient, cds face values
static void facefluxuvw_periodic(Case& c, int ijp, int ijn, double xf, double yf, double zf, double arx, double ary,
                                 double arz, double flomass, double gam, double& cap, double& can, double& sup,
                                 double& svp, double& swp) {
  const double fxn = 0.5, fxp = fxn;
  double xpn = 2 * (xf - c.xc[ijp]), ypn = 2 * (yf - c.yc[ijp]), zpn = 2 * (zf - c.zc[ijp]);
  double dpn = std::sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
  double are = std::sqrt(arx * arx + ary * ary + arz * arz);
  double game = c.vis[ijp] * fxp + c.vis[ijn] * fxn;
  double de = game * (arx * arx + ary * ary + arz * arz) / (xpn * arx + ypn * ary + zpn * arz);
  double ce = std::min(flomass, 0.0), cp = std::max(flomass, 0.0);
  can = -de + ce;
  cap = -de - cp;
  auto gi = [&](std::vector<double>& g, int k) { return G(g, k, ijp) * fxp + G(g, k, ijn) * fxn; };
  double duxi = gi(c.dUdxi, 1), duyi = gi(c.dUdxi, 2), duzi = gi(c.dUdxi, 3);
  double dvxi = gi(c.dVdxi, 1), dvyi = gi(c.dVdxi, 2), dvzi = gi(c.dVdxi, 3);
  double dwxi = gi(c.dWdxi, 1), dwyi = gi(c.dWdxi, 2), dwzi = gi(c.dWdxi, 3);
  double fdue = game * ((duxi + duxi) * arx + (duyi + dvxi) * ary + (duzi + dwxi) * arz);
  double fdve = game * ((duyi + dvxi) * arx + (dvyi + dvyi) * ary + (dvzi + dwyi) * arz);
  double fdwe = game * ((duzi + dwxi) * arx + (dwyi + dvzi) * ary + (dwzi + dwzi) * arz);
  double fdui = game * are / dpn * (duxi * xpn + duyi * ypn + duzi * zpn);
  double fdvi = game * are / dpn * (dvxi * xpn + dvyi * ypn + dvzi * zpn);
  double fdwi = game * are / dpn * (dwxi * xpn + dwyi * ypn + dwzi * zpn);
  double fuuds = cp * c.u[ijp] + ce * c.u[ijn];
  double fvuds = cp * c.v[ijp] + ce * c.v[ijn];
  double fwuds = cp * c.w[ijp] + ce * c.w[ijn];
  double ue, ve, we;
  if (flomass >= 0.0) {  // face_value_cds, interpolation.f90:116-157
    ue = c.u[ijp] + (c.u[ijn] - c.u[ijp]) * fxp;
    ve = c.v[ijp] + (c.v[ijn] - c.v[ijp]) * fxp;
    we = c.w[ijp] + (c.w[ijn] - c.w[ijp]) * fxp;
  } else {
    ue = c.u[ijn] + (c.u[ijp] - c.u[ijn]) * fxn;
    ve = c.v[ijn] + (c.v[ijp] - c.v[ijn]) * fxn;
    we = c.w[ijn] + (c.w[ijp] - c.w[ijn]) * fxn;
  }
  double fuhigh = flomass * ue, fvhigh = flomass * ve, fwhigh = flomass * we;
  sup = -gam * (fuhigh - fuuds) + fdue - fdui;
  svp = -gam * (fvhigh - fvuds) + fdve - fdvi;
  swp = -gam * (fwhigh - fwuds) + fdwe - fdwi;
}

// calcuvw, velocity.f90:50-750 without buoyancy or MHD terms, with the
// unsteady terms of :226-290 and periodic pairs (:393-430).  Returns the
// worst csrsolve status.
int calcuvw(Case& c) {
  const int nC = c.numCells;
  std::fill(c.spu.begin(), c.spu.end(), 0.0);
  std::fill(c.spv.begin(), c.spv.end(), 0.0);
  std::fill(c.sp.begin(), c.sp.end(), 0.0);
  updateVelocityAtBoundary(c);
  grad(c, c.u, c.dUdxi);
  grad(c, c.v, c.dVdxi);
  grad(c, c.w, c.dWdxi);
  gradp_and_sources(c, c.p);
  // unsteady term of the cell loop, velocity.f90:226-290
  if (c.tscheme > 0) {
    for (int inp = 1; inp <= nC; ++inp) {
      double apotime = c.den[inp] * c.vol[inp] / c.timestep;
      if (c.tscheme == 1) {
        c.su[inp] = c.su[inp] + apotime * c.uo[inp];
        c.sv[inp] = c.sv[inp] + apotime * c.vo[inp];
        c.sw[inp] = c.sw[inp] + apotime * c.wo[inp];
        c.spu[inp] = c.spu[inp] + apotime;
        c.spv[inp] = c.spv[inp] + apotime;
        c.sp[inp] = c.sp[inp] + apotime;
      } else if (c.tscheme == 2) {
        c.su[inp] = c.su[inp] + apotime * (2 * c.uo[inp] - 0.5 * c.uoo[inp]);
        c.sv[inp] = c.sv[inp] + apotime * (2 * c.vo[inp] - 0.5 * c.voo[inp]);
        c.sw[inp] = c.sw[inp] + apotime * (2 * c.wo[inp] - 0.5 * c.woo[inp]);
        c.spu[inp] = c.spu[inp] + 1.5 * apotime;
        c.spv[inp] = c.spv[inp] + 1.5 * apotime;
        c.sp[inp] = c.sp[inp] + 1.5 * apotime;
      } else {
        c.su[inp] = c.su[inp] + apotime * (3 * c.uo[inp] - 1.5 * c.uoo[inp] + 1. / 3.0 * c.uooo[inp]);
        c.sv[inp] = c.sv[inp] + apotime * (3 * c.vo[inp] - 1.5 * c.voo[inp] + 1. / 3.0 * c.vooo[inp]);
        c.sw[inp] = c.sw[inp] + apotime * (3 * c.wo[inp] - 1.5 * c.woo[inp] + 1. / 3.0 * c.wooo[inp]);
        c.spu[inp] = c.spu[inp] + 11. / 6.0 * apotime;
        c.spv[inp] = c.spv[inp] + 11. / 6.0 * apotime;
        c.sp[inp] = c.sp[inp] + 11. / 6.0 * apotime;
      }
    }
  }
  // inner faces :286-314
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double cap, can, sup, svp, swp;
    facefluxuvw(c, i, ijp, ijn, c.xf[i], c.yf[i], c.zf[i], c.arx[i], c.ary[i], c.arz[i], c.flmass[i], c.facint[i],
                c.gdsU, cap, can, sup, svp, swp);
    c.a[c.ijk[i]] = can;
    c.a[c.jik[i]] = cap;
    c.su[ijp] = c.su[ijp] + sup; c.sv[ijp] = c.sv[ijp] + svp; c.sw[ijp] = c.sw[ijp] + swp;
    c.su[ijn] = c.su[ijn] - sup; c.sv[ijn] = c.sv[ijn] - svp; c.sw[ijn] = c.sw[ijn] - swp;
  }
  // boundaries :326-562
  int iWall = 0, iPer = 0, l = c.numInnerFaces;
  const int inp_stale = nC + 1;  // loop variable 'inp' after the cell loop at :183 (used at :379)
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    int t = c.bctype[ib];
    if (t == BC_INLET || t == BC_OUTLET || t == BC_PRESSURE) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        double cp, cb, sup, svp, swp;
        facefluxuvw_bnd(c, ijp, ijb, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface], c.arz[iface],
                        c.flmass[iface], cp, cb, sup, svp, swp);
        c.spu[ijp] = c.spu[ijp] - cb; c.spv[ijp] = c.spv[ijp] - cb; c.sp[ijp] = c.sp[ijp] - cb;
        c.su[ijp] = c.su[ijp] - cb * c.u[ijb] + sup;
        c.sv[ijp] = c.sv[ijp] - cb * c.v[ijb] + svp;
        c.sw[ijp] = c.sw[ijp] - cb * c.w[ijb] + swp;
      }
    } else if (t == BC_SYMMETRY) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface];
        double are = std::sqrt(c.arx[iface] * c.arx[iface] + c.ary[iface] * c.ary[iface] + c.arz[iface] * c.arz[iface]);
        double arer = 1.0 / are;
        double nxf = c.arx[iface] * arer, nyf = c.ary[iface] * arer, nzf = c.arz[iface] * arer;
        double dpb = (c.xf[iface] - c.xc[ijp]) * nxf + (c.yf[iface] - c.yc[ijp]) * nyf + (c.zf[iface] - c.zc[ijp]) * nzf;
        double cf = 2 * c.vis[inp_stale] * are / dpb;
        c.su[ijp] = c.su[ijp] - cf * nxf * (nyf * c.v[ijp] + nzf * c.w[ijp]);
        c.sv[ijp] = c.sv[ijp] - cf * nyf * (nxf * c.u[ijp] + nzf * c.w[ijp]);
        c.sw[ijp] = c.sw[ijp] - cf * nzf * (nxf * c.u[ijp] + nyf * c.v[ijp]);
        c.spu[ijp] = c.spu[ijp] + cf * (nxf * nxf);
        c.spv[ijp] = c.spv[ijp] + cf * (nyf * nyf);
        c.sp[ijp] = c.sp[ijp] + cf * (nzf * nzf);
      }
    } else if (t == BC_PERIODIC) {  // :393-430
      ++iPer;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface];
        int ijn = c.owner[c.startFaceTwin[iPer] + i];
        double cap, can, sup, svp, swp;
        facefluxuvw_periodic(c, ijp, ijn, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface],
                             c.arz[iface], c.flmass[iface], c.gdsU, cap, can, sup, svp, swp);
        ++l;
        c.a[c.ijk[l]] = can;
        c.a[c.jik[l]] = cap;
        c.su[ijp] = c.su[ijp] + sup; c.sv[ijp] = c.sv[ijp] + svp; c.sw[ijp] = c.sw[ijp] + swp;
        c.su[ijn] = c.su[ijn] - sup; c.sv[ijn] = c.sv[ijn] - svp; c.sw[ijn] = c.sw[ijn] - swp;
      }
    } else if (t == BC_WALL) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        ++iWall;
        double viss = std::max(c.viscos, c.visw[iWall]);
        double are = std::sqrt(c.arx[iface] * c.arx[iface] + c.ary[iface] * c.ary[iface] + c.arz[iface] * c.arz[iface]);
        double arer = 1.0 / are;
        double nxf = c.arx[iface] * arer, nyf = c.ary[iface] * arer, nzf = c.arz[iface] * arer;
        double dpb = (c.xf[iface] - c.xc[ijp]) * nxf + (c.yf[iface] - c.yc[ijp]) * nyf + (c.zf[iface] - c.zc[ijp]) * nzf;
        double vsol = viss * are / dpb;
        double upb = c.u[ijp] - c.u[ijb], vpb = c.v[ijp] - c.v[ijb], wpb = c.w[ijp] - c.w[ijb];
        c.spu[ijp] = c.spu[ijp] + vsol * (1. - nxf * nxf);
        c.spv[ijp] = c.spv[ijp] + vsol * (1. - nyf * nyf);
        c.sp[ijp] = c.sp[ijp] + vsol * (1. - nzf * nzf);
        c.su[ijp] = c.su[ijp] + vsol * (c.u[ijb] * (1. - nxf * nxf) + vpb * nyf * nxf + wpb * nzf * nxf);
        c.sv[ijp] = c.sv[ijp] + vsol * (upb * nxf * nyf + c.v[ijb] * (1. - nyf * nyf) + wpb * nzf * nyf);
        c.sw[ijp] = c.sw[ijp] + vsol * (upb * nxf * nzf + vpb * nyf * nzf + c.w[ijb] * (1. - nzf * nzf));
      }
    }
  }
  // PISO keeps the explicit convection and diffusion terms, :565-570
  if (c.piso) {
    for (int inp = 1; inp <= nC; ++inp) { c.rU[inp] = c.su[inp]; c.rV[inp] = c.sv[inp]; c.rW[inp] = c.sw[inp]; }
  }
  int worst = 0;
  SolveInfo si;
  // U :611-638  (the diagonal slot still holds the previous matrix's value)
  {
    double urfr = 1.0 / c.urfU[0], urfm = 1.0 - c.urfU[0];
    for (int inp = 1; inp <= nC; ++inp) {
      double s = 0.0;
      for (int k = c.ia[inp]; k <= c.ia[inp + 1] - 1; ++k) s += c.a[k];
      double off = s - c.a[c.diag[inp]];
      c.a[c.diag[inp]] = c.spu[inp] - off;
      c.apu[inp] = 1. / (c.a[c.diag[inp]] + kSmall);
      c.a[c.diag[inp]] = c.a[c.diag[inp]] * urfr;
      c.su[inp] = c.su[inp] + urfm * c.a[c.diag[inp]] * c.u[inp];
    }
    int st = csrsolve(c, c.lSolverU, c.u, c.su, c.resor[1], c.maxiterU, c.tolAbsU, c.tolRelU, si);
    worst = std::min(worst, st);
  }
  // V :667-693 and W :722-748
  for (int comp = 2; comp <= 3; ++comp) {
    for (int inp = 1; inp <= nC; ++inp) { c.a[c.diag[inp]] = 0.0; c.su[inp] = 0.0; }
    double urfr = 1.0 / c.urfU[comp - 1], urfm = 1.0 - c.urfU[comp - 1];
    std::vector<double>& spc = (comp == 2) ? c.spv : c.sp;
    std::vector<double>& apc = (comp == 2) ? c.apv : c.apw;
    std::vector<double>& src = (comp == 2) ? c.sv : c.sw;
    std::vector<double>& fld = (comp == 2) ? c.v : c.w;
    for (int inp = 1; inp <= nC; ++inp) {
      double s = 0.0;
      for (int k = c.ia[inp]; k <= c.ia[inp + 1] - 1; ++k) s += c.a[k];
      double off = s - c.a[c.diag[inp]];
      c.a[c.diag[inp]] = spc[inp] - off;
      apc[inp] = 1. / (c.a[c.diag[inp]] + kSmall);
      c.a[c.diag[inp]] = c.a[c.diag[inp]] * urfr;
      c.su[inp] = src[inp] + urfm * c.a[c.diag[inp]] * fld[inp];
    }
    int st = csrsolve(c, c.lSolverU, fld, c.su, c.resor[comp], c.maxiterU, c.tolAbsU, c.tolRelU, si);
    worst = std::min(worst, st);
  }
  return worst;
}

// ------------------------------------------------------- pressure (SIMPLE)
// facefluxmass2, faceflux_mass.f90:175-249 (dPdxi weights as written)
static void facefluxmass2(Case& c, int i, int ijp, int ijn, double arx, double ary, double arz, double lambda,
                          double& cap, double& can, double& fluxmass) {
  double fxn = lambda, fxp = 1.0 - lambda;
  double xpn = c.xc[ijn] - c.xc[ijp], ypn = c.yc[ijn] - c.yc[ijp], zpn = c.zc[ijn] - c.zc[ijp];
  double dene = c.den[ijp] * fxp + c.den[ijn] * fxn;
  double Kj = c.vol[ijp] * c.apu[ijp] * fxp + c.vol[ijn] * c.apu[ijn] * fxn;
  cap = -dene * Kj * c.Df[i];
  can = cap;
  double ui = c.u[ijp] + (c.u[ijn] - c.u[ijp]) * lambda;
  double vi = c.v[ijp] + (c.v[ijn] - c.v[ijp]) * lambda;
  double wi = c.w[ijp] + (c.w[ijn] - c.w[ijp]) * lambda;
  double dpxi = (G(c.dPdxi, 1, ijn) * fxp + G(c.dPdxi, 1, ijp) * fxn) * xpn;
  double dpyi = (G(c.dPdxi, 2, ijn) * fxp + G(c.dPdxi, 2, ijp) * fxn) * ypn;
  double dpzi = (G(c.dPdxi, 3, ijn) * fxp + G(c.dPdxi, 3, ijp) * fxn) * zpn;
  fluxmass = dene * (ui * arx + vi * ary + wi * arz) + cap * (c.p[ijn] - c.p[ijp] - dpxi - dpyi - dpzi);
}

// fluxmc2, faceflux_mass.f90:650-696
static void fluxmc2(Case& c, int ijp, int ijn, double sx, double sy, double sz, double& fmc) {
  double xpn = c.xc[ijn] - c.xc[ijp], ypn = c.yc[ijn] - c.yc[ijp], zpn = c.zc[ijn] - c.zc[ijp];
  double s2 = sx * sx + sy * sy + sz * sz;
  double dn = xpn * sx + ypn * sy + zpn * sz;
  double rapr = -0.5 * (c.apu[ijp] * c.den[ijp] + c.apu[ijn] * c.den[ijn]);
  double dpx = 0.5 * (G(c.dPdxi, 1, ijn) + G(c.dPdxi, 1, ijp));
  double dpy = 0.5 * (G(c.dPdxi, 2, ijn) + G(c.dPdxi, 2, ijp));
  double dpz = 0.5 * (G(c.dPdxi, 3, ijn) + G(c.dPdxi, 3, ijp));
  fmc = rapr * ((dn * sx - xpn * s2) * dpx + (dn * sy - ypn * s2) * dpy + (dn * sz - zpn * s2) * dpz);
}

// adjustMassFlow, faceflux_mass.f90:833-916
static void adjustMassFlow(Case& c) {
  double flowo = 0.0;
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] != BC_OUTLET) continue;
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
      c.u[ijb] = c.u[ijp]; c.v[ijb] = c.v[ijp]; c.w[ijb] = c.w[ijp];
      c.flmass[iface] = c.den[ijp] * (c.u[ijb] * c.arx[iface] + c.v[ijb] * c.ary[iface] + c.w[ijb] * c.arz[iface]);
      flowo = flowo + c.flmass[iface];
    }
  }
  double fac = c.flomas / (flowo + kSmall);
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] != BC_OUTLET) continue;
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      int iface = c.startFace[ib] + i, ijb = c.iBndValueStart[ib] + i;
      c.flmass[iface] = c.flmass[iface] * fac;
      c.u[ijb] = c.u[ijb] * fac; c.v[ijb] = c.v[ijb] * fac; c.w[ijb] = c.w[ijb] * fac;
    }
  }
}

// continuityErrors, continuityErrors.f90:1-77 (flmass indexed by the owner
// cell as written at :26-27)
void continuityErrors(Case& c) {
  const int nC = c.numCells;
  std::fill(c.su.begin(), c.su.end(), 0.0);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    c.su[ijp] = c.su[ijp] - c.flmass[ijp];
    c.su[ijn] = c.su[ijn] + c.flmass[ijp];
  }
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] != BC_INLET && c.bctype[ib] != BC_OUTLET) continue;
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      int iface = c.startFace[ib] + i, ijp = c.owner[iface];
      c.su[ijp] = c.su[ijp] - c.flmass[iface];
    }
  }
  double wavg = 0.0, sumvol = 0.0;
  for (int inp = 1; inp <= nC; ++inp) {
    wavg = wavg + (c.vol[inp] * std::fabs(c.su[inp] * c.apu[inp]));
    sumvol = sumvol + c.vol[inp];
  }
  wavg = wavg / sumvol;
  double glob = 0.0;
  for (int inp = 1; inp <= nC; ++inp) glob += c.su[inp];
  c.cumulativeContErr = c.cumulativeContErr + glob;
  std::fill(c.su.begin(), c.su.end(), 0.0);
  c.resor[4] = wavg;
}

// facefluxmassPressBnd, faceflux_mass.f90:765-830: mass flux and boundary
// velocity through a pressure face, and its coefficient of the
// pressure-correction equation
static void facefluxmassPressBnd(Case& c, int ijp, int ijb, double xf, double yf, double zf, double arx, double ary,
                                 double arz, double& cap, double& fluxmass) {
  double xpn = xf - c.xc[ijp], ypn = yf - c.yc[ijp], zpn = zf - c.zc[ijp];
  double capp = c.vol[ijp] * c.apu[ijp] / (arx * xpn + ary * ypn + arz * zpn);
  double dpcor = c.p[ijb] - c.p[ijp] -
                 (G(c.dPdxi, 1, ijp) * xpn + G(c.dPdxi, 2, ijp) * ypn + G(c.dPdxi, 3, ijp) * zpn);
  c.u[ijb] = c.u[ijp] - arx * capp * dpcor;
  c.v[ijb] = c.v[ijp] - ary * capp * dpcor;
  c.w[ijb] = c.w[ijp] - arz * capp * dpcor;
  fluxmass = c.den[ijp] * (c.u[ijb] * arx + c.v[ijb] * ary + c.w[ijb] * arz);
  cap = -c.den[ijp] * (arx * arx + ary * ary + arz * arz) * capp;
}

// facefluxmassCorrPressBnd, faceflux_mass.f90:699-762: p' is zero at a
// pressure face, so the correction is driven by -pp(ijp)
static void facefluxmassCorrPressBnd(Case& c, int ijp, int ijb, double xf, double yf, double zf, double arx,
                                     double ary, double arz, double& fluxmass) {
  double xpn = xf - c.xc[ijp], ypn = yf - c.yc[ijp], zpn = zf - c.zc[ijp];
  double cap = c.vol[ijp] * c.apu[ijp] / (arx * xpn + ary * ypn + arz * zpn);
  double dpcor = -c.pp[ijp];
  c.u[ijb] = c.u[ijb] - arx * cap * dpcor;
  c.v[ijb] = c.v[ijb] - ary * cap * dpcor;
  c.w[ijb] = c.w[ijb] - arz * cap * dpcor;
  fluxmass = fluxmass - c.den[ijp] * (arx * arx + ary * ary + arz * arz) * cap * dpcor;
}

// facefluxmass2_periodic, faceflux_mass.f90:313-384: the mass flux through a
// periodic face between ijp (owner of the face) and ijn (owner of its twin),
// with the face's own centre standing in for the twin side (xpn = 2 (xf -
// xc(ijp))).  Df is indexed by the face's position i within its patch, as
// the reference writes it.
static void facefluxmass2_periodic(Case& c, int i, int ijp, int ijn, double xf, double yf, double zf, double arx,
                                   double ary, double arz, double lambda, double& cap, double& can,
                                   double& fluxmass) {
  double fxn = lambda, fxp = 1.0 - lambda;
  double xpn = 2 * (xf - c.xc[ijp]), ypn = 2 * (yf - c.yc[ijp]), zpn = 2 * (zf - c.zc[ijp]);
  double dene = c.den[ijp] * fxp + c.den[ijn] * fxn;
  double Kj = c.vol[ijp] * c.apu[ijp] * fxp + c.vol[ijn] * c.apu[ijn] * fxn;
  cap = -dene * Kj * c.Df[i];
  can = cap;
  Kj = (c.apu[ijp] + c.apu[ijn] + kSmall);
  double ui = (c.u[ijp] * c.apu[ijn] + c.u[ijn] * c.apu[ijp]) / Kj;
  double vi = (c.v[ijp] * c.apv[ijn] + c.v[ijn] * c.apv[ijp]) / Kj;
  double wi = (c.w[ijp] * c.apw[ijn] + c.w[ijn] * c.apw[ijp]) / Kj;
  double dpxi = (G(c.dPdxi, 1, ijn) * fxp + G(c.dPdxi, 1, ijp) * fxn) * xpn;
  double dpyi = (G(c.dPdxi, 2, ijn) * fxp + G(c.dPdxi, 2, ijp) * fxn) * ypn;
  double dpzi = (G(c.dPdxi, 3, ijn) * fxp + G(c.dPdxi, 3, ijp) * fxn) * zpn;
  fluxmass = dene * (ui * arx + vi * ary + wi * arz) + cap * (c.p[ijn] - c.p[ijp] - dpxi - dpyi - dpzi);
}

// the periodic branch of the boundary loops of calcp_simple (:185-225) and
// calcp_piso (:248-289): mass flux, both off-diagonal slots, both diagonals
// and both sources of every pair; l runs on from numInnerFaces
static void periodic_pressure_faces(Case& c, int ib, int& iPer, int& l) {
  ++iPer;
  for (int i = 1; i <= c.nfaces[ib]; ++i) {
    int iface = c.startFace[ib] + i, ijp = c.owner[iface];
    int iftwin = c.startFaceTwin[iPer] + i, ijn = c.owner[iftwin];
    double cap, can;
    facefluxmass2_periodic(c, i, ijp, ijn, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface],
                           c.arz[iface], 0.5, cap, can, c.flmass[iface]);
    ++l;
    c.a[c.ijk[l]] = cap;
    c.a[c.jik[l]] = cap;
    c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - cap;
    c.a[c.diag[ijn]] = c.a[c.diag[ijn]] - cap;
    c.su[ijp] = c.su[ijp] - c.flmass[iface];
    c.su[ijn] = c.su[ijn] + c.flmass[iface];
  }
}

// flux correction through the periodic pairs after a pressure solve
// (calcp_simple.f90:322-342, calcp_piso.f90:437-456, with phi = pp or p):
// the twin face takes the same mass flux
static void periodic_flux_correct(Case& c, int ib, int& iPer, int& l, const std::vector<double>& phi) {
  ++iPer;
  for (int i = 1; i <= c.nfaces[ib]; ++i) {
    int iface = c.startFace[ib] + i, ijp = c.owner[iface];
    int iftwin = c.startFaceTwin[iPer] + i, ijn = c.owner[iftwin];
    ++l;
    c.flmass[iface] = c.flmass[iface] + c.a[c.ijk[l]] * (phi[ijn] - phi[ijp]);
    c.flmass[iftwin] = c.flmass[iface];
  }
}

// calcp_simple, calcp_simple.f90:1-470 for incompressible SIMPLE, with
// pressure boundaries (:162-183, :344-356, :363-369) and periodic pairs
// (:185-225, :322-342).
int calcp_simple(Case& c) {
  const int nC = c.numCells;
  std::fill(c.a.begin(), c.a.end(), 0.0);
  std::fill(c.su.begin(), c.su.end(), 0.0);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double cap, can;
    facefluxmass2(c, i, ijp, ijn, c.arx[i], c.ary[i], c.arz[i], c.facint[i], cap, can, c.flmass[i]);
    c.a[c.ijk[i]] = cap;
    c.a[c.jik[i]] = cap;
    c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - cap;
    c.a[c.diag[ijn]] = c.a[c.diag[ijn]] - cap;
    c.su[ijp] = c.su[ijp] - c.flmass[i];
    c.su[ijn] = c.su[ijn] + c.flmass[i];
  }
  adjustMassFlow(c);
  bool have_pressure = false;
  int iPer = 0, l = c.numInnerFaces;
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] == BC_PERIODIC) {
      periodic_pressure_faces(c, ib, iPer, l);
    } else if (c.bctype[ib] == BC_INLET || c.bctype[ib] == BC_OUTLET) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface];
        c.su[ijp] = c.su[ijp] - c.flmass[iface];
      }
    } else if (c.bctype[ib] == BC_PRESSURE) {
      have_pressure = true;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        double cap;
        facefluxmassPressBnd(c, ijp, ijb, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface],
                             c.arz[iface], cap, c.flmass[iface]);
        c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - cap;
        c.su[ijp] = c.su[ijp] - c.flmass[iface];
        c.pp[ijb] = 0.0;
      }
    }
  }
  int worst = 0;
  for (int ipcorr = 1; ipcorr <= c.npcor; ++ipcorr) {
    SolveInfo si;
    int st = csrsolve(c, c.lSolverP, c.pp, c.su, c.resor[4], c.maxiterP, c.tolAbsP, c.tolRelP, si);
    worst = std::min(worst, st);
    for (int iface = 1; iface <= c.numInnerFaces; ++iface) {
      int ijp = c.owner[iface], ijn = c.neighbour[iface];
      c.flmass[iface] = c.flmass[iface] + c.a[c.ijk[iface]] * (c.pp[ijn] - c.pp[ijp]);
    }
    iPer = 0;
    l = c.numInnerFaces;
    for (int ib = 1; ib <= c.numBoundaries; ++ib) {
      if (c.bctype[ib] == BC_PERIODIC) {
        periodic_flux_correct(c, ib, iPer, l, c.pp);
        continue;
      }
      if (c.bctype[ib] != BC_PRESSURE) continue;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        facefluxmassCorrPressBnd(c, ijp, ijb, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface],
                                 c.arz[iface], c.flmass[iface]);
      }
    }
    // with a pressure boundary the reference p' is zero (:363-369)
    double ppref = have_pressure ? 0.0 : c.pp[c.pRefCell];
    gradp_and_sources(c, c.pp);
    for (int i = 1; i <= nC; ++i) c.u[i] = c.u[i] + c.su[i] * c.apu[i];
    for (int i = 1; i <= nC; ++i) c.v[i] = c.v[i] + c.sv[i] * c.apv[i];
    for (int i = 1; i <= nC; ++i) c.w[i] = c.w[i] + c.sw[i] * c.apw[i];
    for (int i = 1; i <= nC; ++i) c.p[i] = c.p[i] + c.urfP * (c.pp[i] - ppref);
    updateVelocityAtBoundary(c);
    if (ipcorr != c.npcor) {
      std::fill(c.su.begin(), c.su.end(), 0.0);
      for (int i = 1; i <= c.numInnerFaces; ++i) {
        int ijp = c.owner[i], ijn = c.neighbour[i];
        double fmcor;
        fluxmc2(c, ijp, ijn, c.arx[i], c.ary[i], c.arz[i], fmcor);
        c.flmass[i] = c.flmass[i] + fmcor;
        c.su[ijp] = c.su[ijp] - fmcor;
        c.su[ijn] = c.su[ijn] + fmcor;
      }
    }
  }
  continuityErrors(c);
  return worst;
}

// ---------------------------------------------------------------- PISO
// time_shift, time_shift.f90 (velocity levels; the PISO extrapolation
// levels of bdf2/bdf3 are not shifted there, and bdf2/bdf3 PISO is rejected)
void time_shift(Case& c) {
  if (c.tscheme == 3) { c.uooo = c.uoo; c.vooo = c.voo; c.wooo = c.woo; }
  if (c.tscheme == 3 || c.tscheme == 2) { c.uoo = c.uo; c.voo = c.vo; c.woo = c.wo; }
  c.uo = c.u; c.vo = c.v; c.wo = c.w;
}

// facefluxmass_piso, faceflux_mass.f90:389-559
static void facefluxmass_piso(Case& c, int i, int ijp, int ijn, double arx, double ary, double arz, double lambda,
                              double& cap, double& can, double& flmass) {
  double fxn = lambda, fxp = 1.0 - lambda;
  double dene = c.den[ijp] * fxp + c.den[ijn] * fxn;
  double Kj = c.vol[ijp] * c.apu[ijp] * fxp + c.vol[ijn] * c.apu[ijn] * fxn;
  cap = -dene * Kj * c.Df[i];
  can = cap;
  double ui = c.u[ijp] + (c.u[ijn] - c.u[ijp]) * lambda;
  double vi = c.v[ijp] + (c.v[ijn] - c.v[ijp]) * lambda;
  double wi = c.w[ijp] + (c.w[ijn] - c.w[ijp]) * lambda;
  flmass = dene * (ui * arx + vi * ary + wi * arz);
}

// fluxmc, faceflux_mass.f90:564-647 (the projections xpp, xep as written)
static void fluxmc(Case& c, int ijp, int ijn, double xf, double yf, double zf, double arx, double ary, double arz,
                   double lambda, double& fmcor) {
  double fxn = lambda, fxp = 1.0 - lambda;
  double xpn = c.xc[ijn] - c.xc[ijp], ypn = c.yc[ijn] - c.yc[ijp], zpn = c.zc[ijn] - c.zc[ijp];
  double are = std::sqrt(arx * arx + ary * ary + arz * arz);
  double nxx = arx / are, nyy = ary / are, nzz = arz / are;
  double xpp = xf - (xf - c.xc[ijp]) * nxx, ypp = yf - (yf - c.yc[ijp]) * nyy, zpp = zf - (zf - c.zc[ijp]) * nzz;
  double xep = xf - (xf - c.xc[ijn]) * nxx, yep = yf - (yf - c.yc[ijn]) * nyy, zep = zf - (zf - c.zc[ijn]) * nzz;
  xpp = xpp - c.xc[ijp]; ypp = ypp - c.yc[ijp]; zpp = zpp - c.zc[ijp];
  xep = xep - c.xc[ijn]; yep = yep - c.yc[ijn]; zep = zep - c.zc[ijn];
  double rapr = -((c.apu[ijp] * c.den[ijp] * c.vol[ijp] * fxp + c.apu[ijn] * c.den[ijn] * c.vol[ijn] * fxn) * are /
                  (xpn * nxx + ypn * nyy + zpn * nzz));
  fmcor = rapr * ((G(c.dPdxi, 1, ijn) * xep - G(c.dPdxi, 1, ijp) * xpp) +
                  (G(c.dPdxi, 2, ijn) * yep - G(c.dPdxi, 2, ijp) * ypp) +
                  (G(c.dPdxi, 3, ijn) * zep - G(c.dPdxi, 3, ijp) * zpp));
}

// calcp_piso, calcp_piso.f90:86-489, incompressible, with periodic pairs
// (:248-289, :437-456) and without pressure boundaries; nipgrad = 2
// (parameters.f90:62)
int calcp_piso(Case& c) {
  const int nC = c.numCells;
  c.h = c.a;
  int worst = 0;
  for (int icorr = 1; icorr <= c.ncorr; ++icorr) {
    for (int i = 1; i <= nC; ++i) { c.su[i] = c.rU[i]; c.sv[i] = c.rV[i]; c.sw[i] = c.rW[i]; }
    for (int i = 1; i <= c.numInnerFaces; ++i) {
      int ijp = c.owner[i], ijn = c.neighbour[i];
      int k = c.ijk[i];
      c.su[ijp] = c.su[ijp] - c.h[k] * c.u[ijn];
      c.sv[ijp] = c.sv[ijp] - c.h[k] * c.v[ijn];
      c.sw[ijp] = c.sw[ijp] - c.h[k] * c.w[ijn];
      k = c.jik[i];
      c.su[ijn] = c.su[ijn] - c.h[k] * c.u[ijp];
      c.sv[ijn] = c.sv[ijn] - c.h[k] * c.v[ijp];
      c.sw[ijn] = c.sw[ijn] - c.h[k] * c.w[ijp];
    }
    for (int i = 1; i <= nC; ++i) {
      c.u[i] = c.apu[i] * c.su[i];
      c.v[i] = c.apv[i] * c.sv[i];
      c.w[i] = c.apw[i] * c.sw[i];
    }
    std::fill(c.a.begin(), c.a.end(), 0.0);
    std::fill(c.su.begin(), c.su.end(), 0.0);
    for (int i = 1; i <= c.numInnerFaces; ++i) {
      int ijp = c.owner[i], ijn = c.neighbour[i];
      double cap, can;
      facefluxmass_piso(c, i, ijp, ijn, c.arx[i], c.ary[i], c.arz[i], c.facint[i], cap, can, c.flmass[i]);
      c.a[c.ijk[i]] = can;
      c.a[c.jik[i]] = cap;
      c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - can;
      c.a[c.diag[ijn]] = c.a[c.diag[ijn]] - cap;
      c.su[ijp] = c.su[ijp] - c.flmass[i];
      c.su[ijn] = c.su[ijn] + c.flmass[i];
    }
    adjustMassFlow(c);
    int iPer = 0, l = c.numInnerFaces;
    for (int ib = 1; ib <= c.numBoundaries; ++ib) {
      if (c.bctype[ib] == BC_PERIODIC) {
        periodic_pressure_faces(c, ib, iPer, l);
        continue;
      }
      if (c.bctype[ib] != BC_INLET && c.bctype[ib] != BC_OUTLET) continue;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface];
        c.su[ijp] = c.su[ijp] - c.flmass[iface];
      }
    }
    for (int ipcorr = 1; ipcorr <= c.npcor; ++ipcorr) {
      SolveInfo si;
      int st = csrsolve(c, c.lSolverP, c.pp, c.su, c.resor[4], c.maxiterP, c.tolAbsP, c.tolRelP, si);
      worst = std::min(worst, st);
      double pavg = 0.0;
      for (int i = 1; i <= nC; ++i) pavg = pavg + c.pp[i];
      pavg = pavg / (double)nC;
      for (int i = 1; i <= nC; ++i) c.p[i] = (1.0 - c.urfP) * c.p[i] + c.urfP * (c.pp[i] - pavg);
      for (int istage = 1; istage <= 2; ++istage) {
        bpres(c, c.p, istage);
        grad_gauss(c, c.p, c.dPdxi);
      }
      if (ipcorr != c.npcor) {
        for (int i = 1; i <= c.numInnerFaces; ++i) {
          int ijp = c.owner[i], ijn = c.neighbour[i];
          double fmcor;
          fluxmc(c, ijp, ijn, c.xf[i], c.yf[i], c.zf[i], c.arx[i], c.ary[i], c.arz[i], c.facint[i], fmcor);
          c.su[ijp] = c.su[ijp] - fmcor;
          c.su[ijn] = c.su[ijn] + fmcor;
        }
      } else {
        for (int iface = 1; iface <= c.numInnerFaces; ++iface) {
          int ijp = c.owner[iface], ijn = c.neighbour[iface];
          c.flmass[iface] = c.flmass[iface] + c.a[c.ijk[iface]] * (c.p[ijn] - c.p[ijp]);
        }
        continuityErrors(c);
      }
    }
    gradp_and_sources(c, c.p);
    for (int i = 1; i <= nC; ++i) {
      c.u[i] = c.u[i] + c.su[i] * c.apu[i];
      c.v[i] = c.v[i] + c.sv[i] * c.apv[i];
      c.w[i] = c.w[i] + c.sw[i] * c.apw[i];
    }
    // periodic pairs take the flux correction of the last p (:437-456)
    iPer = 0;
    l = c.numInnerFaces;
    for (int ib = 1; ib <= c.numBoundaries; ++ib)
      if (c.bctype[ib] == BC_PERIODIC) periodic_flux_correct(c, ib, iPer, l, c.p);
    updateVelocityAtBoundary(c);
  }
  return worst;
}

// ------------------------------------------------------ scalar transport
// facefluxsc (inner face), scalar_fluxes.f90:32-141
void facefluxsc(Case& c, int i, int ijp, int ijn, double xf, double yf, double zf, double arx, double ary,
                       double arz, double fm, double lambda, double gam, int scheme, const std::vector<double>& fi,
                       std::vector<double>& dfidxi, double dcoef, double& cap, double& can, double& suadd) {
  double fxn = lambda, fxp = 1.0 - lambda;
  double xpn = c.xc[ijn] - c.xc[ijp], ypn = c.yc[ijn] - c.yc[ijp], zpn = c.zc[ijn] - c.zc[ijp];
  double de = dcoef * c.Df[i];
  double ce = std::min(fm, 0.0), cp = std::max(fm, 0.0);
  can = -de + ce;
  cap = -de - cp;
  double dfixi = G(dfidxi, 1, ijp) * fxp + G(dfidxi, 1, ijn) * fxn;
  double dfiyi = G(dfidxi, 2, ijp) * fxp + G(dfidxi, 2, ijn) * fxn;
  double dfizi = G(dfidxi, 3, ijp) * fxp + G(dfidxi, 3, ijn) * fxn;
  dfixi = dfixi * (arx - c.Df[i] * xpn);
  dfiyi = dfiyi * (ary - c.Df[i] * ypn);
  dfizi = dfizi * (arz - c.Df[i] * zpn);
  double fdfie = dcoef * (dfixi + dfiyi + dfizi);
  double fii;
  if (fm >= 0.0) fii = face_value(c, ijp, ijn, xf, yf, zf, fxp, fi, dfidxi, scheme);
  else fii = face_value(c, ijn, ijp, xf, yf, zf, fxn, fi, dfidxi, scheme);
  double fcfie = fm * fii;
  double fcfii = ce * fi[ijn] + cp * fi[ijp];
  fcfie = gam * (fcfie - fcfii);
  suadd = -fcfie + fdfie;
}

// facefluxsc_periodic, scalar_fluxes.f90:147-251: a periodic face between
// ijp and the twin's owner ijn, central weights 1/2, the distance vector
// 2 (xf - xc(ijp)), Df indexed by the face's position i within its patch (as
// the reference writes it), cds face value
void facefluxsc_periodic(Case& c, int i, int ijp, int ijn, double xf, double yf, double zf, double arx,
                                double ary, double arz, double fm, double gam, const std::vector<double>& fi,
                                std::vector<double>& dfidxi, double dcoef, double& cap, double& can,
                                double& suadd) {
  const double fxn = 0.5, fxp = fxn;
  double xpn = 2 * (xf - c.xc[ijp]), ypn = 2 * (yf - c.yc[ijp]), zpn = 2 * (zf - c.zc[ijp]);
  double de = dcoef * c.Df[i];
  double ce = std::min(fm, 0.0), cp = std::max(fm, 0.0);
  can = -de + ce;
  cap = -de - cp;
  double dfixi = G(dfidxi, 1, ijp) * fxp + G(dfidxi, 1, ijn) * fxn;
  double dfiyi = G(dfidxi, 2, ijp) * fxp + G(dfidxi, 2, ijn) * fxn;
  double dfizi = G(dfidxi, 3, ijp) * fxp + G(dfidxi, 3, ijn) * fxn;
  dfixi = dfixi * (arx - c.Df[i] * xpn);
  dfiyi = dfiyi * (ary - c.Df[i] * ypn);
  dfizi = dfizi * (arz - c.Df[i] * zpn);
  double fdfie = dcoef * (dfixi + dfiyi + dfizi);
  double fii;
  if (fm >= 0.0) fii = fi[ijp] + (fi[ijn] - fi[ijp]) * fxp;  // face_value_cds, interpolation.f90:116-157
  else fii = fi[ijn] + (fi[ijp] - fi[ijn]) * fxn;
  double fcfie = fm * fii;
  double fcfii = ce * fi[ijn] + cp * fi[ijp];
  fcfie = gam * (fcfie - fcfii);
  suadd = -fcfie + fdfie;
}

// updateBoundary, updateBoundary.f90:1-77: outlet, symmetry, pressure and
// empty faces take the owner's value; a periodic face and its twin take the
// mean of the pair's two cells (in patch order, so a twin patch listed after
// its periodic patch ends with the owner's value)
void updateBoundary(Case& c, std::vector<double>& phi) {
  int iPer = 0;
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    int t = c.bctype[ib];
    if (t == BC_OUTLET || t == BC_SYMMETRY || t == BC_PRESSURE || t == BC_EMPTY) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        phi[ijb] = phi[ijp];
      }
    } else if (t == BC_PERIODIC) {
      ++iPer;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        int ijn = c.owner[c.startFaceTwin[iPer] + i];
        phi[ijb] = 0.5 * (phi[ijp] + phi[ijn]);
        int ijbt = c.numCells + (c.startFaceTwin[iPer] - c.numInnerFaces) + i;
        phi[ijbt] = phi[ijb];
      }
    }
  }
}

// facefluxsc_boundary, scalar_fluxes.f90:256-337
void facefluxsc_bnd(Case& c, int ijp, double xf, double yf, double zf, double arx, double ary, double arz,
                           double fm, std::vector<double>& dfidxi, double dcoef, double& cap, double& can,
                           double& suadd) {
  double xpn = xf - c.xc[ijp], ypn = yf - c.yc[ijp], zpn = zf - c.zc[ijp];
  double Dfi = (arx * arx + ary * ary + arz * arz) / (xpn * arx + ypn * ary + zpn * arz);
  double de = dcoef * Dfi;
  double ce = std::min(fm, 0.0), cp = std::max(fm, 0.0);
  can = -de + ce;
  cap = -de - cp;
  double dfixi = G(dfidxi, 1, ijp), dfiyi = G(dfidxi, 2, ijp), dfizi = G(dfidxi, 3, ijp);
  dfixi = dfixi * (arx - Dfi * xpn);
  dfiyi = dfiyi * (ary - Dfi * ypn);
  dfizi = dfizi * (arz - Dfi * zpn);
  suadd = dcoef * (dfixi + dfiyi + dfizi);
}

// calculate_temperature, temperature.f90:35-385, steady and laminar-or-given
// vis (no transient, turbulent heat-flux or Crank-Nicolson terms), with
// periodic pairs (:262-313).
// Isothermal walls are bcDFracT == 1, adiabatic walls bcDFracT == 0; the wall
// counter iWall advances only on isothermal walls (:203), so srdw is indexed
// as the reference indexes it.  Adiabatic walls copy T(ijp) to T(ijb) during
// the assembly (:214-225).
int calculate_temperature(Case& c, bool solve) {
  const int nC = c.numCells;
  const double gam = c.gdsT;
  const double prl = 1.0 / c.pranl;
  const double prtr = 1. / c.sigt;
  grad(c, c.T, c.dTdxi);
  std::fill(c.a.begin(), c.a.end(), 0.0);
  std::fill(c.su.begin(), c.su.end(), 0.0);
  std::fill(c.sp.begin(), c.sp.end(), 0.0);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    double dcoef = c.viscos * prl + ((c.vis[ijp] + (c.vis[ijn] - c.vis[ijp]) * c.facint[i]) - c.viscos) * prtr;
    double cap, can, suadd;
    facefluxsc(c, i, ijp, ijn, c.xf[i], c.yf[i], c.zf[i], c.arx[i], c.ary[i], c.arz[i], c.flmass[i], c.facint[i],
               gam, c.cSchemeT, c.T, c.dTdxi, dcoef, cap, can, suadd);
    c.a[c.ijk[i]] = can;
    c.a[c.jik[i]] = cap;
    c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - can;
    c.a[c.diag[ijn]] = c.a[c.diag[ijn]] - cap;
    c.su[ijp] = c.su[ijp] + suadd;
    c.su[ijn] = c.su[ijn] - suadd;
  }
  int iWall = 0, iPer = 0, l = c.numInnerFaces;
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    int t = c.bctype[ib];
    if (t == BC_INLET || t == BC_OUTLET || t == BC_PRESSURE) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        double dcoef = c.viscos * prl + (c.vis[ijp] - c.viscos) / c.sigt;
        double cap, can, suadd;
        facefluxsc_bnd(c, ijp, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface], c.arz[iface],
                       c.flmass[iface], c.dTdxi, dcoef, cap, can, suadd);
        c.sp[ijp] = c.sp[ijp] - can;
        c.su[ijp] = c.su[ijp] - can * c.T[ijb] + suadd;
      }
    } else if (t == BC_WALL && c.bcDFracT[ib] == 1.0) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        ++iWall;
        double dcoef = c.viscos / c.pranl + (c.vis[ijp] - c.viscos) / c.sigt;
        dcoef = dcoef * c.srdw[iWall];
        c.sp[ijp] = c.sp[ijp] + dcoef;
        c.su[ijp] = c.su[ijp] + dcoef * c.T[ijb];
        (void)iface;
      }
    } else if (t == BC_WALL && c.bcDFracT[ib] == 0.0) {
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface], ijb = c.iBndValueStart[ib] + i;
        c.T[ijb] = c.T[ijp];
      }
    } else if (t == BC_PERIODIC) {  // temperature.f90:262-313
      ++iPer;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int iface = c.startFace[ib] + i, ijp = c.owner[iface];
        int ijn = c.owner[c.startFaceTwin[iPer] + i];
        // facint of the face's position i within its patch, as written there
        double dcoef = c.viscos * prl + ((c.vis[ijp] + (c.vis[ijn] - c.vis[ijp]) * c.facint[i]) - c.viscos) * prtr;
        double cap, can, suadd;
        facefluxsc_periodic(c, i, ijp, ijn, c.xf[iface], c.yf[iface], c.zf[iface], c.arx[iface], c.ary[iface],
                            c.arz[iface], c.flmass[iface], gam, c.T, c.dTdxi, dcoef, cap, can, suadd);
        ++l;
        c.a[c.ijk[l]] = can;
        c.a[c.jik[l]] = cap;
        c.a[c.diag[ijp]] = c.a[c.diag[ijp]] - can;
        c.a[c.diag[ijn]] = c.a[c.diag[ijn]] - cap;
        c.su[ijp] = c.su[ijp] + suadd;
        c.su[ijn] = c.su[ijn] - suadd;
      }
    }
  }
  const double urfr = 1.0 / c.urfT, urfm = 1.0 - c.urfT;
  for (int inp = 1; inp <= nC; ++inp) {
    double s = 0.0;
    for (int k = c.ia[inp]; k <= c.ia[inp + 1] - 1; ++k) s += c.a[k];
    double off = s - c.a[c.diag[inp]];
    c.a[c.diag[inp]] = c.sp[inp] - off;
    c.a[c.diag[inp]] = c.a[c.diag[inp]] * urfr;
    c.su[inp] = c.su[inp] + urfm * c.a[c.diag[inp]] * c.T[inp];
  }
  if (!solve) return 0;
  SolveInfo si;
  int st = csrsolve(c, c.lSolverT, c.T, c.su, c.resor[7], c.maxiterT, c.tolAbsT, c.tolRelT, si);
  updateBoundary(c, c.T);
  double fimin = c.T[1];
  for (int i = 2; i <= nC; ++i) fimin = std::min(fimin, c.T[i]);
  if (fimin < 0.0)
    for (int i = 1; i <= nC; ++i) c.T[i] = std::max(c.T[i], kSmall);
  return st;
}

// ---------------------------------------------- convection-diffusion adjoint
void cd_assemble(Case& c, const std::vector<double>& gamma, const std::vector<double>& source) {
  const int nC = c.numCells;
  std::fill(c.a.begin(), c.a.end(), 0.0);
  std::fill(c.su.begin(), c.su.end(), 0.0);
  std::fill(c.sp.begin(), c.sp.end(), 0.0);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    const int ijp = c.owner[i], ijn = c.neighbour[i];
    const double gf = gamma[ijp] * (1.0 - c.facint[i]) + gamma[ijn] * c.facint[i];
    const double de = gf * c.Df[i];
    const double fm = c.flmass[i];
    c.a[c.ijk[i]] = -de + std::min(fm, 0.0);
    c.a[c.jik[i]] = -de - std::max(fm, 0.0);
  }
  for (int ib = 1; ib <= c.numBoundaries; ++ib)
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      const int iface = c.startFace[ib] + i, ijp = c.owner[iface];
      const double xpn = c.xf[iface] - c.xc[ijp], ypn = c.yf[iface] - c.yc[ijp], zpn = c.zf[iface] - c.zc[ijp];
      const double arx = c.arx[iface], ary = c.ary[iface], arz = c.arz[iface];
      const double dfi = (arx * arx + ary * ary + arz * arz) / (xpn * arx + ypn * ary + zpn * arz);
      c.sp[ijp] = c.sp[ijp] + gamma[ijp] * dfi;
    }
  for (int inp = 1; inp <= nC; ++inp) {
    double s = 0.0;
    for (int k = c.ia[inp]; k <= c.ia[inp + 1] - 1; ++k) s += c.a[k];
    const double off = s - c.a[c.diag[inp]];
    c.a[c.diag[inp]] = c.sp[inp] - off;
    c.su[inp] = source[inp] * c.vol[inp];
  }
}

void cd_gradient(Case& c, const std::vector<double>& phi, const std::vector<double>& lambda, std::vector<double>& out) {
  const int nC = c.numCells;
  out.assign(nC + 1, 0.0);
  // face order per cell, as the device gathers it: inner faces ascending,
  // then boundary faces ascending
  std::vector<double> sf(c.numInnerFaces + 1);
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    const int ijp = c.owner[i], ijn = c.neighbour[i];
    sf[i] = (lambda[ijp] - lambda[ijn]) * (phi[ijp] - phi[ijn]) * c.Df[i];
  }
  for (int i = 1; i <= c.numInnerFaces; ++i) {
    const int ijp = c.owner[i], ijn = c.neighbour[i];
    out[ijp] = out[ijp] - sf[i] * (1.0 - c.facint[i]);
    out[ijn] = out[ijn] - sf[i] * c.facint[i];
  }
  for (int ib = 1; ib <= c.numBoundaries; ++ib)
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      const int iface = c.startFace[ib] + i, ijp = c.owner[iface];
      const double xpn = c.xf[iface] - c.xc[ijp], ypn = c.yf[iface] - c.yc[ijp], zpn = c.zf[iface] - c.zc[ijp];
      const double arx = c.arx[iface], ary = c.ary[iface], arz = c.arz[iface];
      const double dfi = (arx * arx + ary * ary + arz * arz) / (xpn * arx + ypn * ary + zpn * arz);
      out[ijp] = out[ijp] - lambda[ijp] * phi[ijp] * dfi;
    }
}

}  // namespace orc
