// ORACLE (test infrastructure only) -- mesh geometry and CSR pattern.
// Restates read_mesh_native's geometry part (src/mesh/geometry.f90:416-740)
// and create_CSR_matrix (src/sparseMatrix/sparse_matrix.f90:86-296) with the
// helpers of src/misc/utils.f90:96-189.
#include <algorithm>
#include <cmath>
#include <utility>

#include "oracle.hpp"

namespace orc {

void setup_case(Case& c, int numNodes, int numCells, int numInnerFaces, int numBoundaryFaces, const double* x,
                const double* y, const double* z, const int* nnodes, const int* nodes, const int* owner,
                const int* neighbour, int numBoundaries, const int* bctype, const int* nfaces,
                const int* startFace, const int* twin) {
  c.numNodes = numNodes;
  c.numCells = numCells;
  c.numInnerFaces = numInnerFaces;
  c.numBoundaryFaces = numBoundaryFaces;
  c.numFaces = numInnerFaces + numBoundaryFaces;
  c.numTotal = numCells + numBoundaryFaces;  // geometry.f90:282
  c.numBoundaries = numBoundaries;
  c.bctype.assign(numBoundaries + 1, 0);
  c.nfaces.assign(numBoundaries + 1, 0);
  c.startFace.assign(numBoundaries + 1, 0);
  c.iBndValueStart.assign(numBoundaries + 1, 0);
  c.nwal = c.nsym = 0;
  c.nper = c.numPeriodic = 0;
  c.startFaceTwin.assign(1, 0);
  for (int i = 1; i <= numBoundaries; ++i) {
    c.bctype[i] = bctype[i - 1];
    c.nfaces[i] = nfaces[i - 1];
    c.startFace[i] = startFace[i - 1];
    if (c.bctype[i] == BC_WALL) c.nwal += c.nfaces[i];
    else if (c.bctype[i] == BC_SYMMETRY) c.nsym += c.nfaces[i];
    else if (c.bctype[i] == BC_PERIODIC) {  // geometry.f90:250-258
      ++c.nper;
      c.numPeriodic += c.nfaces[i];
      c.startFaceTwin.push_back(twin ? twin[i - 1] : 0);
    }
    // geometry.f90:292-294
    c.iBndValueStart[i] = numCells + (c.startFace[i] - numInnerFaces);
  }
  c.x.assign(numNodes + 1, 0.0);
  c.y.assign(numNodes + 1, 0.0);
  c.z.assign(numNodes + 1, 0.0);
  for (int i = 1; i <= numNodes; ++i) { c.x[i] = x[i - 1]; c.y[i] = y[i - 1]; c.z[i] = z[i - 1]; }
  c.nnodes.assign(c.numFaces + 1, 0);
  c.node.assign((size_t)(c.numFaces + 1) * 6, 0);
  c.owner.assign(c.numFaces + 1, 0);
  c.neighbour.assign(numInnerFaces + 1, 0);
  for (int f = 1; f <= c.numFaces; ++f) {
    c.nnodes[f] = nnodes[f - 1];
    for (int k = 0; k < 6; ++k) c.node[(size_t)f * 6 + k] = nodes[(size_t)(f - 1) * 6 + k];
    c.owner[f] = owner[f - 1];
  }
  for (int f = 1; f <= numInnerFaces; ++f) c.neighbour[f] = neighbour[f - 1];

  geometry(c);
  if (c.nper > 0) face_mapping(c);  // geometry.f90:110-112
  create_csr(c);

  const size_t nt = c.numTotal + 1, nc = c.numCells + 1;
  c.u.assign(nt, 0.0); c.v.assign(nt, 0.0); c.w.assign(nt, 0.0);
  for (auto* v : {&c.uo, &c.vo, &c.wo, &c.uoo, &c.voo, &c.woo, &c.uooo, &c.vooo, &c.wooo}) v->assign(nt, 0.0);
  for (auto* v : {&c.rU, &c.rV, &c.rW}) v->assign(nc, 0.0);
  c.p.assign(nt, 0.0); c.pp.assign(nt, 0.0);
  c.vis.assign(nt, 0.0); c.den.assign(nt, 0.0);
  c.flmass.assign(c.numFaces + 1, 0.0);
  c.visw.assign(c.nwal + 1, 0.0);
  c.dUdxi.assign(3 * nt, 0.0); c.dVdxi.assign(3 * nt, 0.0);
  c.dWdxi.assign(3 * nt, 0.0); c.dPdxi.assign(3 * nt, 0.0);
  c.T.assign(nt, 0.0); c.dTdxi.assign(3 * nt, 0.0);
  for (auto* v : {&c.te, &c.ed, &c.fsst}) v->assign(nt, 0.0);
  c.dTEdxi.assign(3 * nt, 0.0); c.dEDdxi.assign(3 * nt, 0.0);
  for (auto* v : {&c.gen, &c.magStrain, &c.walldist}) v->assign(nc, 0.0);
  c.tau.assign(c.nwal + 1, 0.0); c.ypl.assign(c.nwal + 1, 0.0);
  c.bcDFracT.assign(numBoundaries + 1, 0.0);  // geometry.f90:226 bcDFraction = 0
  c.a.assign(c.nnz + 1, 0.0);
  c.su.assign(nc, 0.0); c.sv.assign(nc, 0.0); c.sw.assign(nc, 0.0);
  c.spu.assign(nc, 0.0); c.spv.assign(nc, 0.0); c.sp.assign(nc, 0.0);
  c.apu.assign(nc, 0.0); c.apv.assign(nc, 0.0); c.apw.assign(nc, 0.0);
  c.res.assign(nc, 0.0); c.reso.assign(nc, 0.0); c.pk.assign(nc, 0.0); c.zk.assign(nc, 0.0);
  c.d.assign(nc, 0.0); c.uk.assign(nc, 0.0); c.vk.assign(nc, 0.0);
}

// triangle_area_vector, geometry.f90:1721-1749
static inline void triangle_area_vector(double px, double py, double pz, double qx, double qy, double qz, double& nx,
                                        double& ny, double& nz) {
  const double half = 0.5;
  nx = half * (py * qz - pz * qy);
  ny = half * (pz * qx - px * qz);
  nz = half * (px * qy - py * qx);
}

// geometry.f90:416-740 (interpolation_coeff_variant = 2, geometry.f90:47)
void geometry(Case& c) {
  const double third = 1.0 / 3.0;  // 1./3._dp
  const int nF = c.numFaces, nC = c.numCells, nI = c.numInnerFaces;
  c.arx.assign(nF + 1, 0.0); c.ary.assign(nF + 1, 0.0); c.arz.assign(nF + 1, 0.0);
  c.xf.assign(nF + 1, 0.0); c.yf.assign(nF + 1, 0.0); c.zf.assign(nF + 1, 0.0);
  c.xc.assign(nC + 1, 0.0); c.yc.assign(nC + 1, 0.0); c.zc.assign(nC + 1, 0.0);
  c.vol.assign(nC + 1, 0.0);
  std::vector<double> r8tmp(nC + 1, 0.0);
  auto NODE = [&](int k, int iface) { return c.node[(size_t)iface * 6 + (k - 1)]; };
  for (int iface = 1; iface <= nF; ++iface) {
    int inp = c.owner[iface];
    double areasum = 0.0;
    for (int i = 1; i <= c.nnodes[iface] - 2; ++i) {
      double px = c.x[NODE(i + 1, iface)] - c.x[NODE(1, iface)];
      double py = c.y[NODE(i + 1, iface)] - c.y[NODE(1, iface)];
      double pz = c.z[NODE(i + 1, iface)] - c.z[NODE(1, iface)];
      double qx = c.x[NODE(i + 2, iface)] - c.x[NODE(1, iface)];
      double qy = c.y[NODE(i + 2, iface)] - c.y[NODE(1, iface)];
      double qz = c.z[NODE(i + 2, iface)] - c.z[NODE(1, iface)];
      double nx, ny, nz;
      triangle_area_vector(px, py, pz, qx, qy, qz, nx, ny, nz);
      c.arx[iface] = c.arx[iface] + nx;
      c.ary[iface] = c.ary[iface] + ny;
      c.arz[iface] = c.arz[iface] + nz;
      double cx = third * (c.x[NODE(i + 2, iface)] + c.x[NODE(i + 1, iface)] + c.x[NODE(1, iface)]);
      double cy = third * (c.y[NODE(i + 2, iface)] + c.y[NODE(i + 1, iface)] + c.y[NODE(1, iface)]);
      double cz = third * (c.z[NODE(i + 2, iface)] + c.z[NODE(i + 1, iface)] + c.z[NODE(1, iface)]);
      double are = std::sqrt(nx * nx + ny * ny + nz * nz);
      c.xf[iface] = c.xf[iface] + (are * cx);
      c.yf[iface] = c.yf[iface] + (are * cy);
      c.zf[iface] = c.zf[iface] + (are * cz);
      areasum = areasum + are;
      double riSi = (cx * nx + cy * ny + cz * nz);
      c.vol[inp] = c.vol[inp] + third * riSi;
      c.xc[inp] = c.xc[inp] + 0.75 * riSi * cx;
      c.yc[inp] = c.yc[inp] + 0.75 * riSi * cy;
      c.zc[inp] = c.zc[inp] + 0.75 * riSi * cz;
      r8tmp[inp] = r8tmp[inp] + riSi;
      if (iface <= nI) {
        int inn = c.neighbour[iface];
        riSi = -(cx * nx + cy * ny + cz * nz);
        c.vol[inn] = c.vol[inn] + third * riSi;
        c.xc[inn] = c.xc[inn] + 0.75 * riSi * cx;
        c.yc[inn] = c.yc[inn] + 0.75 * riSi * cy;
        c.zc[inn] = c.zc[inn] + 0.75 * riSi * cz;
        r8tmp[inn] = r8tmp[inn] + riSi;
      }
    }
    c.xf[iface] = c.xf[iface] / areasum;
    c.yf[iface] = c.yf[iface] / areasum;
    c.zf[iface] = c.zf[iface] / areasum;
  }
  for (int inp = 1; inp <= nC; ++inp) {
    c.xc[inp] = c.xc[inp] / r8tmp[inp];
    c.yc[inp] = c.yc[inp] / r8tmp[inp];
    c.zc[inp] = c.zc[inp] / r8tmp[inp];
  }
  // interpolation factor, variant 2 (geometry.f90:581-603)
  c.facint.assign(nI + 1, 0.0);
  for (int iface = 1; iface <= nI; ++iface) {
    int inp = c.owner[iface], inn = c.neighbour[iface];
    double xpn = c.xf[iface] - c.xc[inp];
    double ypn = c.yf[iface] - c.yc[inp];
    double zpn = c.zf[iface] - c.zc[inp];
    double djp = std::sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    xpn = c.xf[iface] - c.xc[inn];
    ypn = c.yf[iface] - c.yc[inn];
    zpn = c.zf[iface] - c.zc[inn];
    double djn = std::sqrt(xpn * xpn + ypn * ypn + zpn * zpn);
    c.facint[iface] = djp / (djp + djn);
  }
  // Df (geometry.f90:650-665)
  c.Df.assign(nI + 1, 0.0);
  for (int iface = 1; iface <= nI; ++iface) {
    int inp = c.owner[iface], inn = c.neighbour[iface];
    double xpn = c.xc[inn] - c.xc[inp];
    double ypn = c.yc[inn] - c.yc[inp];
    double zpn = c.zc[inn] - c.zc[inp];
    double are = c.arx[iface] * c.arx[iface] + c.ary[iface] * c.ary[iface] + c.arz[iface] * c.arz[iface];
    c.Df[iface] = are / (c.arx[iface] * xpn + c.ary[iface] * ypn + c.arz[iface] * zpn);
  }
  // dns/srds, dnw/srdw (geometry.f90:690-740)
  c.dns.assign(c.nsym + 1, 0.0); c.srds.assign(c.nsym + 1, 0.0);
  c.dnw.assign(c.nwal + 1, 0.0); c.srdw.assign(c.nwal + 1, 0.0);
  int iWall = 0, iSym = 0;
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] != BC_SYMMETRY && c.bctype[ib] != BC_WALL) continue;
    for (int i = 1; i <= c.nfaces[ib]; ++i) {
      int iface = c.startFace[ib] + i;
      int ijp = c.owner[iface];
      double are = std::sqrt(c.arx[iface] * c.arx[iface] + c.ary[iface] * c.ary[iface] + c.arz[iface] * c.arz[iface]);
      double nxf = c.arx[iface] / are, nyf = c.ary[iface] / are, nzf = c.arz[iface] / are;
      double dn = (c.xf[iface] - c.xc[ijp]) * nxf + (c.yf[iface] - c.yc[ijp]) * nyf + (c.zf[iface] - c.zc[ijp]) * nzf;
      if (c.bctype[ib] == BC_SYMMETRY) {
        ++iSym; c.dns[iSym] = dn; c.srds[iSym] = are / c.dns[iSym];
      } else {
        ++iWall; c.dnw[iWall] = dn; c.srdw[iWall] = are / c.dnw[iWall];
      }
    }
  }
}

// create_CSR_matrix, sparse_matrix.f90:86-296.  The lexicographic heap sort
// i4vec2_sort_a (utils.f90:443) is replaced by std::sort: the (row,col)
// keys are compared on both components, equal keys are indistinguishable, so
// every correct lexicographic sort yields the same arrays.
void create_csr(Case& c) {
  const int nC = c.numCells, nI = c.numInnerFaces, nP = c.numPeriodic;
  c.nnz = 2 * (nI + nP) + nC;  // sparse_matrix.f90:110
  std::vector<std::pair<int, int>> coo(c.nnz);
  for (int icell = 1; icell <= nC; ++icell) coo[icell - 1] = {icell, icell};
  for (int i = 1; i <= nI; ++i) coo[nC + i - 1] = {c.owner[i], c.neighbour[i]};
  for (int i = 1; i <= nI; ++i) coo[nC + nI + i - 1] = {c.neighbour[i], c.owner[i]};
  // cells coupled through periodic pairs, two entries per pair (:136-165);
  // pairs(l - nI) = (ijp, ijn) in the running order l of the face loops
  std::vector<std::pair<int, int>> pairs;
  {
    int k = nC + 2 * nI, iPer = 0;
    for (int ib = 1; ib <= c.numBoundaries; ++ib) {
      if (c.bctype[ib] != BC_PERIODIC) continue;
      ++iPer;
      for (int i = 1; i <= c.nfaces[ib]; ++i) {
        int ijp = c.owner[c.startFace[ib] + i], ijn = c.owner[c.startFaceTwin[iPer] + i];
        coo[k++] = {ijp, ijn};
        coo[k++] = {ijn, ijp};
        pairs.push_back({ijp, ijn});
      }
    }
  }
  std::sort(coo.begin(), coo.end());
  c.ja.assign(c.nnz + 1, 0);
  std::vector<int> iacoo(c.nnz + 1, 0);
  for (int k = 1; k <= c.nnz; ++k) { iacoo[k] = coo[k - 1].first; c.ja[k] = coo[k - 1].second; }
  // find_main_diag_element_positions (utils.f90:149-167)
  c.diag.assign(nC + 1, 0);
  int id = 1;
  for (int indx = 1; indx <= c.nnz; ++indx)
    if (iacoo[indx] == c.ja[indx]) { c.diag[id] = indx; ++id; }
  // ia via find_index_position (sparse_matrix.f90:195-202, utils.f90:170-189)
  c.ia.assign(nC + 2, 0);
  int istart = 1, iend = 1;
  for (int icell = 1; icell <= nC; ++icell) {
    for (int i = istart; i <= iend; ++i)
      if (iacoo[i] == icell) { c.ia[icell] = i; break; }
    istart = c.ia[icell] + 1;
    iend = c.nnz;
  }
  c.ia[nC + 1] = c.nnz + 1;
  // csr_to_k slot maps (sparse_matrix.f90:251-260, utils.f90:96-147)
  auto csr_to_k = [&](int icell, int jcell) {
    int k = 0;
    for (int l = c.ia[icell]; l <= c.ia[icell + 1] - 1; ++l)
      if (c.ja[l] == jcell) { k = l; break; }
    return k;
  };
  c.ijk.assign(nI + nP + 1, 0);
  c.jik.assign(nI + nP + 1, 0);
  for (int i = 1; i <= nI; ++i) {
    int ijp = c.owner[i], ijn = c.neighbour[i];
    c.ijk[i] = csr_to_k(ijp, ijn);
    c.jik[i] = csr_to_k(ijn, ijp);
  }
  for (int q = 0; q < nP; ++q) {  // :262-292
    c.ijk[nI + 1 + q] = csr_to_k(pairs[q].first, pairs[q].second);
    c.jik[nI + 1 + q] = csr_to_k(pairs[q].second, pairs[q].first);
  }
}

// face_mapping, geometry.f90:1848-1997: face i of a periodic patch is paired
// with the twin-patch face whose owner's centre is nearest (L1 distance) to
// face i's centre; the twin faces' owners, centres and area vectors are then
// reordered so that twin face i belongs to that pair.
void face_mapping(Case& c) {
  int iPer = 0;
  for (int ib = 1; ib <= c.numBoundaries; ++ib) {
    if (c.bctype[ib] != BC_PERIODIC) continue;
    ++iPer;
    const int n = c.nfaces[ib], tw = c.startFaceTwin[iPer];
    std::vector<int> tmp(n + 1, 0), itmp(n + 1, 0);
    for (int i = 1; i <= n; ++i) {
      const int iface = c.startFace[ib] + i;
      double mindist = (double)1e+30f;
      for (int it = 1; it <= n; ++it) {
        const int ijn = c.owner[tw + it];
        const double dist =
            std::fabs(c.xf[iface] - c.xc[ijn]) + std::fabs(c.yf[iface] - c.yc[ijn]) + std::fabs(c.zf[iface] - c.zc[ijn]);
        if (dist < mindist) { mindist = dist; tmp[i] = ijn; itmp[i] = it; }
      }
    }
    for (int i = 1; i <= n; ++i) c.owner[tw + i] = tmp[i];
    std::vector<double> vtmp(n + 1);
    for (std::vector<double>* v : {&c.xf, &c.yf, &c.zf, &c.arx, &c.ary, &c.arz}) {
      for (int i = 1; i <= n; ++i) vtmp[i] = (*v)[tw + itmp[i]];
      for (int i = 1; i <= n; ++i) (*v)[tw + i] = vtmp[i];
    }
  }
}

}  // namespace orc
