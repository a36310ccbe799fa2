#include "fc_node_interp.hpp"

#include <algorithm>
#include <cmath>

namespace {

// geometry.f90:41, a default-real literal
const double kTiny = (double)1e-30f;

struct Moments {
  std::vector<double> rx, ry, rz, ixx, iyy, izz, ixy, ixz, iyz;
  explicit Moments(int n)
      : rx(n, 0.0), ry(n, 0.0), rz(n, 0.0), ixx(n, 0.0), iyy(n, 0.0), izz(n, 0.0), ixy(n, 0.0), ixz(n, 0.0),
        iyz(n, 0.0) {}
  void add(int v, double dx, double dy, double dz) {
    rx[v] = rx[v] + dx;
    ry[v] = ry[v] + dy;
    rz[v] = rz[v] + dz;
    ixx[v] = ixx[v] + dx * dx;
    iyy[v] = iyy[v] + dy * dy;
    izz[v] = izz[v] + dz * dz;
    ixy[v] = ixy[v] + dx * dy;
    ixz[v] = ixz[v] + dx * dz;
    iyz[v] = iyz[v] + dy * dz;
  }
  // min(|1 + lambda . d|, 1), lambda as node_interpolation.f90:386-407
  // writes it (its lamx numerator has ixx izz - iyz^2 where the cofactor
  // would have iyy izz - iyz^2; kept)
  double weight(int v, double dx, double dy, double dz) const {
    const double a = ixx[v], b = iyy[v], c = izz[v], d = ixy[v], e = ixz[v], f = iyz[v];
    const double X = rx[v], Y = ry[v], Z = rz[v];
    const double D = a * (b * c - f * f) - d * (d * c - e * f) + e * (d * f - b * e) + kTiny;
    const double lx = (-(X * (a * c - f * f)) + Y * (d * c - e * f) - Z * (d * f - b * e)) / D;
    const double ly = (X * (d * c - e * f) - Y * (a * c - e * e) + Z * (a * f - d * e)) / D;
    const double lz = (-(X * (d * f - b * e)) + Y * (a * f - d * e) - Z * (a * b - d * d)) / D;
    const double wv = 1.0 + lx * dx + ly * dy + lz * dz;
    const double aw = std::fabs(wv);
    return 1.0 < aw ? 1.0 : aw;
  }
};

double dist(double xa, double ya, double za, double xb, double yb, double zb) {
  const double dx = xa - xb, dy = ya - yb, dz = za - zb;
  return std::sqrt(dx * dx + dy * dy + dz * dz);
}

}  // namespace

void build_node_interp(int nNodes, int nC, int nI, int nF, const int* owner, const int* neighbour,
                       const int* nnodes, const int* nodes, int nomax, const double* x, const double* y,
                       const double* z, const double* xc, const double* yc, const double* zc, const double* xf,
                       const double* yf, const double* zf, int method, NodeInterp& out) {
  auto NODE = [&](int f, int k) { return nodes[(size_t)f * nomax + k]; };
  // weights in the reference's running order
  std::vector<double> wc, wf;
  if (method == 1) {
    std::vector<double> dsum(nNodes, 0.0);
    for (int f = 0; f < nI; ++f)
      for (int k = 0; k < nnodes[f]; ++k) {
        const int v = NODE(f, k);
        const int p = owner[f], q = neighbour[f];
        dsum[v] = dsum[v] + 1. / dist(xc[p], yc[p], zc[p], x[v], y[v], z[v]);
        dsum[v] = dsum[v] + 1. / dist(xc[q], yc[q], zc[q], x[v], y[v], z[v]);
      }
    for (int f = 0; f < nI; ++f)
      for (int k = 0; k < nnodes[f]; ++k) {
        const int v = NODE(f, k);
        const int p = owner[f], q = neighbour[f];
        wc.push_back(1. / (dist(xc[p], yc[p], zc[p], x[v], y[v], z[v]) * dsum[v]));
        wc.push_back(1. / (dist(xc[q], yc[q], zc[q], x[v], y[v], z[v]) * dsum[v]));
      }
    std::fill(dsum.begin(), dsum.end(), 0.0);
    for (int f = nI; f < nF; ++f)
      for (int k = 0; k < nnodes[f]; ++k) {
        const int v = NODE(f, k);
        dsum[v] = dsum[v] + 1. / dist(xf[f], yf[f], zf[f], x[v], y[v], z[v]);
      }
    for (int f = nI; f < nF; ++f)
      for (int k = 0; k < nnodes[f]; ++k) {
        const int v = NODE(f, k);
        wf.push_back(1. / (dist(xf[f], yf[f], zf[f], x[v], y[v], z[v]) * dsum[v]));
      }
  } else {
    {
      Moments M(nNodes);
      for (int f = 0; f < nI; ++f)
        for (int k = 0; k < nnodes[f]; ++k) {
          const int v = NODE(f, k);
          const int p = owner[f], q = neighbour[f];
          M.add(v, xc[p] - x[v], yc[p] - y[v], zc[p] - z[v]);
          M.add(v, xc[q] - x[v], yc[q] - y[v], zc[q] - z[v]);
        }
      for (int f = 0; f < nI; ++f)
        for (int k = 0; k < nnodes[f]; ++k) {
          const int v = NODE(f, k);
          const int p = owner[f], q = neighbour[f];
          wc.push_back(M.weight(v, xc[p] - x[v], yc[p] - y[v], zc[p] - z[v]));
          wc.push_back(M.weight(v, xc[q] - x[v], yc[q] - y[v], zc[q] - z[v]));
        }
      std::vector<double> wsum(nNodes, 0.0);
      size_t i = 0;
      for (int f = 0; f < nI; ++f)
        for (int k = 0; k < nnodes[f]; ++k) {
          const int v = NODE(f, k);
          wsum[v] = wsum[v] + wc[i++];
          wsum[v] = wsum[v] + wc[i++];
        }
      i = 0;
      for (int f = 0; f < nI; ++f)
        for (int k = 0; k < nnodes[f]; ++k) {
          const int v = NODE(f, k);
          wc[i] = wc[i] / wsum[v];
          ++i;
          wc[i] = wc[i] / wsum[v];
          ++i;
        }
    }
    Moments M(nNodes);
    for (int f = nI; f < nF; ++f)
      for (int k = 0; k < nnodes[f]; ++k) {
        const int v = NODE(f, k);
        M.add(v, xf[f] - x[v], yf[f] - y[v], zf[f] - z[v]);
      }
    for (int f = nI; f < nF; ++f)
      for (int k = 0; k < nnodes[f]; ++k) {
        const int v = NODE(f, k);
        wf.push_back(M.weight(v, xf[f] - x[v], yf[f] - y[v], zf[f] - z[v]));
      }
    std::vector<double> wsum(nNodes, 0.0);
    size_t i = 0;
    for (int f = nI; f < nF; ++f)
      for (int k = 0; k < nnodes[f]; ++k) {
        const int v = NODE(f, k);
        wsum[v] = wsum[v] + wf[i++];
      }
    i = 0;
    for (int f = nI; f < nF; ++f)
      for (int k = 0; k < nnodes[f]; ++k) {
        const int v = NODE(f, k);
        wf[i] = wf[i] / wsum[v];
        ++i;
      }
  }
  // per-node lists of the terms interpolate_to_nodes keeps, in its order
  std::vector<char> bnd(nNodes, 0);
  for (int f = nI; f < nF; ++f)
    for (int k = 0; k < nnodes[f]; ++k) bnd[NODE(f, k)] = 1;
  out.nNodes = nNodes;
  out.ptr.assign(nNodes + 1, 0);
  for (int f = 0; f < nI; ++f)
    for (int k = 0; k < nnodes[f]; ++k)
      if (!bnd[NODE(f, k)]) out.ptr[NODE(f, k) + 1] += 2;
  for (int f = nI; f < nF; ++f)
    for (int k = 0; k < nnodes[f]; ++k) out.ptr[NODE(f, k) + 1] += 1;
  for (int v = 0; v < nNodes; ++v) out.ptr[v + 1] += out.ptr[v];
  out.src.assign(out.ptr[nNodes], 0);
  out.w.assign(out.ptr[nNodes], 0.0);
  std::vector<int> pos(out.ptr.begin(), out.ptr.end() - 1);
  size_t i = 0;
  for (int f = 0; f < nI; ++f)
    for (int k = 0; k < nnodes[f]; ++k, i += 2) {
      const int v = NODE(f, k);
      if (bnd[v]) continue;
      out.src[pos[v]] = owner[f];
      out.w[pos[v]++] = wc[i];
      out.src[pos[v]] = neighbour[f];
      out.w[pos[v]++] = wc[i + 1];
    }
  i = 0;
  for (int f = nI; f < nF; ++f)
    for (int k = 0; k < nnodes[f]; ++k, ++i) {
      const int v = NODE(f, k);
      out.src[pos[v]] = nC + (f - nI);
      out.w[pos[v]++] = wf[i];
    }
}
