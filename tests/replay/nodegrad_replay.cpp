// Host replay of the device node-based Gauss gradient: the library's weight
// builder (host/fc_node_interp.cpp) and the per-node and per-cell functions
// of csrc/fc_nodegrad.cuh (the source the CUDA kernels run), on arrays read
// from argv[1]; the gradient is written to argv[2].
// Input (native binary): int method, nN, nC, nI, nF, nT, ncf; int owner[nF],
// neighbour[nI], nnodes[nF], nodes[6 nF], cf_ptr[nC+1], cf_face[ncf]
// (0-based); double x, y, z[nN], xc, yc, zc[nC], xf, yf, zf[nF], arx, ary,
// arz[nF], vol[nC], phi[nT].  Output: double g[3 nT] (SoA, boundary 0).
#include <cstdio>
#include <vector>

#include "fc_node_interp.hpp"
#include "fc_nodegrad.cuh"

template <class T>
static bool rd(std::FILE* f, std::vector<T>& v, size_t n) {
  v.resize(n);
  return std::fread(v.data(), sizeof(T), n, f) == n;
}

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  std::FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int h[7];
  if (std::fread(h, sizeof(int), 7, f) != 7) return 2;
  const int method = h[0], nN = h[1], nC = h[2], nI = h[3], nF = h[4], nT = h[5], ncf = h[6];
  std::vector<int> own, nb, nnodes, nodes, cfp, cff;
  std::vector<double> x, y, z, xc, yc, zc, xf, yf, zf, arx, ary, arz, vol, phi;
  if (!rd(f, own, nF) || !rd(f, nb, nI) || !rd(f, nnodes, nF) || !rd(f, nodes, 6 * (size_t)nF) ||
      !rd(f, cfp, nC + 1) || !rd(f, cff, ncf) || !rd(f, x, nN) || !rd(f, y, nN) || !rd(f, z, nN) || !rd(f, xc, nC) ||
      !rd(f, yc, nC) || !rd(f, zc, nC) || !rd(f, xf, nF) || !rd(f, yf, nF) || !rd(f, zf, nF) || !rd(f, arx, nF) ||
      !rd(f, ary, nF) || !rd(f, arz, nF) || !rd(f, vol, nC) || !rd(f, phi, nT))
    return 3;
  std::fclose(f);
  NodeInterp ni;
  build_node_interp(nN, nC, nI, nF, own.data(), nb.data(), nnodes.data(), nodes.data(), 6, x.data(), y.data(),
                    z.data(), xc.data(), yc.data(), zc.data(), xf.data(), yf.data(), zf.data(), method, ni);
  std::vector<double> uN(nN);
  for (int v = 0; v < nN; ++v) uN[v] = fcng::node_value(v, ni.ptr.data(), ni.src.data(), ni.w.data(), phi.data());
  std::vector<double> g(3 * (size_t)nT, 0.0);
  for (int c = 0; c < nC; ++c)
    fcng::node_gauss_cell(c, cfp.data(), cff.data(), own.data(), nnodes.data(), nodes.data(), 6, uN.data(),
                          arx.data(), ary.data(), arz.data(), vol.data(), g[c], g[nT + c], g[2 * (size_t)nT + c]);
  std::FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  std::fwrite(g.data(), sizeof(double), g.size(), o);
  std::fclose(o);
  return 0;
}
