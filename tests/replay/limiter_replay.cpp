// Host replay of the device slope limiters: the per-cell functions of
// csrc/fc_limiter.cuh (the same source the CUDA kernels run) applied to a
// gradient read from argv[1]; the limited gradient is written to argv[2].
// Input (native binary): int kind, nC, nI, nF, nT, nnz, ncf; int ia[nC+1],
// ja[nnz], dg[nC], cf_ptr[nC+1], cf_face[ncf] (0-based); double xc, yc,
// zc[nC], xf, yf, zf[nF], phi[nT], g[3 nT] (SoA).  Output: double g[3 nT].
#include <cstdio>
#include <vector>

#include "fc_limiter.cuh"

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
  const int kind = h[0], nC = h[1], nI = h[2], nF = h[3], nT = h[4], nnz = h[5], ncf = h[6];
  std::vector<int> ia, ja, dg, cfp, cff;
  std::vector<double> xc, yc, zc, xf, yf, zf, phi, g;
  if (!rd(f, ia, nC + 1) || !rd(f, ja, nnz) || !rd(f, dg, nC) || !rd(f, cfp, nC + 1) || !rd(f, cff, ncf) ||
      !rd(f, xc, nC) || !rd(f, yc, nC) || !rd(f, zc, nC) || !rd(f, xf, nF) || !rd(f, yf, nF) || !rd(f, zf, nF) ||
      !rd(f, phi, nT) || !rd(f, g, 3 * (size_t)nT))
    return 3;
  std::fclose(f);
  const size_t T = (size_t)nT;
  if (kind == FC_LIMITER_MD) {
    for (int c = 0; c < nC; ++c) {
      double gx = g[c], gy = g[T + c], gz = g[2 * T + c];
      fclim::limit_md(c, ia.data(), ja.data(), cfp.data(), cff.data(), nI, xf.data(), yf.data(), zf.data(),
                      xc.data(), yc.data(), zc.data(), phi.data(), gx, gy, gz);
      g[c] = gx; g[T + c] = gy; g[2 * T + c] = gz;
    }
  } else if (kind >= FC_LIMITER_BJ && kind <= FC_LIMITER_R) {
    double lo = phi[0], hi = phi[0];
    for (int c = 0; c < nC; ++c) { lo = fclim::dmin(lo, phi[c]); hi = fclim::dmax(hi, phi[c]); }
    for (int c = 0; c < nC; ++c) {
      const double gx = g[c], gy = g[T + c], gz = g[2 * T + c];
      double s;
      if (kind == FC_LIMITER_BJ)
        s = fclim::limit_factor<FC_LIMITER_BJ>(c, ia.data(), ja.data(), dg.data(), xc.data(), yc.data(), zc.data(),
                                               phi.data(), gx, gy, gz, lo, hi);
      else if (kind == FC_LIMITER_VENKAT)
        s = fclim::limit_factor<FC_LIMITER_VENKAT>(c, ia.data(), ja.data(), dg.data(), xc.data(), yc.data(),
                                                   zc.data(), phi.data(), gx, gy, gz, lo, hi);
      else
        s = fclim::limit_factor<FC_LIMITER_R>(c, ia.data(), ja.data(), dg.data(), xc.data(), yc.data(), zc.data(),
                                              phi.data(), gx, gy, gz, lo, hi);
      g[c] = s * gx; g[T + c] = s * gy; g[2 * T + c] = s * gz;
    }
  }
  std::FILE* o = std::fopen(argv[2], "wb");
  if (!o) return 2;
  std::fwrite(g.data(), sizeof(double), g.size(), o);
  std::fclose(o);
  return 0;
}
