// CPU replay of the multicolour FP32 inner solve (csrc/fc_mc.cu) on the
// library's own layout builder (host/fc_colour.cpp).
//
// Checks, for a 7-point matrix on an nx*ny*nz grid (optionally with extra
// random couplings):
//  - the colouring is proper and every stored index stays inside its buffer;
//  - rows list their lower-colour entries first; padding is inert;
//  - the kernels' pass sequence (setup colour by colour; the forward sweep on
//    the right-hand side; per PCG iteration in Eisenstat's form the backward
//    colours C-2..1, colour 0, the forward colours 1..C-1, the x/r update and
//    the new direction; the final backward sweep) gathers only values written
//    by an earlier pass, i.e. before a kernel boundary;
//  - the replayed PCG converges on an SPD matrix and its solution satisfies
//    A x = b.
// Prints OK on success.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "fc_colour.hpp"

static int fails = 0;
#define CHECK(c, ...)                     \
  do {                                    \
    if (!(c)) {                           \
      std::printf("FAIL: " __VA_ARGS__);  \
      std::printf("\n");                  \
      if (++fails > 20) std::exit(1);     \
    }                                     \
  } while (0)

int main(int argc, char** argv) {
  if (argc < 4) {
    std::printf("usage: colour_replay nx ny nz [random_couplings]\n");
    return 2;
  }
  const int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nz = std::atoi(argv[3]);
  const int extra = argc > 4 ? std::atoi(argv[4]) : 0;
  const int n = nx * ny * nz;
  std::mt19937_64 rng(7);
  std::uniform_real_distribution<double> U(0.1, 1.0);
  // symmetric pattern: 7-point neighbours plus random long-range pairs
  std::vector<std::vector<std::pair<int, double>>> rows(n);
  auto id = [&](int i, int j, int k) { return (k * ny + j) * nx + i; };
  auto couple = [&](int a, int b, double w) {
    rows[a].push_back({b, -w});
    rows[b].push_back({a, -w});
  };
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int r = id(i, j, k);
        if (i + 1 < nx) couple(r, id(i + 1, j, k), U(rng));
        if (j + 1 < ny) couple(r, id(i, j + 1, k), U(rng));
        if (k + 1 < nz) couple(r, id(i, j, k + 1), U(rng));
      }
  if (extra && n > 2) {
    std::uniform_int_distribution<int> R(0, n - 1);
    for (int t = 0; t < n / 3; ++t) {
      int a = R(rng), b = R(rng);
      if (a == b) continue;
      bool dup = false;
      for (auto& e : rows[a]) dup |= e.first == b;
      if (!dup) couple(a, b, 0.3 * U(rng));
    }
  }
  // CSR (0-based), diagonal = sum |off| + shift: SPD
  std::vector<int> ia(n + 1, 0), ja, dg(n);
  std::vector<double> a;
  for (int r = 0; r < n; ++r) {
    std::vector<std::pair<int, double>> e = rows[r];
    double s = 0.0;
    for (auto& x : e) s += std::fabs(x.second);
    e.push_back({r, s + 0.05 + 0.01 * (r % 7)});
    std::sort(e.begin(), e.end());
    for (auto& x : e) {
      if (x.first == r) dg[r] = (int)ja.size();
      ja.push_back(x.first);
      a.push_back(x.second);
    }
    ia[r + 1] = (int)ja.size();
  }
  const int nnz = (int)ja.size();
  ColouredLayout L;
  std::string err;
  if (!build_coloured(n, ia.data(), ja.data(), dg.data(), L, &err)) {
    std::printf("build_coloured failed: %s\n", err.c_str());
    return 1;
  }
  // ---- structure
  CHECK(L.nP % FC_MC_SLICE == 0 && L.nslices * FC_MC_SLICE == L.nP, "slices");
  CHECK((int)L.cslice.size() == L.ncol + 1 && L.cslice[0] == 0 && L.cslice[L.ncol] == L.nslices, "cslice");
  std::vector<int> colour_of(L.nP, -1);
  for (int c = 0; c < L.ncol; ++c)
    for (int r = L.cslice[c] * FC_MC_SLICE; r < L.cslice[c + 1] * FC_MC_SLICE; ++r) colour_of[r] = c;
  int seen = 0;
  for (int r = 0; r < L.nP; ++r) {
    const int o = L.perm[r];
    if (o < 0) {
      CHECK(L.rowinfo[r] == 0 && L.dslot[r] == -1, "padding row %d not inert", r);
      continue;
    }
    ++seen;
    CHECK(o < n && L.iperm[o] == r, "perm/iperm mismatch at %d", r);
    CHECK(L.dslot[r] == dg[o], "dslot of %d", r);
  }
  CHECK(seen == n, "rows covered %d of %d", seen, n);
  CHECK((long long)L.col.size() == L.nent && (long long)L.src.size() == L.nent, "entry arrays");
  CHECK((int)L.cwl.size() == L.ncol && (int)L.cwu.size() == L.ncol, "widths");
  long long covered = 0;
  for (int c = 0; c < L.ncol; ++c) {
    const int r0 = L.cslice[c] * FC_MC_SLICE, rows = (L.cslice[c + 1] - L.cslice[c]) * FC_MC_SLICE;
    covered += (long long)(L.cwl[c] + L.cwu[c]) * rows;
    CHECK(L.ceu[c] == L.cel[c] + (long long)L.cwl[c] * rows, "colour %d block offsets", c);
    for (int r = r0; r < r0 + rows; ++r) {
      const int nlo = L.rowinfo[r] & 0xFFFF, ne = L.rowinfo[r] >> 16;
      CHECK(nlo <= L.cwl[c] && ne - nlo <= L.cwu[c], "row %d counts", r);
      for (int up = 0; up < 2; ++up) {
        const int w = up ? L.cwu[c] : L.cwl[c], nreal = up ? ne - nlo : nlo;
        for (int k = 0; k < w; ++k) {
          const long long e = (up ? L.ceu[c] : L.cel[c]) + (long long)k * rows + (r - r0);
          CHECK(e >= 0 && e < L.nent, "entry out of range");
          const int cc = L.col[e];
          CHECK(cc >= 0 && cc < L.nP, "col out of range");
          if (k >= nreal) {
            CHECK(L.src[e] == -1 && cc == r, "padding entry of row %d", r);
            continue;
          }
          CHECK(L.src[e] >= 0 && L.src[e] < nnz, "src out of range");
          const int o = L.perm[r];
          CHECK(L.src[e] >= ia[o] && L.src[e] < ia[o + 1] && L.iperm[ja[L.src[e]]] == cc, "src is not a_ij");
          CHECK(L.tsrc[e] >= 0 && L.tsrc[e] < nnz && ja[L.tsrc[e]] == o, "tsrc");
          CHECK(colour_of[cc] != colour_of[r], "colouring not proper: %d %d", r, cc);
          if (!up) CHECK(colour_of[cc] < colour_of[r], "lower block entry at row %d", r);
          else CHECK(colour_of[cc] > colour_of[r], "upper block entry at row %d", r);
        }
      }
    }
  }
  CHECK(covered == L.nent, "blocks cover %lld of %lld entries", covered, L.nent);
  // ---- replay of the kernel with phase stamps (a value may be read only
  // if it was written in an earlier phase)
  int phase = 0;
  std::vector<int> dstamp(L.nP, -1);
  std::vector<double> mval(L.nent, 0.0), invd(L.nP), adiag(L.nP), dset(L.nP);
  // the kernel's addressing: block start + k * rows of the colour + row offset
  auto entL = [&](int c, int i, int k) {
    const int r0 = L.cslice[c] * FC_MC_SLICE, rows = (L.cslice[c + 1] - L.cslice[c]) * FC_MC_SLICE;
    return L.cel[c] + (long long)k * rows + (i - r0);
  };
  auto entU = [&](int c, int i, int k) {
    const int r0 = L.cslice[c] * FC_MC_SLICE, rows = (L.cslice[c + 1] - L.cslice[c]) * FC_MC_SLICE;
    return L.ceu[c] + (long long)k * rows + (i - r0);
  };
  for (int c = 0; c < L.ncol; ++c, ++phase)
    for (int i = L.cslice[c] * FC_MC_SLICE; i < L.cslice[c + 1] * FC_MC_SLICE; ++i) {
        const int ds = L.dslot[i];
        const double aii = ds >= 0 ? a[ds] : 1.0;
        double d = aii;
        for (int k = 0; k < L.cwl[c]; ++k) {
          const long long e = entL(c, i, k);
          if (L.src[e] < 0) continue;
          const double v = a[L.src[e]];
          mval[e] = v;
          CHECK(dstamp[L.col[e]] < phase, "d read before its colour finished");
          d -= v * a[L.tsrc[e]] / dset[L.col[e]];
        }
        for (int k = 0; k < L.cwu[c]; ++k) {
          const long long e = entU(c, i, k);
          if (L.src[e] >= 0) mval[e] = a[L.src[e]];
        }
        dset[i] = d;
        dstamp[i] = phase;
        invd[i] = 1.0 / (d + 1e-20);
        adiag[i] = ds >= 0 ? aii : 0.0;
      }
  // Eisenstat form of the coloured DIC-PCG, pass by pass as the graph runs
  // it: every read of a vector that some pass writes is stamped, and must
  // come from an earlier pass (a kernel boundary) or from the row itself.
  std::vector<double> b(n), r(L.nP, 0.0), x(L.nP, 0.0), p(L.nP, 0.0), q(L.nP, 0.0), z(L.nP, 0.0), t(L.nP, 0.0),
      w(L.nP, 0.0), dv(L.nP), kd(L.nP);
  for (int i = 0; i < L.nP; ++i) { dv[i] = dset[i]; kd[i] = adiag[i] - 2.0 * dset[i]; }
  for (int i = 0; i < n; ++i) b[i] = std::sin(0.37 * i) + 0.1;
  for (int i = 0; i < L.nP; ++i) r[i] = L.perm[i] >= 0 ? b[L.perm[i]] : 0.0;
  const int C = L.ncol;
  std::vector<int> st_r(L.nP, -1), st_t(L.nP, -1), st_w(L.nP, -1), st_x(L.nP, -1);
  auto rd = [&](const std::vector<double>& v, std::vector<int>& stamp, int j, int self) {
    CHECK(j == self || stamp[j] < phase, "gathered value %d written in the same pass %d", j, phase);
    return v[j];
  };
  auto rows_of = [&](int c, int& r0, int& r1) { r0 = L.cslice[c] * FC_MC_SLICE; r1 = L.cslice[c + 1] * FC_MC_SLICE; };
  int r0, r1;
  // prologue: (D+L) r~ = b colour by colour
  for (int c = 0; c < C; ++c, ++phase) {
    rows_of(c, r0, r1);
    for (int i = r0; i < r1; ++i) {
      double s = 0.0;
      for (int k = 0; k < L.cwl[c]; ++k) { const long long e = entL(c, i, k); s += mval[e] * rd(r, st_r, L.col[e], i); }
      r[i] = (r[i] - s) * invd[i];
      st_r[i] = phase;
    }
  }
  rows_of(C - 1, r0, r1);
  double rz = 0.0;
  for (int i = 0; i < L.nP; ++i) {
    z[i] = dv[i] * r[i];
    p[i] = z[i];
    if (i >= r0) { t[i] = p[i] * invd[i]; st_t[i] = phase; }
    rz += r[i] * z[i];
  }
  ++phase;
  const double rz0 = rz;
  int it = 0;
  for (; it < 4 * n + 100; ++it) {
    for (int c = C - 2; c >= 1; --c, ++phase) {
      rows_of(c, r0, r1);
      for (int i = r0; i < r1; ++i) {
        double s = 0.0;
        for (int k = 0; k < L.cwu[c]; ++k) { const long long e = entU(c, i, k); s += mval[e] * rd(t, st_t, L.col[e], i); }
        t[i] = (p[i] - s) * invd[i];
        st_t[i] = phase;
      }
    }
    double pq = 0.0;
    rows_of(0, r0, r1);
    for (int i = r0; i < r1; ++i) {
      double s = 0.0;
      for (int k = 0; k < L.cwu[0]; ++k) { const long long e = entU(0, i, k); s += mval[e] * rd(t, st_t, L.col[e], i); }
      const double ti = (p[i] - s) * invd[i];
      w[i] = (p[i] + kd[i] * ti) * invd[i];
      q[i] = ti + w[i];
      st_w[i] = phase;
      pq += p[i] * q[i];
    }
    ++phase;
    for (int c = 1; c < C; ++c, ++phase) {
      rows_of(c, r0, r1);
      for (int i = r0; i < r1; ++i) {
        double s = 0.0;
        for (int k = 0; k < L.cwl[c]; ++k) { const long long e = entL(c, i, k); s += mval[e] * rd(w, st_w, L.col[e], i); }
        CHECK(st_t[i] < phase, "own t written in the same pass");
        w[i] = (p[i] + kd[i] * t[i] - s) * invd[i];
        q[i] = t[i] + w[i];
        st_w[i] = phase;
        pq += p[i] * q[i];
      }
    }
    const double alpha = rz / pq;
    double rzn = 0.0;
    for (int i = 0; i < L.nP; ++i) {
      x[i] += alpha * p[i];
      r[i] -= alpha * q[i];
      z[i] = dv[i] * r[i];
      rzn += r[i] * z[i];
    }
    ++phase;
    if (std::fabs(rzn) <= 1e-26 * std::fabs(rz0)) break;
    const double beta = rzn / rz;
    rz = rzn;
    rows_of(C - 1, r0, r1);
    for (int i = 0; i < L.nP; ++i) {
      p[i] = z[i] + beta * p[i];
      if (i >= r0) { t[i] = p[i] * invd[i]; st_t[i] = phase; }
    }
    ++phase;
  }
  // x = (D+U)^-1 y, colours C-1..0, in place
  for (int c = C - 1; c >= 0; --c, ++phase) {
    rows_of(c, r0, r1);
    for (int i = r0; i < r1; ++i) {
      double s = 0.0;
      for (int k = 0; k < L.cwu[c]; ++k) { const long long e = entU(c, i, k); s += mval[e] * rd(x, st_x, L.col[e], i); }
      x[i] = (x[i] - s) * invd[i];
      st_x[i] = phase;
    }
  }
  // true residual of the solution in the original numbering
  double err_l1 = 0.0, bl1 = 0.0;
  for (int o = 0; o < n; ++o) {
    double s = 0.0;
    for (int k = ia[o]; k < ia[o + 1]; ++k) s += a[k] * x[L.iperm[ja[k]]];
    err_l1 += std::fabs(b[o] - s);
    bl1 += std::fabs(b[o]);
  }
  std::printf("n=%d colours=%d slices=%d entries=%lld iterations=%d rel_res=%.3e\n", n, L.ncol, L.nslices, L.nent,
              it + 1, err_l1 / bl1);
  CHECK(err_l1 / bl1 < 1e-9, "replayed PCG did not converge: %.3e", err_l1 / bl1);
  if (nx > 1 && ny > 1 && nz > 1 && !extra) CHECK(L.ncol == 2, "structured grid should need 2 colours, got %d", L.ncol);
  if (fails) return 1;
  std::printf("OK\n");
  return 0;
}
