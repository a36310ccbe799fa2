// CPU replay of the schedule-ordered sweep (host/fc_schedule.hpp): builds the
// ordered structure for a 7-point pattern (optionally with random long-range
// and one-sided couplings), replays the forward and backward sweeps tile by
// tile with the kernel's ring and exchange rules, and checks the result bit for
// bit against plain substitution in the original numbering, plus the
// exchange/push bookkeeping and the renumbered matrix.  Prints OK on success.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <random>
#include <vector>
#include <string>
#include "fc_schedule.hpp"

static void make_pattern(int nx, int ny, int nz, std::vector<int>& ia, std::vector<int>& ja, std::vector<int>& dg,
                         std::vector<double>& a, std::vector<double>& xyz, unsigned seed, bool extra) {
  int n = nx * ny * nz;
  std::mt19937 rng(seed);
  std::vector<std::vector<int>> cols(n);
  auto id = [&](int i, int j, int k) { return i + nx * (j + ny * k); };
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) {
    int c = id(i, j, k);
    cols[c].push_back(c);
    if (i > 0) cols[c].push_back(id(i - 1, j, k));
    if (i < nx - 1) cols[c].push_back(id(i + 1, j, k));
    if (j > 0) cols[c].push_back(id(i, j - 1, k));
    if (j < ny - 1) cols[c].push_back(id(i, j + 1, k));
    if (k > 0) cols[c].push_back(id(i, j, k - 1));
    if (k < nz - 1) cols[c].push_back(id(i, j, k + 1));
  }
  if (extra) {  // random long-range symmetric couplings (many entries per row)
    for (int t = 0; t < n / 3; ++t) {
      int p = rng() % n, q = rng() % n;
      if (p == q) continue;
      cols[p].push_back(q); cols[q].push_back(p);
    }
    // one-sided entries (non-symmetric pattern)
    for (int t = 0; t < n / 10; ++t) { int p = rng() % n, q = rng() % n; if (p != q) cols[p].push_back(q); }
  }
  ia.assign(n + 1, 0); ja.clear(); dg.assign(n, 0); a.clear();
  std::uniform_real_distribution<double> U(0.5, 1.5);
  for (int c = 0; c < n; ++c) {
    std::sort(cols[c].begin(), cols[c].end());
    cols[c].erase(std::unique(cols[c].begin(), cols[c].end()), cols[c].end());
    for (int j : cols[c]) { if (j == c) dg[c] = (int)ja.size(); ja.push_back(j); a.push_back(j == c ? 0.0 : -U(rng)); }
    ia[c + 1] = (int)ja.size();
  }
  for (int c = 0; c < n; ++c) { double s = 0; for (int k = ia[c]; k < ia[c + 1]; ++k) if (k != dg[c]) s += fabs(a[k]); a[dg[c]] = s + 1.0; }
  xyz.assign(3 * n, 0.0);
  for (int k = 0; k < nz; ++k) for (int j = 0; j < ny; ++j) for (int i = 0; i < nx; ++i) {
    int c = id(i, j, k);
    xyz[c] = i; xyz[n + c] = j; xyz[2 * n + c] = k;
  }
}

int main(int argc, char** argv) {
  int nx = atoi(argv[1]), ny = atoi(argv[2]), nz = atoi(argv[3]), T = atoi(argv[4]);
  bool extra = argc > 5 && atoi(argv[5]);
  int R = argc > 6 ? atoi(argv[6]) : 4, K = argc > 7 ? atoi(argv[7]) : 4;
  const int wmax = argc > 8 ? atoi(argv[8]) : 0;  // cap on the rows of a step (wide levels split)
  std::vector<int> ia, ja, dg; std::vector<double> a, xyz;
  make_pattern(nx, ny, nz, ia, ja, dg, a, xyz, 7, extra);
  int n = nx * ny * nz, nnz = ia[n];
  OrderedSweep O; SweepSchedule S; std::string err;
  if (!build_ordered_sweep(n, ia.data(), ja.data(), dg.data(), nullptr, T, extra ? nullptr : xyz.data(), R, O, S, err,
                           wmax)) {
    printf("build failed: %s\n", err.c_str()); return 1;
  }
  printf("n=%d nnz=%d tiles=%d nsteps=%d nlev=%d maxW=%d maxsteps=%d ring=%lld pushed=%lld cross=%lld ovf=%d/%d\n", n, nnz,
         O.ntiles, O.nsteps, O.nlev, O.maxW, O.max_tile_steps, O.dir[0].ring_entries + O.dir[1].ring_entries,
         O.dir[0].pushed_entries + O.dir[1].pushed_entries, O.dir[0].cross_tile_entries + O.dir[1].cross_tile_entries,
         O.dir[0].ovf_ptr[n], O.dir[1].ovf_ptr[n]);
  // reference: sequential forward and backward substitution in original order (DIC apply style, no d)
  std::vector<double> q(n), yref(n), zref(n);
  std::mt19937 rng(3); std::normal_distribution<double> N01;
  for (auto& v : q) v = N01(rng);
  for (int i = 0; i < n; ++i) { double acc = q[i]; for (int k = ia[i]; k < dg[i]; ++k) acc = std::fma(-a[k], yref[ja[k]], acc); yref[i] = acc * 0.5; }
  for (int i = n - 1; i >= 0; --i) { double acc = yref[i]; for (int k = dg[i] + 1; k < ia[i + 1]; ++k) acc = std::fma(-a[k], zref[ja[k]], acc); zref[i] = acc * 0.5; }
  // ordered replay on the packed layout
  int bad = 0;
  std::vector<int> row_step(n);
  for (int gs = 0; gs < O.nsteps; ++gs) for (int qq = O.step_ptr[gs]; qq < O.step_ptr[gs + 1]; ++qq) row_step[qq] = gs;
  for (int dirn = 0; dirn < 2; ++dirn) {
    const OrderedDir& D = O.dir[dirn];
    size_t xvn = D.xv_ptr[O.nsteps];
    std::vector<int> pushed_cnt(xvn, 0);
    for (int qq = 0; qq < n; ++qq) {
      unsigned s0 = (unsigned)D.srec[4 * qq];
      int np = (s0 >> 8) & 255, poff = D.srec[4 * qq + 1];
      for (int m = 0; m < np; ++m) {
        int pos = D.push[D.push_ptr[row_step[qq]] + poff + m];
        if (pos < 0 || (size_t)pos >= xvn) { printf("push pos out of range\n"); return 1; }
        pushed_cnt[pos]++;
      }
    }
    std::vector<int> needed(xvn, 0);
    auto code_of = [&](int qq, int e) {
      if (e < FC_ELL) { unsigned w = (unsigned)D.srec[4 * qq + 2 + e / 2]; return (int)((w >> (16 * (e & 1))) & 0xFFFF) - 1; }
      return D.ovf_code[D.ovf_ptr[qq] + e - FC_ELL];
    };
    auto slot_of = [&](int qq, int e) { return e < FC_ELL ? D.slot[(size_t)e * O.nE + qq] : D.ovf_slot[D.ovf_ptr[qq] + e - FC_ELL]; };
    for (int qq = 0; qq < n; ++qq) {
      unsigned s0 = (unsigned)D.srec[4 * qq];
      int ne = s0 & 255, xoff = s0 >> 16, m = 0;
      if (ne != D.ne[qq]) { printf("ne mismatch\n"); return 1; }
      for (int e = 0; e < ne; ++e) if (code_of(qq, e) < 0) needed[D.xv_ptr[row_step[qq]] + xoff + m++]++;
    }
    for (size_t p = 0; p < xvn; ++p) if (pushed_cnt[p] != needed[p]) { if (bad < 5) printf("dir %d pos %zu pushed %d needed %d\n", dirn, p, pushed_cnt[p], needed[p]); bad++; }
    std::vector<double> in(n), out(n, NAN), xv(xvn, NAN);
    for (int qq = 0; qq < n; ++qq) in[qq] = dirn == 0 ? q[O.perm[qq]] : yref[O.perm[qq]];
    std::vector<int> next(O.ntiles, 0);
    std::vector<std::vector<double>> ring(O.ntiles);
    for (int t = 0; t < O.ntiles; ++t) ring[t].assign((size_t)R * O.tile_W[t], NAN);
    int done = 0, rounds = 0;
    while (done < O.ntiles) {
      bool progress = false;
      std::vector<std::pair<size_t, double>> pending;
      done = 0;
      for (int t = 0; t < O.ntiles; ++t) {
        int ns = O.tile_step_ptr[t + 1] - O.tile_step_ptr[t];
        if (next[t] >= ns) { done++; continue; }
        int k = next[t], ls = dirn ? ns - 1 - k : k, gs = O.tile_step_ptr[t] + ls;
        int base = O.step_ptr[gs], cnt = O.step_ptr[gs + 1] - base, W = O.tile_W[t];
        bool ready = true;
        for (int sl = 0; sl < cnt && ready; ++sl) {
          int qq = base + sl; unsigned s0 = (unsigned)D.srec[4 * qq]; int ne = s0 & 255, xoff = s0 >> 16, m = 0;
          for (int e = 0; e < ne; ++e) if (code_of(qq, e) < 0) { if (std::isnan(xv[D.xv_ptr[gs] + xoff + m])) { ready = false; break; } m++; }
        }
        if (!ready) continue;
        progress = true;
        std::vector<double> vals(cnt);
        for (int sl = 0; sl < cnt; ++sl) {
          int qq = base + sl; unsigned s0 = (unsigned)D.srec[4 * qq]; int ne = s0 & 255, xoff = s0 >> 16, m = 0;
          double acc = in[qq];
          for (int e = 0; e < ne; ++e) {
            int c = code_of(qq, e), slot = slot_of(qq, e);
            double v;
            if (c >= 0) { if (c >= R * W) { printf("ring code out of range\n"); return 1; } v = ring[t][c]; }
            else { size_t pos = D.xv_ptr[gs] + xoff + m++; v = xv[pos]; xv[pos] = NAN; }
            acc = std::fma(-a[slot], v, acc);
          }
          vals[sl] = acc * 0.5;
        }
        for (int sl = 0; sl < cnt; ++sl) {
          int qq = base + sl; unsigned s0 = (unsigned)D.srec[4 * qq]; int np = (s0 >> 8) & 255, poff = D.srec[4 * qq + 1];
          out[qq] = vals[sl];
          ring[t][(k % R) * W + sl] = vals[sl];
          for (int m = 0; m < np; ++m) pending.push_back({(size_t)D.push[D.push_ptr[gs] + poff + m], vals[sl]});
        }
        next[t]++;
      }
      for (auto& pv : pending) xv[pv.first] = pv.second;
      rounds++;
      if (!progress && done < O.ntiles) { printf("DEADLOCK dir %d after %d rounds\n", dirn, rounds); return 1; }
    }
    const std::vector<double>& ref = dirn == 0 ? yref : zref;
    int mism = 0;
    for (int qq = 0; qq < n; ++qq) if (out[qq] != ref[O.perm[qq]]) mism++;
    printf("dir %d: rounds %d mismatches %d xv %zu pushes %d\n", dirn, rounds, mism, xvn, D.push_ptr[O.nsteps]);
    bad += mism;
  }
  // permuted CSR check
  for (int qq = 0; qq < n; ++qq) {
    int i = O.perm[qq];
    if (O.p_ptr[qq + 1] - O.p_ptr[qq] != ia[i + 1] - ia[i]) bad++;
    for (int o = O.p_ptr[qq], k = ia[i]; o < O.p_ptr[qq + 1]; ++o, ++k)
      if (O.p_slot[o] != k || O.perm[O.p_col[o]] != ja[k]) bad++;
    if (O.dslot[qq] != dg[i]) bad++;
  }
  printf(bad ? "FAIL %d\n" : "OK\n", bad);
  return bad != 0;
}
