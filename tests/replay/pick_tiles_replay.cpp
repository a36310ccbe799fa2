// Tile-count choice of the pattern analysis: pick_sweep_tiles (concurrent
// trials) against the same candidates built one after another here, on a
// structured nx x ny x nz 7-point pattern (argv: nx ny nz sms [coords]).
// Prints "tiles est" of both.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "fc_schedule.hpp"

int main(int argc, char** argv) {
  if (argc < 5) return 2;
  const int nx = atoi(argv[1]), ny = atoi(argv[2]), nz = atoi(argv[3]), sms = atoi(argv[4]);
  const bool coords = argc < 6 || atoi(argv[5]) != 0;
  const int n = nx * ny * nz;
  std::vector<int> ia(n + 1), ja, dg(n);
  std::vector<double> xyz(3 * (size_t)n);
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const int r = (k * ny + j) * nx + i;
        ia[r] = (int)ja.size();
        const int nb[7] = {r - nx * ny, r - nx, r - 1, r, r + 1, r + nx, r + nx * ny};
        const bool ok[7] = {k > 0, j > 0, i > 0, true, i < nx - 1, j < ny - 1, k < nz - 1};
        for (int e = 0; e < 7; ++e)
          if (ok[e]) {
            if (e == 3) dg[r] = (int)ja.size();
            ja.push_back(nb[e]);
          }
        xyz[r] = i;
        xyz[n + r] = j;
        xyz[2 * (size_t)n + r] = k;
      }
  ia[n] = (int)ja.size();
  const double* X = coords ? xyz.data() : nullptr;
  const std::vector<int> cand = {sms, (3 * sms) / 4, sms / 2, sms / 4};
  // one after another, one scratch code array reused between trials
  std::vector<int> lev;
  const int nls = symmetric_levels(n, ia.data(), ja.data(), dg.data(), lev);
  std::vector<int> scratch(ia[n], 0);
  double best = 1e300;
  int tiles = sms;
  for (int c = 0; c < 4; ++c) {
    if (cand[c] < 1 || (c > 0 && cand[c] == cand[c - 1])) continue;
    SweepSchedule S;
    build_sweep_schedule(n, ia.data(), ja.data(), dg.data(), lev, nls, true, cand[c], X, S, scratch);
    const double e = estimate_sweep_us(S, 0.15, 0.001, 1.5);
    if (e < best) { best = e; tiles = cand[c]; }
  }
  double est = 0;
  const int t2 = pick_sweep_tiles(n, ia.data(), ja.data(), dg.data(), X, cand, 0.15, 0.001, 1.5, &est);
  std::printf("%d %.17g\n%d %.17g\n", tiles, best, t2, est);
  return 0;
}
