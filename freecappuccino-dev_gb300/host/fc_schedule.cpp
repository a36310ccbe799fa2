// Tiled pipeline schedule of a sparse triangular sweep: chains, tiles, steps,
// shared-memory ring codes and cross-tile waits (see fc_schedule.hpp).
#include "fc_schedule.hpp"

#include <algorithm>
#include <deque>
#include <limits>
#include <numeric>
#include <set>
#include <thread>
#include <utility>

namespace {

struct Deps {
  const int *ia, *ja, *dg;
  bool fwd;
  int begin(int i) const { return fwd ? ia[i] : dg[i] + 1; }
  int end(int i) const { return fwd ? dg[i] : ia[i + 1]; }
};

}  // namespace

// recursive coordinate bisection of items (chains) weighted by rows into
// nparts parts; split along the axis of largest extent at the weighted
// median.  The two halves of the first levels are cut concurrently (they
// write disjoint entries of part_of).
static void rcb(std::vector<int>& items, const std::vector<double>& cx, const std::vector<double>& cy,
                const std::vector<double>& cz, const std::vector<int>& w, int nparts, int first_part,
                std::vector<int>& part_of, int depth = 0) {
  if (nparts <= 1 || items.size() <= 1) {
    for (int c : items) part_of[c] = first_part;
    return;
  }
  double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
  for (int c : items) {
    const double p[3] = {cx[c], cy[c], cz[c]};
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
  }
  int ax = 0;
  for (int a = 1; a < 3; ++a)
    if (hi[a] - lo[a] > hi[ax] - lo[ax]) ax = a;
  const std::vector<double>& key = ax == 0 ? cx : ax == 1 ? cy : cz;
  // stable sort by the coordinate, on (key, item) pairs kept together
  std::vector<std::pair<double, int>> kv(items.size());
  for (size_t q = 0; q < items.size(); ++q) kv[q] = {key[items[q]], items[q]};
  std::stable_sort(kv.begin(), kv.end(),
                   [](const std::pair<double, int>& a, const std::pair<double, int>& b) { return a.first < b.first; });
  for (size_t q = 0; q < kv.size(); ++q) items[q] = kv[q].second;
  const int nl = nparts / 2;
  long long tot = 0;
  for (int c : items) tot += w[c];
  const long long want = tot * nl / nparts;
  // cut at the widest coordinate gap among the positions whose left weight is
  // within half a part of the balanced cut, so that grid lines sharing a
  // coordinate stay on one side and the tile boundaries follow the mesh
  const long long tol = std::max<long long>(1, tot / nparts / 2);
  size_t cut = 0, best_near = 1;
  double best_gap = -1.0;
  long long acc = 0, best_dist = -1;
  for (size_t q = 1; q < items.size(); ++q) {
    acc += w[items[q - 1]];
    const long long dist = acc > want ? acc - want : want - acc;
    if (best_dist < 0 || dist < best_dist) { best_dist = dist; best_near = q; }
    if (dist <= tol) {
      const double gap = kv[q].first - kv[q - 1].first;
      if (gap > best_gap) { best_gap = gap; cut = q; }
    }
  }
  if (cut == 0) cut = best_near;
  cut = std::max<size_t>(1, std::min(cut, items.size() - 1));
  std::vector<int> left(items.begin(), items.begin() + cut), right(items.begin() + cut, items.end());
  kv.clear();
  kv.shrink_to_fit();
  if (depth < 3 && items.size() > 4096) {
    std::thread th([&]() { rcb(left, cx, cy, cz, w, nl, first_part, part_of, depth + 1); });
    rcb(right, cx, cy, cz, w, nparts - nl, first_part + nl, part_of, depth + 1);
    th.join();
  } else {
    rcb(left, cx, cy, cz, w, nl, first_part, part_of, depth + 1);
    rcb(right, cx, cy, cz, w, nparts - nl, first_part + nl, part_of, depth + 1);
  }
}

// runs body(lo, hi) over [0, n) in contiguous chunks on up to
// hardware_concurrency threads
template <class F>
static void parallel_chunks(int n, F body) {
  const int nt = std::max(1, std::min<int>((int)std::thread::hardware_concurrency(), std::max(1, n / 4)));
  if (nt <= 1) {
    body(0, n);
    return;
  }
  std::vector<std::thread> th;
  for (int k = 0; k < nt; ++k) {
    const int lo = (int)((long long)n * k / nt), hi = (int)((long long)n * (k + 1) / nt);
    th.emplace_back([&body, lo, hi]() { body(lo, hi); });
  }
  for (std::thread& t : th) t.join();
}

void build_sweep_schedule(int n, const int* ia, const int* ja, const int* dg, const std::vector<int>& lev, int nlev,
                          bool forward, int ntiles_target, const double* xyz, SweepSchedule& S,
                          std::vector<int>& code, bool with_waits) {
  S = SweepSchedule();
  S.n = n;
  S.nlev = nlev;
  const Deps D{ia, ja, dg, forward};
  // ---- 1. chains: a row continues the chain of its latest dependency
  std::vector<int> chain_of(n, -1), has_succ(n, 0);
  std::vector<int> chain_first;  // first row (in sweep order) of each chain
  std::vector<int> chain_rows;   // rows per chain
  for (int t = 0; t < n; ++t) {
    const int i = forward ? t : n - 1 - t;
    int best = -1;
    for (int k = D.begin(i); k < D.end(i); ++k) {
      const int j = ja[k];
      if (has_succ[j]) continue;
      if (best < 0 || lev[j] > lev[best] || (lev[j] == lev[best] && (forward ? j > best : j < best))) best = j;
    }
    if (best >= 0) {
      has_succ[best] = 1;
      chain_of[i] = chain_of[best];
      chain_rows[chain_of[i]]++;
    } else {
      chain_of[i] = (int)chain_first.size();
      chain_first.push_back(i);
      chain_rows.push_back(1);
    }
  }
  const int nch = (int)chain_first.size();
  // ---- 2. chain graph (undirected adjacency through dependencies), built
  //         only where the tiles are grown or merged over it: the coordinate
  //         bisection gives at most the target count by itself
  std::vector<int> adj_ptr, adj;
  auto chain_graph = [&]() {
    std::vector<std::pair<int, int>> edges;
    edges.reserve((size_t)n * 2);
    for (int i = 0; i < n; ++i)
      for (int k = D.begin(i); k < D.end(i); ++k) {
        const int a = chain_of[i], b = chain_of[ja[k]];
        if (a != b) { edges.push_back({a, b}); edges.push_back({b, a}); }
      }
    std::sort(edges.begin(), edges.end());
    edges.erase(std::unique(edges.begin(), edges.end()), edges.end());
    adj_ptr.assign(nch + 1, 0);
    for (auto& e : edges) adj_ptr[e.first + 1]++;
    for (int c = 0; c < nch; ++c) adj_ptr[c + 1] += adj_ptr[c];
    adj.resize(edges.size());
    for (size_t q = 0; q < edges.size(); ++q) adj[q] = edges[q].second;  // sorted by (first, second)
  };
  // ---- 3. tiles: grow regions over the chain graph in breadth-first order
  const int T = std::max(1, std::min(ntiles_target, nch));
  const long long target = (n + T - 1) / T;
  std::vector<int> tile_of_chain(nch, -1);
  std::vector<long long> tile_rows;
  if (xyz) {
    std::vector<double> cx(nch, 0.0), cy(nch, 0.0), cz(nch, 0.0);
    for (int i = 0; i < n; ++i) {
      const int c = chain_of[i];
      cx[c] += xyz[i]; cy[c] += xyz[n + i]; cz[c] += xyz[2 * (size_t)n + i];
    }
    for (int c = 0; c < nch; ++c) { cx[c] /= chain_rows[c]; cy[c] /= chain_rows[c]; cz[c] /= chain_rows[c]; }
    std::vector<int> items(nch);
    std::iota(items.begin(), items.end(), 0);
    rcb(items, cx, cy, cz, chain_rows, T, 0, tile_of_chain);
    // drop empty parts
    std::vector<int> used(T, 0);
    for (int c = 0; c < nch; ++c) used[tile_of_chain[c]] = 1;
    std::vector<int> nid(T, -1);
    int m = 0;
    for (int t = 0; t < T; ++t)
      if (used[t]) nid[t] = m++;
    for (int c = 0; c < nch; ++c) tile_of_chain[c] = nid[tile_of_chain[c]];
    tile_rows.assign(m, 0);
    for (int c = 0; c < nch; ++c) tile_rows[tile_of_chain[c]] += chain_rows[c];
  } else {
    chain_graph();
    std::deque<int> q;
    int next_seed = 0;
    while (true) {
      while (next_seed < nch && tile_of_chain[next_seed] >= 0) ++next_seed;
      if (next_seed >= nch) break;
      const int t = (int)tile_rows.size();
      tile_rows.push_back(0);
      q.clear();
      q.push_back(next_seed);
      tile_of_chain[next_seed] = t;
      while (!q.empty() && tile_rows[t] < target) {
        const int c = q.front();
        q.pop_front();
        if (tile_of_chain[c] != t) continue;
        tile_rows[t] += chain_rows[c];
        for (int e = adj_ptr[c]; e < adj_ptr[c + 1] && tile_rows[t] < target; ++e) {
          const int d = adj[e];
          if (tile_of_chain[d] < 0) { tile_of_chain[d] = t; q.push_back(d); }
        }
      }
      // chains queued but not consumed go back to the pool
      for (int c : q)
        if (tile_of_chain[c] == t) tile_of_chain[c] = -1;
    }
  }
  // every chain now has a tile; merge the smallest tiles until at most T remain
  int ntiles = (int)tile_rows.size();
  if (ntiles > T) {
    if (adj_ptr.empty()) chain_graph();
    std::vector<int> remap(ntiles);
    std::iota(remap.begin(), remap.end(), 0);
    auto find = [&](int x) { while (remap[x] != x) x = remap[x] = remap[remap[x]]; return x; };
    // tile adjacency through chain edges
    std::vector<std::pair<int, int>> tedges;
    for (int c = 0; c < nch; ++c)
      for (int e = adj_ptr[c]; e < adj_ptr[c + 1]; ++e) {
        int a = tile_of_chain[c], b = tile_of_chain[adj[e]];
        if (a != b) tedges.push_back({a, b});
      }
    std::sort(tedges.begin(), tedges.end());
    tedges.erase(std::unique(tedges.begin(), tedges.end()), tedges.end());
    int alive = ntiles;
    while (alive > T) {
      int small = -1;
      for (int t = 0; t < ntiles; ++t)
        if (find(t) == t && (small < 0 || tile_rows[t] < tile_rows[small])) small = t;
      int best = -1;
      for (auto& e : tedges) {
        if (find(e.first) != small) continue;
        int o = find(e.second);
        if (o != small && (best < 0 || tile_rows[o] < tile_rows[best])) best = o;
      }
      if (best < 0)  // isolated: merge into the smallest other tile
        for (int t = 0; t < ntiles; ++t)
          if (find(t) == t && t != small && (best < 0 || tile_rows[t] < tile_rows[best])) best = t;
      remap[small] = best;
      tile_rows[best] += tile_rows[small];
      --alive;
    }
    std::vector<int> newid(ntiles, -1);
    int m = 0;
    for (int t = 0; t < ntiles; ++t)
      if (find(t) == t) newid[t] = m++;
    for (int c = 0; c < nch; ++c) tile_of_chain[c] = newid[find(tile_of_chain[c])];
    ntiles = m;
  }
  S.ntiles = ntiles;
  // ---- 4. per tile: steps (distinct levels) and slots (chains sharing a slot
  //         when their level ranges do not overlap)
  std::vector<int> chain_lo(nch, 1 << 30), chain_hi(nch, -1);
  for (int i = 0; i < n; ++i) {
    const int c = chain_of[i];
    chain_lo[c] = std::min(chain_lo[c], lev[i]);
    chain_hi[c] = std::max(chain_hi[c], lev[i]);
  }
  std::vector<std::vector<int>> tile_chains(ntiles);
  for (int c = 0; c < nch; ++c) tile_chains[tile_of_chain[c]].push_back(c);
  std::vector<int> slot_of_chain(nch, 0);
  std::vector<int> row_tile(n), row_step(n), row_slot(n);
  // slots, tile by tile (concurrently): the chains in order of their first
  // level each take the free slot (its last chain ended before that level)
  // that was freed last, the lowest such slot on ties, else a new slot; the
  // free slots are kept ordered by (level after which free, -slot)
  S.tile_slots.assign(ntiles, 1);
  parallel_chunks(ntiles, [&](int t0, int t1) {
    for (int t = t0; t < t1; ++t) {
      auto& ch = tile_chains[t];
      std::sort(ch.begin(), ch.end(), [&](int a, int b) {
        return chain_lo[a] != chain_lo[b] ? chain_lo[a] < chain_lo[b] : a < b;
      });
      std::set<std::pair<int, int>> slot_free;
      int nslots = 0;
      for (int c : ch) {
        auto it = slot_free.lower_bound({chain_lo[c], std::numeric_limits<int>::min()});
        int sl;
        if (it != slot_free.begin()) {
          --it;
          sl = -it->second;
          slot_free.erase(it);
        } else {
          sl = nslots++;
        }
        slot_free.insert({chain_hi[c], -sl});
        slot_of_chain[c] = sl;
      }
      S.tile_slots[t] = std::max(1, nslots);
    }
  });
  for (int t = 0; t < ntiles; ++t) S.max_slots = std::max(S.max_slots, S.tile_slots[t]);
  // the distinct levels of every tile, ascending: marked in a (tile, level)
  // table that then maps a row's level to its step, or sorted per tile when
  // that table would be large
  std::vector<std::vector<int>> tile_levels(ntiles);
  const size_t tab_cells = (size_t)ntiles * (size_t)std::max(1, nlev);
  std::vector<int> step_tab;
  if (tab_cells <= ((size_t)1 << 24)) {
    step_tab.assign(tab_cells, -1);
    for (int i = 0; i < n; ++i) step_tab[(size_t)tile_of_chain[chain_of[i]] * nlev + lev[i]] = -2;
    for (int t = 0; t < ntiles; ++t) {
      int* tab = step_tab.data() + (size_t)t * nlev;
      for (int l = 0; l < nlev; ++l)
        if (tab[l] == -2) {
          tab[l] = (int)tile_levels[t].size();
          tile_levels[t].push_back(l);
        }
    }
  } else {
    for (int i = 0; i < n; ++i) tile_levels[tile_of_chain[chain_of[i]]].push_back(lev[i]);
    for (int t = 0; t < ntiles; ++t) {
      auto& L = tile_levels[t];
      std::sort(L.begin(), L.end());
      L.erase(std::unique(L.begin(), L.end()), L.end());
    }
  }
  S.R = std::max(1, std::min(4, (int)((160 * 1024) / (8LL * std::max(1, S.max_slots)))));
  S.tile_step_ptr.assign(ntiles + 1, 0);
  for (int t = 0; t < ntiles; ++t) S.tile_step_ptr[t + 1] = S.tile_step_ptr[t] + (int)tile_levels[t].size();
  const int nsteps = S.tile_step_ptr[ntiles];
  S.step_level.resize(nsteps);
  S.step_row_ptr.assign(nsteps + 1, 0);
  for (int t = 0; t < ntiles; ++t)
    for (size_t s = 0; s < tile_levels[t].size(); ++s) {
      const int gs = S.tile_step_ptr[t] + (int)s;
      S.step_level[gs] = tile_levels[t][s];
      S.step_row_ptr[gs + 1] = S.step_row_ptr[gs] + S.tile_slots[t];
    }
  S.rows.assign(S.step_row_ptr[nsteps], -1);
  // place every row (its tile's level -> step from the table, else by binary search)
  for (int i = 0; i < n; ++i) {
    const int t = tile_of_chain[chain_of[i]];
    int s;
    if (!step_tab.empty()) {
      s = step_tab[(size_t)t * nlev + lev[i]];
    } else {
      const auto& L = tile_levels[t];
      s = (int)(std::lower_bound(L.begin(), L.end(), lev[i]) - L.begin());
    }
    const int slot = slot_of_chain[chain_of[i]];
    row_tile[i] = t;
    row_step[i] = s;
    row_slot[i] = slot;
    S.rows[S.step_row_ptr[S.tile_step_ptr[t] + s] + slot] = i;
  }
  if (!with_waits) return;
  // ---- 5. entry codes and waits
  std::vector<std::vector<std::pair<int, int>>> waits(nsteps);
  for (int i = 0; i < n; ++i) {
    const int t = row_tile[i], s = row_step[i];
    const int gs = S.tile_step_ptr[t] + s;
    for (int k = D.begin(i); k < D.end(i); ++k) {
      const int j = ja[k];
      if (row_tile[j] == t && s - row_step[j] < S.R) {
        code[k] = (row_step[j] % S.R) * S.tile_slots[t] + row_slot[j];
        S.ring_entries++;
      } else {
        code[k] = -j - 2;
        if (row_tile[j] != t) {
          waits[gs].push_back({row_tile[j], lev[j] + 1});
          S.cross_tile_entries++;
        } else {
          S.global_same_tile_entries++;
        }
      }
    }
  }
  S.wait_ptr.assign(nsteps + 1, 0);
  for (int gs = 0; gs < nsteps; ++gs) {
    auto& w = waits[gs];
    std::sort(w.begin(), w.end());
    // keep the largest requirement per producer tile
    std::vector<std::pair<int, int>> m;
    for (auto& p : w) {
      if (!m.empty() && m.back().first == p.first) m.back().second = std::max(m.back().second, p.second);
      else m.push_back(p);
    }
    for (auto& p : m) { S.wait_tile.push_back(p.first); S.wait_level.push_back(p.second); }
    S.wait_ptr[gs + 1] = (int)S.wait_tile.size();
  }
}

// Critical-path estimate of a sweep: every step of a tile costs
// tau0 + per_row * (rows in the step); a step starts when the tile's previous
// step is done and, for each producer it waits on, hop microseconds after the
// producer published the needed progress.  Returns microseconds.
double estimate_sweep_us(const SweepSchedule& S, double tau0, double per_row, double hop) {
  std::vector<std::vector<double>> pub(S.ntiles);
  std::vector<int> cur(S.ntiles, 0);
  // steps of all tiles in level order (a valid processing order)
  std::vector<std::pair<int, int>> order;  // (level, global step)
  for (int t = 0; t < S.ntiles; ++t)
    for (int gs = S.tile_step_ptr[t]; gs < S.tile_step_ptr[t + 1]; ++gs) order.push_back({S.step_level[gs], gs});
  std::sort(order.begin(), order.end());
  std::vector<int> tile_of_step(S.step_level.size());
  for (int t = 0; t < S.ntiles; ++t)
    for (int gs = S.tile_step_ptr[t]; gs < S.tile_step_ptr[t + 1]; ++gs) tile_of_step[gs] = t;
  double tmax = 0.0;
  for (auto& o : order) {
    const int gs = o.second, t = tile_of_step[gs];
    double st = pub[t].empty() ? 0.0 : pub[t].back();
    for (int w = S.wait_ptr[gs]; w < S.wait_ptr[gs + 1]; ++w) {
      const int q = S.wait_tile[w], need = S.wait_level[w];
      const int q0 = S.tile_step_ptr[q];
      // first published step of q whose next level reaches need
      int lo = 0, hi = (int)pub[q].size() - 1, found = -1;
      while (lo <= hi) {
        const int mid = (lo + hi) / 2;
        const int nxt = (q0 + mid + 1 < S.tile_step_ptr[q + 1]) ? S.step_level[q0 + mid + 1] : S.nlev;
        if (nxt >= need) { found = mid; hi = mid - 1; } else lo = mid + 1;
      }
      if (found >= 0) st = std::max(st, pub[q][found] + hop);
    }
    int rowsn = 0;
    for (int sl = 0; sl < S.tile_slots[t]; ++sl) rowsn += S.rows[S.step_row_ptr[gs] + sl] >= 0;
    const double end = st + tau0 + per_row * rowsn;
    pub[t].push_back(end);
    tmax = std::max(tmax, end);
  }
  return tmax;
}

// ---------------------------------------------------------------------------
int pick_sweep_tiles(int n, const int* ia, const int* ja, const int* dg, const double* xyz, const std::vector<int>& cand,
                     double tau0, double per_row, double hop, double* best_est) {
  std::vector<int> lev;
  const int nls = symmetric_levels(n, ia, ja, dg, lev);
  const int nc = (int)cand.size();
  std::vector<double> est(nc, 1e300);
  auto trial = [&](int c) {
    std::vector<int> code(ia[n], 0);
    SweepSchedule S;
    build_sweep_schedule(n, ia, ja, dg, lev, nls, true, cand[c], xyz, S, code);
    est[c] = estimate_sweep_us(S, tau0, per_row, hop);
  };
  std::vector<std::thread> th;
  for (int c = 0; c < nc; ++c) {
    if (cand[c] < 1) continue;
    bool dup = false;
    for (int d = 0; d < c; ++d) dup = dup || cand[d] == cand[c];
    if (dup) continue;
    th.emplace_back(trial, c);
  }
  for (std::thread& t : th) t.join();
  int best = -1;
  for (int c = 0; c < nc; ++c)
    if (best < 0 || est[c] < est[best]) best = c;
  if (best_est) *best_est = best >= 0 ? est[best] : 0.0;
  return best >= 0 && est[best] < 1e300 ? cand[best] : (nc ? std::max(1, cand[0]) : 1);
}

int symmetric_levels(int n, const int* ia, const int* ja, const int* dg, std::vector<int>& lev) {
  lev.assign(n, 0);
  for (int i = 0; i < n; ++i) {
    int l = lev[i];
    for (int k = ia[i]; k < dg[i]; ++k) l = std::max(l, lev[ja[k]] + 1);
    lev[i] = l;
    for (int k = dg[i] + 1; k < ia[i + 1]; ++k) lev[ja[k]] = std::max(lev[ja[k]], l + 1);
  }
  int nlev = 0;
  for (int i = 0; i < n; ++i) nlev = std::max(nlev, lev[i] + 1);
  return nlev;
}

// Splits the rows of every (tile, level) step wider than wmax into sub-levels:
// lev(i) becomes lev(i) * M + chunk(i), chunk = rank of the row in its step /
// wmax, then the levels are renumbered densely.  Rows of one level do not
// depend on each other, so every dependency still points to a lower level.
// The tiling is recomputed from the new levels (it may move rows between
// tiles), so the split is repeated until no step is wider than wmax (a few
// passes).  Returns the number of levels.
static int split_wide_levels(int n, const int* ia, const int* ja, const int* dg, int ntiles, const double* xyz,
                             int wmax, std::vector<int>& lev, int nlev) {
  std::vector<int> code_tmp;  // not written by a layout-only build
  for (int pass = 0; pass < 8; ++pass) {
    SweepSchedule T;
    build_sweep_schedule(n, ia, ja, dg, lev, nlev, true, ntiles, xyz, T, code_tmp, false);
    std::vector<int> chunk(n, 0);
    int maxc = 0;
    const int nsteps = T.tile_step_ptr[T.ntiles];
    for (int gs = 0; gs < nsteps; ++gs) {
      int cnt = 0;
      for (int q = T.step_row_ptr[gs]; q < T.step_row_ptr[gs + 1]; ++q) {
        const int i = T.rows[q];
        if (i < 0) continue;
        chunk[i] = cnt / wmax;
        ++cnt;
      }
      maxc = std::max(maxc, (cnt - 1) / wmax);
    }
    if (maxc == 0) break;
    const long long M = maxc + 1;
    if ((long long)nlev * M <= (1LL << 26)) {
      // dense ranks of the keys lev * M + chunk through a table of all keys
      std::vector<int> rank((size_t)nlev * M, 0);
      for (int i = 0; i < n; ++i) rank[(size_t)lev[i] * M + chunk[i]] = 1;
      int r = 0;
      for (int& v : rank) v = v ? r++ : -1;
      for (int i = 0; i < n; ++i) lev[i] = rank[(size_t)lev[i] * M + chunk[i]];
      nlev = r;
    } else {
      std::vector<long long> key(n);
      for (int i = 0; i < n; ++i) key[i] = (long long)lev[i] * M + chunk[i];
      std::vector<long long> uk(key);
      std::sort(uk.begin(), uk.end());
      uk.erase(std::unique(uk.begin(), uk.end()), uk.end());
      for (int i = 0; i < n; ++i) lev[i] = (int)(std::lower_bound(uk.begin(), uk.end(), key[i]) - uk.begin());
      nlev = (int)uk.size();
    }
  }
  return nlev;
}

bool build_ordered_sweep(int n, const int* ia, const int* ja, const int* dg, const int* ts, int ntiles,
                         const double* xyz, int R, OrderedSweep& O, SweepSchedule& S, std::string& err, int wmax) {
  O = OrderedSweep();
  O.n = n;
  O.R = std::max(2, R);
  std::vector<int> lev;
  int nlev = symmetric_levels(n, ia, ja, dg, lev);
  if (wmax > 0) nlev = split_wide_levels(n, ia, ja, dg, ntiles, xyz, wmax, lev, nlev);
  O.nlev = nlev;
  std::vector<int> code_tmp((size_t)ia[n], 0);
  build_sweep_schedule(n, ia, ja, dg, lev, nlev, true, ntiles, xyz, S, code_tmp);
  // ---- new numbering: tile, step, slot order, empty slots dropped
  const int T = S.ntiles;
  O.ntiles = T;
  O.nsteps = S.tile_step_ptr[T];
  O.tile_step_ptr = S.tile_step_ptr;
  O.step_ptr.assign(O.nsteps + 1, 0);
  O.tile_W.assign(T, 1);
  O.perm.reserve(n);
  O.iperm.assign(n, -1);
  // per old row: new index, tile, step within the tile, position in the
  // step, kept together so that a dependency costs one cache line
  struct RowInfo { int q, tile, ls, pos; };
  std::vector<RowInfo> rinfo(n);
  std::vector<int> row_tile(n), row_ls(n);
  for (int t = 0; t < T; ++t) {
    O.max_tile_steps = std::max(O.max_tile_steps, S.tile_step_ptr[t + 1] - S.tile_step_ptr[t]);
    for (int gs = S.tile_step_ptr[t]; gs < S.tile_step_ptr[t + 1]; ++gs) {
      O.step_ptr[gs] = (int)O.perm.size();
      int pos = 0;
      for (int q = S.step_row_ptr[gs]; q < S.step_row_ptr[gs + 1]; ++q) {
        const int i = S.rows[q];
        if (i < 0) continue;
        O.iperm[i] = (int)O.perm.size();
        O.perm.push_back(i);
        row_tile[i] = t;
        row_ls[i] = gs - S.tile_step_ptr[t];
        rinfo[i] = {O.iperm[i], t, row_ls[i], pos++};
      }
      O.tile_W[t] = std::max(O.tile_W[t], pos);
    }
  }
  O.step_ptr[O.nsteps] = (int)O.perm.size();
  if ((int)O.perm.size() != n) { err = "ordered sweep: schedule does not cover every row once"; return false; }
  for (int t = 0; t < T; ++t) O.maxW = std::max(O.maxW, O.tile_W[t]);
  const int nE = (n + 3) & ~3;
  O.nE = nE;
  const size_t E = (size_t)FC_ELL * nE;
  // ---- per triangle: entries, codes, exchange and push blocks
  std::vector<int> row_step(n);  // global step of every new row
  for (int gs = 0; gs < O.nsteps; ++gs)
    for (int q = O.step_ptr[gs]; q < O.step_ptr[gs + 1]; ++q) row_step[q] = gs;
  // the two triangles are independent: built concurrently
  auto build_dir = [&](int dirn, std::string& derr) -> bool {
    OrderedDir& D = O.dir[dirn];
    D.ne.assign(nE, 0);
    D.slot.assign(E, -1);
    D.col.assign(E, 0);
    D.srec.assign((size_t)4 * nE, 0);
    D.ovf_ptr.assign(n + 1, 0);
    for (int q = 0; q < n; ++q) {
      const int i = O.perm[q];
      const int k0 = dirn == 0 ? ia[i] : dg[i] + 1, k1 = dirn == 0 ? dg[i] : ia[i + 1];
      D.ne[q] = k1 - k0;
      D.ovf_ptr[q + 1] = D.ovf_ptr[q] + std::max(0, k1 - k0 - FC_ELL);
    }
    const int novf = D.ovf_ptr[n];
    D.ovf_slot.assign(novf, -1);
    D.ovf_code.assign(novf, 0);
    D.ovf_col.assign(novf, 0);
    std::vector<int> nx(n, 0);  // exchange slots of each consumer row
    // pushes in the order they arise (consumer row ascending, entries in CSR
    // order): producer row, consumer row, the consumer's slot number; grouped
    // by producer below (a counting sort keeps that order within a producer)
    std::vector<int> push_src, push_dst, push_m;
    for (int q = 0; q < n; ++q) {
      const int i = O.perm[q], t = row_tile[i];
      const int nst = S.tile_step_ptr[t + 1] - S.tile_step_ptr[t];
      const int W = O.tile_W[t];
      const int my = dirn == 0 ? row_ls[i] : nst - 1 - row_ls[i];
      const int k0 = dirn == 0 ? ia[i] : dg[i] + 1;
      int codes[FC_ELL] = {0, 0, 0, 0};
      for (int e = 0; e < D.ne[q]; ++e) {
        const int k = k0 + e, j = ja[k];
        const RowInfo rj = rinfo[j];
        const int qj = rj.q;
        int c;
        if (rj.tile == t) {
          const int pj = dirn == 0 ? rj.ls : nst - 1 - rj.ls;
          if (pj >= my) { derr = "ordered sweep: dependency not before its consumer in the tile"; return false; }
          if (my - pj <= O.R - 1) c = (pj % O.R) * W + rj.pos;
          else c = -1;
        } else {
          c = -1;
          D.cross_tile_entries++;
        }
        if (c > 65534) { derr = "ordered sweep: ring index does not fit 16 bits"; return false; }
        if (c < 0) {
          push_src.push_back(qj);
          push_dst.push_back(q);
          push_m.push_back(nx[q]++);
          D.pushed_entries++;
        } else {
          D.ring_entries++;
        }
        if (e < FC_ELL) {
          D.slot[(size_t)e * nE + q] = k;
          D.col[(size_t)e * nE + q] = qj;
          codes[e] = c + 1;
        } else {
          const int o = D.ovf_ptr[q] + e - FC_ELL;
          D.ovf_slot[o] = k;
          D.ovf_code[o] = c;
          D.ovf_col[o] = qj;
        }
      }
      D.srec[4 * (size_t)q + 2] = codes[0] | (codes[1] << 16);
      D.srec[4 * (size_t)q + 3] = codes[2] | (codes[3] << 16);
    }
    std::vector<int> cons_ptr(n + 1, 0), cons_q(push_src.size()), cons_m(push_src.size());
    for (int qj : push_src) cons_ptr[qj + 1]++;
    for (int q = 0; q < n; ++q) cons_ptr[q + 1] += cons_ptr[q];
    {
      std::vector<int> fill(cons_ptr.begin(), cons_ptr.end() - 1);
      for (size_t u = 0; u < push_src.size(); ++u) {
        const int o = fill[push_src[u]]++;
        cons_q[o] = push_dst[u];
        cons_m[o] = push_m[u];
      }
    }
    std::vector<int>().swap(push_src);
    std::vector<int>().swap(push_dst);
    std::vector<int>().swap(push_m);
    // exchange blocks (consumer side) and push blocks (producer side), one
    // per step, each starting on a multiple of 4 elements
    D.xv_ptr.assign(O.nsteps + 1, 0);
    D.push_ptr.assign(O.nsteps + 1, 0);
    std::vector<int> xoff(n, 0), poff(n, 0);
    for (int gs = 0; gs < O.nsteps; ++gs) {
      int xs = 0, ps = 0;
      for (int q = O.step_ptr[gs]; q < O.step_ptr[gs + 1]; ++q) {
        xoff[q] = xs;
        poff[q] = ps;
        xs += nx[q];
        ps += cons_ptr[q + 1] - cons_ptr[q];
      }
      if (xs > 65535 || ps > (1 << 30)) { derr = "ordered sweep: exchange block of a step too large"; return false; }
      D.xv_ptr[gs + 1] = D.xv_ptr[gs] + ((xs + 3) & ~3);
      D.push_ptr[gs + 1] = D.push_ptr[gs] + ((ps + 3) & ~3);
    }
    D.push.assign(D.push_ptr[O.nsteps], 0);
    for (int q = 0; q < n; ++q) {
      const int np = cons_ptr[q + 1] - cons_ptr[q];
      if (nx[q] > 255 || np > 255) { derr = "ordered sweep: more than 255 exchanged entries in a row"; return false; }
      D.srec[4 * (size_t)q] = D.ne[q] | (np << 8) | (xoff[q] << 16);
      D.srec[4 * (size_t)q + 1] = poff[q];
      for (int m = 0; m < np; ++m) {
        const int qc = cons_q[cons_ptr[q] + m], mc = cons_m[cons_ptr[q] + m];
        D.push[D.push_ptr[row_step[q]] + poff[q] + m] = D.xv_ptr[row_step[qc]] + xoff[qc] + mc;
      }
    }
    return true;
  };
  std::string err1;
  bool ok1 = true;
  std::thread th1([&]() { ok1 = build_dir(1, err1); });
  const bool ok0 = build_dir(0, err);
  th1.join();
  if (!ok0) return false;
  if (!ok1) { err = err1; return false; }
  // ---- DILU transpose slots of the lower entries, diagonal slots, matrix
  O.lo_tslot.assign(E, 0);
  O.lo_ovf_tslot.assign(O.dir[0].ovf_ptr[n], 0);
  O.dslot.assign(nE, 0);
  O.p_ptr.assign(n + 1, 0);
  for (int q = 0; q < n; ++q) {
    const int i = O.perm[q];
    O.dslot[q] = dg[i];
    O.p_ptr[q + 1] = O.p_ptr[q] + (ia[i + 1] - ia[i]);
    for (int e = 0; e < O.dir[0].ne[q]; ++e) {
      const int k = ia[i] + e;
      const int tsk = ts ? ts[k] : k;
      if (e < FC_ELL) O.lo_tslot[(size_t)e * nE + q] = tsk;
      else O.lo_ovf_tslot[O.dir[0].ovf_ptr[q] + e - FC_ELL] = tsk;
    }
  }
  O.p_col.resize(ia[n]);
  O.p_slot.resize(ia[n]);
  for (int q = 0; q < n; ++q) {
    const int i = O.perm[q];
    int o = O.p_ptr[q];
    for (int k = ia[i]; k < ia[i + 1]; ++k, ++o) {
      O.p_col[o] = O.iperm[ja[k]];
      O.p_slot[o] = k;
    }
  }
  return true;
}
