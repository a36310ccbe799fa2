#include "fc_batch_plan.hpp"

#include <algorithm>
#include <queue>
#include <utility>

namespace {
// per step of a sweep, per row of a tile's sweep, per row of the vector
// passes of one block (microseconds), per group reduction
constexpr double kStepUs = 0.15;
constexpr double kSweepRowUs = 0.001;
constexpr double kVecRowUs = 0.003;
constexpr double kReduceUs = 2.0;
constexpr int kReductions = 6;
constexpr int kSweeps = 4;
}  // namespace

double batch_iteration_us(const BatchCost& c, int g) {
  const double per_block = c.rows / std::max(1, g);
  return kSweeps * (c.levels * kStepUs + per_block * kSweepRowUs) + per_block * kVecRowUs + kReductions * kReduceUs;
}

double batch_makespan_us(const std::vector<BatchCost>& c, const std::vector<int>& g) {
  double m = 0.0;
  for (size_t p = 0; p < c.size() && p < g.size(); ++p) m = std::max(m, c[p].weight * batch_iteration_us(c[p], g[p]));
  return m;
}

std::vector<int> plan_batch_groups(const std::vector<BatchCost>& c, int budget, int gmax, int min_rows) {
  const int np = (int)c.size();
  if (np == 0 || np > budget) return {};
  std::vector<int> g(np, 1), cap(np, 1);
  for (int p = 0; p < np; ++p) {
    const int by_rows = min_rows > 0 ? (int)(c[p].rows / min_rows) : gmax;
    cap[p] = std::max(1, std::min(gmax, by_rows));
  }
  // max-heap on predicted time; ties go to the lower problem index
  using Entry = std::pair<double, int>;
  auto cmp = [](const Entry& a, const Entry& b) { return a.first < b.first || (a.first == b.first && a.second > b.second); };
  std::priority_queue<Entry, std::vector<Entry>, decltype(cmp)> heap(cmp);
  for (int p = 0; p < np; ++p) heap.push({c[p].weight * batch_iteration_us(c[p], 1), p});
  int left = budget - np;
  while (left > 0 && !heap.empty()) {
    const Entry top = heap.top();
    const int p = top.second;
    if (g[p] >= cap[p]) break;  // the slowest problem cannot get faster
    const double t1 = c[p].weight * batch_iteration_us(c[p], g[p] + 1);
    if (!(t1 < top.first)) break;
    heap.pop();
    ++g[p];
    --left;
    heap.push({t1, p});
  }
  return g;
}
