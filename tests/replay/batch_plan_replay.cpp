// Runs the batch planner (host/fc_batch_plan.cpp) on problems read from
// stdin: "budget gmax min_rows np" then np lines "rows levels weight".
// Prints the tiles per problem on one line, then the predicted makespan.
#include <cstdio>
#include <vector>

#include "fc_batch_plan.hpp"

int main() {
  int budget = 0, gmax = 0, min_rows = 0, np = 0;
  if (std::scanf("%d %d %d %d", &budget, &gmax, &min_rows, &np) != 4) return 2;
  std::vector<BatchCost> c(np);
  for (auto& x : c)
    if (std::scanf("%lf %lf %lf", &x.rows, &x.levels, &x.weight) != 3) return 2;
  const std::vector<int> g = plan_batch_groups(c, budget, gmax, min_rows);
  for (size_t p = 0; p < g.size(); ++p) std::printf("%s%d", p ? " " : "", g[p]);
  std::printf("\n%.17g\n", g.empty() ? -1.0 : batch_makespan_us(c, g));
  for (int p = 0; p < np; ++p)
    for (int t = 1; t <= 4; ++t) std::printf("%.17g%s", batch_iteration_us(c[p], t), t == 4 ? "\n" : " ");
  return 0;
}
