// Block partition of a batched persistent solve.
//
// A batched launch solves independent sparse systems at once: the launch
// grid (one resident block per SM) is split into groups, group p runs
// problem p's BiCGStab with its own sweep schedule (one tile per block),
// barrier and reductions.  The reference has no counterpart; it solves such
// systems one csrsolve call after another (e.g. the u, v, w momentum solves
// of calcuvw, velocity.f90:638, :693, :748).
//
// The planner picks the group sizes.  Its model of one iteration of a
// problem on g blocks: four triangular sweeps, each a chain of level steps
// (levels x tau0) plus the rows of a tile (rows / g x per-row cost), vector
// passes over rows / g rows per block, and a fixed cost per group
// reduction.  A weight per problem scales the model: 1 for a plan from the
// model alone, measured time / modelled iteration time for a tuned plan.
#pragma once
#include <vector>

struct BatchCost {
  double rows = 0;     // rows of the system
  double levels = 0;   // depth of the level sets of its triangular sweeps
  double weight = 1;   // iterations x calibration of the model
};

// modelled microseconds of one BiCGStab iteration on g blocks
double batch_iteration_us(const BatchCost& c, int g);

// Group sizes g_p >= 1 with sum g_p <= budget and g_p <= min(gmax, rows /
// min_rows) (at least 1): blocks go one at a time to the problem with the
// largest weight x batch_iteration_us while one more block shortens it.
// Empty when the problems outnumber the budget.
std::vector<int> plan_batch_groups(const std::vector<BatchCost>& c, int budget, int gmax, int min_rows);

// predicted time of the batch under a plan: the slowest group
double batch_makespan_us(const std::vector<BatchCost>& c, const std::vector<int>& g);
