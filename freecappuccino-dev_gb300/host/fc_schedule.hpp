// Tiled pipeline schedule of a sparse triangular sweep (forward over the
// entries left of the diagonal, or backward over those right of it).
//
// The rows are cut into dependency chains (each row continues the chain of
// its most recent dependency, so on a naturally ordered structured mesh the
// chains are the grid lines along the fastest index), the chains are grouped
// into tiles of about n/T rows by growing regions over the chain graph, and
// every tile is given to one thread block.  A block walks its rows level by
// level: rows of one level are independent, values produced inside the tile
// in the last R steps are read from a shared-memory ring, everything else
// from global memory after the producing tile has published enough progress.
#pragma once
#include <vector>

struct SweepSchedule {
  int n = 0;
  int ntiles = 0;
  int nlev = 0;                    // levels of the sweep (0..nlev-1)
  int R = 4;                       // shared-memory ring depth in steps
  int max_slots = 0;               // widest tile (rows of one tile in one level)
  std::vector<int> tile_step_ptr;  // tile t owns global steps [ptr[t], ptr[t+1])
  std::vector<int> step_level;     // level of each global step
  std::vector<int> tile_slots;     // rows per step (padded width) of each tile
  std::vector<int> step_row_ptr;   // offset of each global step's padded row list
  std::vector<int> rows;           // padded row ids, -1 = empty slot
  std::vector<int> kbne;           // per padded slot: first swept CSR entry << 4 | min(entries, 15)
  std::vector<int> wait_ptr;       // per global step: waits [ptr[s], ptr[s+1])
  std::vector<int> wait_tile;      // producer tile of a wait
  std::vector<int> wait_level;     // producer must have published progress >= this level
  // per CSR entry of the swept part: >= 0 ring index (step%R)*slots+slot of
  // the producing row in the same tile, < 0 global row -(code)-2
  std::vector<int> code;           // size nnz, entries of the other part untouched
  long long cross_tile_entries = 0, ring_entries = 0, global_same_tile_entries = 0;
};

// ia, ja, dg: 0-based CSR (sorted rows) and diagonal positions; lev: level of
// every row for the direction (forward: from the lower part, backward: from
// the upper part); code must have nnz entries (shared between directions).
// xyz (optional, 3*n: x,y,z of every row, e.g. the cell centroids) lets the
// tiles be cut by recursive coordinate bisection of the chain centroids:
// dependencies along the mesh then run one way between tiles, so tiles
// pipeline instead of waiting on each other at every level.  Without
// coordinates the tiles are grown over the chain graph.
void build_sweep_schedule(int n, const int* ia, const int* ja, const int* dg, const std::vector<int>& lev, int nlev,
                          bool forward, int ntiles, const double* xyz, SweepSchedule& S, std::vector<int>& code);

// Critical-path estimate (microseconds) of a schedule: per step tau0 +
// per_row * rows, cross-tile waits delayed by hop after publication.
double estimate_sweep_us(const SweepSchedule& S, double tau0, double per_row, double hop);
