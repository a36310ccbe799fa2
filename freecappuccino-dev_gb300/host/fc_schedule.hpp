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
#include <string>
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
// coordinates the tiles are grown over the chain graph.  with_waits false
// stops after the layout (tiles, steps, rows): code, the waits and the entry
// counts are left empty.
void build_sweep_schedule(int n, const int* ia, const int* ja, const int* dg, const std::vector<int>& lev, int nlev,
                          bool forward, int ntiles, const double* xyz, SweepSchedule& S, std::vector<int>& code,
                          bool with_waits = true);

// Critical-path estimate (microseconds) of a schedule: per step tau0 +
// per_row * rows, cross-tile waits delayed by hop after publication.
double estimate_sweep_us(const SweepSchedule& S, double tau0, double per_row, double hop);

// ---------------------------------------------------------------------------
// Schedule-ordered sweep structure.
//
// The rows are renumbered in schedule order: tile by tile, step by step, so
// that every step of every tile is a contiguous range of new row indices and
// a thread block walks consecutive memory.  The forward sweep runs the steps
// of a tile in order, the backward sweep runs them in reverse; this is valid
// for both triangles because the levels are taken over the symmetrised
// pattern (row i waits for every j < i with a_ij != 0 or a_ji != 0).
//
// Per new row and per triangle the first FC_ELL entries (in the row's CSR
// order) are stored column-major (entry e of row q at e*nE + q, nE = n
// rounded up to a multiple of 4 so that every column starts 16-byte
// aligned), the rest in an overflow list.  A dependency produced in the same tile within the last
// R-1 steps is read from the block's shared-memory ring (code >= 0: ring
// index (local step % R) * W + position); every other dependency is pushed:
// its producer stores the value into the consumer's own slot of an exchange
// array xv.  The slots of a step's rows form one contiguous block of xv (in
// row order, entries in CSR order), so the consumer fetches all values the
// step needs with one copy; the producer's targets likewise form one block
// per producing step.
#define FC_ELL 4

struct OrderedDir {
  std::vector<int> ne;        // [nE] entries of this triangle in the row
  std::vector<int> slot;      // [FC_ELL*nE] original CSR slot, -1 past ne (coefficient gather)
  std::vector<int> col;       // [FC_ELL*nE] new index of the entry's column
  // [4*nE] packed row record, one 16-byte load per row:
  //   [0] ne | np << 8 | xoff << 16   (np: pushes of the row's value; xoff:
  //       first exchange slot of the row in its step's exchange block)
  //   [1] poff: first push target of the row in its step's push block
  //   [2], [3] codes of entries 0..3, 16 bits each, stored as code + 1
  //       (0: the value arrives through the exchange block)
  std::vector<int> srec;
  std::vector<int> xv_ptr;    // [nsteps+1] exchange block of each step (multiples of 4)
  std::vector<int> push_ptr;  // [nsteps+1] push block of each step (multiples of 4)
  std::vector<int> push;      // absolute exchange positions the values are pushed to
  std::vector<int> ovf_ptr;   // [n+1] entries e >= FC_ELL
  std::vector<int> ovf_slot, ovf_code, ovf_col;
  long long ring_entries = 0, pushed_entries = 0, cross_tile_entries = 0;
};

struct OrderedSweep {
  int n = 0, nE = 0, ntiles = 0, nsteps = 0, nlev = 0, R = 4, maxW = 0, max_tile_steps = 0;
  std::vector<int> perm, iperm;    // new -> old, old -> new
  std::vector<int> tile_step_ptr;  // [ntiles+1]
  std::vector<int> step_ptr;       // [nsteps+1] first new row of each step
  std::vector<int> tile_W;         // widest step of each tile (ring / staging width)
  OrderedDir dir[2];               // 0: left of the diagonal (forward), 1: right (backward)
  std::vector<int> lo_tslot;       // [FC_ELL*nE] transpose slot of each lower entry (DILU)
  std::vector<int> lo_ovf_tslot;
  std::vector<int> dslot;          // [nE] original diagonal slot (0 in the padding)
  std::vector<int> p_ptr, p_col, p_slot;  // the matrix in new numbering, entries in original order
};

// levels over the symmetrised lower triangle: lev(i) = 1 + max lev(j) over
// j < i with a_ij != 0 or a_ji != 0; returns the number of levels
int symmetric_levels(int n, const int* ia, const int* ja, const int* dg, std::vector<int>& lev);

// The tile count among cand whose forward schedule has the smallest
// critical-path estimate (the trials are built concurrently, one thread
// each; ties go to the earlier candidate, duplicates and counts < 1 are
// skipped).  best_est (optional) receives that estimate.
int pick_sweep_tiles(int n, const int* ia, const int* ja, const int* dg, const double* xyz, const std::vector<int>& cand,
                     double tau0, double per_row, double hop, double* best_est);

// ia, ja, dg 0-based; ts (optional) the transpose slot of every entry;
// ntiles the tile target; xyz (optional) row coordinates for the tiling; R
// the ring depth; wmax > 0 caps the rows of a step (a wider level of a tile
// is split into consecutive steps, whose rows are independent).  S receives
// the underlying tiled schedule (for the critical-path estimate).  Returns
// false with a message if a consistency check fails.
bool build_ordered_sweep(int n, const int* ia, const int* ja, const int* dg, const int* ts, int ntiles,
                         const double* xyz, int R, OrderedSweep& O, SweepSchedule& S, std::string& err,
                         int wmax = 0);
