// Greedy multicolouring and the per-colour ELLPACK layout of the coloured
// matrix (see fc_colour.hpp).
#include "fc_colour.hpp"

#include <algorithm>

bool build_coloured(int n, const int* ia, const int* ja, const int* dg, ColouredLayout& L, std::string* err) {
  L = ColouredLayout();
  L.n = n;
  auto fail = [&](const char* m) {
    if (err) *err = m;
    return false;
  };
  // adjacency of A + A^T without the diagonal
  std::vector<int> ptr(n + 1, 0);
  for (int i = 0; i < n; ++i)
    for (int k = ia[i]; k < ia[i + 1]; ++k) {
      const int j = ja[k];
      if (j == i) continue;
      if (j < 0 || j >= n) return fail("column index out of range");
      ptr[i + 1]++;
      ptr[j + 1]++;
    }
  for (int i = 0; i < n; ++i) ptr[i + 1] += ptr[i];
  std::vector<int> adj(ptr[n]);
  {
    std::vector<int> pos(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < n; ++i)
      for (int k = ia[i]; k < ia[i + 1]; ++k) {
        const int j = ja[k];
        if (j == i) continue;
        adj[pos[i]++] = j;
        adj[pos[j]++] = i;
      }
  }
  // greedy colouring in the original row order: the smallest colour no
  // earlier neighbour holds (on a structured hex mesh this is the red-black
  // checkerboard)
  std::vector<int> colour(n, -1), mark(FC_MC_MAXCOL, -1);
  int ncol = 0;
  for (int i = 0; i < n; ++i) {
    for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
      const int c = colour[adj[q]];
      if (c >= 0) mark[c] = i;
    }
    int c = 0;
    while (c < FC_MC_MAXCOL && mark[c] == i) ++c;
    if (c == FC_MC_MAXCOL) return fail("more colours than FC_MC_MAXCOL");
    colour[i] = c;
    ncol = std::max(ncol, c + 1);
  }
  if (n == 0) ncol = 0;
  L.ncol = ncol;
  // coloured numbering: colour by colour, original order inside a colour,
  // every colour padded to whole slices
  std::vector<int> count(ncol, 0);
  for (int i = 0; i < n; ++i) count[colour[i]]++;
  L.cslice.assign(ncol + 1, 0);
  for (int c = 0; c < ncol; ++c) L.cslice[c + 1] = L.cslice[c] + (count[c] + FC_MC_SLICE - 1) / FC_MC_SLICE;
  L.nslices = L.cslice[ncol];
  L.nP = L.nslices * FC_MC_SLICE;
  L.perm.assign(L.nP, -1);
  L.iperm.assign(n, -1);
  {
    std::vector<int> next(ncol);
    for (int c = 0; c < ncol; ++c) next[c] = L.cslice[c] * FC_MC_SLICE;
    for (int i = 0; i < n; ++i) {
      const int r = next[colour[i]]++;
      L.perm[r] = i;
      L.iperm[i] = r;
    }
  }
  // per row: its lower-colour and higher-colour entries, each in CSR order
  L.rowinfo.assign(L.nP, 0);
  L.dslot.assign(L.nP, -1);
  L.cwl.assign(ncol, 0);
  L.cwu.assign(ncol, 0);
  L.cel.assign(ncol, 0);
  L.ceu.assign(ncol, 0);
  long long next_e = 0;
  for (int c = 0; c < ncol; ++c) {
    int wl = 0, wu = 0;
    const int r0 = L.cslice[c] * FC_MC_SLICE, rows = (L.cslice[c + 1] - L.cslice[c]) * FC_MC_SLICE;
    for (int r = r0; r < r0 + rows; ++r) {
      const int i = L.perm[r];
      if (i < 0) continue;
      int nlo = 0, ne = 0;
      for (int k = ia[i]; k < ia[i + 1]; ++k) {
        const int j = ja[k];
        if (j == i) continue;
        ++ne;
        if (colour[j] < colour[i]) ++nlo;
      }
      if (ne > 0xFFFF) return fail("row with more than 65535 entries");
      L.rowinfo[r] = nlo | (ne << 16);
      L.dslot[r] = dg[i];
      wl = std::max(wl, nlo);
      wu = std::max(wu, ne - nlo);
    }
    L.cwl[c] = wl;
    L.cwu[c] = wu;
    L.cel[c] = next_e;
    L.ceu[c] = next_e + (long long)wl * rows;
    next_e = L.ceu[c] + (long long)wu * rows;
  }
  L.nent = next_e;
  if (L.nent >= (1LL << 31)) return fail("more than 2^31 stored entries");
  L.col.assign(L.nent, 0);
  L.src.assign(L.nent, -1);
  L.tsrc.assign(L.nent, -1);
  auto find_slot = [&](int row, int c) {
    for (int k = ia[row]; k < ia[row + 1]; ++k)
      if (ja[k] == c) return k;
    return -1;
  };
  for (int c = 0; c < ncol; ++c) {
    const int r0 = L.cslice[c] * FC_MC_SLICE, rows = (L.cslice[c + 1] - L.cslice[c]) * FC_MC_SLICE;
    for (int r = r0; r < r0 + rows; ++r) {
      const int i = L.perm[r];
      int kl = 0, ku = 0;
      if (i >= 0)
        for (int k = ia[i]; k < ia[i + 1]; ++k) {
          const int j = ja[k];
          if (j == i) continue;
          const bool lower = colour[j] < colour[i];
          const size_t e = lower ? (size_t)L.cel[c] + (size_t)(kl++) * rows + (r - r0)
                                 : (size_t)L.ceu[c] + (size_t)(ku++) * rows + (r - r0);
          L.col[e] = L.iperm[j];
          L.src[e] = k;
          L.tsrc[e] = find_slot(j, i);
        }
      for (; kl < L.cwl[c]; ++kl) L.col[(size_t)L.cel[c] + (size_t)kl * rows + (r - r0)] = r;
      for (; ku < L.cwu[c]; ++ku) L.col[(size_t)L.ceu[c] + (size_t)ku * rows + (r - r0)] = r;
    }
  }
  return true;
}
