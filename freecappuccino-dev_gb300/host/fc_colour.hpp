// Multicolour layout of a CSR matrix for the FP32 inner solves of the
// mixed-precision path.  Rows are coloured greedily so that no two rows of a
// colour are coupled, and renumbered colour by colour (each colour padded to
// a multiple of 32 rows).  The off-diagonal entries of every colour are
// stored in two ELLPACK blocks of uniform width: the entries coupling to
// lower colours and those coupling to higher colours (entry k of row i of
// colour c at cel[c] (or ceu[c]) + k * rows_c + (i - crow[c])).  Short rows
// are padded with entries pointing at the row itself, whose values are zero.
// Every address of a row is then known from its index and colour alone, and a
// colour of rows updates in one data-parallel pass: the incomplete
// factorisation built on this ordering (DILU, which is DIC for a symmetric
// matrix) is applied in one pass per colour and direction over one block.
#pragma once
#include <string>
#include <vector>

#define FC_MC_SLICE 32
#define FC_MC_MAXCOL 32

struct ColouredLayout {
  int n = 0;          // rows of the original matrix
  int nP = 0;         // rows of the coloured numbering (padded)
  int ncol = 0;       // colours
  int nslices = 0;    // nP / FC_MC_SLICE
  long long nent = 0; // stored entries (sum over colours of rows x (lower + upper width))
  std::vector<int> cslice;     // ncol + 1: first slice of every colour (rows: x FC_MC_SLICE)
  std::vector<int> cwl, cwu;   // ncol: widths of the lower and upper blocks of every colour
  std::vector<long long> cel, ceu;  // ncol: first entry of the lower and upper blocks
  std::vector<int> perm;       // nP: original row of a coloured row, -1 for padding
  std::vector<int> iperm;      // n: coloured row of an original row
  std::vector<int> rowinfo;    // nP: lower entries | all entries << 16
  std::vector<int> col;        // entries: coloured column (the row itself on padding)
  std::vector<int> src;        // entries: CSR slot of a_ij in the original values, -1 on padding
  std::vector<int> tsrc;       // entries: CSR slot of a_ji, -1 if the pattern has none
  std::vector<int> dslot;      // nP: CSR slot of a_ii, -1 for padding rows
};

// ia (n+1), ja (nnz), dg (n) 0-based.  Fails (false, err) when a row has more
// than 65535 off-diagonal entries or the greedy colouring needs more than
// FC_MC_MAXCOL colours.
bool build_coloured(int n, const int* ia, const int* ja, const int* dg, ColouredLayout& L, std::string* err);
