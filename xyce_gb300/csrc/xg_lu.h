// xg_lu.h — the sparse LU of the Newton solve: host symbolic analysis
// (lu_symbolic.cpp) shared with the device refactor/solve (lu_kernels.cu).
//
// The reference factors the Jacobian with KLU through Amesos
// (N_LAS_AmesosSolver.C:231-492): one symbolic analysis per matrix pattern,
// a numeric factorisation with partial pivoting per Newton iteration, then
// the triangular solves.  Here the analysis runs once on the host: an
// approximate-minimum-degree column order, then a left-looking partial-pivot
// factorisation of the first matrix that fixes the row (pivot) order and the
// filled L\U pattern.  Every later factorisation reuses that pivot order and
// pattern and runs on the GPU.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "xg.h"

namespace xg {

struct LuSymbolic {
  int n = 0;
  int64_t nnz_a = 0;
  // B = A(P, Q): row k of B is row P[k] of A, column j of B is column Q[j].
  std::vector<int> P, Q;
  // Filled pattern of L\U of B, row-wise (CSR), columns ascending in each
  // row; L strictly left of the diagonal (unit diagonal implied), U from the
  // diagonal on.
  std::vector<int> rp, ci, diag;
  std::vector<int> lu2a;     // LU position -> CSR index of the A entry, or -1 (fill)
  double refactor_flops = 0;  // multiply-adds + divides of one refactorisation
  double solve_flops = 0;     // multiply-adds of one forward + backward solve
  int levels = 0;             // longest row dependency chain of the factorisation
  int max_width = 0;          // rows in the widest level of that chain
  int n_dense = 0;            // rows/columns ordered last as dense
  double min_pivot = 0, max_pivot = 0;  // |U(k,k)| range of the analysed matrix
  int ordering = 0;           // column order: 0 minimum degree, 1 nested dissection
  // Update schedule of the refactorisation (lu_build_updates): for row i, its
  // L entries p in ascending column k, and for each the entries q of U row k
  // right of the diagonal in ascending column, upos holds the position in
  // row i that U(k, ci[q]) updates.  urp[i] is where row i's updates start.
  std::vector<int64_t> urp;
  std::vector<int> upos;
  // Rows grouped by dependency level for the level-by-level kernels: lrow
  // lists the rows of L level 0, 1, ... (a row's L level is one more than the
  // highest of the rows its L part names), lptr[l] where level l starts;
  // urow/uptr the same for the backward solve, by U level.
  std::vector<int> lrow, lptr, urow, uptr;
  // Within level l the rows with more than kHeavyRowUpdates updates come
  // last, from lheavy[l] on: a warp factors each of those (when the level
  // has at most kMaxHeavyRows of them).
  std::vector<int> lheavy;
  // Trailing rows with long L parts (a supply rail ordered last has one L
  // entry per device on it), and the rows after them, are left out of lrow:
  // one thread would walk them serially.  They are factored one at a time after the levels, each with
  // all threads: every position of the row pulls its updates (tail_pm[j] the
  // row's own multiplier, tail_q[j] the U entry, in the order the row-wise
  // elimination applies them), positions grouped so that a group reads only
  // multipliers of earlier groups.  tail_pos lists the positions by group,
  // tail_gptr[g] where group g starts, tail_rowg[r] the first group of row
  // tail0 + r, tail_pp[t] where the pairs of tail_pos[t] start.  Within a
  // group the positions with more than kTailLongPulls pairs come last, from
  // tail_glong[g] on: a warp sums each of those (the diagonal of a supply
  // rail pulls one pair per device on the rail).
  int tail0 = 0;
  std::vector<int> tail_rowg, tail_gptr, tail_glong, tail_pos, tail_pp, tail_pm, tail_q;
};

constexpr int kTailLongPulls = 32;
constexpr int kHeavyRowUpdates = 32;
constexpr int kMaxHeavyRows = 8;

// The tail starts at the first of the last kTailMaxRows rows with more than
// kTailMinL L entries.
constexpr int kTailMinL = 64;
constexpr int kTailMaxRows = 16;

// Ordering choice: nested dissection is tried when minimum degree leaves a
// dependency chain longer than kNdMinLevels rows with fewer than
// kNdMaxRowsPerLevel rows per level on average; parts of at most kNdLeaf
// vertices are ordered by minimum degree.  The refactorisation time model
// charges kLuLevelSeconds per dependent level and kLuFlopSeconds per
// multiply-add.
constexpr int kNdMinLevels = 64;
constexpr double kNdMaxRowsPerLevel = 8.0;  // and minimum degree averages fewer rows per level
constexpr int kNdLeaf = 16;
constexpr double kLuLevelSeconds = 2e-6;
constexpr double kLuFlopSeconds = 2e-10;
double lu_model_seconds(const LuSymbolic &S);

// Nested-dissection order of the graph of A + A^T (diagonal ignored).
std::vector<int> nd_order(int n, const int *rp, const int *ci, int leaf, int *n_dense);

// Approximate minimum degree order of the graph of A + A^T (diagonal
// ignored).  Returns the elimination order: order[k] = the k-th unknown.
std::vector<int> amd_order(int n, const int *rp, const int *ci, int *n_dense);

// Ordering + pivoting factorisation of A (CSR, n x n) with threshold partial
// pivoting (diagonal preferred when |a_diag| >= pivot_tol * max|column|).
// ordering: 0 minimum degree, 1 nested dissection, -1 chooses (see
// kNdMinLevels; XG_LU_ORDER=amd|nd in the environment overrides that choice).
// Returns 0, or -1 with *err set when A is structurally or numerically
// singular.
int lu_analyze(int n, const int *rp, const int *ci, const double *val, double pivot_tol,
               LuSymbolic *out, std::string *err, int ordering = -1);

// Fills the update schedule (urp, upos), the level lists and the tail from
// the L\U pattern; false if an update falls outside the pattern (cannot
// happen for a pattern lu_analyze made).
bool lu_build_updates(LuSymbolic &S);

// Device address of an LU's status word (bits as xg_lu_status reports), for
// callers that read it back together with other results.
const unsigned *lu_status_device(const xg_lu *lu);

}  // namespace xg
