// xg_direct_solver.h — the linear-solve half of the drop-in: a host-side
// direct solver over xg's GPU sparse LU (include/xg.h, xg_lu_*), written
// against no Xyce type so that it builds anywhere libxg.so does.
// N_LAS_XgSolver.h adapts it to the reference's N_LAS_Solver interface.
//
// It keeps the behaviour of the reference's default direct solver
// (N_LAS_AmesosSolver::solve, src/LinearAlgebraServicesPKG/src/
// N_LAS_AmesosSolver.C:231-492):
//   * the first solve of a pattern analyses it (symbolic factorisation and
//     the pivot order of its values, :388);
//   * each later solve refactors numerically (:405) unless the caller reuses
//     the factors, then solves (:444);
//   * KLU repivots at every numeric factorisation by default (:355-370).
//     The GPU refactor keeps the pivot order instead; when a pivot comes out
//     zero or non-finite the matrix is analysed again (a new pivot order) and
//     factored once more;
//   * a matrix still singular after that returns a zero solution and status
//     0, leaving the decision to the nonlinear solver (:411-436).
#ifndef XG_DIRECT_SOLVER_H
#define XG_DIRECT_SOLVER_H

#include <xg.h>

#include <algorithm>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

namespace xg_integration {

class DirectSolver {
 public:
  // fp32_factors: FP32 factors and solves with n_refine FP64 refinement
  // steps against the FP64 matrix (the mixed-precision form).
  explicit DirectSolver(int cuda_device = 0, bool fp32_factors = false, int n_refine = 2)
      : device_(cuda_device), fp32_(fp32_factors), refine_(fp32_factors ? n_refine : 0) {}
  ~DirectSolver() { release(); }
  DirectSolver(const DirectSolver &) = delete;
  DirectSolver &operator=(const DirectSolver &) = delete;

  void set_precision(bool fp32_factors, int n_refine) {
    if (fp32_factors != fp32_) drop_factors();
    fp32_ = fp32_factors;
    refine_ = fp32_factors ? n_refine : 0;
  }

  // x = A^-1 b.  A: n rows in CSR on the host (columns ascending within a
  // row, as Epetra keeps them after FillComplete).  Returns 0 when x holds
  // the solution or, for a singular matrix, zeros (then singular() is true);
  // an XG_ERR_* code when the GPU call itself fails.
  int solve(int n, const int *rowptr, const int *col, const double *val, const double *b,
            double *x, bool reuse_factors = false) {
    refactored_ = false;
    singular_ = false;
    if (n <= 0) return XG_ERR_ARG;
    const bool same = lu_ && same_pattern(n, rowptr, col);
    if (!same && reuse_factors) return XG_ERR_STATE;  // nothing to reuse
    int rc = XG_OK;
    if (!same) {
      rc = analyse(n, rowptr, col, val);
      if (rc == XG_ERR_SINGULAR) return zero(n, x);
      if (rc) return rc;
    }
    int status = 0;
    rc = xg_lu_solve_host(lu_, val, b, x, refine_, reuse_factors ? 1 : 0, &status);
    if (rc) return rc;
    if ((status & 1) && !reuse_factors) {  // a zero pivot in the kept order: repivot
      rc = analyse(n, rowptr, col, val);
      if (rc == XG_ERR_SINGULAR) return zero(n, x);
      if (rc) return rc;
      rc = xg_lu_solve_host(lu_, val, b, x, refine_, 0, &status);
      if (rc) return rc;
    }
    if (status & 1) return zero(n, x);
    if (status) return XG_ERR_TIMEOUT;
    refactored_ = !reuse_factors;
    return XG_OK;
  }

  bool refactored() const { return refactored_; }  // the last solve factored anew
  bool singular() const { return singular_; }      // the last solve returned zeros
  int analyses() const { return analyses_; }       // pivot orders chosen so far

 private:
  int analyse(int n, const int *rowptr, const int *col, const double *val) {
    drop_factors();
    int rc = XG_OK;
    if (!ctx_ && (rc = xg_ctx_create(device_, &ctx_))) return rc;
    rc = xg_lu_analyze(ctx_, n, rowptr, col, val, fp32_ ? XG_LU_FP32 : XG_LU_FP64, &lu_);
    if (rc) {
      lu_ = nullptr;
      return rc;
    }
    ++analyses_;
    rowptr_.assign(rowptr, rowptr + n + 1);
    col_.assign(col, col + rowptr[n]);
    return XG_OK;
  }
  bool same_pattern(int n, const int *rowptr, const int *col) const {
    return int(rowptr_.size()) == n + 1 && std::equal(rowptr, rowptr + n + 1, rowptr_.begin()) &&
           std::equal(col, col + rowptr[n], col_.begin());
  }
  int zero(int n, double *x) {
    std::fill(x, x + n, 0.0);
    singular_ = true;
    return XG_OK;
  }
  void drop_factors() {
    if (lu_) xg_lu_destroy(lu_);
    lu_ = nullptr;
    rowptr_.clear();
    col_.clear();
  }
  void release() {
    drop_factors();
    if (ctx_) xg_ctx_destroy(ctx_);
    ctx_ = nullptr;
  }

  int device_;
  bool fp32_;
  int refine_;
  xg_ctx *ctx_ = nullptr;
  xg_lu *lu_ = nullptr;
  std::vector<int> rowptr_, col_;
  bool refactored_ = false, singular_ = false;
  int analyses_ = 0;
};

}  // namespace xg_integration

#endif  // XG_DIRECT_SOLVER_H
