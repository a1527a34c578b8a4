// N_LAS_XgSolver.h — xg's GPU sparse LU as one more Xyce linear solver, the
// drop-in for the reference's N_LAS_Solver interface
// (src/LinearAlgebraServicesPKG/include/N_LAS_Solver.h:60-125).
//
// A maintainer adds this header under src/LinearAlgebraServicesPKG/include
// and one branch to N_LAS_SolverFactory::create
// (src/LinearAlgebraServicesPKG/src/N_LAS_SolverFactory.C:87-160):
//
//     else if (type == "XG") return new N_LAS_XgSolver(prob, options);
//
// so that `.OPTIONS LINSOL TYPE=XG` or `-linsolv xg` selects it.  Like the
// factory's other serial solvers it takes the problem as an Epetra linear
// problem (N_LAS_Problem::epetraObj) and reads the CSR arrays of its matrix
// and the views of its right-hand side and solution in place.  The solving
// itself (analysis on the first matrix, GPU refactor and solve, repivot on a
// zero pivot, zero solution for a singular matrix) is
// xg_integration::DirectSolver (xg_direct_solver.h).
//
// Options (LINSOL block):  XG_PRECISION = FP64 (default) | FP32  (FP32
// factors with FP64 iterative refinement), XG_REFINE = refinement steps of
// the FP32 form (default 2), XG_DEVICE = CUDA device (default 0).  Options of
// the other solvers are accepted and ignored, as the reference's solvers do
// with options that are not theirs.
#ifndef Xyce_N_LAS_XgSolver_h
#define Xyce_N_LAS_XgSolver_h

#include <N_LAS_Problem.h>
#include <N_LAS_Solver.h>
#include <N_UTL_OptionBlock.h>
#include <N_UTL_Param.h>

#include <Epetra_CrsMatrix.h>
#include <Epetra_LinearProblem.h>
#include <Epetra_MultiVector.h>

#include <memory>
#include <string>

#include "xg_direct_solver.h"

class N_LAS_XgSolver : public N_LAS_Solver {
 public:
  N_LAS_XgSolver(N_LAS_Problem &prob, N_UTL_OptionBlock &options)
      : N_LAS_Solver(false), problem_(prob.epetraObj()) {
    setDefaultOptions();
    setOptions(options);
  }
  virtual ~N_LAS_XgSolver() {}

  virtual bool setOptions(const N_UTL_OptionBlock &OB) {
    for (N_UTL_OptionBlock::ParameterList::const_iterator it = OB.begin(); it != OB.end(); ++it)
      setParam(*it);
    return true;
  }
  virtual bool setDefaultOptions() {
    fp32_ = false;
    refine_ = 2;
    device_ = 0;
    solver_.reset();
    return true;
  }
  virtual bool setDefaultOption(const std::string &option) {
    if (option == "XG_PRECISION") fp32_ = false;
    else if (option == "XG_REFINE") refine_ = 2;
    else if (option == "XG_DEVICE") device_ = 0;
    solver_.reset();
    return true;
  }
  virtual bool setParam(const N_UTL_Param &param) {
    const std::string tag = param.uTag();
    if (tag == "XG_PRECISION") fp32_ = param.usVal() == "FP32";
    else if (tag == "XG_REFINE") refine_ = param.getImmutableValue<int>();
    else if (tag == "XG_DEVICE") device_ = param.getImmutableValue<int>();
    else return true;
    solver_.reset();
    return true;
  }
  // "Refactored" (N_NLS_NonLinearSolver.C:1036-1040): 1 when the last solve
  // factored the matrix.
  virtual bool getInfo(N_UTL_Param &info) {
    if (info.uTag() == "REFACTORED") info.setVal(solver_ && solver_->refactored() ? 1 : 0);
    return true;
  }

  // x = A^-1 b; 0 on success, as N_LAS_AmesosSolver::solve returns (a
  // singular matrix also returns 0 with a zero solution).
  virtual int solve(bool ReuseFactors = false) {
    Epetra_CrsMatrix *A = dynamic_cast<Epetra_CrsMatrix *>(problem_.GetMatrix());
    if (!A) return -1;
    int *rowptr = 0, *col = 0;
    double *val = 0, *b = 0, *x = 0;
    int ldb = 0, ldx = 0;
    if (A->ExtractCrsDataPointers(rowptr, col, val) || problem_.GetRHS()->ExtractView(&b, &ldb) ||
        problem_.GetLHS()->ExtractView(&x, &ldx))
      return -1;
    if (!solver_) solver_.reset(new xg_integration::DirectSolver(device_, fp32_, refine_));
    return solver_->solve(A->NumMyRows(), rowptr, col, val, b, x, ReuseFactors);
  }

 private:
  Epetra_LinearProblem &problem_;
  bool fp32_ = false;
  int refine_ = 2, device_ = 0;
  std::unique_ptr<xg_integration::DirectSolver> solver_;
};

#endif  // Xyce_N_LAS_XgSolver_h
