/* Stand-in declaration of Trilinos' Epetra_LinearProblem (see Epetra_MultiVector.h). */
#ifndef XG_SHIM_EPETRA_LINEARPROBLEM
#define XG_SHIM_EPETRA_LINEARPROBLEM
#include <Epetra_MultiVector.h>
#include <Epetra_RowMatrix.h>
class Epetra_LinearProblem {
 public:
  virtual ~Epetra_LinearProblem();
  Epetra_RowMatrix *GetMatrix() const;
  Epetra_MultiVector *GetLHS() const;
  Epetra_MultiVector *GetRHS() const;
};
#endif
