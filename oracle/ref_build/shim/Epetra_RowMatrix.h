/* Stand-in declaration of Trilinos' Epetra_RowMatrix (see Epetra_MultiVector.h). */
#ifndef XG_SHIM_EPETRA_ROWMATRIX
#define XG_SHIM_EPETRA_ROWMATRIX
class Epetra_RowMatrix {
 public:
  virtual ~Epetra_RowMatrix();
  virtual int NumMyRows() const = 0;
};
#endif
