/* Stand-in declaration of Trilinos' Epetra_CrsMatrix (see Epetra_MultiVector.h). */
#ifndef XG_SHIM_EPETRA_CRSMATRIX
#define XG_SHIM_EPETRA_CRSMATRIX
#include <Epetra_RowMatrix.h>
class Epetra_CrsMatrix : public Epetra_RowMatrix {
 public:
  virtual ~Epetra_CrsMatrix();
  virtual int NumMyRows() const;
  int NumMyNonzeros() const;
  int ExtractCrsDataPointers(int *&IndexOffset, int *&Indices, double *&Values) const;
};
#endif
