/* Stand-in declaration of Trilinos' Epetra_MultiVector (not in the reference
 * tree): the members the GPU linear-solver drop-in calls, with Epetra's
 * signatures, so that it compiles against the reference headers.  Test
 * infrastructure only; nothing is defined. */
#ifndef XG_SHIM_EPETRA_MULTIVECTOR
#define XG_SHIM_EPETRA_MULTIVECTOR
class Epetra_MultiVector {
 public:
  virtual ~Epetra_MultiVector();
  int ExtractView(double **A, int *MyLDA) const;
  int MyLength() const;
  int NumVectors() const;
};
#endif
