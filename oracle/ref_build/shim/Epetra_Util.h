/* Stand-in for Epetra_Util: the devices only use it for a seeded random
 * perturbation that is unused on the load path. Test infrastructure only. */
#ifndef XG_SHIM_EPETRA_UTIL
#define XG_SHIM_EPETRA_UTIL
class Epetra_Util {
 public:
  Epetra_Util() : s_(12345u) {}
  unsigned int RandomInt() { s_ = s_ * 1103515245u + 12345u; return s_; }
  double RandomDouble() { return (double)(RandomInt() % 1000000u) / 500000.0 - 1.0; }
  int SetSeed(unsigned int s) { s_ = s; return 0; }
  unsigned int Seed() const { return s_; }
 private:
  unsigned int s_;
};
#endif
