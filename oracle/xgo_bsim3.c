/*
 * xgo_bsim3.c — BSIM3 v3.2 load loops of the oracle (TEST INFRASTRUCTURE
 * ONLY; see xgo.h).  Placeholder until the BSIM3 restatement lands.
 */
#include <stdlib.h>

#include "xgo_internal.h"

int xgo_b3_nparams(void) { return 1; }
void *xgo_b3_members_alloc(int n) { return calloc((size_t)n + 1, sizeof(double)); }
void xgo_b3_members_reset(void *m, int n) { (void)m; (void)n; }
int xgo_b3_nlid(void) { return 4; }
int xgo_b3_nint(const xgo_type *T, int i) { (void)T; (void)i; return 0; }
void xgo_b3_lids(const xgo_type *T, int i, const int *ext, int *next, int *lid) {
  (void)T; (void)i; (void)next;
  for (int k = 0; k < 4; ++k) lid[k] = ext[k];
}
int xgo_b3_stamps(const xgo_type *T, int i, int *rows, int *cols) {
  (void)T; (void)i; (void)rows; (void)cols;
  return 0;
}
void xgo_b3_update_state(xgo_circuit *c, int i0, int i1, xgo_io *io) { (void)c; (void)i0; (void)i1; (void)io; }
void xgo_b3_load_vectors(xgo_circuit *c, int i0, int i1, xgo_io *io) { (void)c; (void)i0; (void)i1; (void)io; }
void xgo_b3_load_matrices(xgo_circuit *c, int i0, int i1, xgo_io *io) { (void)c; (void)i0; (void)i1; (void)io; }
