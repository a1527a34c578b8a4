/*
 * xgo.h — CPU oracle for the Newton load.  TEST INFRASTRUCTURE ONLY: a plain-C
 * restatement of the reference Xyce load loops (updateState, loadDAEVectors,
 * loadDAEMatrices per device type, in DeviceMgr's order), used by tests/,
 * smoke() and the CPU-baseline leg of bench.py as the checker.  The engine
 * never links, imports or calls anything in this folder.
 *
 * Inputs are the netlist of include/xg.h plus the per-instance parameter
 * blocks of include/xg_params.h (derived on the host by circuit setup); the
 * oracle restates only the load path.  Parity of this restatement with the
 * reference itself is pinned by the tests against oracle/_ref (the reference's
 * own device sources compiled here) and the golden fixtures generated from it.
 *
 * Compiled with -ffp-contract=off: every product and sum is rounded on its
 * own, as in the reference's x86-64 build.
 */
#ifndef XGO_H
#define XGO_H

#include <stdint.h>

#include "xg.h"
#include "xg_params.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct xgo_circuit xgo_circuit;

/* params[t] = SoA block of device type t (xg_params.h), or NULL if none. */
int xgo_build(const xg_netlist *nl, const xg_device_options *opt,
              const double *const *params, xgo_circuit **out);
void xgo_free(xgo_circuit *c);
int xgo_sizes(const xgo_circuit *c, int *n_unknowns, int *n_state, int *n_store,
              int64_t *nnz);
/* Ground-excluded CSR pattern, ascending columns. */
int xgo_pattern(const xgo_circuit *c, int *rowptr, int *col);
/* Instance members that persist from one load to the next (the diode's
 * limited junction voltage, read back as the next iterate's history). */
int xgo_reset_members(xgo_circuit *c);
/* in_vecs: sol next/curr/last (n_unknowns+1), sta next/curr/last (n_state),
 * sto next/curr/last (n_store).  Outputs over n_unknowns+1 rows (ground last);
 * dfdx/dqdx values over the ground-excluded pattern. */
int xgo_load(xgo_circuit *c, const xg_load_flags *fl, const double *const *in_vecs,
             double *f, double *q, double *dfdxdvp, double *dqdxdvp,
             double *sta_next, double *sto_next, double *dfdx, double *dqdx);
/* Load only a contiguous instance range [i0, i1) of one device type into the
 * given outputs (no zeroing); used to time a bounded sample of a big load. */
int xgo_load_range(xgo_circuit *c, const xg_load_flags *fl, const double *const *in_vecs,
                   int dev_type, int i0, int i1, double *f, double *q, double *dfdxdvp,
                   double *dqdxdvp, double *sta_next, double *sto_next, double *dfdx,
                   double *dqdx);

#ifdef __cplusplus
}
#endif

#endif
