/*
 * xgo.h — CPU oracle for the Newton load.  TEST INFRASTRUCTURE ONLY: a plain-C
 * restatement of the reference Xyce load loops (updateState, loadDAEVectors,
 * loadDAEMatrices per device type, in DeviceMgr's order), used by tests/,
 * smoke() and the CPU-baseline leg of bench.py as the checker.  The engine
 * never links, imports or calls anything in this folder.
 *
 * Inputs are the netlist of include/xg.h plus the per-instance parameter
 * blocks of include/xg_params.h, which the oracle derives with its own
 * restatement of the reference's set-up (xgo_setup_params).  Parity of this restatement with the
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

/* The parameter block of device type t (xg_params.h layout, column k of
 * instance i at out[k*n + i]) derived by the oracle's own set-up
 * (xgo_setup.c, xgo_b3setup.c).  out may be NULL to query the sizes. */
int xgo_setup_params(const xg_netlist *nl, const xg_device_options *opt, int dev_type,
                     double *out, int *n_params, int *n_instances);

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

/* ---- transient analysis (xgo_tran.c) ---------------------------------------- */
typedef struct {
  double tstop, tstep;        /* .TRAN TSTEP TSTOP (TSTEP = starting step) */
  double maxstep;             /* <= 0: 0.1 * tstop */
  double reltol, abstol;      /* local error test: 1e-3, 1e-6 */
  int n_out;                  /* unknowns recorded at every accepted point */
  const int *out_idx;
  int max_points;             /* capacity of t_out / v_out */
  const int *col_order;       /* column order of the sparse LU, or NULL */
  const double *x0;           /* initial guess of the DC operating point
                                 (.NODESET), n_unknowns values, or NULL = 0 */
  int uic;                    /* 1: no DC operating point, start from x0 (.TRAN UIC) */
} xgo_tran_opts;

typedef struct {
  int status;                 /* 0, or the failing Newton / step status */
  int steps, steps_attempted, rejected;
  int newton_iters, factorizations, loads;
  int dcop_iters, dcop_solves;
} xgo_tran_stats;

/* DC operating point, then the transient to tstop; records (t, x[out_idx])
 * at t = 0 and at every accepted step. 0 on success. */
int xgo_tran_run(xgo_circuit *c, const xgo_tran_opts *o, double *t_out, double *v_out,
                 int *n_points, xgo_tran_stats *st);
/* Minimum-degree column order of the n x n CSR pattern (xgo_order.c):
 * order[k] = the k-th pivot column. */
int xgo_min_degree(int n, const int *rowptr, const int *col, int *order);
/* The integrator's formulas the transient driver applies (xgo_tran.c; each
 * held by the tests to the reference's own compiled code). */
void xgo_tia_update_coeffs(int order, double h, double h_sum, double *psi, double *beta,
                           double *alphas, double *ck);
void xgo_tia_predictor(int n, int order, const double *beta, const double *xh0, const double *xh1,
                       const double *xh2, const double *qh0, double *xn0, double *qn0);
void xgo_tia_residual(int n, int order, double h, double alphas, int limiter, const double *Q,
                      const double *qn0, const double *F, const double *qh2, const double *fvp,
                      const double *qvp, double *rhs);
void xgo_tia_jacobian(int64_t nnz, int order, double h, double alphas, const double *dqdx,
                      const double *dfdx, double *jac);
double xgo_tia_error_estimate(int n, double ck, const double *x_curr, const double *corr,
                              double reltol, double abstol);
int xgo_nls_converged(int transient, int step, int max_step, double rhs_tol, double dx_tol,
                      double small_update, double max_rhs, double upd, double rhs_rel, double rate,
                      int *count, double *stall_rate);
void xgo_tia_complete_step(int n, const double *in, double *const *hist, const double *x_next,
                           const double *Q, const double *F, double *out);
void xgo_tia_reject_step(const double *in, double *out);
/* x = A^-1 b with the driver's sparse LU (CSR A, column order or NULL). */
int xgo_sparse_solve(int n, const int *rowptr, const int *col, const double *val,
                     const int *col_order, const double *b, double *x);

#ifdef __cplusplus
}
#endif

#endif
