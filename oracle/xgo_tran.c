/*
 * xgo_tran.c — CPU transient driver (TEST INFRASTRUCTURE ONLY; see xgo.h).
 *
 * A plain-C restatement of the reference's transient analysis on top of the
 * oracle's Newton load, used as the waveform checker of the GPU time stepper
 * and as the CPU baseline of Newton iterations per second:
 *
 *  - DC operating point: damped Newton with the DC defaults
 *    (N_NLS_DampedNewton.C:374-629, N_NLS_NLParams.h: RHSTol 1e-6, deltaXTol
 *    1.0 scaled by 0.01 on the first solve, relTol 1e-3, absTol 1e-12, 200
 *    steps), residual -F + dFdxdVp and Jacobian dFdx + 1e-20 dQdx
 *    (N_TIA_NoTimeIntegration.C:140-198), init-junction on the first
 *    iteration (N_DEV_DeviceMgr.C:3557-3560);
 *  - time integration by the "OneStep" trapezoid method (TIAParams default
 *    method 7): predictor, residual and Jacobian
 *    (N_TIA_OneStep.C:115-352), coefficient update (:1355-1480), history
 *    update (:1209-1300), initial step (:1482-1640), step completion and
 *    rejection (:1695-2190);
 *  - Newton per step with the transient defaults (N_NLS_NLParams.C:128-139:
 *    20 steps, RHSTol 1e-2, deltaXTol 0.33, absTol 1e-6, relTol 1e-2) and the
 *    convergence test N_NLS_DampedNewton.C:1787-1919;
 *  - local error test estOverTol = ck * WRMS(x - xpredicted) with weights
 *    relErrorTol * |x_curr|_inf + absErrorTol (N_TIA_DataStore.C:1240-1390,
 *    newLte), accept when <= 1 (N_TIA_StepErrorControl.C:668-800);
 *  - breakpoints at every PULSE corner (N_DEV_SourceData.C:1114-1198), the
 *    stop time (N_TIA_StepErrorControl.C:520-609) and the restart at a
 *    breakpoint (N_ANP_Transient.C:1130-1168).
 *
 * The linear solve is a left-looking sparse LU with threshold partial
 * pivoting on every Newton iteration, as KLU with repivoting does
 * (N_LAS_AmesosSolver.C:355-444), over a caller-given column order.
 */
#include <float.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "xgo_internal.h"

/* ---- sparse LU ------------------------------------------------------------ */

typedef struct {
  int n;
  int64_t nnz;
  const int *Q;
  int *cp, *cr, *cpos;             /* A by columns, with the CSR index */
  int *Lp, *Li, *Up, *Ui;
  double *Lx, *Ux;
  int64_t lcap, ucap;
  int *pinv, *P;
  double *x;
  int *xi, *stk, *pstk, *vis;
} xlu_t;

static void *xmalloc(size_t n) {
  void *p = malloc(n ? n : 1);
  return p;
}

static xlu_t *xlu_new(int n, const int *rp, const int *ci, const int *Q) {
  xlu_t *f = (xlu_t *)calloc(1, sizeof(xlu_t));
  f->n = n;
  f->nnz = rp[n];
  f->Q = Q;
  f->cp = (int *)calloc(n + 1, sizeof(int));
  f->cr = (int *)xmalloc(sizeof(int) * f->nnz);
  f->cpos = (int *)xmalloc(sizeof(int) * f->nnz);
  for (int64_t p = 0; p < f->nnz; ++p) f->cp[ci[p] + 1]++;
  for (int j = 0; j < n; ++j) f->cp[j + 1] += f->cp[j];
  int *fill = (int *)xmalloc(sizeof(int) * n);
  memcpy(fill, f->cp, sizeof(int) * n);
  for (int i = 0; i < n; ++i)
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
      int q = fill[ci[p]]++;
      f->cr[q] = i;
      f->cpos[q] = p;
    }
  free(fill);
  f->lcap = f->ucap = 4 * f->nnz + n;
  f->Lp = (int *)xmalloc(sizeof(int) * (n + 1));
  f->Up = (int *)xmalloc(sizeof(int) * (n + 1));
  f->Li = (int *)xmalloc(sizeof(int) * f->lcap);
  f->Lx = (double *)xmalloc(sizeof(double) * f->lcap);
  f->Ui = (int *)xmalloc(sizeof(int) * f->ucap);
  f->Ux = (double *)xmalloc(sizeof(double) * f->ucap);
  f->pinv = (int *)xmalloc(sizeof(int) * n);
  f->P = (int *)xmalloc(sizeof(int) * n);
  f->x = (double *)calloc(n, sizeof(double));
  f->xi = (int *)xmalloc(sizeof(int) * n);
  f->stk = (int *)xmalloc(sizeof(int) * n);
  f->pstk = (int *)xmalloc(sizeof(int) * n);
  f->vis = (int *)xmalloc(sizeof(int) * n);
  return f;
}

static void xlu_free(xlu_t *f) {
  if (!f) return;
  free(f->cp); free(f->cr); free(f->cpos);
  free(f->Lp); free(f->Li); free(f->Lx); free(f->Up); free(f->Ui); free(f->Ux);
  free(f->pinv); free(f->P); free(f->x); free(f->xi); free(f->stk); free(f->pstk); free(f->vis);
  free(f);
}

static int grow(int **i, double **x, int64_t *cap, int64_t need) {
  if (need <= *cap) return 0;
  int64_t c = *cap * 2 > need ? *cap * 2 : need;
  int *ni = (int *)realloc(*i, sizeof(int) * c);
  double *nx = (double *)realloc(*x, sizeof(double) * c);
  if (!ni || !nx) return -1;
  *i = ni;
  *x = nx;
  *cap = c;
  return 0;
}

/* Factor A (values in CSR order); 0, or -1 when singular. */
static int xlu_factor(xlu_t *f, const double *val, double tol) {
  const int n = f->n;
  int64_t lnz = 0, unz = 0;
  for (int i = 0; i < n; ++i) { f->pinv[i] = -1; f->vis[i] = -1; }
  f->Lp[0] = f->Up[0] = 0;
  for (int k = 0; k < n; ++k) {
    const int col = f->Q ? f->Q[k] : k;
    int top = n;
    for (int q = f->cp[col]; q < f->cp[col + 1]; ++q) {
      int r0 = f->cr[q];
      if (f->vis[r0] == k) continue;
      int head = 0;
      f->stk[0] = r0;
      while (head >= 0) {
        int r = f->stk[head], jc = f->pinv[r];
        if (f->vis[r] != k) {
          f->vis[r] = k;
          f->pstk[head] = jc < 0 ? 0 : f->Lp[jc];
        }
        int pend = jc < 0 ? 0 : f->Lp[jc + 1], leaf = 1;
        for (int p = f->pstk[head]; p < pend; ++p) {
          int ch = f->Li[p];
          if (f->vis[ch] == k) continue;
          f->pstk[head] = p + 1;
          f->stk[++head] = ch;
          leaf = 0;
          break;
        }
        if (leaf) { --head; f->xi[--top] = r; }
      }
    }
    for (int q = top; q < n; ++q) f->x[f->xi[q]] = 0.0;
    for (int q = f->cp[col]; q < f->cp[col + 1]; ++q) f->x[f->cr[q]] = val[f->cpos[q]];
    for (int q = top; q < n; ++q) {
      int r = f->xi[q], j = f->pinv[r];
      if (j < 0) continue;
      double xj = f->x[r];
      for (int p = f->Lp[j]; p < f->Lp[j + 1]; ++p) f->x[f->Li[p]] -= f->Lx[p] * xj;
    }
    int best = -1;
    double amax = 0.0;
    for (int q = top; q < n; ++q) {
      int r = f->xi[q];
      if (f->pinv[r] >= 0) continue;
      double a = fabs(f->x[r]);
      if (best < 0 || a > amax) { amax = a; best = r; }
    }
    if (best < 0 || !(amax > 0.0) || !isfinite(amax)) return -1;
    int piv = best;
    if (f->vis[col] == k && f->pinv[col] < 0 && fabs(f->x[col]) >= tol * amax) piv = col;
    double pivot = f->x[piv];
    if (grow(&f->Ui, &f->Ux, &f->ucap, unz + (n - top) + 1) ||
        grow(&f->Li, &f->Lx, &f->lcap, lnz + (n - top)))
      return -2;
    for (int q = top; q < n; ++q) {
      int r = f->xi[q];
      if (f->pinv[r] >= 0) { f->Ui[unz] = f->pinv[r]; f->Ux[unz++] = f->x[r]; }
    }
    f->Ui[unz] = k;
    f->Ux[unz++] = pivot;
    f->Up[k + 1] = (int)unz;
    for (int q = top; q < n; ++q) {
      int r = f->xi[q];
      if (f->pinv[r] < 0 && r != piv) { f->Li[lnz] = r; f->Lx[lnz++] = f->x[r] / pivot; }
    }
    f->Lp[k + 1] = (int)lnz;
    f->pinv[piv] = k;
    f->P[k] = piv;
  }
  for (int64_t p = 0; p < lnz; ++p) f->Li[p] = f->pinv[f->Li[p]];
  return 0;
}

/* x = A^-1 b (b and x of length n; may alias) */
static void xlu_solve(xlu_t *f, const double *b, double *x) {
  const int n = f->n;
  double *y = f->x;
  for (int k = 0; k < n; ++k) y[k] = b[f->P[k]];
  for (int k = 0; k < n; ++k) {
    double yk = y[k];
    for (int p = f->Lp[k]; p < f->Lp[k + 1]; ++p) y[f->Li[p]] -= f->Lx[p] * yk;
  }
  for (int k = n - 1; k >= 0; --k) {
    int pd = f->Up[k + 1] - 1;
    y[k] /= f->Ux[pd];
    double yk = y[k];
    for (int p = f->Up[k]; p < pd; ++p) y[f->Ui[p]] -= f->Ux[p] * yk;
  }
  for (int k = 0; k < n; ++k) x[f->Q ? f->Q[k] : k] = y[k];
}

/* ---- transient --------------------------------------------------------------- */

typedef struct {
  xgo_circuit *c;
  int n, nr, nsta, nsto;
  int64_t nnz;
  xlu_t *lu;
  double *sol[3], *sta[3], *sto[3];  /* next, curr, last */
  double *f, *q, *fvp, *qvp, *dfdx, *dqdx, *jac, *rhs, *dx, *w;
  double *xh0, *xh1, *xh2, *qh0, *qh1, *qh2, *xn0, *qn0;
  int64_t *diag;                     /* CSR position of (i, i), or -1 */
  double gshunt;                     /* DC homotopy conductance on node rows */
  /* Newton bookkeeping kept from one solve to the next */
  int stall_count;
  double stall_rate;
  int first_solve;
  xgo_tran_stats *st;
} tctx;

static double inf_norm(const double *v, int n) {
  double m = 0;
  for (int i = 0; i < n; ++i) if (fabs(v[i]) > m || v[i] != v[i]) m = v[i] != v[i] ? v[i] : fabs(v[i]);
  return m;
}
static double two_norm(const double *v, int n) {
  double s = 0;
  for (int i = 0; i < n; ++i) s += v[i] * v[i];
  return sqrt(s);
}
static double wrms(const double *v, const double *w, int n) {
  double s = 0;
  for (int i = 0; i < n; ++i) { double t = v[i] / w[i]; s += t * t; }
  return sqrt(s / n);
}

/* ---- the integrator's formulas, one function each, exported so that the
 * tests hold them to the reference's own compiled code ------------------ */

/* OneStep::updateCoeffs (N_TIA_OneStep.C:1355-1480): the step history psi,
 * the predictor coefficients beta, the leading coefficient alphas and the
 * error constant ck of a trapezoid (order 2) or backward-Euler step. */
void xgo_tia_update_coeffs(int order, double h, double h_sum, double *psi, double *beta,
                           double *alphas, double *ck) {
  if (order == 2) psi[2] = psi[1];
  psi[1] = psi[0];
  psi[0] = h;
  beta[0] = 1.0;
  *alphas = -1.0;
  if (order == 2) {
    double r = h / psi[1];
    beta[1] = r + r * r / 2;
    beta[2] = -1.0 * h * h / psi[1] / psi[2] / 2;
    *ck = (h / h_sum) / 3.0;
  } else {
    beta[1] = h / psi[1];
    *ck = h / h_sum;
  }
}

/* OneStep::obtainPredictor (N_TIA_OneStep.C:115-205): xn0 = xh0 +
 * beta_1 xh1 (+ beta_2 xh2 at order 2), qn0 = qh0. */
void xgo_tia_predictor(int n, int order, const double *beta, const double *xh0, const double *xh1,
                       const double *xh2, const double *qh0, double *xn0, double *qn0) {
  for (int i = 0; i < n; ++i) {
    double x = xh0[i];
    x = beta[1] * xh1[i] + x;
    if (order == 2) x = beta[2] * xh2[i] + x;
    xn0[i] = x;
    qn0[i] = qh0[i];
  }
}

/* OneStep::obtainResidual (N_TIA_OneStep.C:215-290): the Newton right-hand
 * side -[(Q - qn0)/h + f F + f qh2] + (-alphas/h) dQdxdVp + f dFdxdVp, with
 * f = 1/2 at order 2 (the qh2 term then) and 1 at order 1; the limiter terms
 * only when limiting changed a junction voltage.  alphas = -1. */
void xgo_tia_residual(int n, int order, double h, double alphas, int limiter, const double *Q,
                      const double *qn0, const double *F, const double *qh2, const double *fvp,
                      const double *qvp, double *rhs) {
  const double fs = order == 2 ? 0.5 : 1.0, qs = -alphas / h;
  for (int i = 0; i < n; ++i) {
    double r = 1.0 * Q[i] + -1.0 * qn0[i];
    r = order == 2 ? (1.0 / h) * r + 0.5 * F[i] : (1.0 / h) * r + 1.0 * F[i];
    if (order == 2) r = 1.0 * r + 0.5 * qh2[i];
    r = -1.0 * r;
    if (limiter) {
      r = 1.0 * r + 1.0 * (qs * qvp[i]);
      r = 1.0 * r + fs * fvp[i];
    }
    rhs[i] = r;
  }
}

/* OneStep::obtainJacobian (N_TIA_OneStep.C:297-352): J = (-alphas/h) dQdx +
 * f dFdx over the matrix values. */
void xgo_tia_jacobian(int64_t nnz, int order, double h, double alphas, const double *dqdx,
                      const double *dfdx, double *jac) {
  const double qs = -alphas / h, fs = order == 2 ? 0.5 : 1.0;
  for (int64_t p = 0; p < nnz; ++p) jac[p] = qs * dqdx[p] + fs * dfdx[p];
}

/* computeErrorEstimate = ck * WRMS_errorNorm (N_TIA_OneStep.h:97), with the
 * weights of DataStore::setErrorWtVector (N_TIA_DataStore.C:1200-1370;
 * newLte, every unknown treated as a voltage): reltol |x_curr|_inf + abstol,
 * and the norm sqrt(sum((corr_i / w)^2) / n) of the Newton correction
 * corr = x - predictor (N_TIA_DataStore.C:1380-1400). */
double xgo_tia_error_estimate(int n, double ck, const double *x_curr, const double *corr,
                              double reltol, double abstol) {
  double xmax = 0.0;
  for (int i = 0; i < n; ++i) xmax = fabs(x_curr[i]) > xmax ? fabs(x_curr[i]) : xmax;
  const double wt = reltol * xmax + abstol;
  double s2 = 0.0;
  for (int i = 0; i < n; ++i) {
    const double e = corr[i] / wt;
    s2 += e * e;
  }
  return ck * sqrt(s2 / n);
}

/* Damped Newton convergence test, N_NLS_DampedNewton.C:1787-1919: the
 * status of a Newton step (1, 2, 3, 4: converged; -1, -2, -3: failed; 0:
 * go on) from the residual's max norm, the weighted norm of the update, the
 * residual's reduction and its rate.  *count / *stall_rate carry the stall
 * counter from one step to the next.  small_update: the solver's
 * smallUpdateTol (1e-6). */
int xgo_nls_converged(int transient, int step, int max_step, double rhs_tol, double dx_tol,
                      double small_update, double max_rhs, double upd, double rhs_rel, double rate,
                      int *count, double *stall_rate) {
  const double eps = DBL_EPSILON, rate_max = 0.5 * DBL_MAX, min_red = 0.9, stag = 1e-3;
  if (max_rhs <= eps && max_rhs <= rhs_tol) return 1;
  if (max_rhs <= rhs_tol && upd <= dx_tol) return 2;
  if (step > max_step && transient)
    if (rhs_rel <= min_red && rate <= 1.0) return 3;
  if (upd <= small_update) return 4;
  if (step > max_step) return -1;
  else if (rate > rate_max) return -2;
  if (transient && fabs(rate - 1.0) <= stag) {
    if (*count == 0 || rate < *stall_rate) *stall_rate = rate;
    (*count)++;
  } else {
    *count = 0;
  }
  if (transient && *count == 5) {
    *count = 0;
    return (rhs_rel < min_red && *stall_rate <= 1.0) ? 3 : -3;
  }
  return 0;
}

/* Step control after an accepted step: OneStep::completeStep
 * (N_TIA_OneStep.C:1945-2190) with the history update (updateHistory,
 * :1209-1300).  in[17]: order, steps taken, error-test failures, estOverTol,
 * h, t, t_next, stop time, min step, max step, last step, h_sum, psi[3],
 * Newton status, saved step.  hist: the solution history 0..2 then the
 * charge history 0..2 (n each, rotated in place); x_next, Q, F: the accepted
 * point.  out[12]: order, steps, failures, h, t, t_next, last step, h_sum,
 * saved step, psi[3]. */
void xgo_tia_complete_step(int n, const double *in, double *const *hist, const double *x_next,
                           const double *Q, const double *F, double *out) {
  const double tol_aim = 0.5, r_min = 0.25, r_max = 0.9, r_hincr_test = 2.0, r_hincr = 2.0;
  int order = (int)in[0], n_steps = (int)in[1] + 1;
  const double est = in[3], h = in[4], t = in[6], stop_time = in[7], min_step = in[8];
  const double max_step = in[9];
  double next_time = in[6], h_sum = in[11], saved = in[16];
  double hn = h, rr = pow(tol_aim / (est + 0.0001), 1.0 / (order + 1.0));
  if (n_steps >= 2 && order == 1) {
    order = 2;
    rr = pow(tol_aim / (est + 0.0001), 1.0 / (order + 1.0));
    if (rr <= 1.05) order = 1;
  }
  if (rr >= r_hincr_test) {
    rr = r_hincr;
    hn = rr * h;
  } else if (rr <= 1) {
    rr = fmax(r_min, fmin(r_max, rr));
    hn = rr * h;
  }
  /* updateHistory, with the order chosen for the next step: a trapezoid
   * step keeps F of the accepted point */
  double *xh0 = hist[0], *xh1 = hist[1], *xh2 = hist[2], *qh0 = hist[3], *qh1 = hist[4], *qh2 = hist[5];
  if (order == 2) {
    memcpy(xh2, xh1, sizeof(double) * n);
    memcpy(qh2, F, sizeof(double) * n);
  }
  for (int i = 0; i < n; ++i) {
    xh1[i] = 1.0 * x_next[i] + -1.0 * xh0[i];
    qh1[i] = 1.0 * Q[i] + -1.0 * qh0[i];
  }
  memcpy(xh0, x_next, sizeof(double) * n);
  memcpy(qh0, Q, sizeof(double) * n);
  hn = fmax(hn, min_step);
  hn = fmin(hn, max_step);
  if (stop_time - t >= min_step) {
    double next_pt = t + hn;
    if (next_pt > stop_time) {
      saved = hn;
      next_pt = stop_time;
      hn = stop_time - t;
    }
    next_time = next_pt;
    h_sum = hn + h;
  }
  out[0] = order;
  out[1] = n_steps;
  out[2] = 0;
  out[3] = hn;
  out[4] = t;
  out[5] = next_time;
  out[6] = h;
  out[7] = h_sum;
  out[8] = saved;
  for (int k = 0; k < 3; ++k) out[9 + k] = in[12 + k];
}

/* Step control after a failed step: OneStep::rejectStep
 * (N_TIA_OneStep.C:1695-1930), in the reference's default build (no
 * Xyce_USE_Q_NORM: r_factor 1, r_safety 2, r_fudge 1e-4, and newOrder 1,
 * which the one-step method never changes, N_TIA_StepErrorControl.C:155-176).
 * A Newton failure retries an eighth of the step, a first local-error
 * failure r = (2 (est + 1e-4))^(-1/2) clamped to [0.25, 0.9], a later one a
 * quarter; each at order 1.  in / out as xgo_tia_complete_step. */
void xgo_tia_reject_step(const double *in, double *out) {
  const double r_min = 0.25, r_max = 0.9, r_factor = 1.0, r_safety = 2.0, r_fudge = 0.0001;
  const int new_order = 1;
  int order = (int)in[0], nef = (int)in[2] + 1;
  const double est = in[3], h = in[4], t = in[5], stop_time = in[7], min_step = in[8];
  const double max_step = in[9], h_last = in[10];
  double psi[3] = {in[12], in[13], in[14]};
  for (int i = 1; i <= order; ++i) psi[i - 1] = psi[i]; /* restoreHistory */
  double hn = h;
  if (in[15] <= 0) {
    hn = h / 8;
    order = 1;
  } else if (nef == 1) {
    double rr = r_factor * pow(r_safety * (est + r_fudge), -1.0 / (new_order + 1.0));
    rr = fmax(r_min, fmin(r_max, rr));
    hn = rr * h;
    order = 1;
  } else {
    hn = r_min * h;
    order = 1;
  }
  hn = fmax(hn, min_step);
  hn = fmin(hn, max_step);
  double next_pt = t + hn;
  if (next_pt > stop_time) {
    next_pt = stop_time;
    hn = stop_time - t;
  }
  out[0] = order;
  out[1] = in[1];
  out[2] = nef;
  out[3] = hn;
  out[4] = t;
  out[5] = next_pt;
  out[6] = h_last;
  out[7] = hn + h_last;
  out[8] = in[16];
  for (int k = 0; k < 3; ++k) out[9 + k] = psi[k];
}

static int do_load(tctx *T, const xg_load_flags *fl) {
  const double *in[9] = {T->sol[0], T->sol[1], T->sol[2], T->sta[0], T->sta[1], T->sta[2],
                         T->sto[0], T->sto[1], T->sto[2]};
  /* sto next holds the previous iterate on entry; the load overwrites it */
  double *sto_out = (double *)xmalloc(sizeof(double) * (T->nsto ? T->nsto : 1));
  double *sta_out = (double *)xmalloc(sizeof(double) * (T->nsta ? T->nsta : 1));
  int rc = xgo_load(T->c, fl, in, T->f, T->q, T->fvp, T->qvp, sta_out, sto_out, T->dfdx, T->dqdx);
  memcpy(T->sta[0], sta_out, sizeof(double) * T->nsta);
  memcpy(T->sto[0], sto_out, sizeof(double) * T->nsto);
  free(sto_out);
  free(sta_out);
  T->st->loads++;
  return rc;
}

static int converged(tctx *T, int transient, int step, int max_step, double rhs_tol, double dx_tol,
                     double max_rhs, double upd, double rhs_rel, double rate) {
  return xgo_nls_converged(transient, step, max_step, rhs_tol, dx_tol, 1e-6, max_rhs, upd, rhs_rel,
                           rate, &T->stall_count, &T->stall_rate);
}

/* One Newton solve.  transient: trapezoid/BE residual with step h and order;
 * otherwise the DC operating point.  Returns the convergence status. */
static int newton(tctx *T, int transient, double h, int order, double time, int init_tran) {
  const int n = T->n;
  const int max_step = transient ? 20 : 200;
  const double rhs_tol = transient ? 1e-2 : 1e-6;
  double dx_tol = transient ? 0.33 : 1.0;
  const double abs_tol = transient ? 1e-6 : 1e-12, rel_tol = transient ? 1e-2 : 1e-3;
  if (T->first_solve) { dx_tol *= 0.01; T->first_solve = 0; }
  const double fs = (transient && order == 2) ? 0.5 : 1.0;
  xg_load_flags fl;
  memset(&fl, 0, sizeof(fl));
  fl.dcop = !transient;
  fl.tranop = !transient;
  fl.transient = transient;
  fl.time = time;
  fl.init_tran = init_tran;
  fl.pdt = transient ? 1.0 / h : 0.0;
  int any_limit = 0;
#define RESIDUAL()                                                                        \
  do {                                                                                    \
    if (transient) {                                                                      \
      xgo_tia_residual(n, order, h, -1.0, 1, T->q, T->qn0, T->f, T->qh2, T->fvp, T->qvp,  \
                       T->rhs);                                                           \
    } else {                                                                              \
      for (int i = 0; i < n; ++i) T->rhs[i] = -T->f[i] + T->fvp[i];                       \
      if (T->gshunt > 0)                                                                  \
        for (int i = 0; i < T->c->n_nodes; ++i)                                           \
          if (T->diag[i] >= 0) T->rhs[i] -= T->gshunt * T->sol[0][i];                     \
    }                                                                                     \
    any_limit = inf_norm(T->fvp, n) != 0.0 || inf_norm(T->qvp, n) != 0.0;                 \
  } while (0)
  fl.newton_iter = 0;
  fl.init_jct = !transient && T->st->dcop_solves == 0;
  if (do_load(T, &fl)) return -10;
  RESIDUAL();
  double norm_rhs = two_norm(T->rhs, n), max_rhs = inf_norm(T->rhs, n);
  if (norm_rhs < DBL_EPSILON) return 1;
  const double norm_init = norm_rhs;
  double norm_old = norm_rhs;
  if (transient)
    for (int i = 0; i < n; ++i)
      T->w[i] = rel_tol * fmax(fabs(T->sol[1][i]), fabs(T->sol[0][i])) + abs_tol;
  int status = 0, step = 0;
  while (status == 0) {
    ++step;
    if (transient) {
      xgo_tia_jacobian(T->nnz, order, h, -1.0, T->dqdx, T->dfdx, T->jac);
    } else {
      for (int64_t p = 0; p < T->nnz; ++p) T->jac[p] = 1.0e-20 * T->dqdx[p] + fs * T->dfdx[p];
    }
    if (!transient && T->gshunt > 0)
      for (int i = 0; i < T->c->n_nodes; ++i)
        if (T->diag[i] >= 0) T->jac[T->diag[i]] += T->gshunt;
    T->st->factorizations++;
    if (xlu_factor(T->lu, T->jac, 1e-3)) return -5;
    xlu_solve(T->lu, T->rhs, T->dx);
    for (int i = 0; i < n; ++i) T->sol[0][i] += T->dx[i];
    fl.newton_iter = step;
    fl.init_jct = 0;
    fl.init_fix = !transient && T->st->dcop_solves == 0 && any_limit;
    if (do_load(T, &fl)) return -10;
    RESIDUAL();
    if (!transient)
      for (int i = 0; i < n; ++i)
        T->w[i] = rel_tol * fmax(fabs(T->sol[1][i]), fabs(T->sol[0][i])) + abs_tol;
    double upd = wrms(T->dx, T->w, n);
    norm_rhs = two_norm(T->rhs, n);
    max_rhs = inf_norm(T->rhs, n);
    double rhs_rel = norm_rhs / norm_init, rate = norm_rhs / norm_old;
    norm_old = norm_rhs;
    T->st->newton_iters++;
    status = converged(T, transient, step, max_step, rhs_tol, dx_tol, max_rhs, upd, rhs_rel, rate);
    if (getenv("XGO_TRAN_DEBUG") && !transient)
      fprintf(stderr, "  dc step %d g=%.1e max_rhs=%.3e upd=%.3e rate=%.3e status=%d\n", step,
              T->gshunt, max_rhs, upd, rate, status);
    if (max_rhs != 0.0 && !(max_rhs < 0.0) && !(max_rhs > 0.0)) status = -6;
  }
#undef RESIDUAL
  return status;
}

static int cmp_double(const void *a, const void *b) {
  double x = *(const double *)a, y = *(const double *)b;
  return x < y ? -1 : x > y;
}

/* PULSE corners of voltage and current sources up to tstop, sorted, without
 * duplicates (PulseData::getBreakPoints). */
static double *breakpoints(const xgo_circuit *c, double tstop, int *nbp) {
  int cap = 64, nb = 0;
  double *bp = (double *)xmalloc(sizeof(double) * cap);
  for (int src = 0; src < 2; ++src) {
    const xgo_type *V = &c->T[src == 0 ? XG_DEV_VSRC : XG_DEV_ISRC];
    for (int i = 0; i < V->n; ++i) {
      if (P(V, XG_V_KIND, i) != XG_SRC_PULSE) continue;
      double td = P(V, XG_V_TD, i), tr = P(V, XG_V_TR, i), tf = P(V, XG_V_TF, i);
      double pw = P(V, XG_V_PW, i), per = P(V, XG_V_PER, i);
      for (int k = 0;; ++k) {
        double base = per > 0 ? per * k : 0.0;
        double pts[4] = {base + td, base + td + tr, base + td + tr + pw, base + td + tr + pw + tf};
        for (int j = 0; j < 4; ++j) {
          if (pts[j] <= 0.0 || pts[j] >= tstop) continue;
          if (nb == cap) { cap *= 2; bp = (double *)realloc(bp, sizeof(double) * cap); }
          bp[nb++] = pts[j];
        }
        if (per <= 0 || base + td >= tstop) break;
      }
    }
  }
  if (nb == cap) bp = (double *)realloc(bp, sizeof(double) * (cap + 1));
  bp[nb++] = tstop;
  qsort(bp, nb, sizeof(double), cmp_double);
  int m = 0;
  for (int i = 0; i < nb; ++i)
    if (m == 0 || bp[i] > bp[m - 1]) bp[m++] = bp[i];
  *nbp = m;
  return bp;
}

int xgo_tran_run(xgo_circuit *c, const xgo_tran_opts *o, double *t_out, double *v_out,
                 int *n_points, xgo_tran_stats *st) {
  memset(st, 0, sizeof(*st));
  tctx T;
  memset(&T, 0, sizeof(T));
  T.c = c;
  T.st = st;
  T.n = c->n_unk;
  T.nr = c->n_unk + 1;
  T.nsta = c->n_sta;
  T.nsto = c->n_sto;
  T.nnz = c->nnz;
  T.first_solve = 1;
  const int n = T.n, nr = T.nr;
  for (int k = 0; k < 3; ++k) {
    T.sol[k] = (double *)calloc(nr, sizeof(double));
    T.sta[k] = (double *)calloc(T.nsta + 1, sizeof(double));
    T.sto[k] = (double *)calloc(T.nsto + 1, sizeof(double));
  }
  double **vs[] = {&T.f, &T.q, &T.fvp, &T.qvp, &T.rhs, &T.dx, &T.w, &T.xh0, &T.xh1, &T.xh2,
                   &T.qh0, &T.qh1, &T.qh2, &T.xn0, &T.qn0};
  for (size_t k = 0; k < sizeof(vs) / sizeof(vs[0]); ++k) *vs[k] = (double *)calloc(nr, sizeof(double));
  T.dfdx = (double *)calloc(T.nnz + 1, sizeof(double));
  T.dqdx = (double *)calloc(T.nnz + 1, sizeof(double));
  T.jac = (double *)calloc(T.nnz + 1, sizeof(double));
  T.lu = xlu_new(n, c->rowptr, c->col, o->col_order);
  xgo_reset_members(c);
  int nbp = 0;
  double *bp = breakpoints(c, o->tstop, &nbp);
  const double bp_tol = 1e-18;
  int np = 0, rc = 0;
#define RECORD(tt)                                                              \
  do {                                                                          \
    if (np < o->max_points) {                                                   \
      t_out[np] = (tt);                                                         \
      for (int k = 0; k < o->n_out; ++k) v_out[(int64_t)np * o->n_out + k] = T.sol[1][o->out_idx[k]]; \
      ++np;                                                                     \
    }                                                                           \
  } while (0)

  /* DC operating point: plain Newton from zero; if that fails, gmin
   * stepping (a shunt conductance on every node row, 1e-2 down to 1e-12 by
   * decades, each solve starting from the last) and a final plain solve */
  T.diag = (int64_t *)xmalloc(sizeof(int64_t) * nr);
  for (int i = 0; i < n; ++i) {
    T.diag[i] = -1;
    for (int p = c->rowptr[i]; p < c->rowptr[i + 1]; ++p)
      if (c->col[p] == i) T.diag[i] = p;
  }
  if (o->x0) memcpy(T.sol[0], o->x0, sizeof(double) * n);
  memcpy(T.sol[1], T.sol[0], sizeof(double) * nr);
  int s = 1;
  if (o->uic) {
    /* start from x0: one load there supplies F and Q for the history */
    xg_load_flags fl;
    memset(&fl, 0, sizeof(fl));
    fl.dcop = 1;
    fl.tranop = 1;
    if (do_load(&T, &fl)) s = -10;
  } else {
    s = newton(&T, 0, 0.0, 1, 0.0, 0);
  }
  st->dcop_solves = 1;
  if (s <= 0 && !o->uic) {
    if (o->x0) memcpy(T.sol[0], o->x0, sizeof(double) * n);
    else memset(T.sol[0], 0, sizeof(double) * nr);
    memset(T.sto[0], 0, sizeof(double) * (T.nsto + 1));
    xgo_reset_members(c);
    for (double g = 1e-2; g >= 0.99e-12 && s != -100; g *= 0.1) {
      T.gshunt = g;
      memcpy(T.sol[1], T.sol[0], sizeof(double) * nr);
      s = newton(&T, 0, 0.0, 1, 0.0, 0);
      if (s <= 0) break;
    }
    T.gshunt = 0.0;
    if (s > 0) {
      memcpy(T.sol[1], T.sol[0], sizeof(double) * nr);
      s = newton(&T, 0, 0.0, 1, 0.0, 0);
    }
  }
  st->dcop_iters = st->newton_iters;
  if (s <= 0) { rc = -1; st->status = s; goto done; }
  memcpy(T.sol[1], T.sol[0], sizeof(double) * nr);
  memcpy(T.sol[2], T.sol[0], sizeof(double) * nr);
  memcpy(T.sta[1], T.sta[0], sizeof(double) * T.nsta);
  memcpy(T.sta[2], T.sta[0], sizeof(double) * T.nsta);
  memcpy(T.sto[1], T.sto[0], sizeof(double) * T.nsto);
  memcpy(T.sto[2], T.sto[0], sizeof(double) * T.nsto);
  RECORD(0.0);
  {
    const double tstop = o->tstop, reltol = o->reltol, abstol = o->abstol;
    const double max_step = o->maxstep > 0 ? o->maxstep : 0.1 * tstop;
    const double h0_max_factor = 0.005;
    const double starting = o->tstep > 0 ? o->tstep : 1e-10;
    double t = 0.0, h = starting, h_last = starting, h_sum = 2 * starting, saved = 1e-10;
    double next_time = 0.0, stop_time = tstop;
    double psi[3] = {0, 0, 0}, beta[3] = {1, 0, 0}, ck = 1;
    int order = 1, n_steps = 0, nef = 0, beginning = 1, accepted_last = 1, first_step = 1;
    int bpi = 0;
    const int debug = getenv("XGO_TRAN_DEBUG") != NULL;
    while (t < tstop && fabs(t - tstop) > bp_tol) {
      /* stop time: the first breakpoint after t */
      while (bpi < nbp && bp[bpi] <= t + bp_tol) ++bpi;
      stop_time = bpi < nbp ? bp[bpi] : tstop;
      if (beginning && accepted_last) {
        /* OneStep::initialize */
        double tts = stop_time - t, hh;
        if (t == 0.0) hh = h0_max_factor * fabs(tts);
        else hh = 0.1 * fmin(saved, fabs(tts));
        if (starting > 0.0 && t == 0.0) hh = fmin(starting, hh);
        if (hh > max_step) hh = max_step;
        h = (t != 0.0) ? fmin(h, hh) : hh;
        h_sum = 2.0 * h;
        h_last = h;
        next_time = t + h;
        memcpy(T.xh0, T.sol[1], sizeof(double) * n);
        memset(T.xh1, 0, sizeof(double) * n);
        memcpy(T.qh0, T.q, sizeof(double) * n);
        for (int i = 0; i < n; ++i) T.qh1[i] = -h * T.f[i];
        n_steps = 0;
        order = 1;
        psi[0] = h;
      }
      double alphas;
      xgo_tia_update_coeffs(order, h, h_sum, psi, beta, &alphas, &ck);
      xgo_tia_predictor(n, order, beta, T.xh0, T.xh1, T.xh2, T.qh0, T.xn0, T.qn0);
      memcpy(T.sol[0], T.xn0, sizeof(double) * n);
      memcpy(T.sta[0], T.sta[1], sizeof(double) * T.nsta);
      memcpy(T.sto[0], T.sto[1], sizeof(double) * T.nsto);
      int ns = newton(&T, 1, h, order, next_time, first_step);
      st->steps_attempted++;
      if (debug)
        fprintf(stderr, "t=%.6e h=%.3e order=%d beg=%d newton=%d iters=%d stop=%.6e\n", t, h, order,
                beginning, ns, st->newton_iters, stop_time);
      /* evaluateStepError */
      int ok = ns >= 0;
      double est = 0.0;
      if (ok && st->steps >= 1 && !beginning) {
        for (int i = 0; i < n; ++i) T.dx[i] = T.sol[0][i] - T.xn0[i];  /* the Newton correction */
        est = xgo_tia_error_estimate(n, ck, T.sol[1], T.dx, reltol, abstol);
        ok = est <= 1.0;
        if (debug) fprintf(stderr, "   est=%.3e ck=%.3e\n", est, ck);
      }
      if (ok) {
        /* completeStep, with the minimum step from machine precision at the
         * new time (StepErrorControl::updateMinTimeStep) */
        first_step = 0;
        st->steps++;
        double in[17] = {order, n_steps, nef, est, h, t, next_time, stop_time,
                         next_time * 10.0 * DBL_EPSILON, max_step, h_last, h_sum, psi[0], psi[1],
                         psi[2], ns, saved};
        double out[12];
        double *hist[6] = {T.xh0, T.xh1, T.xh2, T.qh0, T.qh1, T.qh2};
        xgo_tia_complete_step(n, in, hist, T.sol[0], T.q, T.f, out);
        order = (int)out[0];
        n_steps = (int)out[1];
        nef = (int)out[2];
        h = out[3];
        t = out[4];
        next_time = out[5];
        h_last = out[6];
        h_sum = out[7];
        saved = out[8];
        /* rotate the accepted point into current / last */
        memcpy(T.sol[2], T.sol[1], sizeof(double) * nr);
        memcpy(T.sol[1], T.sol[0], sizeof(double) * nr);
        memcpy(T.sta[2], T.sta[1], sizeof(double) * T.nsta);
        memcpy(T.sta[1], T.sta[0], sizeof(double) * T.nsta);
        memcpy(T.sto[2], T.sto[1], sizeof(double) * T.nsto);
        memcpy(T.sto[1], T.sto[0], sizeof(double) * T.nsto);
        RECORD(t);
        beginning = fabs(t - stop_time) <= bp_tol && fabs(t - tstop) > bp_tol;
        accepted_last = 1;
      } else {
        /* rejectStep */
        st->rejected++;
        accepted_last = 0;
        if (nef + 1 >= 15) { rc = -2; st->status = -7; goto done; }
        double in[17] = {order, n_steps, nef, est, h, t, next_time, stop_time,
                         t * 10.0 * DBL_EPSILON, max_step, h_last, h_sum, psi[0], psi[1], psi[2],
                         ns, saved};
        double out[12];
        xgo_tia_reject_step(in, out);
        order = (int)out[0];
        nef = (int)out[2];
        h = out[3];
        next_time = out[5];
        h_sum = out[7];
        for (int k = 0; k < 3; ++k) psi[k] = out[9 + k];
        if (h < 1e-21) { rc = -3; st->status = -8; goto done; }
      }
    }
  }
done:
  *n_points = np;
#undef RECORD
  free(bp);
  xlu_free(T.lu);
  for (int k = 0; k < 3; ++k) { free(T.sol[k]); free(T.sta[k]); free(T.sto[k]); }
  for (size_t k = 0; k < sizeof(vs) / sizeof(vs[0]); ++k) free(*vs[k]);
  free(T.dfdx); free(T.dqdx); free(T.jac); free(T.diag);
  return rc;
}

/* Standalone sparse solve with the same LU (checks the linear algebra). */
int xgo_sparse_solve(int n, const int *rowptr, const int *col, const double *val,
                     const int *col_order, const double *b, double *x) {
  xlu_t *f = xlu_new(n, rowptr, col, col_order);
  int rc = xlu_factor(f, val, 1e-3);
  if (!rc) xlu_solve(f, b, x);
  xlu_free(f);
  return rc;
}
