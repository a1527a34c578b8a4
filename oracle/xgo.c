/*
 * xgo.c — CPU oracle for the Newton load (TEST INFRASTRUCTURE ONLY; see xgo.h).
 *
 * A serial restatement, in plain C, of what the reference does for one load:
 *   DeviceMgr::updateState -> every Master::updateState   (N_DEV_DeviceMgr.C:2201-2285)
 *   DeviceMgr::loadDAEVectors -> every Master::loadDAEVectors (N_DEV_DeviceMgr.C:2520-2661)
 *   DeviceMgr::loadDAEMatrices -> every Master::loadDAEMatrices (N_DEV_DeviceMgr.C:2329-2479)
 * with device types visited in load order, instances in creation order and
 * stamps in statement order, each `+=` / `-=` applied one at a time.
 */
#include "xgo.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "xgo_internal.h"

/* ---- helpers -------------------------------------------------------------- */

static int cmp_i64(const void *a, const void *b) {
  int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return (x > y) - (x < y);
}

int xgo_slot(const xgo_circuit *c, int r, int col) {
  if (r >= c->n_unk || col >= c->n_unk) return -1; /* ground row/col */
  int lo = c->rowptr[r], hi = c->rowptr[r + 1] - 1;
  while (lo <= hi) {
    int mid = (lo + hi) >> 1;
    if (c->col[mid] == col) return mid;
    if (c->col[mid] < col) lo = mid + 1; else hi = mid - 1;
  }
  return -2; /* not in pattern: a bug in the stamp enumeration */
}

static int cached_slot(xgo_circuit *c, int r, int col) {
  if (c->recording) {
    int s = xgo_slot(c, r, col);
    if (c->n_slots == c->cap_slots) {
      c->cap_slots = c->cap_slots ? 2 * c->cap_slots : 1024;
      c->slot_rc = (int *)realloc(c->slot_rc, sizeof(int) * 3 * (size_t)c->cap_slots);
    }
    int *e = c->slot_rc + 3 * c->n_slots++;
    e[0] = r; e[1] = col; e[2] = s;
    return s;
  }
  if (c->slot_rc && c->cursor < c->n_slots) {
    const int *e = c->slot_rc + 3 * c->cursor;
    if (e[0] == r && e[1] == col) {
      ++c->cursor;
      return e[2];
    }
  }
  return xgo_slot(c, r, col);
}

/* dFdx / dQdx `+=` (sign +1) or `-=` (sign -1) on one entry. */
void xgo_madd(xgo_circuit *c, double *vals, int r, int col, double v) {
  int s = cached_slot(c, r, col);
  if (s >= 0) vals[s] += v;
  else if (s == -2) c->bad_slot = 1;
}
void xgo_msub(xgo_circuit *c, double *vals, int r, int col, double v) {
  int s = cached_slot(c, r, col);
  if (s >= 0) vals[s] -= v;
  else if (s == -2) c->bad_slot = 1;
}

static int type_count(const xg_netlist *nl, int t) {
  switch (t) {
    case XG_DEV_RES: return nl->res.n;
    case XG_DEV_CAP: return nl->cap.n;
    case XG_DEV_VSRC: return nl->vsrc.n;
    case XG_DEV_ISRC: return nl->isrc.n;
    case XG_DEV_DIODE: return nl->diode.n;
    case XG_DEV_MOS1: return nl->mos1.n;
    case XG_DEV_BSIM3: return nl->bsim3.n;
  }
  return 0;
}

static int nparams_of(int t) {
  switch (t) {
    case XG_DEV_RES: return XG_R_NPARAMS;
    case XG_DEV_CAP: return XG_C_NPARAMS;
    case XG_DEV_VSRC: case XG_DEV_ISRC: return XG_V_NPARAMS;
    case XG_DEV_DIODE: return XG_D_NPARAMS;
    case XG_DEV_MOS1: return XG_M1_NPARAMS;
    case XG_DEV_BSIM3: return xgo_b3_nparams();
  }
  return 0;
}

/* ---- build ---------------------------------------------------------------- */

int xgo_build(const xg_netlist *nl, const xg_device_options *opt,
              const double *const *params, xgo_circuit **out) {
  xgo_circuit *c = (xgo_circuit *)calloc(1, sizeof *c);
  if (!c) return XG_ERR_OOM;
  c->opt = *opt;
  c->n_nodes = nl->n_nodes;
  if (nl->type_order && nl->n_type_order > 0) {
    c->n_order = nl->n_type_order;
    for (int i = 0; i < c->n_order; ++i) c->order[i] = nl->type_order[i];
  } else {
    c->n_order = XG_NUM_DEV_TYPES;
    for (int i = 0; i < XG_NUM_DEV_TYPES; ++i) c->order[i] = i;
  }
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) {
    xgo_type *T = &c->T[t];
    T->n = type_count(nl, t);
    T->np = nparams_of(t);
    T->p = params ? params[t] : NULL;
    if (T->n > 0 && !T->p) { free(c); return XG_ERR_ARG; }
  }

  /* LIDs: nodes, then internal unknowns by type order and instance. */
  int next = nl->n_nodes;
  for (int k = 0; k < c->n_order; ++k) {
    int t = c->order[k];
    xgo_type *T = &c->T[t];
    if (!T->n) continue;
    T->nlid = xgo_nlid(t);
    T->lid = (int *)malloc(sizeof(int) * (size_t)T->nlid * T->n);
    for (int i = 0; i < T->n; ++i) xgo_assign_lids(c, nl, t, i, &next);
  }
  c->n_unk = next;
  /* ground was recorded as -1 during assignment: map it to n_unk */
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) {
    xgo_type *T = &c->T[t];
    for (int64_t j = 0; j < (int64_t)T->nlid * T->n; ++j)
      if (T->lid[j] < 0) T->lid[j] = c->n_unk;
  }
  /* State / store layout. */
  int sta = 0, sto = 0;
  for (int k = 0; k < c->n_order; ++k) {
    int t = c->order[k];
    xgo_type *T = &c->T[t];
    if (!T->n) continue;
    T->sta0 = sta;
    T->sto0 = sto;
    T->nsta = xgo_nsta(c, t);
    T->nsto = xgo_nsto(t);
    if (t == XG_DEV_DIODE) {
      /* one state slot per diode whose CJO == 0 (N_DEV_Diode.C:392-393);
       * the load never touches it, it only shifts later types' slots */
      for (int i = 0; i < T->n; ++i) sta += P(T, XG_D_TJCTCAP, i) == 0.0 ? 1 : 0;
    } else {
      sta += T->nsta * T->n;
    }
    sto += T->nsto * T->n;
  }
  c->n_sta = sta;
  c->n_sto = sto;

  /* Pattern: every stamp (row, col) of every instance, ground excluded. */
  int64_t cap = 0;
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) cap += (int64_t)c->T[t].n * xgo_max_stamps(t);
  int64_t *keys = (int64_t *)malloc(sizeof(int64_t) * (size_t)(cap + 1));
  int64_t nk = 0;
  const int64_t W = (int64_t)c->n_unk + 1;
  for (int k = 0; k < c->n_order; ++k) {
    int t = c->order[k];
    for (int i = 0; i < c->T[t].n; ++i) {
      int rows[64], cols[64];
      int ns = xgo_stamps(c, t, i, rows, cols);
      for (int s = 0; s < ns; ++s)
        if (rows[s] < c->n_unk && cols[s] < c->n_unk) keys[nk++] = rows[s] * W + cols[s];
    }
  }
  qsort(keys, (size_t)nk, sizeof(int64_t), cmp_i64);
  int64_t nu = 0;
  for (int64_t j = 0; j < nk; ++j)
    if (nu == 0 || keys[j] != keys[nu - 1]) keys[nu++] = keys[j];
  c->nnz = nu;
  c->rowptr = (int *)calloc((size_t)c->n_unk + 1, sizeof(int));
  c->col = (int *)malloc(sizeof(int) * (size_t)(nu + 1));
  for (int64_t j = 0; j < nu; ++j) {
    c->rowptr[keys[j] / W + 1]++;
    c->col[j] = (int)(keys[j] % W);
  }
  for (int r = 0; r < c->n_unk; ++r) c->rowptr[r + 1] += c->rowptr[r];
  free(keys);

  c->diode_vd = (double *)calloc((size_t)c->T[XG_DEV_DIODE].n + 1, sizeof(double));
  c->b3_member = xgo_b3_members_alloc(c->T[XG_DEV_BSIM3].n);

  /* record every instance's stamp positions: one matrix load of a transient
   * Newton iteration on zero vectors (the values are discarded) */
  {
    const size_t nr = (size_t)c->n_unk + 1;
    const size_t nz = nr + (size_t)c->n_sta + (size_t)c->n_sto + 3;
    double *zv = (double *)calloc(nz, sizeof(double));
    double *zs = (double *)calloc(nz, sizeof(double));
    double *m0 = (double *)calloc((size_t)c->nnz + 1, sizeof(double));
    double *m1 = (double *)calloc((size_t)c->nnz + 1, sizeof(double));
    xg_load_flags fl;
    memset(&fl, 0, sizeof fl);
    fl.transient = 1;
    fl.newton_iter = 1;
    xgo_io io;
    memset(&io, 0, sizeof io);
    io.fl = &fl;
    io.sol = io.sol_curr = io.sol_last = zv;
    io.sta_curr = io.sta_last = io.sto_curr = io.sto_last = zv;
    io.sta = io.sto = io.f = io.q = io.dfdxdvp = io.dqdxdvp = zs;
    io.dfdx = m0;
    io.dqdx = m1;
    for (int k = 0; k < c->n_order; ++k)
      if (c->T[c->order[k]].n) xgo_update_state(c, c->order[k], 0, c->T[c->order[k]].n, &io);
    c->recording = 1;
    for (int k = 0; k < c->n_order; ++k) {
      int t = c->order[k];
      int nt = c->T[t].n;
      if (!nt) continue;
      c->slot_off[t] = (int64_t *)malloc(sizeof(int64_t) * ((size_t)nt + 1));
      for (int i = 0; i < nt; ++i) {
        c->slot_off[t][i] = c->n_slots;
        xgo_load_matrices(c, t, i, i + 1, &io);
      }
      c->slot_off[t][nt] = c->n_slots;
    }
    c->recording = 0;
    c->bad_slot = 0;
    xgo_reset_members(c);
    free(zv);
    free(zs);
    free(m0);
    free(m1);
  }
  *out = c;
  return XG_OK;
}

void xgo_free(xgo_circuit *c) {
  if (!c) return;
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) {
    free(c->T[t].lid);
    free(c->T[t].m);
  }
  free(c->rowptr);
  free(c->col);
  free(c->diode_vd);
  free(c->b3_member);
  free(c->slot_rc);
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) free(c->slot_off[t]);
  free(c);
}

int xgo_sizes(const xgo_circuit *c, int *n_unknowns, int *n_state, int *n_store, int64_t *nnz) {
  *n_unknowns = c->n_unk;
  *n_state = c->n_sta;
  *n_store = c->n_sto;
  *nnz = c->nnz;
  return XG_OK;
}

int xgo_pattern(const xgo_circuit *c, int *rowptr, int *col) {
  memcpy(rowptr, c->rowptr, sizeof(int) * ((size_t)c->n_unk + 1));
  memcpy(col, c->col, sizeof(int) * (size_t)c->nnz);
  return XG_OK;
}

int xgo_reset_members(xgo_circuit *c) {
  memset(c->diode_vd, 0, sizeof(double) * ((size_t)c->T[XG_DEV_DIODE].n + 1));
  xgo_b3_members_reset(c->b3_member, c->T[XG_DEV_BSIM3].n);
  return XG_OK;
}

/* ---- load ----------------------------------------------------------------- */

static int run_load(xgo_circuit *c, const xg_load_flags *fl, const double *const *in,
                    int only_type, int i0, int i1, xgo_io *io) {
  io->sol = in[0]; io->sol_curr = in[1]; io->sol_last = in[2];
  io->sta_curr = in[4]; io->sta_last = in[5];
  io->sto_curr = in[7]; io->sto_last = in[8];
  io->fl = fl;
  /* Master::updateState, every type in load order (N_DEV_DeviceMgr.C:2263-2270). */
  for (int k = 0; k < c->n_order; ++k) {
    int t = c->order[k];
    if (!c->T[t].n || (only_type >= 0 && t != only_type)) continue;
    int a = only_type >= 0 ? i0 : 0, b = only_type >= 0 ? i1 : c->T[t].n;
    xgo_update_state(c, t, a, b, io);
  }
  /* Master::loadDAEVectors (N_DEV_DeviceMgr.C:2604-2616). */
  for (int k = 0; k < c->n_order; ++k) {
    int t = c->order[k];
    if (!c->T[t].n || (only_type >= 0 && t != only_type)) continue;
    int a = only_type >= 0 ? i0 : 0, b = only_type >= 0 ? i1 : c->T[t].n;
    xgo_load_vectors(c, t, a, b, io);
  }
  /* Master::loadDAEMatrices (N_DEV_DeviceMgr.C:2385-2397), one instance at
   * a time so each starts at its cached stamp positions. */
  for (int k = 0; k < c->n_order; ++k) {
    int t = c->order[k];
    if (!c->T[t].n || (only_type >= 0 && t != only_type)) continue;
    int a = only_type >= 0 ? i0 : 0, b = only_type >= 0 ? i1 : c->T[t].n;
    for (int i = a; i < b; ++i) {
      c->cursor = c->slot_off[t] ? c->slot_off[t][i] : c->n_slots;
      xgo_load_matrices(c, t, i, i + 1, io);
    }
  }
  return c->bad_slot ? XG_ERR_ARG : XG_OK;
}

int xgo_load(xgo_circuit *c, const xg_load_flags *fl, const double *const *in_vecs,
             double *f, double *q, double *dfdxdvp, double *dqdxdvp,
             double *sta_next, double *sto_next, double *dfdx, double *dqdx) {
  const size_t nr = (size_t)c->n_unk + 1;
  /* The caller zeroes the outputs (N_TIA_Assembler.C:156-161). */
  memset(f, 0, nr * sizeof(double));
  memset(q, 0, nr * sizeof(double));
  memset(dfdxdvp, 0, nr * sizeof(double));
  memset(dqdxdvp, 0, nr * sizeof(double));
  memset(dfdx, 0, (size_t)c->nnz * sizeof(double));
  memset(dqdx, 0, (size_t)c->nnz * sizeof(double));
  /* next sta/sto start as the caller's vectors: sto next holds the previous
   * Newton iterate, read by the limiters before it is overwritten. */
  if (c->n_sta) memcpy(sta_next, in_vecs[3], (size_t)c->n_sta * sizeof(double));
  if (c->n_sto) memcpy(sto_next, in_vecs[6], (size_t)c->n_sto * sizeof(double));
  xgo_io io;
  memset(&io, 0, sizeof io);
  io.f = f; io.q = q; io.dfdxdvp = dfdxdvp; io.dqdxdvp = dqdxdvp;
  io.sta = sta_next; io.sto = sto_next; io.dfdx = dfdx; io.dqdx = dqdx;
  return run_load(c, fl, in_vecs, -1, 0, 0, &io);
}

int xgo_load_range(xgo_circuit *c, const xg_load_flags *fl, const double *const *in_vecs,
                   int dev_type, int i0, int i1, double *f, double *q, double *dfdxdvp,
                   double *dqdxdvp, double *sta_next, double *sto_next, double *dfdx,
                   double *dqdx) {
  if (dev_type < 0 || dev_type >= XG_NUM_DEV_TYPES || i0 < 0 || i1 > c->T[dev_type].n || i0 > i1)
    return XG_ERR_ARG;
  xgo_io io;
  memset(&io, 0, sizeof io);
  io.f = f; io.q = q; io.dfdxdvp = dfdxdvp; io.dqdxdvp = dqdxdvp;
  io.sta = sta_next; io.sto = sto_next; io.dfdx = dfdx; io.dqdx = dqdx;
  return run_load(c, fl, in_vecs, dev_type, i0, i1, &io);
}
