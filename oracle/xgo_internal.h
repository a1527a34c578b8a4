/* xgo_internal.h — oracle internals (TEST INFRASTRUCTURE ONLY; see xgo.h). */
#ifndef XGO_INTERNAL_H
#define XGO_INTERNAL_H

#include "xgo.h"

typedef struct {
  int n, np;               /* instances, params per instance            */
  const double *p;         /* SoA param block: p[k * n + i]             */
  int nlid;                /* solution LIDs per instance                */
  int *lid;                /* lid[i * nlid + j], ground = n_unk         */
  int sta0, nsta, sto0, nsto;
  void *m;                 /* per-instance members (type specific)      */
} xgo_type;

struct xgo_circuit {
  xg_device_options opt;
  int n_nodes, n_unk, n_sta, n_sto;
  int order[XG_NUM_DEV_TYPES], n_order;
  xgo_type T[XG_NUM_DEV_TYPES];
  int *rowptr, *col;
  int64_t nnz;
  int bad_slot;
  double *diode_vd;        /* Diode Instance::Vd carried between loads  */
  void *b3_member;         /* BSIM3 members carried between loads       */
  /* Matrix positions of each instance's dFdx/dQdx stamps in call order,
   * found once at build (the reference caches the same positions as
   * pointers, registerJacLIDs/setupPointers); a call whose (row, col) does
   * not match the cached entry falls back to a search. */
  int *slot_rc;            /* [3 * k]: row, col, position */
  int64_t *slot_off[XG_NUM_DEV_TYPES];
  int64_t n_slots, cap_slots, cursor;
  int recording;
};

typedef struct {
  const xg_load_flags *fl;
  const double *sol, *sol_curr, *sol_last;
  const double *sta_curr, *sta_last, *sto_curr, *sto_last;
  double *sta, *sto;       /* next state / store (written)              */
  double *f, *q, *dfdxdvp, *dqdxdvp, *dfdx, *dqdx;
} xgo_io;

#define P(T, k, i) ((T)->p[(int64_t)(k) * (T)->n + (i)])

int xgo_slot(const xgo_circuit *c, int r, int col);
void xgo_madd(xgo_circuit *c, double *vals, int r, int col, double v);
void xgo_msub(xgo_circuit *c, double *vals, int r, int col, double v);

/* per-type dispatch (xgo_devices.c) */
int xgo_nlid(int t);
void xgo_assign_lids(xgo_circuit *c, const xg_netlist *nl, int t, int i, int *next);
int xgo_nsta(const xgo_circuit *c, int t);
int xgo_nsto(int t);
int xgo_max_stamps(int t);
int xgo_stamps(const xgo_circuit *c, int t, int i, int *rows, int *cols);
void xgo_update_state(xgo_circuit *c, int t, int i0, int i1, xgo_io *io);
void xgo_load_vectors(xgo_circuit *c, int t, int i0, int i1, xgo_io *io);
void xgo_load_matrices(xgo_circuit *c, int t, int i0, int i1, xgo_io *io);

/* DeviceSupport restatements (xgo_support.c) */
double xgo_limvds(double vnew, double vold);
double xgo_pnjlim(double vnew, double vold, double vt, double vcrit, int *icheck);
double xgo_fetlim(double vnew, double vold, double vto);
void xgo_qmeyer(double vgs, double vgd, double vgb, double von, double vdsat,
                double *capgs, double *capgd, double *capgb, double phi, double cox);

/* set-up (xgo_setup.c, xgo_b3setup.c) */
int xgo_card_eq(const char *a, const char *b);
int xgo_b3_setup(const xg_netlist *nl, const xg_device_options *opt, double *out);

/* BSIM3 (xgo_bsim3.c) */
int xgo_b3_nparams(void);
void *xgo_b3_members_alloc(int n);
void xgo_b3_members_reset(void *m, int n);
int xgo_b3_nlid(void);
int xgo_b3_nint(const xgo_type *T, int i);
void xgo_b3_lids(const xgo_type *T, int i, const int *ext, int *next, int *lid);
int xgo_b3_stamps(const xgo_type *T, int i, int *rows, int *cols);
void xgo_b3_update_state(xgo_circuit *c, int i0, int i1, xgo_io *io);
void xgo_b3_load_vectors(xgo_circuit *c, int i0, int i1, xgo_io *io);
void xgo_b3_load_matrices(xgo_circuit *c, int i0, int i1, xgo_io *io);

#endif
