/*
 * xg.h — C ABI of the GB300 Newton-load engine (libxg).
 *
 * The engine evaluates SPICE device models (MOSFET level 1, BSIM3 v3.2, junction
 * diode, resistor, capacitor, independent V/I sources) in FP64 on one GPU and
 * stamps their residual and Jacobian contributions into the sparse MNA system.
 * Every sum is taken in a fixed order — device type, then instance, then the
 * statement order of the reference load loop — so F, Q, dF/dx and dQ/dx are
 * identical run to run and match a serial CPU load bit for bit wherever the
 * per-term arithmetic matches.
 *
 * Reference interfaces replaced (paths inside the Xyce source tree):
 *   Device::updateState / updateSecondaryState / loadDAEVectors / loadDAEMatrices
 *       src/DeviceModelPKG/Core/include/N_DEV_Device.h:200-265
 *   DeviceMgr::updateState / loadDAEVectors / loadDAEMatrices (orchestration)
 *       src/DeviceModelPKG/Core/src/N_DEV_DeviceMgr.C:2201-2285, 2329-2479, 2520-2661
 *   Topology stamp -> CSR offset registration
 *       src/TopoManagerPKG/src/N_TOP_CktGraphBasic.C:1092-1142
 *   N_LAS_Matrix row access + linearCombo, N_LAS_Solver::solve
 *       src/LinearAlgebraServicesPKG/src/N_LAS_Matrix.C:835-879
 *       src/LinearAlgebraServicesPKG/include/N_LAS_Solver.h:60-125
 *
 * Conventions
 *   - Every entry point returns int: XG_OK (0) or a negative XG_ERR_* code.
 *     No C++ exception crosses this boundary. xg_last_error() gives a message.
 *   - Pointers named host_* are host memory; pointers named dev_* are device
 *     memory on the context's GPU. Sizes are element counts unless noted.
 *   - Node numbering: circuit nodes are 0..n_nodes-1, ground is -1.  Solution
 *     vectors have one extra trailing slot (index n_unknowns) holding ground,
 *     like the reference's SOLUTION_OVERLAP_GND map (N_LAS_Builder.C:334-341);
 *     contributions to ground are discarded and never reach the solved system.
 *   - Unknown order: circuit nodes first, then each device's internal
 *     unknowns (source branch currents, MOSFET drain'/source' nodes, diode
 *     anode' node) in device-type load order, instance order.
 *   - State (sta) and store (sto) slots are laid out per device type in load
 *     order, instance order, each instance's slots contiguous in the order the
 *     reference registers them (registerStateLIDs / registerStoreLIDs).
 */
#ifndef XG_H
#define XG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XG_ABI_VERSION 1

/* ---- status codes --------------------------------------------------------- */
#define XG_OK               0
#define XG_ERR_ARG         -1   /* bad argument / size / index                   */
#define XG_ERR_CUDA        -2   /* CUDA runtime error                            */
#define XG_ERR_OOM         -3   /* device or host allocation failed              */
#define XG_ERR_SINGULAR    -4   /* zero pivot in LU refactorisation              */
#define XG_ERR_NAN         -5   /* non-finite value in a load or solve           */
#define XG_ERR_TIMEOUT     -6   /* a bounded device wait gave up                 */
#define XG_ERR_STATE       -7   /* call made in the wrong order                  */
#define XG_ERR_UNSUPPORTED -8   /* model option / parameter not implemented      */
#define XG_ERR_NOCONV      -9   /* Newton iteration did not converge             */

/* ---- device types (also the default load order) ---------------------------- */
enum xg_dev_type {
  XG_DEV_RES   = 0,   /* resistor            N_DEV_Resistor.C   */
  XG_DEV_CAP   = 1,   /* capacitor           N_DEV_Capacitor.C  */
  XG_DEV_VSRC  = 2,   /* independent V src   N_DEV_Vsrc.C       */
  XG_DEV_ISRC  = 3,   /* independent I src   N_DEV_ISRC.C       */
  XG_DEV_DIODE = 4,   /* junction diode      N_DEV_Diode.C      */
  XG_DEV_MOS1  = 5,   /* MOSFET level 1      N_DEV_MOSFET1.C    */
  XG_DEV_BSIM3 = 6,   /* BSIM3 v3.2 (lvl 9/49) N_DEV_MOSFET_B3.C */
  XG_NUM_DEV_TYPES = 7
};

/* Source waveform kinds for XG_DEV_VSRC / XG_DEV_ISRC (N_DEV_SourceData.C). */
enum xg_src_kind { XG_SRC_DC = 0, XG_SRC_PULSE = 1 };

/* ---- netlist description (input to setup) ---------------------------------- */

/* A .MODEL card: parameters by (case-insensitive) name, as in a netlist.
 * polarity: +1 for NMOS / diode, -1 for PMOS (the reference's model dtype). */
typedef struct {
  int type;                 /* enum xg_dev_type: XG_DEV_DIODE, XG_DEV_MOS1, XG_DEV_BSIM3 */
  int polarity;
  int n_params;
  const char *const *names;
  const double *values;
} xg_model_desc;

/* MOSFET instances (level 1 or BSIM3). Optional arrays may be NULL (default). */
typedef struct {
  int n;
  const int *d, *g, *s, *b;   /* terminal nodes                             */
  const int *model;           /* index into xg_netlist.models               */
  const double *w, *l;        /* channel width / length [m]                 */
  const double *ad, *as;      /* drain / source area   [m^2]   (optional)   */
  const double *pd, *ps;      /* drain / source perim. [m]     (optional)   */
  const double *nrd, *nrs;    /* drain / source squares        (optional)   */
  const double *m;            /* parallel multiplier           (optional)   */
} xg_mos_desc;

typedef struct {
  int n;
  const int *a, *c;           /* anode / cathode */
  const int *model;
  const double *area;         /* optional, default 1 */
} xg_diode_desc;

/* Two-terminal linear elements: resistor [ohm], capacitor [F], DC current [A]. */
typedef struct {
  int n;
  const int *p, *m;
  const double *value;
} xg_twoterm_desc;

/* Independent voltage / current sources. wave holds 7 doubles per source:
 *   DC:    {v, 0, 0, 0, 0, 0, 0}
 *   PULSE: {v1, v2, td, tr, tf, pw, per}   (N_DEV_SourceData.C:775-1031)   */
typedef struct {
  int n;
  const int *p, *m;
  const int *kind;            /* enum xg_src_kind */
  const double *wave;         /* 7 * n */
} xg_src_desc;

typedef struct {
  int n_nodes;                /* circuit nodes, ground excluded */
  int n_models;
  const xg_model_desc *models;
  /* Load order of device types; NULL = enum order. n_type_order entries. */
  int n_type_order;
  const int *type_order;
  xg_twoterm_desc res, cap;
  xg_src_desc vsrc, isrc;
  xg_diode_desc diode;
  xg_mos_desc mos1, bsim3;
} xg_netlist;

/* Device options (DeviceOptions, N_DEV_DeviceOptions.C:66-160). */
typedef struct {
  double gmin;                /* default 1e-12 */
  double temp;                /* circuit temperature [K], default 300.15 */
  double tnom;                /* nominal temperature [K], default 300.15 */
  int    voltlim;             /* voltageLimiterFlag, default 1 */
  int    newmeyer;            /* must be 0 (Meyer back-averaging path) */
  int    fma;                 /* 0: every product/sum rounded separately, bit-
                                 identical to a serial CPU load; 1: kernels built
                                 with fused multiply-add (faster, ~1 ulp/term) */
} xg_device_options;

/* Per-load solver flags (SolverState, N_DEV_SolverState.h:85-160). */
typedef struct {
  int dcop, tranop, acop, transient;
  int init_jct, init_fix;
  int newton_iter;
  int inputop;
  double pdt;                 /* alpha / h of the integrator */
  double time;                /* current time [s], for PULSE sources */
  int init_tran;              /* first transient step (SolverState::initTranFlag) */
} xg_load_flags;

/* ---- vector ids ------------------------------------------------------------ */
enum xg_vec_id {
  XG_VEC_SOL_NEXT = 0, XG_VEC_SOL_CURR, XG_VEC_SOL_LAST,   /* n_unknowns + 1 */
  XG_VEC_STA_NEXT, XG_VEC_STA_CURR, XG_VEC_STA_LAST,       /* n_state        */
  XG_VEC_STO_NEXT, XG_VEC_STO_CURR, XG_VEC_STO_LAST,       /* n_store        */
  XG_VEC_F, XG_VEC_Q, XG_VEC_DFDXDVP, XG_VEC_DQDXDVP,      /* n_unknowns + 1 */
  XG_VEC_DFDX, XG_VEC_DQDX,                                /* nnz values     */
  XG_NUM_VECS
};

typedef struct xg_ctx xg_ctx;
typedef struct xg_circuit xg_circuit;

typedef struct {
  int n_unknowns;             /* solved unknowns (ground excluded) */
  int n_state, n_store;
  int64_t nnz;                /* non-zeros of the solved Jacobian pattern */
  int64_t n_terms;            /* stamp terms produced per load */
  int64_t scratch_bytes;      /* device scratch held for per-load terms */
  int n_instances[XG_NUM_DEV_TYPES];
} xg_circuit_info;

/* ---- library ----------------------------------------------------------------- */
int  xg_abi_version(void);
const char *xg_last_error(void);
const char *xg_status_string(int status);
/* Kernels this library has launched since it was loaded (all contexts). */
long long xg_launch_count(void);

/* Sustained FP64 fused-multiply-add throughput of a GPU [flop/s] (2 flops per
 * DFMA), measured with a short DFMA-chain kernel: the roofline denominator of
 * the device-evaluation kernels, which are bound by the FP64 pipe.  A
 * measurement utility with no counterpart in the reference. */
int xg_probe_fp64_rate(int cuda_device, double *flops_per_second);
/* The FMA load build's FP64 reciprocal (Newton-Raphson from the hardware's
 * approximation) of n values on the current device, for testing it against
 * 1.0 / b.  No counterpart in the reference. */
int xg_probe_reciprocal(int n, const double *host_b, double *host_out);

/* ---- context: one GPU, one stream (replaces the DeviceMgr singleton) -------- */
int xg_ctx_create(int cuda_device, xg_ctx **out);
int xg_ctx_destroy(xg_ctx *ctx);
int xg_ctx_set_options(xg_ctx *ctx, const xg_device_options *opt);
int xg_ctx_get_options(const xg_ctx *ctx, xg_device_options *opt);
int xg_ctx_synchronize(xg_ctx *ctx);
/* The CUDA stream all work of this context is queued on (cudaStream_t). */
int xg_ctx_stream(xg_ctx *ctx, void **stream_out);

/* ---- circuit setup (DeviceMgr::addDeviceModel/addDeviceInstance, Topology
 *      registerLIDs/registerJacLIDs, Instance::updateTemperature) ----------- */
int xg_circuit_create(xg_ctx *ctx, const xg_netlist *nl, xg_circuit **out);
int xg_circuit_destroy(xg_circuit *c);
int xg_circuit_get_info(const xg_circuit *c, xg_circuit_info *info);
/* CSR pattern of the solved Jacobian (ground row/col excluded): rowptr has
 * n_unknowns+1 entries, colidx nnz entries, columns ascending in each row. */
int xg_circuit_get_pattern(const xg_circuit *c, int *host_rowptr, int *host_colidx);
/* Per-instance parameter block of one device type as derived by setup
 * (layout: include/xg_params.h, column k of instance i at [k*n + i]).
 * host_out may be NULL to query n_params / n_instances only. */
int xg_circuit_get_params(const xg_circuit *c, int dev_type, double *host_out,
                          int *n_params, int *n_instances);
/* The same parameter block computed on the host alone (no GPU needed): for
 * callers that inspect setup, and for CPU-side checks of it. */
int xg_setup_params(const xg_netlist *nl, const xg_device_options *opt, int dev_type,
                    double *host_out, int *n_params, int *n_instances);

/* ---- vectors ------------------------------------------------------------------ */
int xg_vec_size(const xg_circuit *c, int vec_id, int64_t *n);
int xg_vec_upload(xg_circuit *c, int vec_id, const double *host_src);
int xg_vec_download(xg_circuit *c, int vec_id, double *host_dst);
int xg_vec_device_ptr(xg_circuit *c, int vec_id, double **dev_ptr);
/* next <- curr <- last rotation of sol/sta/sto after an accepted step. */
int xg_rotate_history(xg_circuit *c);

/* ---- the Newton load ---------------------------------------------------------
 * xg_update_state       : Device::updateState for every type/instance: limited
 *                         junction voltages, currents, charges, caps; writes
 *                         next sta/sto and the per-instance stamp terms.
 * xg_load_dae_vectors   : Device::loadDAEVectors: F, Q, dFdxdVp, dQdxdVp.
 * xg_load_dae_matrices  : Device::loadDAEMatrices: dFdx, dQdx values.
 * xg_load               : all three, fused (the path a Newton iteration uses).
 * Outputs are zeroed inside the call (the reference's caller zeroes them,
 * N_TIA_Assembler.C:156-161). All calls are asynchronous on the context stream.
 */
int xg_update_state(xg_circuit *c, const xg_load_flags *flags);
int xg_load_dae_vectors(xg_circuit *c);
int xg_load_dae_matrices(xg_circuit *c);
int xg_load(xg_circuit *c, const xg_load_flags *flags);

/* ---- sparse LU of the Newton solve -------------------------------------------
 * Replaces the KLU solver behind N_LAS_AmesosSolver::solve
 * (N_LAS_AmesosSolver.C:231-492): symbolic analysis once per pattern (:388),
 * numeric factorisation per Newton iteration (:405), solve (:444).
 * xg_lu_analyze   : host: a column order (approximate minimum degree, or
 *                   nested dissection when minimum degree leaves a long
 *                   dependency chain and dissection models faster), then a
 *                   left-looking threshold-partial-pivot factorisation of the
 *                   given values (KLU's tol 0.001, diagonal preferred) that
 *                   fixes the pivot order and the L\U pattern; uploads them.
 * xg_lu_refactor  : GPU numeric refactorisation of new values (device CSR
 *                   values in the analysed pattern) with that pivot order.
 *                   Asynchronous; a zero or non-finite pivot is reported by
 *                   xg_lu_status (the reference repivots; here the caller
 *                   analyses again).
 * xg_lu_solve     : GPU forward/backward solves, x = A^-1 b (device buffers,
 *                   length n, distinct).  With XG_LU_FP32 the factors and
 *                   solves are FP32 and n_refine steps of FP64 iterative
 *                   refinement follow (r = b - A x with the FP64 matrix).
 * xg_lu_status    : synchronises; status bits 1 = zero/non-finite pivot (bad_row
 *                   = first such row of B), 2 = a wait gave up, 4 = pattern error.
 */
enum xg_lu_precision { XG_LU_FP64 = 0, XG_LU_FP32 = 1 };
typedef struct xg_lu xg_lu;
typedef struct {
  int n;
  int64_t nnz_a, nnz_lu;      /* matrix and L\U non-zeros */
  int precision;
  int levels;                 /* longest row dependency chain of the refactor */
  int n_dense;                /* dense rows ordered last */
  double refactor_flops;      /* multiply-adds + divides of one refactor */
  double solve_flops;         /* multiply-adds of one forward + backward solve */
  double min_pivot, max_pivot;/* |U(k,k)| range of the analysed matrix */
  int ordering;               /* column order: 0 minimum degree, 1 nested dissection */
  int solve_chain;            /* trailing rows the grid-wide solves hand to one CTA,
                                 solved 32 columns at a time (0: none, or the
                                 factor runs on another path) */
} xg_lu_info;
int xg_lu_analyze(xg_ctx *ctx, int n, const int *host_rowptr, const int *host_colidx,
                  const double *host_values, int precision, xg_lu **out);
int xg_lu_refactor(xg_lu *lu, const double *dev_values);
int xg_lu_solve(xg_lu *lu, const double *dev_b, double *dev_x, int n_refine);
/* xg_lu_refactor followed by xg_lu_solve, one Newton step's linear algebra
 * (NumericFactorization then Solve, N_LAS_AmesosSolver.C:405-444); small
 * factors do both in one launch from one staging of the factor. */
int xg_lu_refactor_solve(xg_lu *lu, const double *dev_values, const double *dev_b, double *dev_x,
                         int n_refine);
int xg_lu_status(xg_lu *lu, int *status, int *bad_row);
/* xg_lu_solve_host — the same refactor (skipped with reuse_factors) and
 * solve for a caller whose matrix and vectors live in host memory, as the
 * reference's solvers receive them from Epetra (N_LAS_AmesosSolver::solve,
 * N_LAS_AmesosSolver.C:231-444, values in the analysed CSR pattern).  The
 * values and b go up, x comes back; synchronous.  *status gets the bits of
 * xg_lu_status (1: zero or non-finite pivot; the caller repivots by
 * analysing again).  Device staging for the three arrays is allocated on the
 * first call. */
int xg_lu_solve_host(xg_lu *lu, const double *host_values, const double *host_b, double *host_x,
                     int n_refine, int reuse_factors, int *status);
/* Polls a device wait of this factorisation's refactor and solves makes
 * before it gives up, sets status bit 2 and returns (default 1,048,576, about
 * 0.1-0.5 s).  Every launch ends even when a wait gives up; its results are
 * then not valid.  Lowering it makes the waits run out, which is how the
 * timeout path is tested.  No counterpart in the reference, whose host KLU
 * has no device waits.  Synchronises the stream first. */
int xg_lu_set_wait_limit(xg_lu *lu, int polls);
int xg_lu_get_info(const xg_lu *lu, xg_lu_info *info);
/* host copies of the analysis: P, Q (n each), L\U row pointers (n+1), columns (nnz_lu) */
int xg_lu_get_symbolic(const xg_lu *lu, int *P, int *Q, int *lu_rowptr, int *lu_colidx);
int xg_lu_destroy(xg_lu *lu);
/* host-only analysis pieces (no GPU): the AMD order alone, and the full
 * analysis returning P, Q, the L\U non-zero count and (info may be NULL) the
 * statistics xg_lu_get_info reports */
int xg_lu_order(int n, const int *host_rowptr, const int *host_colidx, int *order, int *n_dense);
int xg_lu_analyze_host(int n, const int *host_rowptr, const int *host_colidx,
                       const double *host_values, int *P, int *Q, int64_t *nnz_lu,
                       xg_lu_info *info);

/* ---- transient analysis on the GPU -----------------------------------------
 * DC operating point, then .TRAN TSTEP TSTOP with the trapezoid ("OneStep")
 * integrator, every Newton iteration on the device: xg_load, the trapezoid
 * combine of residual and Jacobian (N_TIA_OneStep.C:215-352), the sparse LU
 * above, the damped-Newton convergence test (N_NLS_DampedNewton.C:1787-1919),
 * the local error test and step/order control (N_TIA_OneStep.C:1355-2190,
 * N_TIA_StepErrorControl.C:520-800) and breakpoints at PULSE corners.
 * host_x0: the DC solve's starting guess (.NODESET; NULL = zeros), or with
 * uic the initial condition itself (no DC solve).  Records t and x[out_idx]
 * at t = 0 and every accepted step, up to max_points. */
typedef struct {
  double tstop, tstep;        /* TSTEP is also the first step's upper bound */
  double maxstep;             /* <= 0: 0.1 * tstop */
  double reltol, abstol;      /* local error test; <= 0: 1e-3, 1e-6 */
  int lu_precision;           /* XG_LU_FP64 or XG_LU_FP32 (+ refinement) */
  int n_refine;               /* refinement steps per solve (FP32 factors) */
  int uic;
} xg_tran_options;
typedef struct {
  int status;                 /* last failing Newton / step status, 0 if none */
  int steps, steps_attempted, rejected;
  int newton_iters, factorizations, loads;
  int dcop_iters, dcop_solves, analyses;
  double t_end;
} xg_tran_stats;
int xg_tran_run(xg_circuit *c, const xg_tran_options *o, const double *host_x0, int n_out,
                const int *out_idx, int max_points, double *host_t, double *host_v,
                int *n_points, xg_tran_stats *st);

/* ---- batched transients (serving) ---------------------------------------------
 * Many independent requests (.STEP / Monte-Carlo variants, uneven sizes)
 * stepped together on one GPU: the block-diagonal union of their netlists is
 * loaded in one pass, and one warp per request refactors and solves its own
 * sparse system (pivot order analysed per request at creation; FP32 factors
 * with FP64 refinement or FP64), while a device-side state machine per request
 * runs the damped-Newton test, local error test and step control of
 * xg_tran_run.  One batch iteration (one Newton iteration of every request) is
 * a fixed sequence of launches, captured into a CUDA graph on the batch's own
 * stream; batches created while others run overlap on the device.
 * Requests start from their initial condition (UIC).  Each request steps to
 * the breakpoints of its own PULSE sources and restarts at first order there,
 * as xg_tran_run does.  x0[r] and out_idx[r] use request r's own unknown
 * numbering (nodes, then its internal unknowns). */
typedef struct xg_batch xg_batch;
typedef struct {
  double tstep;               /* first-step bound (.TRAN TSTEP) */
  double maxstep;             /* <= 0: 0.1 * tstop of each request */
  double reltol, abstol;      /* local error test; <= 0: 1e-3, 1e-6 */
  int lu_precision;           /* XG_LU_FP64 or XG_LU_FP32 */
  int n_refine;               /* FP64 refinement steps with FP32 factors */
  int n_out;                  /* recorded unknowns per request */
  int max_points;             /* recorded points per request */
} xg_batch_options;
int xg_batch_create(xg_ctx *ctx, int n_requests, const xg_netlist *const *netlists,
                    const double *const *x0, const double *tstop, const int *const *out_idx,
                    const xg_batch_options *o, xg_batch **out);
/* enqueue `iterations` batch iterations (asynchronous, on the batch's stream) */
int xg_batch_run(xg_batch *b, int iterations);
/* The request states as the newest finished xg_batch_run left them (each
 * run ends with a snapshot), and the number of finished requests in them.
 * wait = 0: *n_done = -1 when no run has finished since the last poll (later
 * runs may still be on the device); wait = 1 synchronises first. */
int xg_batch_poll(xg_batch *b, int wait, int *n_done);
/* Runs enqueued and not finished yet. */
int xg_batch_inflight(xg_batch *b, int *n);
/* request i's recorded (t, x[out_idx]) and counters (after a poll) */
int xg_batch_results(xg_batch *b, int i, double *host_t, double *host_v, int *n_points,
                     xg_tran_stats *st);
int xg_batch_info(const xg_batch *b, int *n_requests, int64_t *device_bytes);
int xg_batch_destroy(xg_batch *b);

/* ---- slotted batches (continuous batching at request granularity) ------------
 * A slotted batch is created empty with a fixed number of slots of one shape
 * (a size class: the largest request a slot holds).  Requests are submitted
 * into free slots while the batch runs; a finished request's results are read
 * and its slot released for the next one, so a short request never waits for
 * a long one, and a request arriving mid-run starts at the next batch
 * iteration instead of waiting for a new batch.  Each request's arithmetic is
 * the same as in a batch of its own (its load, reduction order, pivot order,
 * Newton test and step control depend on it alone), so its results do not
 * depend on which other requests share the batch.
 *   - Device memory for every slot is allocated at creation
 *     (xg_slot_bytes per slot): submitting allocates nothing on the device.
 *   - xg_batch_submit sets the requests up on the host (device parameters,
 *     pattern, reduction lists), evaluates their first Jacobian on the device
 *     with a load restricted to their slots (on a stream of its own, beside
 *     the running iterations), analyses each one's pivot order, and activates
 *     them at the next batch iteration.  It returns when that activation is
 *     enqueued; it may run on another thread than xg_batch_run/poll.
 *   - xg_batch_run, xg_batch_poll and xg_batch_results work as for any batch,
 *     with slot numbers for request numbers; a free slot counts as done. */
typedef struct {
  int max_unknowns;                       /* nodes + internal unknowns */
  int max_instances[XG_NUM_DEV_TYPES];    /* per device type */
  int64_t max_nnz;                        /* Jacobian entries */
  int64_t max_lu_nnz;                     /* L\U entries after the pivot analysis */
  int64_t max_schedule;                   /* level-schedule ints (0: no level path) */
  int max_breakpoints;                    /* PULSE corners up to tstop, and tstop */
} xg_slot_shape;
/* The shape of one request: its set-up, first Jacobian (at x0, step tstep)
 * and pivot analysis, exactly as xg_batch_submit does them. */
int xg_slot_need(xg_ctx *ctx, const xg_netlist *nl, const double *x0, double tstop, double tstep,
                 xg_slot_shape *need);
/* Device bytes of one slot of this shape under these options (host
 * arithmetic only: no device needed). */
int xg_slot_bytes(const xg_slot_shape *shape, const xg_batch_options *o, int64_t *bytes);
int xg_batch_create_slots(xg_ctx *ctx, int n_slots, const xg_slot_shape *shape,
                          const xg_batch_options *o, xg_batch **out);
/* Submit n requests.  slots[i] receives request i's slot, or -1 when no slot
 * was free (the request was not taken).  A request larger than the shape, or
 * whose set-up fails, is refused with an error and nothing of the call is
 * admitted. */
int xg_batch_submit(xg_batch *b, int n, const xg_netlist *const *netlists, const double *const *x0,
                    const double *tstop, const int *const *out_idx, int *slots);
/* Free a finished slot for the next request (its results are gone then). */
int xg_batch_release(xg_batch *b, int slot);
/* The slots whose request has finished (as of the last poll) and that are
 * not yet released: up to max_slots of them in slots[], their count in *n. */
int xg_batch_finished(const xg_batch *b, int max_slots, int *slots, int *n);
/* Free slots, and slots whose request is still running. */
int xg_batch_slots(const xg_batch *b, int *n_free, int *n_running);
/* Free and total device memory of the context's device (cudaMemGetInfo). */
int xg_mem_info(xg_ctx *ctx, int64_t *free_bytes, int64_t *total_bytes);

/* xg_load_noalloc — the same load as xg_load, for callers that cannot
 * allocate device memory at the point where they load: host simulators that
 * give the GPU a fixed memory budget up front and own every later byte
 * themselves, and real-time loops that must never block in the allocator.
 * It calls no cudaMalloc, cudaFree or allocating library routine.  No
 * counterpart exists in the reference.
 *   - The per-load stamp terms live in one fixed device array inside the
 *     library, at most 2,097,152 terms (16 MiB); every GPU that loads the
 *     library keeps it reserved until exit.  Circuits needing more terms
 *     (xg_circuit_info.n_terms) are rejected with XG_ERR_ARG.
 *   - Outputs go to dev_out (device memory, dev_out_len >= the circuit's
 *     output count 4*(n_unknowns+1) + 2*nnz), laid out
 *     [F | Q | dFdxdVp | dQdxdVp] (n_unknowns+1 each, ground last) then dF/dx
 *     and dQ/dx values on the pattern of xg_circuit_get_pattern.  Next state
 *     and store are written in the circuit as xg_load writes them.
 *   - The first call on a device looks the array's device address up
 *     (cudaGetSymbolAddress) with that device current and keeps it for the
 *     life of the process.  A cudaDeviceReset invalidates the kept address:
 *     reload the library after one.
 *   - All calls share the array: calls whose work overlaps on the GPU race
 *     and must be serialised by the caller. */
int xg_load_noalloc(xg_circuit *c, const xg_load_flags *flags, double *dev_out,
                    int64_t dev_out_len);

#ifdef __cplusplus
}
#endif

#endif /* XG_H */
