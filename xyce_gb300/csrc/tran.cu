// tran.cu — the transient time stepper on the GPU: the rows downstream of the
// Newton load.
//
//  * trapezoid combine (N_TIA_OneStep.C:215-352): residual
//      RHS = -[(Q - qn0)/h + 1/2 F + 1/2 F_prev] + dQdxdVp/h + 1/2 dFdxdVp
//    (order 1: -[(Q - qn0)/h + F] + dQdxdVp/h + dFdxdVp) and Jacobian
//      J = dQdx/h + 1/2 dFdx   (order 1: dQdx/h + dFdx);
//    DC (N_TIA_NoTimeIntegration.C:140-198): RHS = -F + dFdxdVp,
//    J = dFdx + 1e-20 dQdx;  one kernel over the rows and the non-zeros;
//  * Newton (N_NLS_DampedNewton.C:374-629): load, combine, GPU LU refactor and
//    solve (lu_kernels.cu), update, norms; the convergence test
//    (:1787-1919) runs on the host from a handful of reduced scalars;
//  * step control (N_TIA_OneStep.C:1355-2190, N_TIA_StepErrorControl.C:520-800):
//    predictor, local error estimate ck * WRMS(x - xpredicted), accept or
//    reject, order 1 -> 2, breakpoints at PULSE corners.
// Every vector stays on the device; per Newton iteration the host reads back
// a few partial sums (reduced in a fixed order, so runs repeat bit for bit).
// The DC operating point starts from a caller guess (.NODESET) and falls back
// to gmin stepping (shunts on node rows, 1e-2 down to 1e-12).

#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "xg.h"
#include "xg_internal.h"
#include "xg_lu.h"

namespace xg {
namespace {

constexpr int kRedBlocks = 128;  // fixed partition of every reduction
constexpr int kThreads = 256;

enum Partial : int { P_RHS2 = 0, P_RHSMAX, P_LIMMAX, P_DXW2, P_ERR2, P_XMAX, P_N };

__device__ __forceinline__ void block_reduce(double *sh, double v, bool is_max, double *out) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      sh[threadIdx.x] = is_max ? fmax(sh[threadIdx.x], sh[threadIdx.x + s]) : sh[threadIdx.x] + sh[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
  __syncthreads();
}

struct CombineArgs {
  int n, n_nodes;
  int64_t nnz;
  int transient, order;
  double inv_h, fs, qs, gshunt;
  const double *f, *q, *fvp, *qvp, *qn0, *qh2, *x;
  const double *dfdx, *dqdx;
  const int64_t *diag;  // (i, i) position per row, -1 if absent
  double *rhs, *jac;
  double *partials;     // [P_N][kRedBlocks]
};

// The trapezoid / DC combine, plus partial norms of the residual.
__global__ void __launch_bounds__(kThreads) tran_combine(CombineArgs a) {
  __shared__ double sh[kThreads];
  const int stride = gridDim.x * blockDim.x;
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  double s2 = 0.0, mx = 0.0, lim = 0.0;
  for (int i = t0; i < a.n; i += stride) {
    double r;
    if (a.transient) {
      r = (a.q[i] - a.qn0[i]) * a.inv_h;
      r = a.order == 2 ? r + 0.5 * a.f[i] + 0.5 * a.qh2[i] : r + a.f[i];
      r = -r;
      r += a.qvp[i] * a.inv_h;
      r += a.fs * a.fvp[i];
    } else {
      r = -a.f[i] + a.fvp[i];
      if (a.gshunt > 0.0 && i < a.n_nodes && a.diag[i] >= 0) r -= a.gshunt * a.x[i];
    }
    a.rhs[i] = r;
    s2 += r * r;
    mx = fmax(mx, fabs(r));
    lim = fmax(lim, fmax(fabs(a.fvp[i]), fabs(a.qvp[i])));
  }
  for (int64_t p = t0; p < a.nnz; p += stride) a.jac[p] = a.qs * a.dqdx[p] + a.fs * a.dfdx[p];
  block_reduce(sh, s2, false, a.partials + P_RHS2 * kRedBlocks + blockIdx.x);
  block_reduce(sh, mx, true, a.partials + P_RHSMAX * kRedBlocks + blockIdx.x);
  block_reduce(sh, lim, true, a.partials + P_LIMMAX * kRedBlocks + blockIdx.x);
}

// gmin shunts on the node rows' diagonals (after the combine wrote J).
__global__ void tran_shunt(int n_nodes, const int64_t *diag, double g, double *jac) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += gridDim.x * blockDim.x)
    if (diag[i] >= 0) jac[diag[i]] += g;
}

// Newton weights rel * max(|x_curr|, |x|) + abs.
__global__ void tran_weights(int n, const double *xc, const double *x, double rel, double abs_tol,
                             double *w) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    w[i] = rel * fmax(fabs(xc[i]), fabs(x[i])) + abs_tol;
}

// x += dx; optionally refresh the weights from the updated x (DC); partial
// sums of (dx / w)^2.  Also copies the LU status word behind the partials, so
// one read brings both back.
__global__ void __launch_bounds__(kThreads) tran_update(int n, const double *dx, double *x,
                                                        const double *xc, int reweight, double rel,
                                                        double abs_tol, double *w, double *partials,
                                                        const unsigned *lu_status) {
  __shared__ double sh[kThreads];
  if (blockIdx.x == 0 && threadIdx.x == 0)
    *reinterpret_cast<unsigned *>(partials + P_N * kRedBlocks) = *lu_status;
  double s2 = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double xi = x[i] + dx[i];
    x[i] = xi;
    double wi = reweight ? rel * fmax(fabs(xc[i]), fabs(xi)) + abs_tol : w[i];
    if (reweight) w[i] = wi;
    double t = dx[i] / wi;
    s2 += t * t;
  }
  block_reduce(sh, s2, false, partials + P_DXW2 * kRedBlocks + blockIdx.x);
}

// Predictor x = xh0 + b1 xh1 (+ b2 xh2), also kept as xn0; qn0 = qh0.
__global__ void tran_predict(int n, int order, double b1, double b2, const double *xh0,
                             const double *xh1, const double *xh2, double *xn0, double *x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double v = xh0[i];
    v = b1 * xh1[i] + v;
    if (order == 2) v = b2 * xh2[i] + v;
    xn0[i] = v;
    x[i] = v;
  }
}

// Partial sums of (x - xn0)^2 and the max of |x_curr|.
__global__ void __launch_bounds__(kThreads) tran_lte(int n, const double *x, const double *xn0,
                                                     const double *xc, double *partials) {
  __shared__ double sh[kThreads];
  double s2 = 0.0, mx = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double e = x[i] - xn0[i];
    s2 += e * e;
    mx = fmax(mx, fabs(xc[i]));
  }
  block_reduce(sh, s2, false, partials + P_ERR2 * kRedBlocks + blockIdx.x);
  block_reduce(sh, mx, true, partials + P_XMAX * kRedBlocks + blockIdx.x);
}

// OneStep::initialize history: xh0 = x, xh1 = 0, qh0 = Q, qh1 = -h F.
__global__ void tran_init_hist(int n, double h, const double *x, const double *q, const double *f,
                               double *xh0, double *xh1, double *qh0, double *qh1) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    xh0[i] = x[i];
    xh1[i] = 0.0;
    qh0[i] = q[i];
    qh1[i] = -h * f[i];
  }
}

// OneStep::updateHistory with the next step's order.
__global__ void tran_history(int n, int order, const double *x, const double *q, const double *f,
                             double *xh0, double *xh1, double *xh2, double *qh0, double *qh1,
                             double *qh2) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (order == 2) {
      xh2[i] = xh1[i];
      qh2[i] = f[i];
    }
    xh1[i] = x[i] - xh0[i];
    qh1[i] = q[i] - qh0[i];
    xh0[i] = x[i];
    qh0[i] = q[i];
  }
}

__global__ void tran_record(int n_out, const int *idx, const double *x, double *row) {
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_out; k += gridDim.x * blockDim.x)
    row[k] = x[idx[k]];
}

// ---------------------------------------------------------------------------

struct Run {
  xg_circuit *c = nullptr;
  CircuitView v{};
  cudaStream_t s = nullptr;
  int n = 0, nr = 0, n_nodes = 0;
  int64_t nnz = 0;
  xg_tran_stats *st = nullptr;
  const xg_tran_options *o = nullptr;
  xg_lu *lu = nullptr;
  // device work
  double *rhs = nullptr, *jac = nullptr, *dx = nullptr, *w = nullptr, *partials = nullptr;
  double *xh0 = nullptr, *xh1 = nullptr, *xh2 = nullptr, *qh0 = nullptr, *qh1 = nullptr,
         *qh2 = nullptr, *xn0 = nullptr;
  int64_t *diag = nullptr;
  double *h_part = nullptr;  // pinned host copy of the partials
  double gshunt = 0.0;
  int stall_count = 0;
  double stall_rate = 0.0;
  bool first_solve = true;
  int grid = 1;
  std::string err;

  double *vec(int id) {
    double *p = nullptr;
    xg_vec_device_ptr(c, id, &p);
    return p;
  }
  int fail_cuda(cudaError_t e, const char *what) {
    err = std::string(what) + ": " + cudaGetErrorString(e);
    return XG_ERR_CUDA;
  }
  // read back the partials of the given kinds (and the LU status word when
  // asked) with one synchronisation, and reduce them in block order
  // (the status word is the one tran_update copied behind the partials)
  int reduce(std::initializer_list<int> kinds, double *out, unsigned *lu_status = nullptr) {
    int k0 = P_N, k1 = 0;
    for (int k : kinds) {
      k0 = std::min(k0, k);
      k1 = std::max(k1, k + 1);
    }
    if (lu_status) k1 = P_N;
    const size_t count = size_t(k1 - k0) * kRedBlocks + (lu_status ? 1 : 0);
    cudaError_t e = cudaMemcpyAsync(h_part + k0 * kRedBlocks, partials + k0 * kRedBlocks,
                                    sizeof(double) * count, cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return fail_cuda(e, "partials");
    unsigned *h_status = reinterpret_cast<unsigned *>(h_part + P_N * kRedBlocks);
    e = cudaStreamSynchronize(s);
    if (lu_status) *lu_status = *h_status;
    if (e != cudaSuccess) return fail_cuda(e, "stream");
    for (int k : kinds) {
      const bool is_max = k == P_RHSMAX || k == P_LIMMAX || k == P_XMAX;
      double acc = 0.0;
      for (int b = 0; b < kRedBlocks; ++b) {
        double p = h_part[k * kRedBlocks + b];
        acc = is_max ? (p != p ? p : std::max(acc, p)) : acc + p;
      }
      out[k] = acc;
    }
    return XG_OK;
  }

  int load(const xg_load_flags &fl) {
    st->loads++;
    return xg_load(c, &fl);
  }

  int combine(bool transient, int order, double h, double out[P_N], bool fetch = true) {
    CombineArgs a;
    a.n = n;
    a.n_nodes = n_nodes;
    a.nnz = nnz;
    a.transient = transient;
    a.order = order;
    a.inv_h = transient ? 1.0 / h : 0.0;
    a.fs = (transient && order == 2) ? 0.5 : 1.0;
    a.qs = transient ? 1.0 / h : 1.0e-20;
    a.gshunt = transient ? 0.0 : gshunt;
    a.f = vec(XG_VEC_F);
    a.q = vec(XG_VEC_Q);
    a.fvp = vec(XG_VEC_DFDXDVP);
    a.qvp = vec(XG_VEC_DQDXDVP);
    a.qn0 = qh0;
    a.qh2 = qh2;
    a.x = vec(XG_VEC_SOL_NEXT);
    a.dfdx = vec(XG_VEC_DFDX);
    a.dqdx = vec(XG_VEC_DQDX);
    a.diag = diag;
    a.rhs = rhs;
    a.jac = jac;
    a.partials = partials;
    tran_combine<<<kRedBlocks, kThreads, 0, s>>>(a); xg::count_launches(1);
    if (!transient && gshunt > 0.0) {
      tran_shunt<<<grid, kThreads, 0, s>>>(n_nodes, diag, gshunt, jac);
      xg::count_launches(1);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail_cuda(e, "tran_combine");
    return fetch ? reduce({P_RHS2, P_RHSMAX, P_LIMMAX}, out) : XG_OK;
  }

  // N_NLS_DampedNewton::converged_
  int converged(bool transient, int step, int max_step, double rhs_tol, double dx_tol,
                double max_rhs, double upd, double rhs_rel, double rate) {
    const double eps = DBL_EPSILON, rate_max = 0.5 * DBL_MAX, min_red = 0.9, stag = 1e-3;
    const double small_update = 1e-6;
    if (max_rhs <= eps && max_rhs <= rhs_tol) return 1;
    if (max_rhs <= rhs_tol && upd <= dx_tol) return 2;
    if (step > max_step && transient)
      if (rhs_rel <= min_red && rate <= 1.0) return 3;
    if (upd <= small_update) return 4;
    if (step > max_step) return -1;
    else if (rate > rate_max) return -2;
    if (transient && std::fabs(rate - 1.0) <= stag) {
      if (stall_count == 0 || rate < stall_rate) stall_rate = rate;
      stall_count++;
    } else {
      stall_count = 0;
    }
    if (transient && stall_count == 5) {
      stall_count = 0;
      return (rhs_rel < min_red && stall_rate <= 1.0) ? 3 : -3;
    }
    return 0;
  }

  // One Newton solve; returns the convergence status (>0 converged), or a
  // library error code through *rc.
  int newton(bool transient, double h, int order, double time, int init_tran, int *rc) {
    *rc = XG_OK;
    const int max_step = transient ? 20 : 200;
    const double rhs_tol = transient ? 1e-2 : 1e-6;
    double dx_tol = transient ? 0.33 : 1.0;
    const double abs_tol = transient ? 1e-6 : 1e-12, rel_tol = transient ? 1e-2 : 1e-3;
    if (first_solve) {
      dx_tol *= 0.01;
      first_solve = false;
    }
    xg_load_flags fl;
    std::memset(&fl, 0, sizeof(fl));
    fl.dcop = !transient;
    fl.tranop = !transient;
    fl.transient = transient;
    fl.time = time;
    fl.init_tran = init_tran;
    fl.pdt = transient ? 1.0 / h : 0.0;
    fl.newton_iter = 0;
    fl.init_jct = !transient && st->dcop_solves == 0;
    double r[P_N];
    if ((*rc = load(fl))) return 0;
    if ((*rc = combine(transient, order, h, r))) return 0;
    double norm_rhs = std::sqrt(r[P_RHS2]), max_rhs = r[P_RHSMAX];
    bool any_limit = r[P_LIMMAX] != 0.0;
    if (norm_rhs < DBL_EPSILON) return 1;
    const double norm_init = norm_rhs;
    double norm_old = norm_rhs;
    double *x = vec(XG_VEC_SOL_NEXT), *xc = vec(XG_VEC_SOL_CURR);
    if (transient) {
      tran_weights<<<grid, kThreads, 0, s>>>(n, xc, x, rel_tol, abs_tol, w);
      xg::count_launches(1);
    }
    int status = 0, step = 0;
    while (status == 0) {
      ++step;
      st->factorizations++;
      if ((*rc = xg_lu_refactor_solve(lu, jac, rhs, dx, o->n_refine))) return 0;
      tran_update<<<kRedBlocks, kThreads, 0, s>>>(n, dx, x, xc, !transient, rel_tol, abs_tol, w,
                                                  partials, lu_status_device(lu));
      xg::count_launches(1);
      fl.newton_iter = step;
      fl.init_jct = 0;
      fl.init_fix = !transient && st->dcop_solves == 0 && any_limit;
      if ((*rc = load(fl))) return 0;
      if ((*rc = combine(transient, order, h, r, false))) return 0;
      unsigned lu_status = 0;
      if ((*rc = reduce({P_RHS2, P_RHSMAX, P_LIMMAX, P_DXW2}, r, &lu_status))) return 0;
      any_limit = r[P_LIMMAX] != 0.0;
      if (lu_status) return -5;
      const double upd = std::sqrt(r[P_DXW2] / n);
      norm_rhs = std::sqrt(r[P_RHS2]);
      max_rhs = r[P_RHSMAX];
      const double rhs_rel = norm_rhs / norm_init, rate = norm_rhs / norm_old;
      norm_old = norm_rhs;
      st->newton_iters++;
      status = converged(transient, step, max_step, rhs_tol, dx_tol, max_rhs, upd, rhs_rel, rate);
      if (max_rhs != 0.0 && !(max_rhs < 0.0) && !(max_rhs > 0.0)) status = -6;
    }
    return status;
  }
};

}  // namespace

std::vector<double> pulse_breakpoints(const Plan &P, double tstop, const int *lo,
                                      const int *hi) {
  std::vector<double> bp;
  for (int which = 0; which < 2; ++which) {
    const TypeData &V = P.T[which == 0 ? XG_DEV_VSRC : XG_DEV_ISRC];
    const int i0 = lo ? lo[which] : 0, i1 = hi ? hi[which] : V.n;
    for (int i = i0; i < i1; ++i) {
      auto p = [&](int k) { return V.params[(size_t)k * V.n + i]; };
      if (p(XG_V_KIND) != XG_SRC_PULSE) continue;
      const double td = p(XG_V_TD), tr = p(XG_V_TR), tf = p(XG_V_TF), pw = p(XG_V_PW),
                   per = p(XG_V_PER);
      for (int k = 0;; ++k) {
        const double base = per > 0 ? per * k : 0.0;
        const double pts[4] = {base + td, base + td + tr, base + td + tr + pw, base + td + tr + pw + tf};
        for (double t : pts)
          if (t > 0.0 && t < tstop) bp.push_back(t);
        if (per <= 0 || base + td >= tstop) break;
      }
    }
  }
  bp.push_back(tstop);
  std::sort(bp.begin(), bp.end());
  bp.erase(std::unique(bp.begin(), bp.end()), bp.end());
  return bp;
}

}  // namespace xg

extern "C" int xg_tran_run(xg_circuit *c, const xg_tran_options *o, const double *host_x0,
                           int n_out, const int *out_idx, int max_points, double *host_t,
                           double *host_v, int *n_points, xg_tran_stats *st) {
  using namespace xg;
  if (!c || !o || !st || !n_points || (n_out > 0 && (!out_idx || !host_v)) || !host_t ||
      max_points <= 0 || o->tstop <= 0 || (o->lu_precision != XG_LU_FP64 &&
                                           o->lu_precision != XG_LU_FP32) || o->n_refine < 0) {
    set_error("xg_tran_run: bad argument");
    return XG_ERR_ARG;
  }
  std::memset(st, 0, sizeof(*st));
  *n_points = 0;
  Run R;
  R.c = c;
  R.st = st;
  R.o = o;
  if (circuit_view(c, &R.v)) {
    set_error("xg_tran_run: bad circuit");
    return XG_ERR_ARG;
  }
  const Plan &P = *R.v.plan;
  R.s = (cudaStream_t)R.v.stream;
  R.n = P.n_unknowns;
  R.nr = P.n_unknowns + 1;
  R.n_nodes = P.n_nodes;
  R.nnz = P.nnz;
  const int n = R.n, nr = R.nr;
  for (int k = 0; k < n_out; ++k)
    if (out_idx[k] < 0 || out_idx[k] >= n) {
      set_error("xg_tran_run: output index out of range");
      return XG_ERR_ARG;
    }
  if (cudaSetDevice(R.v.device) != cudaSuccess) return XG_ERR_CUDA;
  R.grid = std::max(1, std::min(4 * sm_count(), (n + kThreads - 1) / kThreads));
  int rc = XG_OK;
  double *d_rec = nullptr;
  int *d_idx = nullptr;
  bool reanalysed = false, reused = false;
  uint64_t lu_key = 0;
  auto cleanup = [&]() {
    void *ptrs[] = {R.rhs, R.jac, R.dx, R.w, R.partials, R.xh0, R.xh1, R.xh2, R.qh0, R.qh1,
                    R.qh2, R.xn0, R.diag, d_rec, d_idx};
    cudaStreamSynchronize(R.s);
    for (void *p : ptrs)
      if (p) cudaFree(p);
    if (R.h_part) cudaFreeHost(R.h_part);
    // the first analysis stays with the circuit for the next transient
    if (R.lu && !reanalysed && lu_key) circuit_lu_keep(c, R.lu, lu_key);
    else if (R.lu) xg_lu_destroy(R.lu);
  };
#define TRY_CUDA(call)                                          \
  do {                                                          \
    cudaError_t e_ = (call);                                    \
    if (e_ != cudaSuccess) {                                    \
      set_error(std::string(#call) + ": " + cudaGetErrorString(e_)); \
      cleanup();                                                \
      return e_ == cudaErrorMemoryAllocation ? XG_ERR_OOM : XG_ERR_CUDA; \
    }                                                           \
  } while (0)
  double **bufs[] = {&R.rhs, &R.dx, &R.w, &R.xh0, &R.xh1, &R.xh2, &R.qh0, &R.qh1, &R.qh2, &R.xn0};
  for (double **b : bufs) TRY_CUDA(cudaMalloc((void **)b, sizeof(double) * nr));
  TRY_CUDA(cudaMalloc((void **)&R.jac, sizeof(double) * std::max<int64_t>(R.nnz, 1)));
  TRY_CUDA(cudaMalloc((void **)&R.partials, sizeof(double) * (P_N * kRedBlocks + 1)));
  TRY_CUDA(cudaMallocHost((void **)&R.h_part, sizeof(double) * (P_N * kRedBlocks + 1)));
  TRY_CUDA(cudaMalloc((void **)&R.diag, sizeof(int64_t) * nr));
  TRY_CUDA(cudaMalloc((void **)&d_rec, sizeof(double) * std::max(1, n_out) * (size_t)max_points));
  TRY_CUDA(cudaMalloc((void **)&d_idx, sizeof(int) * std::max(1, n_out)));
  for (double **b : bufs) TRY_CUDA(cudaMemsetAsync(*b, 0, sizeof(double) * nr, R.s));
  {
    std::vector<int64_t> hd(nr, -1);
    for (int i = 0; i < n; ++i)
      for (int p = P.rowptr[i]; p < P.rowptr[i + 1]; ++p)
        if (P.colidx[p] == i) hd[i] = p;
    TRY_CUDA(cudaMemcpy(R.diag, hd.data(), sizeof(int64_t) * nr, cudaMemcpyHostToDevice));
  }
  if (n_out) TRY_CUDA(cudaMemcpy(d_idx, out_idx, sizeof(int) * n_out, cudaMemcpyHostToDevice));

  // initial state: x0 (or zero) in next/curr/last; state and store zero
  {
    std::vector<double> x0(nr, 0.0);
    if (host_x0) std::memcpy(x0.data(), host_x0, sizeof(double) * n);
    std::vector<double> z(std::max(P.n_state, P.n_store) + 1, 0.0);
    for (int id : {XG_VEC_SOL_NEXT, XG_VEC_SOL_CURR, XG_VEC_SOL_LAST})
      if ((rc = xg_vec_upload(c, id, x0.data()))) { cleanup(); return rc; }
    for (int id : {XG_VEC_STA_NEXT, XG_VEC_STA_CURR, XG_VEC_STA_LAST})
      if (P.n_state && (rc = xg_vec_upload(c, id, z.data()))) { cleanup(); return rc; }
    for (int id : {XG_VEC_STO_NEXT, XG_VEC_STO_CURR, XG_VEC_STO_LAST})
      if (P.n_store && (rc = xg_vec_upload(c, id, z.data()))) { cleanup(); return rc; }
  }
  // LU analysis on a matrix of the circuit's pattern: the Jacobian of a
  // first trapezoid step of length tstep at the starting point (static and
  // capacitive parts both present); zero diagonals get a 1e-12 placeholder
  double r[P_N];
  bool first_analysis = true;
  auto analyse = [&](bool transient_matrix, double h) -> int {
    xg_load_flags fl;
    std::memset(&fl, 0, sizeof(fl));
    fl.dcop = !transient_matrix;
    fl.tranop = !transient_matrix;
    fl.transient = transient_matrix;
    int e = R.load(fl);
    if (!e) e = R.combine(transient_matrix, 1, h, r);
    if (e) return e;
    std::vector<double> hj(std::max<int64_t>(R.nnz, 1));
    cudaError_t ce = cudaMemcpy(hj.data(), R.jac, sizeof(double) * R.nnz, cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return R.fail_cuda(ce, "jacobian");
    for (int i = 0; i < n; ++i)
      for (int p = P.rowptr[i]; p < P.rowptr[i + 1]; ++p)
        if (P.colidx[p] == i && hj[p] == 0.0) hj[p] = 1e-12;
    if (R.lu) xg_lu_destroy(R.lu);
    R.lu = nullptr;
    if (first_analysis) {
      // FNV-1a over the matrix values and the precision
      uint64_t hsh = 1469598103934665603ull;
      const unsigned char *bytes = reinterpret_cast<const unsigned char *>(hj.data());
      for (size_t k = 0; k < sizeof(double) * size_t(R.nnz); ++k) hsh = (hsh ^ bytes[k]) * 1099511628211ull;
      hsh = (hsh ^ uint64_t(o->lu_precision + 1)) * 1099511628211ull;
      lu_key = hsh ? hsh : 1;
      first_analysis = false;
      if ((R.lu = circuit_lu_take(c, lu_key))) {
        reused = true;
        return XG_OK;
      }
    } else {
      reanalysed = true;
    }
    return xg_lu_analyze(R.v.ctx, n, P.rowptr.data(), P.colidx.data(), hj.data(), o->lu_precision,
                         &R.lu);
  };
  const double tstep = o->tstep > 0 ? o->tstep : 1e-10;
  if ((rc = analyse(true, tstep))) { cleanup(); return rc; }
  st->analyses = reused ? 0 : 1;
  // Newton with one re-analysis (new pivot order) when the refactor meets a
  // zero pivot, as the reference's KLU repivots
  auto newton = [&](bool transient, double h, int order, double time, int init_tran) -> int {
    int e = XG_OK;
    int s = R.newton(transient, h, order, time, init_tran, &e);
    if (e) return -1000 + e;
    if (s == -5) {
      if ((e = analyse(transient, transient ? h : tstep))) return -1000 + e;
      st->analyses++;
      // restore the starting iterate and retry once
      cudaError_t ce = cudaSuccess;
      if (transient) {
        ce = cudaMemcpyAsync(R.vec(XG_VEC_SOL_NEXT), R.xn0, sizeof(double) * n,
                             cudaMemcpyDeviceToDevice, R.s);
        int64_t ls = 0, lo = 0;
        xg_vec_size(c, XG_VEC_STA_NEXT, &ls);
        xg_vec_size(c, XG_VEC_STO_NEXT, &lo);
        if (ce == cudaSuccess && ls)
          ce = cudaMemcpyAsync(R.vec(XG_VEC_STA_NEXT), R.vec(XG_VEC_STA_CURR), sizeof(double) * ls,
                               cudaMemcpyDeviceToDevice, R.s);
        if (ce == cudaSuccess && lo)
          ce = cudaMemcpyAsync(R.vec(XG_VEC_STO_NEXT), R.vec(XG_VEC_STO_CURR), sizeof(double) * lo,
                               cudaMemcpyDeviceToDevice, R.s);
      } else {
        ce = cudaMemcpyAsync(R.vec(XG_VEC_SOL_NEXT), R.vec(XG_VEC_SOL_CURR), sizeof(double) * n,
                             cudaMemcpyDeviceToDevice, R.s);
      }
      if (ce != cudaSuccess) return -1000 + R.fail_cuda(ce, "restart");
      s = R.newton(transient, h, order, time, init_tran, &e);
      if (e) return -1000 + e;
    }
    return s;
  };
  int np = 0;
  auto record = [&](double t) {
    if (np >= max_points) return;
    host_t[np] = t;
    if (n_out)
      tran_record<<<1, 128, 0, R.s>>>(n_out, d_idx, R.vec(XG_VEC_SOL_CURR), d_rec + (size_t)np * n_out); xg::count_launches(1);
    ++np;
  };
  auto copy_vec = [&](int dst, int src, int64_t len) -> int {
    if (!len) return XG_OK;
    cudaError_t e = cudaMemcpyAsync(R.vec(dst), R.vec(src), sizeof(double) * len,
                                    cudaMemcpyDeviceToDevice, R.s);
    return e == cudaSuccess ? XG_OK : R.fail_cuda(e, "copy");
  };
  // restart from x0 for the DC solve (the analysis loads moved no vector but
  // the store and the diode/BSIM3 members)
  auto reset_start = [&]() -> int {
    std::vector<double> x0(nr, 0.0);
    if (host_x0) std::memcpy(x0.data(), host_x0, sizeof(double) * n);
    std::vector<double> z(std::max(P.n_state, P.n_store) + 1, 0.0);
    int e;
    for (int id : {XG_VEC_SOL_NEXT, XG_VEC_SOL_CURR, XG_VEC_SOL_LAST})
      if ((e = xg_vec_upload(c, id, x0.data()))) return e;
    for (int id : {XG_VEC_STA_NEXT, XG_VEC_STA_CURR, XG_VEC_STA_LAST, XG_VEC_STO_NEXT,
                   XG_VEC_STO_CURR, XG_VEC_STO_LAST}) {
      int64_t len = 0;
      xg_vec_size(c, id, &len);
      if (len && (e = xg_vec_upload(c, id, z.data()))) return e;
    }
    return circuit_reset_members(c);
  };
  if ((rc = reset_start())) { cleanup(); return rc; }

  // ---- DC operating point ---------------------------------------------------
  int s = 1;
  if (o->uic) {
    xg_load_flags fl;
    std::memset(&fl, 0, sizeof(fl));
    fl.dcop = 1;
    fl.tranop = 1;
    if ((rc = R.load(fl)) || (rc = R.combine(false, 1, 0.0, r))) { cleanup(); return rc; }
  } else {
    s = newton(false, 0.0, 1, 0.0, 0);
    st->dcop_solves = 1;
    if (s <= 0 && s > -1000) {
      // gmin stepping from the starting point
      if ((rc = reset_start())) { cleanup(); return rc; }
      for (double g = 1e-2; g >= 0.99e-12; g *= 0.1) {
        R.gshunt = g;
        if ((rc = copy_vec(XG_VEC_SOL_CURR, XG_VEC_SOL_NEXT, nr))) { cleanup(); return rc; }
        s = newton(false, 0.0, 1, 0.0, 0);
        if (s <= 0) break;
      }
      R.gshunt = 0.0;
      if (s > 0) {
        if ((rc = copy_vec(XG_VEC_SOL_CURR, XG_VEC_SOL_NEXT, nr))) { cleanup(); return rc; }
        s = newton(false, 0.0, 1, 0.0, 0);
      }
    }
  }
  st->dcop_solves = 1;
  st->dcop_iters = st->newton_iters;
  if (s <= -1000) { cleanup(); return s + 1000; }
  if (s <= 0) {
    st->status = s;
    cleanup();
    set_error("xg_tran_run: DC operating point did not converge");
    return XG_ERR_NOCONV;
  }
  // the DC point becomes current and last
  if ((rc = copy_vec(XG_VEC_SOL_CURR, XG_VEC_SOL_NEXT, nr)) ||
      (rc = copy_vec(XG_VEC_SOL_LAST, XG_VEC_SOL_NEXT, nr)) ||
      (rc = copy_vec(XG_VEC_STA_CURR, XG_VEC_STA_NEXT, P.n_state)) ||
      (rc = copy_vec(XG_VEC_STA_LAST, XG_VEC_STA_NEXT, P.n_state)) ||
      (rc = copy_vec(XG_VEC_STO_CURR, XG_VEC_STO_NEXT, P.n_store)) ||
      (rc = copy_vec(XG_VEC_STO_LAST, XG_VEC_STO_NEXT, P.n_store))) {
    cleanup();
    return rc;
  }
  record(0.0);

  // ---- time integration -------------------------------------------------------
  const std::vector<double> bp = pulse_breakpoints(P, o->tstop);
  const double bp_tol = 1e-18;
  const double tstop = o->tstop, reltol = o->reltol > 0 ? o->reltol : 1e-3,
               abstol = o->abstol > 0 ? o->abstol : 1e-6;
  const double max_step = o->maxstep > 0 ? o->maxstep : 0.1 * tstop;
  const double tol_aim = 0.5, r_min = 0.25, r_max = 0.9, r_hincr_test = 2.0, r_hincr = 2.0;
  const double h0_max_factor = 0.005;
  double t = 0.0, h = tstep, h_last = tstep, h_sum = 2 * tstep, saved = 1e-10;
  double next_time = 0.0, stop_time = tstop;
  double psi[3] = {0, 0, 0}, beta[3] = {1, 0, 0}, ck = 1;
  int order = 1, n_steps = 0, nef = 0;
  bool beginning = true, accepted_last = true, first_step = true;
  size_t bpi = 0;
  while (t < tstop && std::fabs(t - tstop) > bp_tol) {
    while (bpi < bp.size() && bp[bpi] <= t + bp_tol) ++bpi;
    stop_time = bpi < bp.size() ? bp[bpi] : tstop;
    if (beginning && accepted_last) {
      // OneStep::initialize
      const double tts = stop_time - t;
      double hh = t == 0.0 ? h0_max_factor * std::fabs(tts) : 0.1 * std::min(saved, std::fabs(tts));
      if (t == 0.0) hh = std::min(tstep, hh);
      if (hh > max_step) hh = max_step;
      h = t != 0.0 ? std::min(h, hh) : hh;
      h_sum = 2.0 * h;
      h_last = h;
      next_time = t + h;
      tran_init_hist<<<R.grid, kThreads, 0, R.s>>>(n, h, R.vec(XG_VEC_SOL_CURR), R.vec(XG_VEC_Q),
                                                   R.vec(XG_VEC_F), R.xh0, R.xh1, R.qh0, R.qh1); xg::count_launches(1);
      n_steps = 0;
      order = 1;
      psi[0] = h;
    }
    // updateCoeffs
    if (order == 2) psi[2] = psi[1];
    psi[1] = psi[0];
    psi[0] = h;
    if (order == 2) {
      const double rr = h / psi[1];
      beta[1] = rr + rr * rr / 2;
      beta[2] = -1.0 * h * h / psi[1] / psi[2] / 2;
      ck = (h / h_sum) / 3.0;
    } else {
      beta[1] = h / psi[1];
      ck = h / h_sum;
    }
    tran_predict<<<R.grid, kThreads, 0, R.s>>>(n, order, beta[1], beta[2], R.xh0, R.xh1, R.xh2,
                                               R.xn0, R.vec(XG_VEC_SOL_NEXT)); xg::count_launches(1);
    if ((rc = copy_vec(XG_VEC_STA_NEXT, XG_VEC_STA_CURR, P.n_state)) ||
        (rc = copy_vec(XG_VEC_STO_NEXT, XG_VEC_STO_CURR, P.n_store))) {
      cleanup();
      return rc;
    }
    // qn0 = qh0: the combine reads qh0 directly
    const int ns = newton(true, h, order, next_time, first_step ? 1 : 0);
    if (ns <= -1000) { cleanup(); return ns + 1000; }
    st->steps_attempted++;
    bool ok = ns >= 0;
    double est = 0.0;
    if (ok && st->steps >= 1 && !beginning) {
      tran_lte<<<kRedBlocks, kThreads, 0, R.s>>>(n, R.vec(XG_VEC_SOL_NEXT), R.xn0,
                                                 R.vec(XG_VEC_SOL_CURR), R.partials); xg::count_launches(1);
      double q[P_N];
      if ((rc = R.reduce({P_ERR2, P_XMAX}, q))) { cleanup(); return rc; }
      const double wt = reltol * q[P_XMAX] + abstol;
      est = ck * std::sqrt(q[P_ERR2] / n) / wt;
      ok = est <= 1.0;
    }
    if (ok) {
      // completeStep
      first_step = false;
      n_steps++;
      nef = 0;
      t = next_time;
      double hn = h, rr;
      h_last = h;
      rr = std::pow(tol_aim / (est + 0.0001), 1.0 / (order + 1.0));
      if (n_steps >= 2 && order == 1) {
        order = 2;
        rr = std::pow(tol_aim / (est + 0.0001), 1.0 / (order + 1.0));
        if (rr <= 1.05) order = 1;
      }
      if (rr >= r_hincr_test) {
        rr = r_hincr;
        hn = rr * h;
      } else if (rr <= 1) {
        rr = std::max(r_min, std::min(r_max, rr));
        hn = rr * h;
      }
      st->steps++;
      tran_history<<<R.grid, kThreads, 0, R.s>>>(n, order, R.vec(XG_VEC_SOL_NEXT), R.vec(XG_VEC_Q),
                                                 R.vec(XG_VEC_F), R.xh0, R.xh1, R.xh2, R.qh0,
                                                 R.qh1, R.qh2); xg::count_launches(1);
      const double min_step = t * 10.0 * DBL_EPSILON;
      hn = std::max(hn, min_step);
      hn = std::min(hn, max_step);
      if (stop_time - t >= min_step) {
        next_time = t + hn;
        if (next_time > stop_time) {
          saved = hn;
          next_time = stop_time;  // the breakpoint itself, not t + (stop - t)
          hn = stop_time - t;
        }
        h_sum = hn + h_last;
      }
      h = hn;
      if ((rc = xg_rotate_history(c))) { cleanup(); return rc; }
      record(t);
      beginning = std::fabs(t - stop_time) <= bp_tol && std::fabs(t - tstop) > bp_tol;
      accepted_last = true;
    } else {
      // rejectStep
      st->rejected++;
      accepted_last = false;
      nef++;
      for (int i = 1; i <= order; ++i) psi[i - 1] = psi[i];
      if (nef >= 15) {
        st->status = -7;
        cleanup();
        set_error("xg_tran_run: too many local error test failures");
        return XG_ERR_NOCONV;
      }
      double hn;
      if (ns <= 0) {
        hn = h / 8;
      } else if (nef == 1) {
        // the default build's rejectStep (no Q-norm): r_factor 1, r_safety 2,
        // r_fudge 1e-4 and the one-step method's new order 1
        double rr = 1.0 * std::pow(2.0 * (est + 0.0001), -1.0 / (1 + 1.0));
        rr = std::max(r_min, std::min(r_max, rr));
        hn = rr * h;
      } else {
        hn = r_min * h;
      }
      order = 1;
      hn = std::max(hn, t * 10.0 * DBL_EPSILON);
      hn = std::min(hn, max_step);
      next_time = t + hn;
      if (next_time > stop_time) {
        next_time = stop_time;
        hn = stop_time - t;
      }
      h_sum = hn + h_last;
      h = hn;
      if (h < 1e-21) {
        st->status = -8;
        cleanup();
        set_error("xg_tran_run: time step too small");
        return XG_ERR_NOCONV;
      }
    }
  }
  st->t_end = t;
  *n_points = np;
  if (n_out && np) {
    cudaError_t e = cudaMemcpyAsync(host_v, d_rec, sizeof(double) * (size_t)np * n_out,
                                    cudaMemcpyDeviceToHost, R.s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(R.s);
    if (e != cudaSuccess) {
      set_error(std::string("xg_tran_run: ") + cudaGetErrorString(e));
      cleanup();
      return XG_ERR_CUDA;
    }
  }
  cleanup();
#undef TRY_CUDA
  return XG_OK;
}
