// serve.cu — many independent transients stepped together on one GPU (the
// serving path: .STEP / Monte-Carlo variants of a circuit, each a request).
//
// A batch is the block-diagonal union of its requests' netlists, set up once
// as one circuit: one launch per device type evaluates every instance of every
// request, and the fixed-order reduction stamps every request's matrices, with
// each instance reading its own request's load flags (time, Newton iteration,
// first step).  What the reference does per circuit on the host, the batch does
// per request on the device, with no host round trip inside the time loop:
//
//   batch_solve    one warp per request: refactor its Jacobian with the pivot
//                  order analysed for it at set-up, solve, FP64 refinement when
//                  the factors are FP32, update x, weighted norm of the update;
//   load           the union's evaluation kernels and reduction;
//   batch_combine  one warp per request: trapezoid residual and Jacobian
//                  (N_TIA_OneStep.C:215-352) and the norms the tests need;
//   batch_control  one thread per request: damped-Newton convergence test
//                  (N_NLS_DampedNewton.C:1787-1919), local error test, step and
//                  order control (N_TIA_OneStep.C:1355-2190), finish;
//   batch_vector   one warp per request: history update, state rotation,
//                  waveform record, predictor of the next step.
//
// One batch iteration is these six launches; a run of them is captured once
// into a CUDA graph on the batch's own stream and replayed, so batches admitted
// at different times overlap on the device.  Requests start from their
// initial condition (.TRAN ... UIC); their sources carry no breakpoints.

#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "xg.h"
#include "xg_internal.h"
#include "xg_lu.h"

namespace xg {
namespace {

enum Phase : int { PH_DONE = 0, PH_INIT = 1, PH_START = 2, PH_ITER = 3 };
enum Action : int { A_INIT = 1, A_ACCEPT = 2, A_PREDICT = 4, A_RESTART = 8 };
enum Part : int { Q_RHS2 = 0, Q_RHSMAX, Q_LIMMAX, Q_DXW2, Q_ERR2, Q_XMAX, Q_LUFAIL, Q_N };

struct CState {
  double t, h, h_last, h_sum, saved, next_time, tstop, tstep, max_step, reltol, abstol;
  double stop_time;              // the next breakpoint (or tstop)
  double psi[3], beta[3], ck;
  double norm_init, norm_old, stall_rate;
  int order, n_steps, nef, beginning, first_step;
  int phase, nstep, stall_count, action, status, failed;
  int steps, steps_attempted, rejected, newton_iters, loads, n_rec;
  int bpi;                       // index of stop_time in the request's breakpoints
  int hist_order;                // order of the history update of an accepted step
};

struct BatchDev {
  int nc;
  const int *uptr, *uidx;        // unknowns of request c (union ids, local order)
  const int *sptr, *sidx;        // its state slots: ranges (start, length) sptr[c]..sptr[c+1]
  const int *optr, *oidx;        // its store slots, the same way
  const int *jptr, *jidx;        // its Jacobian entries (its rows), the same way
  const int *arp, *aci;          // union Jacobian pattern
  const int *lrp_off;            // request c's local row pointers start here (n_c + 1)
  const int64_t *lnz_off;        // its L\U entries start here
  const int *lrp, *lci, *ldiag;  // local CSR of L\U (row pointers relative to lnz_off;
                                 // diagonal positions per unknown, from uptr[c])
  const int64_t *lu2a;           // L\U entry -> union Jacobian entry, -1 for fill
  const int *lP, *lQ;            // local pivot order
  void *lval, *lrd;              // L\U values and reciprocal pivots (FP64 or FP32)
  double *y, *r, *dd;            // solve workspace per union unknown
  int *map;                      // column -> position, per union unknown
  double *x, *xc, *xl, *sta, *stac, *stal, *sto, *stoc, *stol;
  const double *f, *q, *fvp, *qvp, *dfdx, *dqdx;
  double *jac, *rhs, *dx, *w, *xh0, *xh1, *xh2, *qh0, *qh1, *qh2, *xn0;
  double *part;                  // [nc][Q_N]
  CState *cs;
  Flags *flags;                  // per request load flags
  const int *out_idx;            // [nc][n_out] union ids
  int n_out, max_points;
  double *rec_t, *rec_v;         // [nc][max_points], [nc][max_points][n_out]
  int n_refine;
  // level schedule per request (batch_solve_lvl): lvl[c] != 0 when request c
  // uses it; its int blob (lvl_blob layout) starts at sched_off[c]
  const int *lvl;
  const int64_t *sched_off;
  const int *sched;
  // breakpoints of request c (its PULSE corners, then its tstop):
  // bp[bp_ptr[c]] .. bp[bp_ptr[c + 1] - 1], sorted
  const int *bp_ptr;
  const double *bp;
};

// 1/u by Newton-Raphson on the reciprocal from a single-precision seed (two
// steps, each doubling the correct bits); IEEE division outside the range
// where the seed is representable.
__device__ __forceinline__ double recip_nr(double u) {
  const double a = fabs(u);
  if (!(a > 1e-30 && a < 1e30)) return 1.0 / u;
  double x = double(1.0f / float(u));
  x = x * (2.0 - u * x);
  x = x * (2.0 - u * x);
  return x;
}
// FP32 factors: a single-precision reciprocal, no FP64 instruction
__device__ __forceinline__ float recip_nr(float u) { return 1.0f / u; }

// A zero, infinite or NaN pivot, from the bits (no FP64 instruction).
__device__ __forceinline__ bool bad_pivot(double u) {
  const unsigned long long v = (unsigned long long)__double_as_longlong(u);
  return (v << 1) == 0 || ((v >> 52) & 0x7ff) == 0x7ff;
}
__device__ __forceinline__ bool bad_pivot(float u) {
  const unsigned v = __float_as_uint(u);
  return (v << 1) == 0 || ((v >> 23) & 0xff) == 0xff;
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max_d(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// ---- batch_solve: factor, solve, refine, update (one warp per request) -------
template <class T>
__global__ void __launch_bounds__(128) batch_solve(BatchDev b) {
  const int c = blockIdx.x * 4 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= b.nc) return;
  if (b.cs[c].phase != PH_ITER || b.lvl[c]) return;
  const int u0 = b.uptr[c], n = b.uptr[c + 1] - u0;
  const int *rp = b.lrp + b.lrp_off[c];
  const int64_t z0 = b.lnz_off[c];
  const int *ci = b.lci + z0;
  const int *diag = b.ldiag + u0;
  T *val = (T *)b.lval + z0;
  T *rd = (T *)b.lrd + u0;
  int *map = b.map + u0;
  const int *P = b.lP + u0, *Q = b.lQ + u0;
  const int64_t nz = b.lnz_off[c + 1] - z0;
  for (int64_t p = lane; p < nz; p += 32) {
    const int64_t s = b.lu2a[z0 + p];
    val[p] = s >= 0 ? T(b.jac[s]) : T(0);
  }
  __syncwarp();
  int bad = 0;
  if (lane == 0) {
    for (int row = 0; row < n; ++row) {
      const int s = rp[row], dp = diag[row], e = rp[row + 1];
      for (int p = s; p < e; ++p) map[ci[p]] = p;
      for (int p = s; p < dp; ++p) {
        const int k = ci[p];
        const T l = val[p] * rd[k];
        val[p] = l;
        for (int q = diag[k] + 1; q < rp[k + 1]; ++q) {
          const int pos = map[ci[q]];
          if (pos > p && pos < e && ci[pos] == ci[q]) val[pos] -= l * val[q];
          else bad = 1;
        }
      }
      const T u = val[dp];
      if (bad_pivot(u)) bad = 1;
      rd[row] = recip_nr(u);
    }
  }
  __syncwarp();
  // solve J dx = rhs, then refine against the FP64 Jacobian; the work vector
  // is in the factors' precision
  T *y = reinterpret_cast<T *>(b.y + u0);
  for (int pass = 0; pass <= b.n_refine; ++pass) {
    const double *src = pass == 0 ? b.rhs : b.r;
    for (int k = lane; k < n; k += 32) y[k] = T(src[b.uidx[u0 + P[k]]]);
    __syncwarp();
    if (lane == 0) {
      for (int row = 0; row < n; ++row) {
        T acc = y[row];
        for (int p = rp[row]; p < diag[row]; ++p) acc -= val[p] * y[ci[p]];
        y[row] = acc;
      }
      for (int row = n - 1; row >= 0; --row) {
        T acc = y[row];
        for (int p = diag[row] + 1; p < rp[row + 1]; ++p) acc -= val[p] * y[ci[p]];
        y[row] = acc * rd[row];
      }
    }
    __syncwarp();
    for (int k = lane; k < n; k += 32) {
      const int g = b.uidx[u0 + Q[k]];
      if (pass == 0) b.dx[g] = double(y[k]);
      else b.dx[g] += double(y[k]);
    }
    __syncwarp();
    if (pass < b.n_refine) {
      // r = rhs - J dx over this request's rows (FP64)
      for (int k = lane; k < n; k += 32) {
        const int g = b.uidx[u0 + k];
        double acc = b.rhs[g];
        for (int p = b.arp[g]; p < b.arp[g + 1]; ++p) acc -= b.jac[p] * b.dx[b.aci[p]];
        b.r[g] = acc;
      }
      __syncwarp();
    }
  }
  // x += dx, weighted norm of the update
  double s2 = 0.0;
  for (int k = lane; k < n; k += 32) {
    const int g = b.uidx[u0 + k];
    b.x[g] += b.dx[g];
    const double t = b.dx[g] / b.w[g];
    s2 += t * t;
  }
  s2 = warp_sum_d(s2);
  bad = __shfl_sync(0xffffffffu, bad, 0);
  if (lane == 0) {
    b.part[c * Q_N + Q_DXW2] = s2;
    b.part[c * Q_N + Q_LUFAIL] = bad;
  }
}

// Shared-memory variant: one warp per block stages its request's L\U values,
// pattern, map and vectors in shared memory, so lane 0's walk costs shared-
// memory latencies instead of L2 round trips.  Used when the largest
// request's footprint fits (smem_bytes_request).
__host__ __device__ inline size_t smem_bytes_request(int n, int64_t nz, size_t tsz) {
  auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
  return a16(tsz * size_t(nz)) + 2 * a16(tsz * size_t(n)) +
         sizeof(int) * (size_t(nz) + 3 * size_t(n) + 1);
}

template <class T>
__global__ void __launch_bounds__(32) batch_solve_smem(BatchDev b) {
  extern __shared__ __align__(16) char sm[];
  const int c = blockIdx.x, lane = threadIdx.x;
  if (c >= b.nc) return;
  if (b.cs[c].phase != PH_ITER || b.lvl[c]) return;
  const int u0 = b.uptr[c], n = b.uptr[c + 1] - u0;
  const int64_t z0 = b.lnz_off[c];
  const int nz = int(b.lnz_off[c + 1] - z0);
  auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
  T *val = (T *)sm;
  T *rd = (T *)(sm + a16(sizeof(T) * nz));
  T *y = (T *)(sm + a16(sizeof(T) * nz) + a16(sizeof(T) * n));
  int *ci = (int *)(sm + a16(sizeof(T) * nz) + 2 * a16(sizeof(T) * n));
  int *rp = ci + nz, *diag = rp + n + 1, *map = diag + n;
  const int *grp = b.lrp + b.lrp_off[c];
  for (int p = lane; p < nz; p += 32) {
    const int64_t s = b.lu2a[z0 + p];
    val[p] = s >= 0 ? T(b.jac[s]) : T(0);
    ci[p] = b.lci[z0 + p];
  }
  for (int i = lane; i <= n; i += 32) rp[i] = grp[i];
  for (int i = lane; i < n; i += 32) diag[i] = b.ldiag[u0 + i];
  __syncwarp();
  int bad = 0;
  if (lane == 0) {
    for (int row = 0; row < n; ++row) {
      const int s = rp[row], dp = diag[row], e = rp[row + 1];
      for (int p = s; p < e; ++p) map[ci[p]] = p;
      for (int p = s; p < dp; ++p) {
        const int k = ci[p];
        const T l = val[p] * rd[k];
        val[p] = l;
        for (int q = diag[k] + 1; q < rp[k + 1]; ++q) {
          const int pos = map[ci[q]];
          if (pos > p && pos < e && ci[pos] == ci[q]) val[pos] -= l * val[q];
          else bad = 1;
        }
      }
      const T u = val[dp];
      if (bad_pivot(u)) bad = 1;
      rd[row] = recip_nr(u);
    }
  }
  __syncwarp();
  const int *P = b.lP + u0, *Q = b.lQ + u0;
  for (int pass = 0; pass <= b.n_refine; ++pass) {
    const double *src = pass == 0 ? b.rhs : b.r;
    for (int k = lane; k < n; k += 32) y[k] = T(src[b.uidx[u0 + P[k]]]);
    __syncwarp();
    if (lane == 0) {
      for (int row = 0; row < n; ++row) {
        T acc = y[row];
        for (int p = rp[row]; p < diag[row]; ++p) acc -= val[p] * y[ci[p]];
        y[row] = acc;
      }
      for (int row = n - 1; row >= 0; --row) {
        T acc = y[row];
        for (int p = diag[row] + 1; p < rp[row + 1]; ++p) acc -= val[p] * y[ci[p]];
        y[row] = acc * rd[row];
      }
    }
    __syncwarp();
    for (int k = lane; k < n; k += 32) {
      const int g = b.uidx[u0 + Q[k]];
      if (pass == 0) b.dx[g] = double(y[k]);
      else b.dx[g] += double(y[k]);
    }
    __syncwarp();
    if (pass < b.n_refine) {
      for (int k = lane; k < n; k += 32) {
        const int g = b.uidx[u0 + k];
        double acc = b.rhs[g];
        for (int p = b.arp[g]; p < b.arp[g + 1]; ++p) acc -= b.jac[p] * b.dx[b.aci[p]];
        b.r[g] = acc;
      }
      __syncwarp();
    }
  }
  double s2 = 0.0;
  for (int k = lane; k < n; k += 32) {
    const int g = b.uidx[u0 + k];
    b.x[g] += b.dx[g];
    const double t = b.dx[g] / b.w[g];
    s2 += t * t;
  }
  s2 = warp_sum_d(s2);
  bad = __shfl_sync(0xffffffffu, bad, 0);
  if (lane == 0) {
    b.part[c * Q_N + Q_DXW2] = s2;
    b.part[c * Q_N + Q_LUFAIL] = bad;
  }
}

// ---- batch_solve_lvl: the level schedule, one warp per request ----------------
// The walk above runs one lane over every row, so the batch iteration takes as
// long as the largest request's rows in sequence.  Here each request's factor
// comes with its dependency levels (nested dissection makes a ring of 501
// stages ~30 levels deep): the rows of a level go to the lanes, the trailing
// supply-rail rows are pulled position by position, and everything sits in
// shared memory.  Per request the sums are in a fixed order, so a request's
// result does not depend on the batch around it.

// The blob, all ints: a header, then the arrays in this order.
enum LvlHdr { H_LEVELS, H_ULEVELS, H_TAIL0, H_NTAIL, H_NGROUPS, H_NPOS, H_NPAIRS, H_NUP, H_N };
__host__ __device__ inline int64_t lvl_blob_len(int n, const int *h) {
  return H_N + (n + 1) + h[H_NUP] + h[H_TAIL0] + (h[H_LEVELS] + 1) + n + (h[H_ULEVELS] + 1) +
         (h[H_NTAIL] + 1) + (h[H_NGROUPS] + 1) + h[H_NPOS] + (h[H_NPOS] + 1) + 2 * int64_t(h[H_NPAIRS]);
}
__host__ __device__ inline size_t smem_bytes_lvl(int n, int64_t nz, int64_t blob, size_t tsz) {
  auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
  return a16(tsz * size_t(nz)) + 2 * a16(tsz * size_t(n)) +
         sizeof(int) * (size_t(nz) + 2 * size_t(n) + 1 + size_t(blob));
}

template <class T>
__device__ __forceinline__ T warp_sum_t(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

constexpr int kLvlThreads = 128;  // threads per request in batch_solve_lvl

template <class T>
__global__ void __launch_bounds__(kLvlThreads) batch_solve_lvl(BatchDev b) {
  extern __shared__ __align__(16) char sm[];
  const int c = blockIdx.x, lane = threadIdx.x & 31, tid = threadIdx.x, nt = blockDim.x;
  if (c >= b.nc) return;
  if (b.cs[c].phase != PH_ITER || !b.lvl[c]) return;
  const int u0 = b.uptr[c], n = b.uptr[c + 1] - u0;
  const int64_t z0 = b.lnz_off[c];
  const int nz = int(b.lnz_off[c + 1] - z0);
  const int64_t s0 = b.sched_off[c];
  const int blob = int(b.sched_off[c + 1] - s0);
  auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
  T *val = (T *)sm;
  T *rd = (T *)(sm + a16(sizeof(T) * nz));
  T *y = (T *)(sm + a16(sizeof(T) * nz) + a16(sizeof(T) * n));
  int *ci = (int *)(sm + a16(sizeof(T) * nz) + 2 * a16(sizeof(T) * n));
  int *rp = ci + nz, *diag = rp + n + 1, *h = diag + n;
  const int *grp = b.lrp + b.lrp_off[c];
  for (int p = tid; p < nz; p += nt) {
    const int64_t s = b.lu2a[z0 + p];
    val[p] = s >= 0 ? T(b.jac[s]) : T(0);
    ci[p] = b.lci[z0 + p];
  }
  for (int i = tid; i <= n; i += nt) rp[i] = grp[i];
  for (int i = tid; i < n; i += nt) diag[i] = b.ldiag[u0 + i];
  for (int i = tid; i < blob; i += nt) h[i] = b.sched[s0 + i];
  __syncthreads();
  const int levels = h[H_LEVELS], ulevels = h[H_ULEVELS], tail0 = h[H_TAIL0];
  const int ntail = h[H_NTAIL], ngroups = h[H_NGROUPS], npos = h[H_NPOS], npairs = h[H_NPAIRS];
  const int *urp = h + H_N, *upos = urp + (n + 1), *lrow = upos + h[H_NUP];
  const int *lptr = lrow + tail0, *urow = lptr + (levels + 1), *uptr = urow + n;
  const int *trowg = uptr + (ulevels + 1), *tgptr = trowg + (ntail + 1), *tpos = tgptr + (ngroups + 1);
  const int *tpp = tpos + npos, *tpm = tpp + (npos + 1), *tq = tpm + npairs;
  bool bad = false;
  // factor: the levels, one row per lane
  for (int lv = 0; lv < levels; ++lv) {
    for (int t = lptr[lv] + tid; t < lptr[lv + 1]; t += nt) {
      const int i = lrow[t];
      const int dp = diag[i];
      int u = urp[i];
      for (int p = rp[i]; p < dp; ++p) {
        const int k = ci[p];
        const T l = val[p] * rd[k];
        val[p] = l;
        const int q0 = diag[k] + 1, len = rp[k + 1] - q0;
        for (int j = 0; j < len; ++j) val[upos[u + j]] -= l * val[q0 + j];
        u += len;
      }
      const T piv = val[dp];
      bad |= bad_pivot(piv);
      rd[i] = recip_nr(piv);
    }
    __syncthreads();
  }
  // the tail rows: positions pull their updates, group by group; a group of
  // one position (the rail's diagonal) is summed by the whole warp
  for (int r = 0; r < ntail; ++r) {
    const int i = tail0 + r, dp = diag[i];
    for (int g = trowg[r]; g < trowg[r + 1]; ++g) {
      if (tgptr[g + 1] - tgptr[g] == 1) {
        if (tid < 32) {
          const int t = tgptr[g], p = tpos[t];
          T part = T(0);
          for (int j = tpp[t] + lane; j < tpp[t + 1]; j += 32) part += val[tpm[j]] * val[tq[j]];
          part = warp_sum_t(part);
          if (lane == 0) {
            const T acc = val[p] - part;
            val[p] = p < dp ? acc * rd[ci[p]] : acc;
          }
        }
      } else {
        for (int t = tgptr[g] + tid; t < tgptr[g + 1]; t += nt) {
          const int p = tpos[t];
          T acc = val[p];
          for (int j = tpp[t]; j < tpp[t + 1]; ++j) acc -= val[tpm[j]] * val[tq[j]];
          val[p] = p < dp ? acc * rd[ci[p]] : acc;
        }
      }
      __syncthreads();
    }
    if (tid == 0) {
      const T piv = val[dp];
      bad |= bad_pivot(piv);
      rd[i] = recip_nr(piv);
    }
    __syncthreads();
  }
  const int *P = b.lP + u0, *Q = b.lQ + u0;
  for (int pass = 0; pass <= b.n_refine; ++pass) {
    const double *src = pass == 0 ? b.rhs : b.r;
    for (int k = tid; k < n; k += nt) y[k] = T(src[b.uidx[u0 + P[k]]]);
    __syncthreads();
    for (int lv = 0; lv < levels; ++lv) {
      for (int t = lptr[lv] + tid; t < lptr[lv + 1]; t += nt) {
        const int i = lrow[t];
        T acc = y[i];
        for (int p = rp[i]; p < diag[i]; ++p) acc -= val[p] * y[ci[p]];
        y[i] = acc;
      }
      __syncthreads();
    }
    if (tid < 32)
      for (int i = tail0; i < n; ++i) {
        T part = T(0);
        for (int p = rp[i] + lane; p < diag[i]; p += 32) part += val[p] * y[ci[p]];
        part = warp_sum_t(part);
        if (lane == 0) y[i] -= part;
        __syncwarp();
      }
    __syncthreads();
    for (int lv = 0; lv < ulevels; ++lv) {
      for (int t = uptr[lv] + tid; t < uptr[lv + 1]; t += nt) {
        const int i = urow[t];
        T acc = y[i];
        for (int p = diag[i] + 1; p < rp[i + 1]; ++p) acc -= val[p] * y[ci[p]];
        y[i] = acc * rd[i];
      }
      __syncthreads();
    }
    for (int k = tid; k < n; k += nt) {
      const int g = b.uidx[u0 + Q[k]];
      if (pass == 0) b.dx[g] = double(y[k]);
      else b.dx[g] += double(y[k]);
    }
    __syncthreads();
    if (pass < b.n_refine) {
      for (int k = tid; k < n; k += nt) {
        const int g = b.uidx[u0 + k];
        double acc = b.rhs[g];
        for (int p = b.arp[g]; p < b.arp[g + 1]; ++p) acc -= b.jac[p] * b.dx[b.aci[p]];
        b.r[g] = acc;
      }
      __syncthreads();
    }
  }
  __shared__ double sh[kLvlThreads / 32];
  double s2 = 0.0;
  for (int k = tid; k < n; k += nt) {
    const int g = b.uidx[u0 + k];
    b.x[g] += b.dx[g];
    const double t = b.dx[g] / b.w[g];
    s2 += t * t;
  }
  s2 = warp_sum_d(s2);
  if (lane == 0) sh[tid >> 5] = s2;
  const int any_bad = __syncthreads_or(bad ? 1 : 0) ? 1 : 0;
  if (tid == 0) {
    double acc = sh[0];
    for (int w = 1; w < nt / 32; ++w) acc += sh[w];
    b.part[c * Q_N + Q_DXW2] = acc;
    b.part[c * Q_N + Q_LUFAIL] = any_bad;
  }
}

// ---- batch_combine: residual, Jacobian and norms (one warp per request) ------
// One block of kBatchThreads per request (not a warp): a request of 500
// stages has thousands of unknowns, state slots and Jacobian entries, and its
// supply row alone has one entry per device on the rail.
constexpr int kBatchThreads = 256;
// batch_vector's phases are chains of dependent gathers (request -> union
// id -> history): a thread per unknown for requests up to 512 unknowns
// keeps each phase one round trip deep
constexpr int kVectorThreads = 512;

// Block-wide sum and max in a fixed order (lane butterfly, then warps in
// order): the same result whatever the batch around the request.
__device__ void block_sum_max(double *vals, int nsum, int nmax, double *sh) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int j = 0; j < nsum; ++j) vals[j] = warp_sum_d(vals[j]);
  for (int j = nsum; j < nsum + nmax; ++j) vals[j] = warp_max_d(vals[j]);
  const int m = nsum + nmax;
  if (lane == 0)
    for (int j = 0; j < m; ++j) sh[wid * m + j] = vals[j];
  __syncthreads();
  // lane j of warp 0 combines value j over the warps, in warp order; the
  // results reach every lane of warp 0 (thread 0 reads them)
  if (wid == 0) {
    double acc = 0.0;
    if (lane < m) {
      acc = sh[lane];
      for (int w = 1; w < nw; ++w) acc = lane < nsum ? acc + sh[w * m + lane] : fmax(acc, sh[w * m + lane]);
    }
    for (int j = 0; j < m; ++j) vals[j] = __shfl_sync(0xffffffffu, acc, j);
  }
}

// ---- batch_combine: residual, Jacobian and norms (one block per request) ------
__global__ void __launch_bounds__(kBatchThreads) batch_combine(BatchDev b) {
  __shared__ double sh[(kBatchThreads / 32) * 5];
  const int c = blockIdx.x;
  if (c >= b.nc) return;
  const CState &cs = b.cs[c];
  if (cs.phase == PH_DONE || cs.phase == PH_INIT) return;
  const int u0 = b.uptr[c], n = b.uptr[c + 1] - u0;
  const int order = cs.order;
  const double inv_h = 1.0 / cs.h, fs = order == 2 ? 0.5 : 1.0;
  double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};  // sums: rhs^2, err^2; maxima: rhs, limiter, x
  for (int k = threadIdx.x; k < n; k += blockDim.x) {
    const int g = b.uidx[u0 + k];
    double r = (b.q[g] - b.qh0[g]) * inv_h;
    r = order == 2 ? r + 0.5 * b.f[g] + 0.5 * b.qh2[g] : r + b.f[g];
    r = -r;
    r += b.qvp[g] * inv_h;
    r += fs * b.fvp[g];
    b.rhs[g] = r;
    v[0] += r * r;
    const double e = b.x[g] - b.xn0[g];
    v[1] += e * e;
    v[2] = fmax(v[2], fabs(r));
    v[3] = fmax(v[3], fmax(fabs(b.fvp[g]), fabs(b.qvp[g])));
    v[4] = fmax(v[4], fabs(b.xc[g]));
  }
  // the Jacobian entries of the request's rows, as runs of consecutive
  // entries spread over the block (a supply row's hundreds of entries too)
  for (int k = b.jptr[c]; k < b.jptr[c + 1]; ++k) {
    const int p0 = b.jidx[2 * k], p1 = p0 + b.jidx[2 * k + 1];
    for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) b.jac[p] = inv_h * b.dqdx[p] + fs * b.dfdx[p];
  }
  block_sum_max(v, 2, 3, sh);
  if (threadIdx.x == 0) {
    double *pp = b.part + c * Q_N;
    pp[Q_RHS2] = v[0];
    pp[Q_ERR2] = v[1];
    pp[Q_RHSMAX] = v[2];
    pp[Q_LIMMAX] = v[3];
    pp[Q_XMAX] = v[4];
  }
}

// ---- batch_control: Newton test and step control (one thread per request) ----
__device__ int converged(CState &cs, int step, double max_rhs, double upd, double rhs_rel,
                         double rate) {
  const double eps = DBL_EPSILON, rate_max = 0.5 * DBL_MAX, min_red = 0.9, stag = 1e-3;
  const int max_step = 20;
  const double rhs_tol = 1e-2, dx_tol = 0.33, small_update = 1e-6;
  if (max_rhs <= eps && max_rhs <= rhs_tol) return 1;
  if (max_rhs <= rhs_tol && upd <= dx_tol) return 2;
  if (step > max_step && rhs_rel <= min_red && rate <= 1.0) return 3;
  if (upd <= small_update) return 4;
  if (step > max_step) return -1;
  if (rate > rate_max) return -2;
  if (fabs(rate - 1.0) <= stag) {
    if (cs.stall_count == 0 || rate < cs.stall_rate) cs.stall_rate = rate;
    cs.stall_count++;
  } else {
    cs.stall_count = 0;
  }
  if (cs.stall_count == 5) {
    cs.stall_count = 0;
    return (rhs_rel < min_red && cs.stall_rate <= 1.0) ? 3 : -3;
  }
  return 0;
}

__device__ void update_coeffs(CState &cs) {
  const double h = cs.h;
  if (cs.order == 2) cs.psi[2] = cs.psi[1];
  cs.psi[1] = cs.psi[0];
  cs.psi[0] = h;
  cs.beta[0] = 1.0;
  if (cs.order == 2) {
    const double rr = h / cs.psi[1];
    cs.beta[1] = rr + rr * rr / 2;
    cs.beta[2] = -1.0 * h * h / cs.psi[1] / cs.psi[2] / 2;
    cs.ck = (h / cs.h_sum) / 3.0;
  } else {
    cs.beta[1] = h / cs.psi[1];
    cs.beta[2] = 0.0;
    cs.ck = h / cs.h_sum;
  }
}

__device__ void start_step(CState &cs, Flags &fl) {
  update_coeffs(cs);
  cs.action |= A_PREDICT;
  cs.phase = PH_START;
  fl = Flags{};
  fl.transient = 1;
  fl.time = cs.next_time;
  fl.pdt = 1.0 / cs.h;
  fl.newton_iter = 0;
  fl.init_tran = cs.first_step;
  cs.loads++;
}

constexpr double kBpTol = 1e-18;

// The first breakpoint after t (the breakpoint list ends with tstop).
__device__ void next_breakpoint(const BatchDev &b, int c, CState &cs) {
  const int e = b.bp_ptr[c + 1];
  int k = b.bp_ptr[c] + cs.bpi;
  while (k < e && b.bp[k] <= cs.t + kBpTol) ++k;
  cs.bpi = k - b.bp_ptr[c];
  cs.stop_time = k < e ? b.bp[k] : cs.tstop;
}

__global__ void batch_control(BatchDev b) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= b.nc) return;
  CState &cs = b.cs[c];
  Flags &fl = b.flags[c];
  const double *pp = b.part + c * Q_N;
  const int n = b.uptr[c + 1] - b.uptr[c];
  cs.action = 0;
  if (cs.phase == PH_DONE) return;
  if (cs.phase == PH_INIT) {
    // OneStep::initialize at t = 0, towards the first breakpoint
    next_breakpoint(b, c, cs);
    const double tts = cs.stop_time - cs.t;
    double hh = 0.005 * fabs(tts);
    hh = fmin(cs.tstep, hh);
    if (hh > cs.max_step) hh = cs.max_step;
    cs.h = hh;
    cs.h_sum = 2.0 * hh;
    cs.h_last = hh;
    cs.next_time = cs.t + hh;
    cs.n_steps = 0;
    cs.order = 1;
    cs.psi[0] = hh;
    cs.action = A_INIT;
    start_step(cs, fl);
    return;
  }
  int status = 0;
  if (cs.phase == PH_START) {
    const double norm = sqrt(pp[Q_RHS2]);
    if (norm < DBL_EPSILON) {
      status = 1;
    } else {
      cs.norm_init = cs.norm_old = norm;
      cs.nstep = 0;
      cs.phase = PH_ITER;
      fl.newton_iter = 1;
      cs.loads++;
      return;
    }
  } else {  // PH_ITER
    cs.nstep++;
    cs.newton_iters++;
    if (pp[Q_LUFAIL] != 0.0) {
      status = -5;
    } else {
      const double upd = sqrt(pp[Q_DXW2] / n);
      const double norm = sqrt(pp[Q_RHS2]), max_rhs = pp[Q_RHSMAX];
      const double rel = norm / cs.norm_init, rate = norm / cs.norm_old;
      cs.norm_old = norm;
      status = converged(cs, cs.nstep, max_rhs, upd, rel, rate);
      if (max_rhs != 0.0 && !(max_rhs < 0.0) && !(max_rhs > 0.0)) status = -6;
      if (status == 0) {
        fl.newton_iter = cs.nstep + 1;
        cs.loads++;
        return;
      }
    }
  }
  // the Newton solve of this step has ended: local error test, accept or reject
  cs.steps_attempted++;
  bool ok = status >= 0;
  double est = 0.0;
  if (ok && cs.steps >= 1 && !cs.beginning) {
    const double wt = cs.reltol * pp[Q_XMAX] + cs.abstol;
    est = cs.ck * sqrt(pp[Q_ERR2] / n) / wt;
    ok = est <= 1.0;
  }
  const double tol_aim = 0.5, r_min = 0.25, r_max = 0.9;
  if (ok) {
    cs.first_step = 0;
    cs.beginning = 0;
    cs.n_steps++;
    cs.nef = 0;
    cs.t = cs.next_time;
    double hn = cs.h;
    cs.h_last = cs.h;
    double rr = pow(tol_aim / (est + 0.0001), 1.0 / (cs.order + 1.0));
    if (cs.n_steps >= 2 && cs.order == 1) {
      cs.order = 2;
      rr = pow(tol_aim / (est + 0.0001), 1.0 / (cs.order + 1.0));
      if (rr <= 1.05) cs.order = 1;
    }
    if (rr >= 2.0) hn = 2.0 * cs.h;
    else if (rr <= 1) hn = fmax(r_min, fmin(r_max, rr)) * cs.h;
    cs.steps++;
    cs.action |= A_ACCEPT;
    const double min_step = cs.t * 10.0 * DBL_EPSILON;
    hn = fmax(hn, min_step);
    hn = fmin(hn, cs.max_step);
    if (cs.stop_time - cs.t >= min_step) {
      cs.next_time = cs.t + hn;
      if (cs.next_time > cs.stop_time) {
        cs.saved = hn;
        cs.next_time = cs.stop_time;  // the breakpoint itself, not t + (stop - t)
        hn = cs.stop_time - cs.t;
      }
      cs.h_sum = hn + cs.h_last;
    }
    cs.h = hn;
    cs.hist_order = cs.order;
    if (!(cs.t < cs.tstop) || fabs(cs.t - cs.tstop) <= kBpTol) {
      cs.phase = PH_DONE;
      return;
    }
    cs.beginning = fabs(cs.t - cs.stop_time) <= kBpTol && fabs(cs.t - cs.tstop) > kBpTol;
    next_breakpoint(b, c, cs);
    if (cs.beginning) {
      // OneStep::initialize at a breakpoint: a first-order restart with a
      // step of at most a tenth of the one cut short there
      const double tts = cs.stop_time - cs.t;
      double hh = 0.1 * fmin(cs.saved, fabs(tts));
      if (hh > cs.max_step) hh = cs.max_step;
      cs.h = fmin(cs.h, hh);
      cs.h_sum = 2.0 * cs.h;
      cs.h_last = cs.h;
      cs.next_time = cs.t + cs.h;
      cs.n_steps = 0;
      cs.order = 1;
      cs.psi[0] = cs.h;
      cs.action |= A_RESTART;
    }
  } else {
    cs.rejected++;
    cs.nef++;
    for (int i = 1; i <= cs.order; ++i) cs.psi[i - 1] = cs.psi[i];
    double hn;
    if (status <= 0) hn = cs.h / 8;
    // first local-error failure: the default build's rejectStep (no Q-norm):
    // r_factor 1, r_safety 2, r_fudge 1e-4, the one-step method's new order 1
    else if (cs.nef == 1) hn = fmax(r_min, fmin(r_max, 1.0 * pow(2.0 * (est + 0.0001), -1.0 / (1 + 1.0)))) * cs.h;
    else hn = r_min * cs.h;
    cs.order = 1;
    hn = fmax(hn, cs.t * 10.0 * DBL_EPSILON);
    hn = fmin(hn, cs.max_step);
    cs.next_time = cs.t + hn;
    if (cs.next_time > cs.stop_time) {
      cs.next_time = cs.stop_time;
      hn = cs.stop_time - cs.t;
    }
    cs.h_sum = hn + cs.h_last;
    cs.h = hn;
    if (cs.nef >= 15 || cs.h < 1e-21) {
      cs.failed = 1;
      cs.status = status != 0 ? status : -7;
      cs.phase = PH_DONE;
      return;
    }
  }
  start_step(cs, fl);
}

// ---- batch_vector: history, rotation, record, predictor (warp per request) ---
__global__ void __launch_bounds__(kVectorThreads) batch_vector(BatchDev b) {
  const int c = blockIdx.x, tid = threadIdx.x, nt = blockDim.x;
  if (c >= b.nc) return;
  CState &cs = b.cs[c];
  const int act = cs.action;
  if (!act) return;
  const int u0 = b.uptr[c], n = b.uptr[c + 1] - u0;
  if (act & A_INIT) {
    for (int k = tid; k < n; k += nt) {
      const int g = b.uidx[u0 + k];
      b.xh0[g] = b.xc[g];
      b.xh1[g] = 0.0;
      b.qh0[g] = b.q[g];
      b.qh1[g] = -cs.h_last * b.f[g];
    }
    // the initial point is the first recorded one
    for (int j = tid; j < b.n_out; j += nt)
      b.rec_v[(size_t)c * b.max_points * b.n_out + j] = b.xc[b.out_idx[c * b.n_out + j]];
    if (tid == 0) {
      b.rec_t[(size_t)c * b.max_points] = 0.0;
      cs.n_rec = 1;
    }
    __syncthreads();
  }
  if (act & A_ACCEPT) {
    const int order = cs.hist_order;
    for (int k = tid; k < n; k += nt) {
      const int g = b.uidx[u0 + k];
      if (order == 2) {
        b.xh2[g] = b.xh1[g];
        b.qh2[g] = b.f[g];
      }
      b.xh1[g] = b.x[g] - b.xh0[g];
      b.qh1[g] = b.q[g] - b.qh0[g];
      b.xh0[g] = b.x[g];
      b.qh0[g] = b.q[g];
      b.xl[g] = b.xc[g];
      b.xc[g] = b.x[g];
    }
    // state / store of the accepted point become current (the load kernels
    // read current and next, never last; they are ranges of slots)
    for (int k = b.sptr[c]; k < b.sptr[c + 1]; ++k)
      for (int s = b.sidx[2 * k] + tid; s < b.sidx[2 * k] + b.sidx[2 * k + 1]; s += nt)
        b.stac[s] = b.sta[s];
    for (int k = b.optr[c]; k < b.optr[c + 1]; ++k)
      for (int s = b.oidx[2 * k] + tid; s < b.oidx[2 * k] + b.oidx[2 * k + 1]; s += nt)
        b.stoc[s] = b.sto[s];
    __syncthreads();
    const int np = cs.n_rec;
    if (np < b.max_points) {
      for (int j = tid; j < b.n_out; j += nt)
        b.rec_v[((size_t)c * b.max_points + np) * b.n_out + j] = b.xc[b.out_idx[c * b.n_out + j]];
      if (tid == 0) {
        b.rec_t[(size_t)c * b.max_points + np] = cs.t;
        cs.n_rec = np + 1;
      }
    }
  }
  __syncthreads();
  if (act & A_RESTART) {
    // the accepted point at a breakpoint starts a new first-order history
    for (int k = tid; k < n; k += nt) {
      const int g = b.uidx[u0 + k];
      b.xh0[g] = b.xc[g];
      b.xh1[g] = 0.0;
      b.qh0[g] = b.q[g];
      b.qh1[g] = -cs.h_last * b.f[g];
    }
    __syncthreads();
  }
  if ((act & A_PREDICT) && cs.phase != PH_DONE) {
    const double b1 = cs.beta[1], b2 = cs.beta[2];
    const int order = cs.order;
    for (int k = tid; k < n; k += nt) {
      const int g = b.uidx[u0 + k];
      double v = b.xh0[g];
      v = b1 * b.xh1[g] + v;
      if (order == 2) v = b2 * b.xh2[g] + v;
      b.xn0[g] = v;
      b.x[g] = v;
      b.w[g] = 1e-2 * fmax(fabs(b.xc[g]), fabs(v)) + 1e-6;
    }
    // the limiters read the previous iterate from next store: start from the
    // current one (every state slot is rewritten by the next load)
    for (int k = b.optr[c]; k < b.optr[c + 1]; ++k)
      for (int s = b.oidx[2 * k] + tid; s < b.oidx[2 * k] + b.oidx[2 * k + 1]; s += nt)
        b.sto[s] = b.stoc[s];
  }
}

template <class V>
int to_dev(V **d, const std::vector<V> &h) {
  if (cudaMalloc((void **)d, sizeof(V) * std::max<size_t>(h.size(), 1)) != cudaSuccess) return XG_ERR_OOM;
  if (!h.empty() && cudaMemcpy(*d, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return XG_ERR_CUDA;
  return XG_OK;
}

}  // namespace
}  // namespace xg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

struct xg_batch {
  xg_ctx *ctx = nullptr;
  xg_circuit *ckt = nullptr;
  cudaStream_t stream = nullptr;
  int nc = 0, n_out = 0, max_points = 0, precision = XG_LU_FP64;
  xg::BatchDev dev{};
  std::vector<void *> allocs;
  std::vector<int> n_unk;              // unknowns per request
  int *d_cid[XG_NUM_DEV_TYPES] = {};   // instance -> request, per type
  cudaGraphExec_t graph = nullptr;
  int graph_iters = 0;
  int graph_launches_per_iter = 0;
  size_t solve_smem = 0;               // > 0: batch_solve_smem with this much shared memory
  int n_walk = 0;                      // requests walked row by row (not on the level path)
  size_t solve_lvl = 0;                // > 0: batch_solve_lvl (for its requests) with this much
  int64_t bytes = 0;
  // pinned host mirror of the request states
  xg::CState *h_cs = nullptr;
};

namespace {

// The union of the requests' netlists: nodes and models offset, instances
// concatenated per device type (each request's instances stay in order).
struct UnionNetlist {
  xg_netlist nl{};
  std::vector<xg_model_desc> models;
  std::vector<std::vector<int>> ints;
  std::vector<std::vector<double>> dbls;
  std::vector<int> type_order;
  int *iv(size_t n) { ints.emplace_back(n); return ints.back().data(); }
  double *dv(size_t n) { dbls.emplace_back(n); return dbls.back().data(); }
};

int build_union(int n, const xg_netlist *const *nls, UnionNetlist *U,
                std::vector<std::array<int, XG_NUM_DEV_TYPES>> *inst0, std::vector<int> *node0) {
  for (int r = 1; r < n; ++r) {
    const xg_netlist &a = *nls[0], &bb = *nls[r];
    bool same = a.n_type_order == bb.n_type_order;
    for (int k = 0; same && k < a.n_type_order; ++k) same = a.type_order[k] == bb.type_order[k];
    if (!same) {
      xg::set_error("xg_batch_create: requests differ in device-type load order");
      return XG_ERR_ARG;
    }
  }
  xg_netlist &u = U->nl;
  std::memset(&u, 0, sizeof(u));
  int nodes = 0, models = 0;
  inst0->assign(n + 1, {});
  node0->assign(n + 1, 0);
  std::vector<int> model0(n + 1, 0);
  for (int r = 0; r < n; ++r) {
    (*node0)[r] = nodes;
    model0[r] = models;
    nodes += nls[r]->n_nodes;
    models += nls[r]->n_models;
    for (int m = 0; m < nls[r]->n_models; ++m) U->models.push_back(nls[r]->models[m]);
  }
  (*node0)[n] = nodes;
  u.n_nodes = nodes;
  u.n_models = models;
  u.models = U->models.data();
  if (nls[0]->type_order && nls[0]->n_type_order) {
    U->type_order.assign(nls[0]->type_order, nls[0]->type_order + nls[0]->n_type_order);
    u.n_type_order = nls[0]->n_type_order;
    u.type_order = U->type_order.data();
  }
  auto node = [&](int r, int v) { return v < 0 ? -1 : v + (*node0)[r]; };
  auto count = [&](int t, const xg_netlist &a) {
    switch (t) {
      case XG_DEV_RES: return a.res.n; case XG_DEV_CAP: return a.cap.n;
      case XG_DEV_VSRC: return a.vsrc.n; case XG_DEV_ISRC: return a.isrc.n;
      case XG_DEV_DIODE: return a.diode.n; case XG_DEV_MOS1: return a.mos1.n;
      default: return a.bsim3.n;
    }
  };
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t) {
    int tot = 0;
    for (int r = 0; r < n; ++r) {
      (*inst0)[r][t] = tot;
      tot += count(t, *nls[r]);
    }
    (*inst0)[n][t] = tot;
  }
  // two-terminal R, C
  for (int which = 0; which < 2; ++which) {
    const int t = which == 0 ? XG_DEV_RES : XG_DEV_CAP;
    const int tot = (*inst0)[n][t];
    if (!tot) continue;
    int *p = U->iv(tot), *m = U->iv(tot);
    double *val = U->dv(tot);
    for (int r = 0; r < n; ++r) {
      const xg_twoterm_desc &d = which == 0 ? nls[r]->res : nls[r]->cap;
      for (int i = 0; i < d.n; ++i) {
        const int k = (*inst0)[r][t] + i;
        p[k] = node(r, d.p[i]);
        m[k] = node(r, d.m[i]);
        val[k] = d.value[i];
      }
    }
    xg_twoterm_desc &o = which == 0 ? u.res : u.cap;
    o.n = tot; o.p = p; o.m = m; o.value = val;
  }
  // sources
  for (int which = 0; which < 2; ++which) {
    const int t = which == 0 ? XG_DEV_VSRC : XG_DEV_ISRC;
    const int tot = (*inst0)[n][t];
    if (!tot) continue;
    int *p = U->iv(tot), *m = U->iv(tot), *kind = U->iv(tot);
    double *wave = U->dv((size_t)tot * 7);
    for (int r = 0; r < n; ++r) {
      const xg_src_desc &d = which == 0 ? nls[r]->vsrc : nls[r]->isrc;
      for (int i = 0; i < d.n; ++i) {
        const int k = (*inst0)[r][t] + i;
        p[k] = node(r, d.p[i]);
        m[k] = node(r, d.m[i]);
        kind[k] = d.kind ? d.kind[i] : XG_SRC_DC;
        for (int j = 0; j < 7; ++j) wave[(size_t)k * 7 + j] = d.wave[(size_t)i * 7 + j];
      }
    }
    xg_src_desc &o = which == 0 ? u.vsrc : u.isrc;
    o.n = tot; o.p = p; o.m = m; o.kind = kind; o.wave = wave;
  }
  // diodes
  if (int tot = (*inst0)[n][XG_DEV_DIODE]) {
    int *a = U->iv(tot), *cc = U->iv(tot), *mod = U->iv(tot);
    double *area = U->dv(tot);
    for (int r = 0; r < n; ++r) {
      const xg_diode_desc &d = nls[r]->diode;
      for (int i = 0; i < d.n; ++i) {
        const int k = (*inst0)[r][XG_DEV_DIODE] + i;
        a[k] = node(r, d.a[i]);
        cc[k] = node(r, d.c[i]);
        mod[k] = d.model[i] + model0[r];
        area[k] = d.area ? d.area[i] : 1.0;
      }
    }
    u.diode.n = tot; u.diode.a = a; u.diode.c = cc; u.diode.model = mod; u.diode.area = area;
  }
  // MOSFETs: optional per-instance arrays stay NULL (the model default) only
  // when no request gives them
  for (int which = 0; which < 2; ++which) {
    const int t = which == 0 ? XG_DEV_MOS1 : XG_DEV_BSIM3;
    const int tot = (*inst0)[n][t];
    if (!tot) continue;
    int *dd = U->iv(tot), *g = U->iv(tot), *s = U->iv(tot), *bb = U->iv(tot), *mod = U->iv(tot);
    double *geo[9];
    for (int j = 0; j < 9; ++j) {
      int given = 0, reqs = 0;
      for (int r = 0; r < n; ++r) {
        const xg_mos_desc &d = which == 0 ? nls[r]->mos1 : nls[r]->bsim3;
        if (!d.n) continue;
        const double *src[9] = {d.w, d.l, d.ad, d.as, d.pd, d.ps, d.nrd, d.nrs, d.m};
        ++reqs;
        given += src[j] != nullptr;
      }
      if (given && given != reqs) {
        xg::set_error("xg_batch_create: requests differ in which MOSFET geometry arrays they give");
        return XG_ERR_ARG;
      }
      geo[j] = given ? U->dv(tot) : nullptr;
    }
    for (int r = 0; r < n; ++r) {
      const xg_mos_desc &d = which == 0 ? nls[r]->mos1 : nls[r]->bsim3;
      const double *src[9] = {d.w, d.l, d.ad, d.as, d.pd, d.ps, d.nrd, d.nrs, d.m};
      for (int i = 0; i < d.n; ++i) {
        const int k = (*inst0)[r][t] + i;
        dd[k] = node(r, d.d[i]);
        g[k] = node(r, d.g[i]);
        s[k] = node(r, d.s[i]);
        bb[k] = node(r, d.b[i]);
        mod[k] = d.model[i] + model0[r];
        for (int j = 0; j < 9; ++j)
          if (geo[j]) geo[j][k] = src[j][i];
      }
    }
    xg_mos_desc &o = which == 0 ? u.mos1 : u.bsim3;
    o.n = tot; o.d = dd; o.g = g; o.s = s; o.b = bb; o.model = mod;
    o.w = geo[0]; o.l = geo[1]; o.ad = geo[2]; o.as = geo[3]; o.pd = geo[4]; o.ps = geo[5];
    o.nrd = geo[6]; o.nrs = geo[7]; o.m = geo[8];
  }
  return XG_OK;
}

}  // namespace

namespace {

void free_batch(xg_batch *b) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (void *p : b->allocs) cudaFree(p);
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t)
    if (b->d_cid[t]) cudaFree(b->d_cid[t]);
  if (b->h_cs) cudaFreeHost(b->h_cs);
  if (b->ckt) xg_circuit_destroy(b->ckt);
  if (b->stream) cudaStreamDestroy(b->stream);
}

template <class V>
int dev_copy(xg_batch *b, V **d, const std::vector<V> &h) {
  int rc = xg::to_dev(d, h);
  if (*d) b->allocs.push_back((void *)*d);
  b->bytes += int64_t(sizeof(V) * h.size());
  return rc;
}

int dev_zero(xg_batch *b, double **d, size_t n) {
  if (cudaMalloc((void **)d, sizeof(double) * std::max<size_t>(n, 1)) != cudaSuccess) return XG_ERR_OOM;
  b->allocs.push_back(*d);
  b->bytes += int64_t(sizeof(double) * n);
  return cudaMemset(*d, 0, sizeof(double) * std::max<size_t>(n, 1)) == cudaSuccess ? XG_OK : XG_ERR_CUDA;
}

// One batch iteration: solve, load, combine, control, vector.
int enqueue_iteration(xg_batch *b) {
  using namespace xg;
  CircuitView v;
  circuit_view(b->ckt, &v);
  const Plan &P = *v.plan;
  cudaStream_t s = b->stream;
  const int blocks4 = (b->nc + 3) / 4;
  if (!b->n_walk) {
    // every request is on the level path
  } else if (b->solve_smem) {
    if (b->precision == XG_LU_FP32) batch_solve_smem<float><<<b->nc, 32, b->solve_smem, s>>>(b->dev);
    else batch_solve_smem<double><<<b->nc, 32, b->solve_smem, s>>>(b->dev);
    count_launches(1);
  } else {
    if (b->precision == XG_LU_FP32) batch_solve<float><<<blocks4, 128, 0, s>>>(b->dev);
    else batch_solve<double><<<blocks4, 128, 0, s>>>(b->dev);
    count_launches(1);
  }
  if (b->solve_lvl) {
    if (b->precision == XG_LU_FP32)
      batch_solve_lvl<float><<<b->nc, kLvlThreads, b->solve_lvl, s>>>(b->dev);
    else
      batch_solve_lvl<double><<<b->nc, kLvlThreads, b->solve_lvl, s>>>(b->dev);
    count_launches(1);
  }
  Flags unused{};
  for (int k = 0; k < P.n_order; ++k) {
    const int t = P.order[k];
    const TypeData &T = P.T[t];
    if (!T.n) continue;
    DevType dt{T.n, T.nterm, T.sta0, T.sto0, T.term0, T.d_params, T.d_lid, b->d_cid[t], b->dev.flags};
    int rc = v.fma ? fast::launch_eval(t, dt, v.opt, unused, v.io, s)
                   : exact::launch_eval(t, dt, v.opt, unused, v.io, s);
    if (rc) return rc;
  }
  double *out = nullptr;
  xg_vec_device_ptr(b->ckt, XG_VEC_F, &out);
  const ReduceArgs ra = reduce_args(P, v.io.terms, v.red_ptr, v.red_idx, v.long_out, v.short_order, out, 0, P.n_out);
  int rc = v.fma ? fast::launch_reduce(ra, s) : exact::launch_reduce(ra, s);
  if (rc) return rc;
  batch_combine<<<b->nc, kBatchThreads, 0, s>>>(b->dev);
  // one warp per 32 requests: the step control is FP64-heavy (pow, sqrt,
  // divisions), and spread over as many SMs as there are warps
  batch_control<<<(b->nc + 31) / 32, 32, 0, s>>>(b->dev);
  batch_vector<<<b->nc, kVectorThreads, 0, s>>>(b->dev);
  count_launches(3);
  return cudaGetLastError() == cudaSuccess ? XG_OK : XG_ERR_CUDA;
}

}  // namespace

extern "C" int xg_batch_create(xg_ctx *ctx, int n, const xg_netlist *const *nls,
                               const double *const *x0, const double *tstop, const int *const *out_idx,
                               const xg_batch_options *o, xg_batch **out) {
  using namespace xg;
  if (!ctx || n <= 0 || !nls || !tstop || !o || !out || o->max_points <= 0 || o->n_out < 0 ||
      (o->n_out && !out_idx) || (o->lu_precision != XG_LU_FP64 && o->lu_precision != XG_LU_FP32) ||
      o->n_refine < 0) {
    set_error("xg_batch_create: bad argument");
    return XG_ERR_ARG;
  }
  *out = nullptr;
  std::unique_ptr<xg_batch, void (*)(xg_batch *)> b(new xg_batch, [](xg_batch *p) {
    free_batch(p);
    delete p;
  });
  b->ctx = ctx;
  b->nc = n;
  b->n_out = o->n_out;
  b->max_points = o->max_points;
  b->precision = o->lu_precision;
  UnionNetlist U;
  std::vector<std::array<int, XG_NUM_DEV_TYPES>> inst0;
  std::vector<int> node0;
  int rc = build_union(n, nls, &U, &inst0, &node0);
  if (rc) return rc;
  if ((rc = xg_circuit_create(ctx, &U.nl, &b->ckt))) return rc;
  CircuitView v;
  circuit_view(b->ckt, &v);
  const Plan &P = *v.plan;
  const int NU = P.n_unknowns;
  int device = 0;
  void *ctx_stream = nullptr;
  ctx_info(ctx, &device, &ctx_stream);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    set_error("xg_batch_create: cudaStreamCreate failed");
    return XG_ERR_CUDA;
  }
  // requests of instances, unknowns, state and store slots
  std::vector<std::vector<int>> l2u(n), sl(n), ol(n);
  std::vector<int> owner(NU, -1);
  for (int r = 0; r < n; ++r)
    for (int k = node0[r]; k < node0[r + 1]; ++k) {
      l2u[r].push_back(k);
      owner[k] = r;
    }
  for (int k = 0; k < P.n_order; ++k) {
    const int t = P.order[k];
    const TypeData &T = P.T[t];
    if (!T.n) continue;
    std::vector<int> cid(T.n);
    for (int r = 0; r < n; ++r) {
      const int i0 = inst0[r][t], i1 = inst0[r + 1][t];
      for (int i = i0; i < i1; ++i) {
        cid[i] = r;
        for (int j = 0; j < T.nlid; ++j) {
          const int g = T.lid[(size_t)j * T.n + i];
          if (g < NU && owner[g] < 0) {
            owner[g] = r;
            l2u[r].push_back(g);
          }
        }
      }
      if (t != XG_DEV_DIODE)
        for (int s = T.sta0 + i0 * T.nsta; s < T.sta0 + i1 * T.nsta; ++s) sl[r].push_back(s);
      for (int s = T.sto0 + i0 * T.nsto; s < T.sto0 + i1 * T.nsto; ++s) ol[r].push_back(s);
    }
    if (to_dev(&b->d_cid[t], cid)) {
      set_error("xg_batch_create: out of device memory");
      return XG_ERR_OOM;
    }
  }
  for (int g = 0; g < NU; ++g)
    if (owner[g] < 0) {
      set_error("xg_batch_create: an unknown belongs to no request");
      return XG_ERR_ARG;
    }
  std::vector<int> uptr(n + 1, 0), uidx, sptr(n + 1, 0), sidx, optr(n + 1, 0), oidx, jptr(n + 1, 0),
      jidx;
  // slot lists -> runs of consecutive slots (start, length)
  auto runs = [](const std::vector<int> &v, std::vector<int> *out) {
    int cnt = 0;
    for (size_t k = 0; k < v.size();) {
      size_t e = k + 1;
      while (e < v.size() && v[e] == v[e - 1] + 1) ++e;
      out->push_back(v[k]);
      out->push_back(int(e - k));
      ++cnt;
      k = e;
    }
    return cnt;
  };
  for (int r = 0; r < n; ++r) {
    uptr[r + 1] = uptr[r] + int(l2u[r].size());
    uidx.insert(uidx.end(), l2u[r].begin(), l2u[r].end());
    sptr[r + 1] = sptr[r] + runs(sl[r], &sidx);
    optr[r + 1] = optr[r] + runs(ol[r], &oidx);
    b->n_unk.push_back(int(l2u[r].size()));
    // Jacobian entries of the request's rows: consecutive rows merge
    std::vector<int> rows(l2u[r]);
    std::sort(rows.begin(), rows.end());
    int nj = 0;
    for (size_t k = 0; k < rows.size();) {
      size_t e = k + 1;
      while (e < rows.size() && rows[e] == rows[e - 1] + 1) ++e;
      const int p0 = P.rowptr[rows[k]], p1 = P.rowptr[rows[e - 1] + 1];
      if (p1 > p0) {
        jidx.push_back(p0);
        jidx.push_back(p1 - p0);
        ++nj;
      }
      k = e;
    }
    jptr[r + 1] = jptr[r] + nj;
  }
  // starting point and a first Jacobian (dF/dx + dQ/dx / tstep) for the
  // per-request pivot analysis
  std::vector<double> xu(NU + 1, 0.0);
  for (int r = 0; r < n; ++r)
    if (x0 && x0[r])
      for (int k = 0; k < int(l2u[r].size()); ++k) xu[l2u[r][k]] = x0[r][k];
  for (int id : {XG_VEC_SOL_NEXT, XG_VEC_SOL_CURR, XG_VEC_SOL_LAST})
    if ((rc = xg_vec_upload(b->ckt, id, xu.data()))) return rc;
  const double tstep = o->tstep > 0 ? o->tstep : 1e-12;
  xg_load_flags fl{};
  fl.transient = 1;
  fl.pdt = 1.0 / tstep;
  if ((rc = xg_load(b->ckt, &fl))) return rc;
  std::vector<double> dfdx(P.nnz), dqdx(P.nnz);
  if ((rc = xg_vec_download(b->ckt, XG_VEC_DFDX, dfdx.data())) ||
      (rc = xg_vec_download(b->ckt, XG_VEC_DQDX, dqdx.data())))
    return rc;
  if ((rc = circuit_reset_members(b->ckt))) return rc;
  std::vector<int> lrp_off(n + 1, 0), lrp, lci, ldiag, lP, lQ, sched, lvl_req(n, 0);
  std::vector<int64_t> lnz_off(n + 1, 0), lu2a, sched_off(n + 1, 0);
  // Each request's analysis is independent: analyse them on the host's cores,
  // then concatenate in request order.
  struct ReqLU {
    LuSymbolic S;
    std::vector<int64_t> gpos;
    std::vector<int> blob;
    int rc = XG_OK;
    std::string err;
  };
  std::vector<ReqLU> req(n);
  auto analyse = [&](int r, std::vector<int> &g2l) {
    ReqLU &R = req[r];
    const int nr_ = int(l2u[r].size());
    for (int k = 0; k < nr_; ++k) g2l[l2u[r][k]] = k;
    std::vector<int> rp(nr_ + 1, 0), ci;
    std::vector<double> val;
    for (int k = 0; k < nr_; ++k) {
      const int g = l2u[r][k];
      std::vector<std::pair<int, int64_t>> row;
      for (int p = P.rowptr[g]; p < P.rowptr[g + 1]; ++p) row.push_back({g2l[P.colidx[p]], p});
      std::sort(row.begin(), row.end());
      for (auto &e : row) {
        ci.push_back(e.first);
        R.gpos.push_back(e.second);
        double a = dfdx[e.second] + dqdx[e.second] / tstep;
        if (e.first == k && a == 0.0) a = 1e-12;
        val.push_back(a);
      }
      rp[k + 1] = int(ci.size());
    }
    LuSymbolic &S = R.S;
    // the level schedule runs each request's levels on the lanes of a warp,
    // so the column order is chosen for depth as for a single circuit
    if (lu_analyze(nr_, rp.data(), ci.data(), val.data(), 1e-3, &S, &R.err, -1)) {
      R.rc = XG_ERR_SINGULAR;
      R.err = "xg_batch_create: request " + std::to_string(r) + ": " + R.err;
      return;
    }
    if (!lu_build_updates(S)) {
      R.rc = XG_ERR_ARG;
      R.err = "xg_batch_create: internal error, an update falls outside the L\\U pattern";
      return;
    }
    const int hdr[H_N] = {int(S.lptr.size()) - 1, int(S.uptr.size()) - 1, S.tail0,
                          int(S.tail_rowg.size()) - 1, int(S.tail_gptr.size()) - 1,
                          int(S.tail_pos.size()), int(S.tail_pm.size()), int(S.upos.size())};
    R.blob.assign(hdr, hdr + H_N);
    for (int64_t v : S.urp) R.blob.push_back(int(v));
    for (const std::vector<int> *a : {&S.upos, &S.lrow, &S.lptr, &S.urow, &S.uptr, &S.tail_rowg,
                                      &S.tail_gptr, &S.tail_pos, &S.tail_pp, &S.tail_pm, &S.tail_q})
      R.blob.insert(R.blob.end(), a->begin(), a->end());
    if (int64_t(R.blob.size()) != lvl_blob_len(nr_, hdr)) {
      R.rc = XG_ERR_ARG;
      R.err = "xg_batch_create: internal error in the level schedule";
    }
    std::vector<int64_t>().swap(S.urp);
    std::vector<int>().swap(S.upos);
  };
  {
    const int nthreads = std::max(1, std::min<int>(std::min(16, n), int(std::thread::hardware_concurrency())));
    std::atomic<int> next{0};
    auto worker = [&]() {
      std::vector<int> g2l(NU, -1);
      for (int r = next++; r < n; r = next++) analyse(r, g2l);
    };
    std::vector<std::thread> pool;
    for (int t = 1; t < nthreads; ++t) pool.emplace_back(worker);
    worker();
    for (auto &t : pool) t.join();
  }
  for (int r = 0; r < n; ++r) {
    const ReqLU &R = req[r];
    if (R.rc) {
      set_error(R.err);
      return R.rc;
    }
    const LuSymbolic &S = R.S;
    const int nr_ = int(l2u[r].size());
    sched.insert(sched.end(), R.blob.begin(), R.blob.end());
    sched_off[r + 1] = int64_t(sched.size());
    lrp_off[r + 1] = lrp_off[r] + nr_ + 1;
    lnz_off[r + 1] = lnz_off[r] + S.rp[nr_];
    lrp.insert(lrp.end(), S.rp.begin(), S.rp.end());
    lci.insert(lci.end(), S.ci.begin(), S.ci.end());
    ldiag.insert(ldiag.end(), S.diag.begin(), S.diag.end());
    for (int a : S.lu2a) lu2a.push_back(a >= 0 ? R.gpos[a] : -1);
    lP.insert(lP.end(), S.P.begin(), S.P.end());
    lQ.insert(lQ.end(), S.Q.begin(), S.Q.end());
  }
  std::vector<ReqLU>().swap(req);
  std::vector<int> outs((size_t)n * std::max(1, o->n_out), 0);
  for (int r = 0; r < n; ++r)
    for (int j = 0; j < o->n_out; ++j) {
      const int k = out_idx[r][j];
      if (k < 0 || k >= int(l2u[r].size())) {
        set_error("xg_batch_create: output index out of range");
        return XG_ERR_ARG;
      }
      outs[(size_t)r * o->n_out + j] = l2u[r][k];
    }
  // breakpoints per request, from its own PULSE sources and tstop
  std::vector<int> bp_ptr(n + 1, 0);
  std::vector<double> bpv;
  for (int r = 0; r < n; ++r) {
    const int lo[2] = {inst0[r][XG_DEV_VSRC], inst0[r][XG_DEV_ISRC]};
    const int hi[2] = {inst0[r + 1][XG_DEV_VSRC], inst0[r + 1][XG_DEV_ISRC]};
    const std::vector<double> bp = pulse_breakpoints(P, tstop[r], lo, hi);
    bpv.insert(bpv.end(), bp.begin(), bp.end());
    bp_ptr[r + 1] = (int)bpv.size();
  }
  BatchDev &d = b->dev;
  {
    int *t_bp_ptr;
    double *t_bp;
    if (dev_copy(b.get(), &t_bp_ptr, bp_ptr) || dev_copy(b.get(), &t_bp, bpv)) {
      set_error("xg_batch_create: out of device memory");
      return XG_ERR_OOM;
    }
    d.bp_ptr = t_bp_ptr;
    d.bp = t_bp;
  }
  d.nc = n;
  d.n_out = o->n_out;
  d.max_points = o->max_points;
  d.n_refine = o->lu_precision == XG_LU_FP32 ? o->n_refine : 0;
  int *t_uptr, *t_uidx, *t_sptr, *t_sidx, *t_optr, *t_oidx, *t_lrp_off, *t_lrp, *t_lci, *t_ldiag,
      *t_lP, *t_lQ, *t_out, *t_arp, *t_aci, *t_jptr, *t_jidx;
  int64_t *t_lnz_off, *t_lu2a, *t_sched_off;
  int *t_sched, *t_lvl;
  if (dev_copy(b.get(), &t_uptr, uptr) || dev_copy(b.get(), &t_uidx, uidx) ||
      dev_copy(b.get(), &t_sptr, sptr) || dev_copy(b.get(), &t_sidx, sidx) ||
      dev_copy(b.get(), &t_optr, optr) || dev_copy(b.get(), &t_oidx, oidx) ||
      dev_copy(b.get(), &t_jptr, jptr) || dev_copy(b.get(), &t_jidx, jidx) ||
      dev_copy(b.get(), &t_lrp_off, lrp_off) || dev_copy(b.get(), &t_lnz_off, lnz_off) ||
      dev_copy(b.get(), &t_lrp, lrp) || dev_copy(b.get(), &t_lci, lci) ||
      dev_copy(b.get(), &t_ldiag, ldiag) || dev_copy(b.get(), &t_lu2a, lu2a) ||
      dev_copy(b.get(), &t_lP, lP) || dev_copy(b.get(), &t_lQ, lQ) ||
      dev_copy(b.get(), &t_out, outs) || dev_copy(b.get(), &t_arp, P.rowptr) ||
      dev_copy(b.get(), &t_aci, P.colidx)) {
    set_error("xg_batch_create: out of device memory");
    return XG_ERR_OOM;
  }
  d.uptr = t_uptr; d.uidx = t_uidx; d.sptr = t_sptr; d.sidx = t_sidx; d.optr = t_optr; d.oidx = t_oidx;
  d.jptr = t_jptr; d.jidx = t_jidx;
  d.arp = t_arp; d.aci = t_aci; d.lrp_off = t_lrp_off; d.lnz_off = t_lnz_off; d.lrp = t_lrp;
  d.lci = t_lci; d.ldiag = t_ldiag; d.lu2a = t_lu2a; d.lP = t_lP; d.lQ = t_lQ; d.out_idx = t_out;
  const size_t tsz = o->lu_precision == XG_LU_FP32 ? sizeof(float) : sizeof(double);
  {
    // requests whose level schedule fits in shared memory use it
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    size_t need_lvl = 0;
    if (!std::getenv("XG_BATCH_NO_LVL"))
      for (int r = 0; r < n; ++r) {
        const size_t sb = smem_bytes_lvl(uptr[r + 1] - uptr[r], lnz_off[r + 1] - lnz_off[r],
                                         sched_off[r + 1] - sched_off[r], tsz);
        if (sb + 1024 <= size_t(optin)) {
          lvl_req[r] = 1;
          need_lvl = std::max(need_lvl, sb);
        }
      }
    if (need_lvl) {
      cudaError_t e = o->lu_precision == XG_LU_FP32
                          ? cudaFuncSetAttribute(batch_solve_lvl<float>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(need_lvl))
                          : cudaFuncSetAttribute(batch_solve_lvl<double>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(need_lvl));
      if (e == cudaSuccess) {
        b->solve_lvl = need_lvl;
      } else {
        cudaGetLastError();
        std::fill(lvl_req.begin(), lvl_req.end(), 0);
      }
    }
    if (dev_copy(b.get(), &t_sched_off, sched_off) || dev_copy(b.get(), &t_sched, sched) ||
        dev_copy(b.get(), &t_lvl, lvl_req)) {
      set_error("xg_batch_create: out of device memory");
      return XG_ERR_OOM;
    }
    d.sched_off = t_sched_off;
    d.sched = t_sched;
    d.lvl = t_lvl;
    b->n_walk = n - int(std::count(lvl_req.begin(), lvl_req.end(), 1));
  }
  {
    size_t need = 0;
    for (int r = 0; r < n; ++r)
      if (!lvl_req[r])
        need = std::max(need, smem_bytes_request(uptr[r + 1] - uptr[r], lnz_off[r + 1] - lnz_off[r], tsz));
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    if (need + 1024 <= size_t(optin) && !std::getenv("XG_BATCH_NO_SMEM")) {
      cudaError_t e = o->lu_precision == XG_LU_FP32
                          ? cudaFuncSetAttribute(batch_solve_smem<float>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(need))
                          : cudaFuncSetAttribute(batch_solve_smem<double>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, int(need));
      if (e == cudaSuccess) b->solve_smem = need;
      else cudaGetLastError();
    }
  }
  {
    void *pv = nullptr, *pr = nullptr;
    int *pm = nullptr;
    if (cudaMalloc(&pv, tsz * std::max<int64_t>(lnz_off[n], 1)) != cudaSuccess ||
        cudaMalloc(&pr, tsz * std::max(NU, 1)) != cudaSuccess ||
        cudaMalloc((void **)&pm, sizeof(int) * std::max(NU, 1)) != cudaSuccess) {
      if (pv) cudaFree(pv);
      if (pr) cudaFree(pr);
      set_error("xg_batch_create: out of device memory");
      return XG_ERR_OOM;
    }
    b->allocs.push_back(pv);
    b->allocs.push_back(pr);
    b->allocs.push_back(pm);
    b->bytes += int64_t(tsz * (lnz_off[n] + NU) + sizeof(int) * NU);
    d.lval = pv;
    d.lrd = pr;
    d.map = pm;
  }
  double **vecs[] = {&d.y, &d.r, &d.dd, &d.jac, &d.rhs, &d.dx, &d.w, &d.xh0, &d.xh1, &d.xh2,
                     &d.qh0, &d.qh1, &d.qh2, &d.xn0};
  for (double **p : vecs) {
    const size_t len = p == &d.jac ? size_t(std::max<int64_t>(P.nnz, 1)) : size_t(NU + 1);
    if (dev_zero(b.get(), p, len)) {
      set_error("xg_batch_create: out of device memory");
      return XG_ERR_OOM;
    }
  }
  if (dev_zero(b.get(), &d.part, size_t(n) * Q_N) ||
      dev_zero(b.get(), &d.rec_t, size_t(n) * o->max_points) ||
      dev_zero(b.get(), &d.rec_v, size_t(n) * o->max_points * std::max(1, o->n_out))) {
    set_error("xg_batch_create: out of device memory");
    return XG_ERR_OOM;
  }
  xg_vec_device_ptr(b->ckt, XG_VEC_SOL_NEXT, &d.x);
  xg_vec_device_ptr(b->ckt, XG_VEC_SOL_CURR, &d.xc);
  xg_vec_device_ptr(b->ckt, XG_VEC_SOL_LAST, &d.xl);
  xg_vec_device_ptr(b->ckt, XG_VEC_STA_NEXT, &d.sta);
  xg_vec_device_ptr(b->ckt, XG_VEC_STA_CURR, &d.stac);
  xg_vec_device_ptr(b->ckt, XG_VEC_STA_LAST, &d.stal);
  xg_vec_device_ptr(b->ckt, XG_VEC_STO_NEXT, &d.sto);
  xg_vec_device_ptr(b->ckt, XG_VEC_STO_CURR, &d.stoc);
  xg_vec_device_ptr(b->ckt, XG_VEC_STO_LAST, &d.stol);
  double *pf, *pq, *pfv, *pqv, *pdf, *pdq;
  xg_vec_device_ptr(b->ckt, XG_VEC_F, &pf);
  xg_vec_device_ptr(b->ckt, XG_VEC_Q, &pq);
  xg_vec_device_ptr(b->ckt, XG_VEC_DFDXDVP, &pfv);
  xg_vec_device_ptr(b->ckt, XG_VEC_DQDXDVP, &pqv);
  xg_vec_device_ptr(b->ckt, XG_VEC_DFDX, &pdf);
  xg_vec_device_ptr(b->ckt, XG_VEC_DQDX, &pdq);
  d.f = pf; d.q = pq; d.fvp = pfv; d.qvp = pqv; d.dfdx = pdf; d.dqdx = pdq;
  // initial states: x0 everywhere, state and store zero, first load in DC mode
  for (int id : {XG_VEC_SOL_NEXT, XG_VEC_SOL_CURR, XG_VEC_SOL_LAST})
    if ((rc = xg_vec_upload(b->ckt, id, xu.data()))) return rc;
  {
    std::vector<double> z(std::max(P.n_state, P.n_store) + 1, 0.0);
    for (int id : {XG_VEC_STA_NEXT, XG_VEC_STA_CURR, XG_VEC_STA_LAST})
      if (P.n_state && (rc = xg_vec_upload(b->ckt, id, z.data()))) return rc;
    for (int id : {XG_VEC_STO_NEXT, XG_VEC_STO_CURR, XG_VEC_STO_LAST})
      if (P.n_store && (rc = xg_vec_upload(b->ckt, id, z.data()))) return rc;
  }
  std::vector<CState> cs(n);
  std::vector<Flags> fls(n);
  for (int r = 0; r < n; ++r) {
    CState &c = cs[r];
    std::memset(&c, 0, sizeof(c));
    c.tstop = tstop[r];
    c.tstep = tstep;
    c.max_step = o->maxstep > 0 ? o->maxstep : 0.1 * tstop[r];
    c.reltol = o->reltol > 0 ? o->reltol : 1e-3;
    c.abstol = o->abstol > 0 ? o->abstol : 1e-6;
    c.saved = 1e-10;
    c.phase = PH_INIT;
    c.first_step = 1;
    c.beginning = 1;
    c.order = 1;
    c.loads = 1;
    Flags f{};
    f.dcop = 1;
    f.tranop = 1;
    fls[r] = f;
  }
  CState *t_cs;
  Flags *t_fl;
  if (dev_copy(b.get(), &t_cs, cs) || dev_copy(b.get(), &t_fl, fls)) {
    set_error("xg_batch_create: out of device memory");
    return XG_ERR_OOM;
  }
  d.cs = t_cs;
  d.flags = t_fl;
  if (cudaMallocHost((void **)&b->h_cs, sizeof(CState) * n) != cudaSuccess) {
    set_error("xg_batch_create: out of pinned host memory");
    return XG_ERR_OOM;
  }
  std::memcpy(b->h_cs, cs.data(), sizeof(CState) * n);
  xg_circuit_info info;
  xg_circuit_get_info(b->ckt, &info);
  b->bytes += info.scratch_bytes;
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t)
    b->bytes += int64_t(P.T[t].params.size() * sizeof(double) + P.T[t].lid.size() * sizeof(int));
  b->bytes += int64_t(9 * (NU + 1) + P.n_out) * int64_t(sizeof(double));
  // the set-up loads ran on the context's stream; running batches keep going
  if (cudaStreamSynchronize((cudaStream_t)ctx_stream) != cudaSuccess) {
    set_error("xg_batch_create: set-up failed");
    return XG_ERR_CUDA;
  }
  *out = b.release();
  return XG_OK;
}

extern "C" int xg_batch_run(xg_batch *b, int iterations) {
  if (!b || iterations <= 0) {
    xg::set_error("xg_batch_run: bad argument");
    return XG_ERR_ARG;
  }
  // One capture or graph launch at a time across threads: a server sets up
  // and first runs a batch on a helper thread while its main thread keeps
  // launching the others, and the launch counter's capture bookkeeping below
  // assumes no other launch lands in between.
  static std::mutex run_mutex;
  std::lock_guard<std::mutex> lock(run_mutex);
  if (!b->graph || b->graph_iters != iterations) {
    if (b->graph) {
      cudaStreamSynchronize(b->stream);
      cudaGraphExecDestroy(b->graph);
      b->graph = nullptr;
    }
    cudaGraph_t g;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
      xg::set_error("xg_batch_run: stream capture failed");
      return XG_ERR_CUDA;
    }
    const long long before = xg_launch_count();
    int rc = XG_OK;
    for (int k = 0; k < iterations && !rc; ++k) rc = enqueue_iteration(b);
    // the captured launches run when the graph is launched, not here
    const long long captured = xg_launch_count() - before;
    b->graph_launches_per_iter = int(captured / iterations);
    xg::count_launches(-int(captured));
    cudaError_t e = cudaStreamEndCapture(b->stream, &g);
    if (rc || e != cudaSuccess) {
      xg::set_error("xg_batch_run: capture of the batch iteration failed");
      return XG_ERR_CUDA;
    }
    e = cudaGraphInstantiate(&b->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      xg::set_error(std::string("xg_batch_run: cudaGraphInstantiate: ") + cudaGetErrorString(e));
      return XG_ERR_CUDA;
    }
    b->graph_iters = iterations;
  }
  if (cudaGraphLaunch(b->graph, b->stream) != cudaSuccess) {
    xg::set_error("xg_batch_run: cudaGraphLaunch failed");
    return XG_ERR_CUDA;
  }
  xg::count_launches(iterations * b->graph_launches_per_iter);
  return XG_OK;
}

extern "C" int xg_batch_poll(xg_batch *b, int wait, int *n_done) {
  if (!b || !n_done) {
    xg::set_error("xg_batch_poll: bad argument");
    return XG_ERR_ARG;
  }
  if (!wait && cudaStreamQuery(b->stream) == cudaErrorNotReady) {
    *n_done = -1;  // still running
    return XG_OK;
  }
  if (cudaMemcpyAsync(b->h_cs, b->dev.cs, sizeof(xg::CState) * b->nc, cudaMemcpyDeviceToHost,
                      b->stream) != cudaSuccess ||
      cudaStreamSynchronize(b->stream) != cudaSuccess) {
    xg::set_error("xg_batch_poll: copy failed");
    return XG_ERR_CUDA;
  }
  int d = 0;
  for (int i = 0; i < b->nc; ++i) d += b->h_cs[i].phase == xg::PH_DONE;
  *n_done = d;
  return XG_OK;
}

extern "C" int xg_batch_results(xg_batch *b, int i, double *t, double *v, int *n_points,
                                xg_tran_stats *st) {
  if (!b || i < 0 || i >= b->nc || !n_points) {
    xg::set_error("xg_batch_results: bad argument");
    return XG_ERR_ARG;
  }
  const xg::CState &c = b->h_cs[i];
  const int np = std::min(c.n_rec, b->max_points);
  *n_points = np;
  if (np && t &&
      cudaMemcpy(t, b->dev.rec_t + (size_t)i * b->max_points, sizeof(double) * np,
                 cudaMemcpyDeviceToHost) != cudaSuccess)
    return XG_ERR_CUDA;
  if (np && v && b->n_out &&
      cudaMemcpy(v, b->dev.rec_v + (size_t)i * b->max_points * b->n_out,
                 sizeof(double) * np * b->n_out, cudaMemcpyDeviceToHost) != cudaSuccess)
    return XG_ERR_CUDA;
  if (st) {
    std::memset(st, 0, sizeof(*st));
    st->status = c.failed ? c.status : 0;
    st->steps = c.steps;
    st->steps_attempted = c.steps_attempted;
    st->rejected = c.rejected;
    st->newton_iters = c.newton_iters;
    st->factorizations = c.newton_iters;
    st->loads = c.loads;
    st->t_end = c.t;
  }
  return XG_OK;
}

extern "C" int xg_batch_info(const xg_batch *b, int *n_requests, int64_t *device_bytes) {
  if (!b) {
    xg::set_error("xg_batch_info: bad argument");
    return XG_ERR_ARG;
  }
  if (n_requests) *n_requests = b->nc;
  if (device_bytes) *device_bytes = b->bytes;
  return XG_OK;
}

extern "C" int xg_batch_destroy(xg_batch *b) {
  if (!b) return XG_OK;
  free_batch(b);
  delete b;
  return XG_OK;
}
