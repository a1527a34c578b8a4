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
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "xg.h"
#include "xg_internal.h"
#include "xg_lu.h"
#include "xg_smem.cuh"

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
  int gen;                       // slotted batches: which request of the slot this is
};

struct BatchDev {
  int nc;
  // Request c's ranges below run from xptr[c] to xend[c]: in a batch made
  // from a fixed set of requests xend = xptr + 1 (the ranges are packed); in
  // a slotted batch each slot owns a fixed region and xend marks how much of
  // it the request in the slot uses.
  const int *uend, *send, *oend, *jend, *bp_end;
  const int64_t *lnz_end, *sched_end;
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
  const int u0 = b.uptr[c], n = b.uend[c] - u0;
  const int *rp = b.lrp + b.lrp_off[c];
  const int64_t z0 = b.lnz_off[c];
  const int *ci = b.lci + z0;
  const int *diag = b.ldiag + u0;
  T *val = (T *)b.lval + z0;
  T *rd = (T *)b.lrd + u0;
  int *map = b.map + u0;
  const int *P = b.lP + u0, *Q = b.lQ + u0;
  const int64_t nz = b.lnz_end[c] - z0;
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
  const int u0 = b.uptr[c], n = b.uend[c] - u0;
  const int64_t z0 = b.lnz_off[c];
  const int nz = int(b.lnz_end[c] - z0);
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
  const int u0 = b.uptr[c], n = b.uend[c] - u0;
  const int64_t z0 = b.lnz_off[c];
  const int nz = int(b.lnz_end[c] - z0);
  const int64_t s0 = b.sched_off[c];
  const int blob = int(b.sched_end[c] - s0);
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
  const int u0 = b.uptr[c], n = b.uend[c] - u0;
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
  for (int k = b.jptr[c]; k < b.jend[c]; ++k) {
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
  const int e = b.bp_end[c];
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
  const int n = b.uend[c] - b.uptr[c];
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
      fl.skip = 1;
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
      fl.skip = 1;
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
  const int u0 = b.uptr[c], n = b.uend[c] - u0;
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
    for (int k = b.sptr[c]; k < b.send[c]; ++k)
      for (int s = b.sidx[2 * k] + tid; s < b.sidx[2 * k] + b.sidx[2 * k + 1]; s += nt)
        b.stac[s] = b.sta[s];
    for (int k = b.optr[c]; k < b.oend[c]; ++k)
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
    for (int k = b.optr[c]; k < b.oend[c]; ++k)
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

namespace xg {
struct SlotPool;
void free_pool(SlotPool *p);
int pool_gen(SlotPool *p, int slot);  // which request slot `slot` holds now
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
  // pinned host mirror of the request states (the last poll's snapshot)
  xg::CState *h_cs = nullptr;
  // every xg_batch_run ends with a copy of the request states into one of
  // these pinned buffers and an event, so a poll can read the snapshot of a
  // finished run while later runs are still on the device
  static constexpr int kRing = 4;
  xg::CState *h_ring[kRing] = {};
  cudaEvent_t ring_ev[kRing] = {};
  long long issued = 0, reported = 0;  // snapshots taken; the last one polled
  // slotted batches: the pool behind the slots (null for a fixed batch)
  xg::SlotPool *pool = nullptr;
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

// One request's pivot order and L\U pattern, from its first Jacobian: the
// level schedule runs each request's levels on the lanes of a warp, so the
// column order is chosen for depth as for a single circuit.  gpos (filled by
// the caller) is the batch Jacobian entry of each local entry.
struct ReqLU {
  xg::LuSymbolic S;
  std::vector<int64_t> gpos;
  std::vector<int> blob;  // the level schedule (lvl_blob_len layout)
  int rc = XG_OK;
  std::string err;
};

void analyse_request(int nr, const std::vector<int> &rp, const std::vector<int> &ci,
                     const std::vector<double> &val, const std::string &who, ReqLU *out) {
  using namespace xg;
  ReqLU &R = *out;
  LuSymbolic &S = R.S;
  if (lu_analyze(nr, rp.data(), ci.data(), val.data(), 1e-3, &S, &R.err, -1)) {
    R.rc = XG_ERR_SINGULAR;
    R.err = who + ": " + R.err;
    return;
  }
  if (!lu_build_updates(S)) {
    R.rc = XG_ERR_ARG;
    R.err = who + ": internal error, an update falls outside the L\\U pattern";
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
  if (int64_t(R.blob.size()) != lvl_blob_len(nr, hdr)) {
    R.rc = XG_ERR_ARG;
    R.err = who + ": internal error in the level schedule";
  }
  std::vector<int64_t>().swap(S.urp);
  std::vector<int>().swap(S.upos);
}

void free_batch(xg_batch *b) {
  if (b->stream) cudaStreamSynchronize(b->stream);
  if (b->pool) xg::free_pool(b->pool);
  b->pool = nullptr;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (void *p : b->allocs) cudaFree(p);
  for (int t = 0; t < XG_NUM_DEV_TYPES; ++t)
    if (b->d_cid[t]) cudaFree(b->d_cid[t]);
  if (b->h_cs) cudaFreeHost(b->h_cs);
  for (int k = 0; k < xg_batch::kRing; ++k) {
    if (b->h_ring[k]) cudaFreeHost(b->h_ring[k]);
    if (b->ring_ev[k]) cudaEventDestroy(b->ring_ev[k]);
  }
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

}  // namespace

namespace xg {
// One capture or graph launch at a time across threads (a server sets up and
// first runs a batch on a helper thread while its main thread keeps launching
// the others), and no launch onto a batch's stream while it is captured.
std::mutex &launch_mutex() {
  static std::mutex m;
  return m;
}
int enqueue_pool_iteration(xg_batch *b);
}  // namespace xg

namespace {

// One batch iteration: solve, load, combine, control, vector.
int enqueue_iteration(xg_batch *b) {
  using namespace xg;
  if (b->pool) return enqueue_pool_iteration(b);
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
  const ReduceArgs ra = reduce_args(P, v.io.terms, v.red, out, 0, P.n_out);
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
    analyse_request(nr_, rp, ci, val, "xg_batch_create: request " + std::to_string(r), &R);
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
    d.bp_end = t_bp_ptr + 1;
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
  d.uend = t_uptr + 1; d.send = t_sptr + 1; d.oend = t_optr + 1; d.jend = t_jptr + 1;
  d.lnz_end = t_lnz_off + 1;
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
      const void *fn = o->lu_precision == XG_LU_FP32 ? (const void *)batch_solve_lvl<float>
                                                     : (const void *)batch_solve_lvl<double>;
      const bool ok = allow_dynamic_smem(fn, need_lvl) == cudaSuccess;
      if (ok) b->solve_lvl = need_lvl;
      else std::fill(lvl_req.begin(), lvl_req.end(), 0);
    }
    if (dev_copy(b.get(), &t_sched_off, sched_off) || dev_copy(b.get(), &t_sched, sched) ||
        dev_copy(b.get(), &t_lvl, lvl_req)) {
      set_error("xg_batch_create: out of device memory");
      return XG_ERR_OOM;
    }
    d.sched_off = t_sched_off;
    d.sched_end = t_sched_off + 1;
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
      const void *fn = o->lu_precision == XG_LU_FP32 ? (const void *)batch_solve_smem<float>
                                                     : (const void *)batch_solve_smem<double>;
      if (allow_dynamic_smem(fn, need) == cudaSuccess) b->solve_smem = need;
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
  std::lock_guard<std::mutex> lock(xg::launch_mutex());
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
  if (!b->h_ring[0]) {
    for (int k = 0; k < xg_batch::kRing; ++k)
      if (cudaMallocHost((void **)&b->h_ring[k], sizeof(xg::CState) * b->nc) != cudaSuccess ||
          cudaEventCreateWithFlags(&b->ring_ev[k], cudaEventDisableTiming) != cudaSuccess) {
        xg::set_error("xg_batch_run: out of pinned host memory");
        return XG_ERR_OOM;
      }
  }
  if (cudaGraphLaunch(b->graph, b->stream) != cudaSuccess) {
    xg::set_error("xg_batch_run: cudaGraphLaunch failed");
    return XG_ERR_CUDA;
  }
  xg::count_launches(iterations * b->graph_launches_per_iter);
  const int k = int(b->issued % xg_batch::kRing);
  if (cudaMemcpyAsync(b->h_ring[k], b->dev.cs, sizeof(xg::CState) * b->nc, cudaMemcpyDeviceToHost,
                      b->stream) != cudaSuccess ||
      cudaEventRecord(b->ring_ev[k], b->stream) != cudaSuccess) {
    xg::set_error("xg_batch_run: snapshot failed");
    return XG_ERR_CUDA;
  }
  ++b->issued;
  return XG_OK;
}

// The newest finished snapshot not yet polled (0: none); snapshots finish in
// the order of their runs on the batch's stream.
static long long newest_snapshot(xg_batch *b) {
  long long newest = 0;
  for (long long j = std::max(b->reported + 1, b->issued - xg_batch::kRing + 1); j <= b->issued; ++j) {
    if (cudaEventQuery(b->ring_ev[(j - 1) % xg_batch::kRing]) != cudaSuccess) break;
    newest = j;
  }
  cudaGetLastError();  // a not-ready query is not an error
  return newest;
}

extern "C" int xg_batch_inflight(xg_batch *b, int *n) {
  if (!b || !n) {
    xg::set_error("xg_batch_inflight: bad argument");
    return XG_ERR_ARG;
  }
  long long done = b->reported;
  for (long long j = std::max(b->reported + 1, b->issued - xg_batch::kRing + 1); j <= b->issued; ++j) {
    if (cudaEventQuery(b->ring_ev[(j - 1) % xg_batch::kRing]) != cudaSuccess) break;
    done = j;
  }
  cudaGetLastError();
  *n = int(b->issued - done);
  return XG_OK;
}

extern "C" int xg_batch_poll(xg_batch *b, int wait, int *n_done) {
  if (!b || !n_done) {
    xg::set_error("xg_batch_poll: bad argument");
    return XG_ERR_ARG;
  }
  if (wait && cudaStreamSynchronize(b->stream) != cudaSuccess) {
    xg::set_error("xg_batch_poll: the batch failed");
    return XG_ERR_CUDA;
  }
  const long long j = newest_snapshot(b);
  if (j) {
    // the states as the newest finished run left them
    std::memcpy(b->h_cs, b->h_ring[(j - 1) % xg_batch::kRing], sizeof(xg::CState) * b->nc);
    b->reported = j;
  } else if (!wait) {
    *n_done = -1;  // no run has finished since the last poll
    return XG_OK;
  } else if (cudaMemcpyAsync(b->h_cs, b->dev.cs, sizeof(xg::CState) * b->nc, cudaMemcpyDeviceToHost,
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
  if (b->pool && c.gen != xg::pool_gen(b->pool, i)) {
    // the last poll predates the slot's request: nothing recorded yet
    *n_points = 0;
    if (st) std::memset(st, 0, sizeof(*st));
    return XG_OK;
  }
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

// ===========================================================================
// Slotted batches: continuous batching at request granularity
// ===========================================================================
//
// A slotted batch is a batch whose per-request arrays have a fixed region per
// slot instead of being packed.  Slot c owns unknowns [c*ucap, (c+1)*ucap),
// Jacobian entries [c*jcap, ...), the instances [c*icap_t, ...) of each device
// type in that type's parameter, LID, term, state and store arrays, and its
// own regions of the L\U, schedule, reduction, breakpoint and record arrays.
// The batch kernels above read request c's ranges through xptr[c]..xend[c],
// so a slot holds a request of any size up to its shape, and a slot that is
// free, or whose request has finished, is skipped by every kernel: its phase
// is done and its load flags say skip.
//
// The load of a slotted batch is its own: the evaluation kernels run over
// every type's whole instance array (an unused place has circuit -1), and
// pool_reduce sums each live slot's outputs from that request's own reduction
// lists (the same term order as a batch of its own; every sum is taken in
// order, so the result does not depend on the other slots).
//
// Submitting a request writes its data into a free slot with one copy-list
// kernel (seg_copy) on the batch's set-up stream, evaluates the slot's first
// Jacobian there with a load restricted to the slots being set up (their own
// circuit and flag arrays), analyses the pivot order on the host, writes the
// L\U arrays, and then, on the batch's own stream and so between two batch
// iterations, copies the request's starting state and flags into place.

namespace xg {

constexpr int kTypes = XG_NUM_DEV_TYPES;
constexpr int kB3Mem = 20;  // BSIM3 members carried between loads, per instance

// A copy list run on the device: 32-bit words copied from a staging payload,
// or filled with one word.
struct Seg {
  uint32_t *dst;
  int64_t src;   // word offset in the payload; < 0: fill
  int64_t n;     // words
  uint32_t fill;
  uint32_t pad;
};

__global__ void __launch_bounds__(256) seg_copy(const Seg *segs, int nseg, const uint32_t *payload) {
  const int lane = threadIdx.x & 31;
  const int nw = int((gridDim.x * blockDim.x) >> 5);
  for (int w = int((blockIdx.x * blockDim.x + threadIdx.x) >> 5); w < nseg; w += nw) {
    const Seg sg = segs[w];
    if (sg.src >= 0)
      for (int64_t k = lane; k < sg.n; k += 32) sg.dst[k] = payload[sg.src + k];
    else
      for (int64_t k = lane; k < sg.n; k += 32) sg.dst[k] = sg.fill;
  }
}

// One output of a slot: the sum, in order, of ref[beg .. beg+cnt) terms.
struct RedEntry {
  int64_t out;
  int64_t beg;
  int32_t cnt;
  int32_t pad;
};
static_assert(sizeof(RedEntry) == 24, "RedEntry is six words");

struct PoolRed {
  const RedEntry *ent;   // slot c's entries start at c * ecap
  int64_t ecap;
  const int *ne, *nl;    // entries of slot c, and how many of them (first) are long
  const uint32_t *ref;   // term of each reduction entry
  const double *terms;
  double *out;
};

constexpr int kLongOut = 64;  // outputs with more terms go to a block each
constexpr int kPoolRedThreads = 256;

// Blocks (c, y) of a slot c that is live (phase not done), or listed.  Long
// outputs (a supply rail's row) take a block each, y-strided: in the exact
// build the block fetches 256 terms at a time and one thread adds them in
// order; in the FMA build every thread adds a strided share, then a fixed
// butterfly per warp and the warps in order.  Short outputs take a thread
// each, summed ((0 + t0) + t1)....  The same sums in the same order as the
// fixed batch's reduction, so a request's outputs do not depend on which
// kind of batch, or which other requests, it runs with.
__global__ void __launch_bounds__(kPoolRedThreads) pool_reduce(PoolRed r, const CState *cs, const int *slots,
                                                               int split) {
  __shared__ double buf[kPoolRedThreads];
  __shared__ double part[kPoolRedThreads / 32];
  const int c = slots ? slots[blockIdx.x] : int(blockIdx.x);
  if (!slots && cs[c].phase == PH_DONE) return;
  const RedEntry *E = r.ent + int64_t(c) * r.ecap;
  const int ne = r.ne[c], nl = r.nl[c];
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int k = blockIdx.y; k < nl; k += gridDim.y) {
    const RedEntry e = E[k];
    if (split) {
      double s = 0.0;
#pragma unroll 4
      for (int j = tid; j < e.cnt; j += kPoolRedThreads) s += r.terms[r.ref[e.beg + j]];
#pragma unroll
      for (int m = 16; m > 0; m >>= 1) s += __shfl_xor_sync(0xffffffffu, s, m);
      if (lane == 0) part[wid] = s;
      __syncthreads();
      if (tid == 0) {
        double t = part[0];
        for (int q = 1; q < kPoolRedThreads / 32; ++q) t += part[q];
        r.out[e.out] = t;
      }
      __syncthreads();
    } else {
      double s = 0.0;
      for (int base = 0; base < e.cnt; base += kPoolRedThreads) {
        const int m = min(kPoolRedThreads, e.cnt - base);
        if (tid < m) buf[tid] = r.terms[r.ref[e.beg + base + tid]];
        __syncthreads();
        if (tid == 0)
          for (int j = 0; j < m; ++j) s += buf[j];
        __syncthreads();
      }
      if (tid == 0) r.out[e.out] = s;
    }
  }
  for (int k = nl + int(blockIdx.y) * kPoolRedThreads + tid; k < ne; k += int(gridDim.y) * kPoolRedThreads) {
    const RedEntry e = E[k];
    double s = 0.0;
    for (int j = 0; j < e.cnt; ++j) s += r.terms[r.ref[e.beg + j]];
    r.out[e.out] = s;
  }
}

// Activation, on the batch's stream between two iterations: the starting
// state and flags written by the set-up stream go into place.
constexpr int kActivateMax = 64;
struct SlotList {
  int n;
  int slot[kActivateMax];
};
__global__ void activate_slots(SlotList l, CState *cs, const CState *cs_next, Flags *fl,
                               const Flags *fl_next) {
  const int k = threadIdx.x;
  if (k >= l.n) return;
  const int c = l.slot[k];
  cs[c] = cs_next[c];
  fl[c] = fl_next[c];
}

// Capacities of one slot.
struct SlotCaps {
  int ucap = 0;           // unknown rows: the shape's + 1 (ground stays outside)
  int64_t jcap = 0, lucap = 0, blobcap = 0, rcap = 0, ecap = 0;
  int bpcap = 0;
  int icap[kTypes] = {};
};

SlotCaps slot_caps(const xg_slot_shape &sh) {
  SlotCaps k;
  k.ucap = sh.max_unknowns + 1;
  k.jcap = std::max<int64_t>(sh.max_nnz, 1);
  k.lucap = std::max<int64_t>(sh.max_lu_nnz, 1);
  k.blobcap = std::max<int64_t>(sh.max_schedule, 0);
  k.bpcap = std::max(sh.max_breakpoints, 1);
  for (int t = 0; t < kTypes; ++t) {
    k.icap[t] = std::max(sh.max_instances[t], 0);
    k.rcap += int64_t(k.icap[t]) * type_layout(t).nterm;
  }
  k.rcap = std::max<int64_t>(k.rcap, 1);
  k.ecap = 4 * int64_t(k.ucap) + 2 * k.jcap;
  return k;
}

// Device bytes of one slot: what xg_batch_create_slots allocates per slot.
int64_t slot_bytes(const SlotCaps &k, int precision, int n_out, int max_points) {
  const int64_t tsz = precision == XG_LU_FP32 ? 4 : 8;
  const int64_t u = k.ucap, j = k.jcap;
  int64_t b = 0;
  for (int t = 0; t < kTypes; ++t) {
    const TypeLayout &L = type_layout(t);
    const int64_t n = k.icap[t];
    b += n * (8 * L.np + 4 * L.nlid + 2 * 4 + 8 * L.nterm + 3 * 8 * (L.nsta + L.nsto));
  }
  b += 8 * int64_t(k.icap[XG_DEV_DIODE]) + 8 * kB3Mem * int64_t(k.icap[XG_DEV_BSIM3]);
  b += 4 * k.rcap + int64_t(sizeof(RedEntry)) * k.ecap + 2 * 4;
  b += 8 * (4 * u + 2 * j);                 // outputs F Q dFdxdVp dQdxdVp dFdx dQdx
  b += 8 * 3 * u;                            // solutions
  b += 8 * 13 * u + 8 * j + 4 * u + 4 * j;   // work vectors, jac, arp, aci
  b += 4 * u;                                // unknown list
  b += (tsz + 4 + 8) * k.lucap + 4 * (u + 1) + 4 * 4 * u + tsz * u;  // L\U
  b += 4 * k.blobcap;
  b += 8 * int64_t(max_points) * (1 + std::max(1, n_out)) + 4 * std::max(1, n_out);
  b += 8 * k.bpcap;
  b += 2 * int64_t(sizeof(CState)) + 3 * int64_t(sizeof(Flags)) + 8 * Q_N;
  b += 4 * (2 * kTypes) * 2 + 4 * 2 + 4 * 16;  // state/store runs, Jacobian run, per-slot ints
  return b;
}

struct SlotPool {
  xg_slot_shape shape{};
  SlotCaps k;
  int n_slots = 0, precision = XG_LU_FP64, n_out = 0, max_points = 0, n_refine = 0;
  double tstep = 1e-12, maxstep = 0.0, reltol = 1e-3, abstol = 1e-6;
  xg_device_options dopt{};
  DevOptions opt{};
  int NU = 0;               // pool unknowns; the ground is unknown NU
  int64_t NNZ = 0;
  int NT[kTypes] = {};
  int64_t sta0[kTypes] = {}, sto0[kTypes] = {}, term0[kTypes] = {};
  int64_t n_state = 0, n_store = 0, n_terms = 0, n_out_vals = 0;
  size_t solve_smem = 0, solve_lvl = 0;
  int red_y = 1;            // reduction blocks per slot
  // device
  double *params[kTypes] = {};
  int *lid[kTypes] = {}, *cid[kTypes] = {}, *cid_stage[kTypes] = {};
  double *terms = nullptr, *out = nullptr;
  uint32_t *ref = nullptr;
  RedEntry *ent = nullptr;
  int *ne = nullptr, *nl = nullptr;
  double *sol[3] = {}, *sta[3] = {}, *sto[3] = {};
  double *diode_vd = nullptr, *b3_mem = nullptr;
  CState *cs_next = nullptr;
  Flags *fl_next = nullptr, *fl_stage = nullptr;
  int *d_list = nullptr;     // the slots of one submit (restricted reduction)
  // writable views of BatchDev's per-slot arrays
  int *uend = nullptr, *send = nullptr, *oend = nullptr, *jend = nullptr, *bp_end = nullptr;
  int *sidx = nullptr, *oidx = nullptr, *jidx = nullptr, *arp = nullptr, *aci = nullptr;
  int *lrp = nullptr, *lci = nullptr, *ldiag = nullptr, *lP = nullptr, *lQ = nullptr;
  int64_t *lu2a = nullptr, *lnz_end = nullptr, *sched_end = nullptr;
  int *sched = nullptr, *lvl = nullptr, *out_idx = nullptr;
  double *bp = nullptr;
  double *work[13] = {};
  double *jac = nullptr, *part = nullptr;
  std::vector<void *> allocs;
  // staging (grown on demand)
  cudaStream_t side = nullptr;
  cudaEvent_t ready = nullptr;
  void *h_stage = nullptr, *d_stage = nullptr;
  size_t stage_cap = 0;
  double *h_jac = nullptr;  // pinned: first Jacobians read back
  size_t h_jac_cap = 0;
  // host state
  std::vector<char> used;
  std::vector<int> gen;
  std::mutex mu;         // used / gen
  std::mutex submit_mu;  // one submit at a time
};

int pool_gen(SlotPool *p, int slot) {
  std::lock_guard<std::mutex> lock(p->mu);
  return p->gen[slot];
}

void free_pool(SlotPool *p) {
  if (!p) return;
  if (p->side) cudaStreamSynchronize(p->side);
  for (void *a : p->allocs) cudaFree(a);
  if (p->d_stage) cudaFree(p->d_stage);
  if (p->h_stage) cudaFreeHost(p->h_stage);
  if (p->h_jac) cudaFreeHost(p->h_jac);
  if (p->ready) cudaEventDestroy(p->ready);
  if (p->side) cudaStreamDestroy(p->side);
  delete p;
}

namespace {

template <class V>
int pool_alloc(SlotPool *p, V **d, int64_t n, int fill_byte = 0) {
  const size_t bytes = sizeof(V) * size_t(std::max<int64_t>(n, 1));
  if (cudaMalloc((void **)d, bytes) != cudaSuccess) return XG_ERR_OOM;
  p->allocs.push_back((void *)*d);
  return cudaMemset(*d, fill_byte, bytes) == cudaSuccess ? XG_OK : XG_ERR_CUDA;
}

template <class V>
int pool_upload(SlotPool *p, const V **d, const std::vector<V> &h) {
  V *x = nullptr;
  int rc = pool_alloc(p, &x, int64_t(h.size()));
  if (!rc && !h.empty() &&
      cudaMemcpy(x, h.data(), sizeof(V) * h.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    rc = XG_ERR_CUDA;
  *d = x;
  return rc;
}

// A host-side copy list: segments plus their payload, device addresses final.
struct Staging {
  std::vector<Seg> segs;
  std::vector<uint32_t> payload;
  void put(void *dst, const void *src, int64_t words) {
    if (words <= 0) return;
    Seg s{(uint32_t *)dst, int64_t(payload.size()), words, 0u, 0u};
    segs.push_back(s);
    const uint32_t *w = (const uint32_t *)src;
    payload.insert(payload.end(), w, w + words);
  }
  void fill(void *dst, uint32_t word, int64_t words) {
    if (words <= 0) return;
    segs.push_back(Seg{(uint32_t *)dst, -1, words, word, 0u});
  }
  template <class V> void put_vec(V *dst, const std::vector<V> &v) {
    static_assert(sizeof(V) % 4 == 0, "word-sized elements");
    put(dst, v.data(), int64_t(v.size() * sizeof(V) / 4));
  }
  template <class V> void put_one(V *dst, const V &v) {
    static_assert(sizeof(V) % 4 == 0, "word-sized elements");
    put(dst, &v, int64_t(sizeof(V) / 4));
  }
  void zero_d(double *dst, int64_t n) { fill(dst, 0u, 2 * n); }
  void append(const Staging &o) {
    const int64_t base = int64_t(payload.size());
    for (Seg s : o.segs) {
      if (s.src >= 0) s.src += base;
      segs.push_back(s);
    }
    payload.insert(payload.end(), o.payload.begin(), o.payload.end());
  }
};

// Upload a copy list on the set-up stream and run it.
int run_staging(SlotPool *p, const Staging &st) {
  if (st.segs.empty()) return XG_OK;
  const size_t seg_bytes = st.segs.size() * sizeof(Seg);
  const size_t bytes = seg_bytes + st.payload.size() * 4;
  if (bytes > p->stage_cap) {
    if (cudaStreamSynchronize(p->side) != cudaSuccess) return XG_ERR_CUDA;
    if (p->d_stage) cudaFree(p->d_stage);
    if (p->h_stage) cudaFreeHost(p->h_stage);
    p->d_stage = p->h_stage = nullptr;
    p->stage_cap = 0;
    const size_t cap = std::max<size_t>(bytes + bytes / 2, 1 << 20);
    if (cudaMalloc(&p->d_stage, cap) != cudaSuccess || cudaMallocHost(&p->h_stage, cap) != cudaSuccess)
      return XG_ERR_OOM;
    p->stage_cap = cap;
  }
  // the pinned buffer is reused: the previous copy out of it has finished
  if (cudaStreamSynchronize(p->side) != cudaSuccess) return XG_ERR_CUDA;
  std::memcpy(p->h_stage, st.segs.data(), seg_bytes);
  std::memcpy((char *)p->h_stage + seg_bytes, st.payload.data(), st.payload.size() * 4);
  if (cudaMemcpyAsync(p->d_stage, p->h_stage, bytes, cudaMemcpyHostToDevice, p->side) != cudaSuccess)
    return XG_ERR_CUDA;
  const int nseg = int(st.segs.size());
  const int blocks = std::min((nseg + 7) / 8, 4 * sm_count());
  seg_copy<<<blocks, 256, 0, p->side>>>((const Seg *)p->d_stage, nseg,
                                        (const uint32_t *)((char *)p->d_stage + seg_bytes));
  count_launches(1);
  return cudaGetLastError() == cudaSuccess ? XG_OK : XG_ERR_CUDA;
}

LoadIO pool_io(const SlotPool *p) {
  return LoadIO{p->sol[0], p->sta[1], p->sto[1], p->sta[0], p->sto[0], p->terms,
                p->diode_vd, p->b3_mem, p->sta[1]};
}

PoolRed pool_red(const SlotPool *p) {
  return PoolRed{p->ent, p->k.ecap, p->ne, p->nl, p->ref, p->terms, p->out};
}

// The evaluation launches over every type's whole instance array, with the
// given circuit and flag arrays (the live ones, or the set-up ones).
int pool_eval(const SlotPool *p, int *const *cid, const Flags *flags, cudaStream_t s) {
  const LoadIO io = pool_io(p);
  for (int t = 0; t < kTypes; ++t) {
    if (!p->NT[t]) continue;
    const TypeLayout &L = type_layout(t);
    DevType dt{p->NT[t], L.nterm, int(p->sta0[t]), int(p->sto0[t]), p->term0[t], p->params[t],
               p->lid[t], cid[t], flags};
    Flags unused{};
    const int rc = p->dopt.fma ? fast::launch_eval(t, dt, p->opt, unused, io, s)
                               : exact::launch_eval(t, dt, p->opt, unused, io, s);
    if (rc) return rc;
  }
  return XG_OK;
}

// One request, set up on the host and placed in its slot.
struct Placed {
  Plan P;
  int slot = -1;
  int gen = 0;  // which request of the slot this one is
  std::vector<double> bp;
  Staging st1, st2;  // before / after the first Jacobian
  ReqLU lu;
  int rc = XG_OK;
  std::string err;
};

// Relocate request P into slot c: everything the set-up load and the batch
// kernels read, except the L\U arrays.
void stage_request(SlotPool *p, Placed &R, const double *x0, const int *out_idx) {
  const Plan &P = R.P;
  const SlotCaps &k = p->k;
  const int c = R.slot, nr = P.n_unknowns;
  const int u0 = c * k.ucap;
  const int64_t j0 = int64_t(c) * k.jcap, r0 = int64_t(c) * k.rcap;
  const int64_t W = int64_t(p->NU) + 1, Wr = int64_t(nr) + 1;
  Staging &st = R.st1;
  int ib[kTypes];
  for (int t = 0; t < kTypes; ++t) ib[t] = c * k.icap[t];
  // device parameters, LIDs (into the slot's unknowns; ground to the pool's),
  // circuits of the live and set-up loads
  std::vector<int> cs_runs, os_runs;
  for (int t = 0; t < kTypes; ++t) {
    const TypeData &T = P.T[t];
    const TypeLayout &L = type_layout(t);
    const int n = T.n;
    if (n) {
      for (int q = 0; q < L.np; ++q)
        st.put(p->params[t] + int64_t(q) * p->NT[t] + ib[t], T.params.data() + int64_t(q) * n, 2 * int64_t(n));
      std::vector<int> rl(size_t(L.nlid) * n);
      for (size_t j = 0; j < rl.size(); ++j) rl[j] = T.lid[j] == nr ? p->NU : u0 + T.lid[j];
      for (int q = 0; q < L.nlid; ++q)
        st.put(p->lid[t] + int64_t(q) * p->NT[t] + ib[t], rl.data() + int64_t(q) * n, n);
      st.fill(p->cid_stage[t] + ib[t], uint32_t(c), n);
    }
    if (k.icap[t]) {
      st.fill(p->cid[t] + ib[t], uint32_t(c), n);
      st.fill(p->cid[t] + ib[t] + n, 0xffffffffu, k.icap[t] - n);
      for (int v = 0; v < 3; ++v) {
        if (L.nsta) st.zero_d(p->sta[v] + p->sta0[t] + int64_t(ib[t]) * L.nsta, int64_t(k.icap[t]) * L.nsta);
        if (L.nsto) st.zero_d(p->sto[v] + p->sto0[t] + int64_t(ib[t]) * L.nsto, int64_t(k.icap[t]) * L.nsto);
      }
    }
    if (n && L.nsta && t != XG_DEV_DIODE) {
      cs_runs.push_back(int(p->sta0[t] + int64_t(ib[t]) * L.nsta));
      cs_runs.push_back(n * L.nsta);
    }
    if (n && L.nsto) {
      os_runs.push_back(int(p->sto0[t] + int64_t(ib[t]) * L.nsto));
      os_runs.push_back(n * L.nsto);
    }
  }
  if (k.icap[XG_DEV_DIODE]) st.zero_d(p->diode_vd + ib[XG_DEV_DIODE], k.icap[XG_DEV_DIODE]);
  if (k.icap[XG_DEV_BSIM3])
    for (int q = 0; q < kB3Mem; ++q)
      st.zero_d(p->b3_mem + int64_t(q) * p->NT[XG_DEV_BSIM3] + ib[XG_DEV_BSIM3], k.icap[XG_DEV_BSIM3]);
  // reduction: the request's lists, terms and outputs renumbered into the pool
  std::vector<uint32_t> ref(P.red_idx.size());
  {
    int64_t lo[kTypes], hi[kTypes];
    for (int t = 0; t < kTypes; ++t) {
      lo[t] = P.T[t].term0;
      hi[t] = P.T[t].n ? P.T[t].term0 + int64_t(P.T[t].n) * P.T[t].nterm : lo[t];
    }
    for (size_t j = 0; j < ref.size(); ++j) {
      const int64_t tau = P.red_idx[j];
      int t = 0;
      while (t < kTypes - 1 && !(P.T[t].n && tau >= lo[t] && tau < hi[t])) ++t;
      const int64_t off = tau - lo[t], n = P.T[t].n;
      ref[j] = uint32_t(p->term0[t] + (off / n) * p->NT[t] + ib[t] + off % n);
    }
  }
  st.put_vec(p->ref + r0, ref);
  std::vector<RedEntry> lng, sht;
  for (int64_t o = 0; o < P.n_out; ++o) {
    const int64_t b0 = P.red_ptr[o], cnt = P.red_ptr[o + 1] - b0;
    if (!cnt) continue;
    int64_t po;
    if (o < 4 * Wr) {
      po = (o / Wr) * W + u0 + o % Wr;
    } else {
      const int64_t e = o - 4 * Wr;
      po = e < P.nnz ? 4 * W + j0 + e : 4 * W + p->NNZ + j0 + (e - P.nnz);
    }
    RedEntry re{po, r0 + b0, int32_t(cnt), 0};
    (cnt > kLongOut ? lng : sht).push_back(re);
  }
  std::stable_sort(sht.begin(), sht.end(), [](const RedEntry &a, const RedEntry &b2) { return a.cnt < b2.cnt; });
  const int nlong = int(lng.size());
  lng.insert(lng.end(), sht.begin(), sht.end());
  st.put_vec(p->ent + int64_t(c) * k.ecap, lng);
  st.put_one(p->ne + c, int(lng.size()));
  st.put_one(p->nl + c, nlong);
  for (int q = 0; q < 4; ++q) st.zero_d(p->out + q * W + u0, k.ucap);
  st.zero_d(p->out + 4 * W + j0, k.jcap);
  st.zero_d(p->out + 4 * W + p->NNZ + j0, k.jcap);
  // solutions x0 (ground excluded), work vectors and histories zero
  std::vector<double> xs(size_t(k.ucap), 0.0);
  if (x0) std::copy(x0, x0 + nr, xs.begin());
  for (int v = 0; v < 3; ++v) st.put(p->sol[v] + u0, xs.data(), 2 * int64_t(k.ucap));
  for (double *w : p->work) st.zero_d(w + u0, k.ucap);
  st.zero_d(p->jac + j0, k.jcap);
  st.zero_d(p->part + int64_t(c) * Q_N, Q_N);
  // Jacobian pattern of the slot's rows
  std::vector<int> ap(size_t(k.ucap)), ac(size_t(P.nnz));
  for (int r = 0; r < k.ucap; ++r) ap[r] = int(j0 + P.rowptr[std::min(r, nr)]);
  for (int64_t e = 0; e < P.nnz; ++e) ac[e] = u0 + P.colidx[e];
  st.put_vec(p->arp + u0, ap);
  st.put_vec(p->aci + j0, ac);
  // the request's ranges
  st.put_one(p->uend + c, u0 + nr);
  st.put_one(p->jend + c, c + (P.nnz > 0 ? 1 : 0));
  const int jr[2] = {int(j0), int(P.nnz)};
  st.put(p->jidx + 2 * c, jr, 2);
  st.put_vec(p->sidx + 2 * kTypes * c, cs_runs);
  st.put_one(p->send + c, kTypes * c + int(cs_runs.size() / 2));
  st.put_vec(p->oidx + 2 * kTypes * c, os_runs);
  st.put_one(p->oend + c, kTypes * c + int(os_runs.size() / 2));
  st.put_vec(p->bp + int64_t(c) * k.bpcap, R.bp);
  st.put_one(p->bp_end + c, c * k.bpcap + int(R.bp.size()));
  if (p->n_out) {
    std::vector<int> oi(size_t(p->n_out));
    for (int j = 0; j < p->n_out; ++j) oi[j] = u0 + out_idx[j];
    st.put_vec(p->out_idx + int64_t(c) * p->n_out, oi);
  }
  // no L\U yet: empty ranges, the walker path
  st.put_one(p->lnz_end + c, int64_t(c) * k.lucap);
  st.put_one(p->sched_end + c, int64_t(c) * k.blobcap);
  st.put_one(p->lvl + c, 0);
  // the set-up load's flags: a transient load at x0 with pdt = 1/tstep
  Flags fs{};
  fs.transient = 1;
  fs.pdt = 1.0 / p->tstep;
  st.put_one(p->fl_stage + c, fs);
}

// The L\U arrays of a placed request, its reset state and its starting
// request state.
void stage_lu(SlotPool *p, Placed &R, double tstop) {
  const Plan &P = R.P;
  const SlotCaps &k = p->k;
  const int c = R.slot, nr = P.n_unknowns;
  const int u0 = c * k.ucap;
  const int64_t j0 = int64_t(c) * k.jcap, z0 = int64_t(c) * k.lucap;
  const LuSymbolic &S = R.lu.S;
  Staging &st = R.st2;
  st.put_vec(p->lrp + int64_t(c) * (k.ucap + 1), S.rp);
  st.put_vec(p->lci + z0, S.ci);
  st.put_vec(p->ldiag + u0, S.diag);
  std::vector<int64_t> l2a(S.lu2a.size());
  for (size_t q = 0; q < l2a.size(); ++q) l2a[q] = S.lu2a[q] >= 0 ? j0 + S.lu2a[q] : -1;
  st.put_vec(p->lu2a + z0, l2a);
  st.put_vec(p->lP + u0, S.P);
  st.put_vec(p->lQ + u0, S.Q);
  st.put_one(p->lnz_end + c, z0 + int64_t(S.rp[nr]));
  const size_t tsz = p->precision == XG_LU_FP32 ? sizeof(float) : sizeof(double);
  const bool lvl = p->solve_lvl && int64_t(R.lu.blob.size()) <= k.blobcap &&
                   smem_bytes_lvl(nr, S.rp[nr], int64_t(R.lu.blob.size()), tsz) <= p->solve_lvl;
  if (lvl) st.put_vec(p->sched + int64_t(c) * k.blobcap, R.lu.blob);
  st.put_one(p->sched_end + c, int64_t(c) * k.blobcap + (lvl ? int64_t(R.lu.blob.size()) : 0));
  st.put_one(p->lvl + c, lvl ? 1 : 0);
  // the set-up load wrote state, store and members: start again from zero,
  // and take the slot out of the set-up load
  for (int t = 0; t < kTypes; ++t) {
    const TypeLayout &L = type_layout(t);
    const int ib = c * k.icap[t];
    if (!k.icap[t]) continue;
    for (int v = 0; v < 3; ++v) {
      if (L.nsta) st.zero_d(p->sta[v] + p->sta0[t] + int64_t(ib) * L.nsta, int64_t(k.icap[t]) * L.nsta);
      if (L.nsto) st.zero_d(p->sto[v] + p->sto0[t] + int64_t(ib) * L.nsto, int64_t(k.icap[t]) * L.nsto);
    }
    st.fill(p->cid_stage[t] + ib, 0xffffffffu, k.icap[t]);
  }
  if (k.icap[XG_DEV_DIODE]) st.zero_d(p->diode_vd + c * k.icap[XG_DEV_DIODE], k.icap[XG_DEV_DIODE]);
  if (k.icap[XG_DEV_BSIM3])
    for (int q = 0; q < kB3Mem; ++q)
      st.zero_d(p->b3_mem + int64_t(q) * p->NT[XG_DEV_BSIM3] + c * k.icap[XG_DEV_BSIM3], k.icap[XG_DEV_BSIM3]);
  // the starting request state (as a batch of its own starts it)
  CState cs;
  std::memset(&cs, 0, sizeof(cs));
  cs.tstop = tstop;
  cs.tstep = p->tstep;
  cs.max_step = p->maxstep > 0 ? p->maxstep : 0.1 * tstop;
  cs.reltol = p->reltol;
  cs.abstol = p->abstol;
  cs.saved = 1e-10;
  cs.phase = PH_INIT;
  cs.first_step = 1;
  cs.beginning = 1;
  cs.order = 1;
  cs.loads = 1;
  cs.gen = R.gen;
  st.put_one(p->cs_next + c, cs);
  Flags f{};
  f.dcop = 1;
  f.tranop = 1;
  st.put_one(p->fl_next + c, f);
}

// Host work spread over threads (each request is independent).
template <class F>
void for_each_parallel(int n, F f) {
  const int nt = std::max(1, std::min<int>(std::min(16, n), int(std::thread::hardware_concurrency())));
  std::atomic<int> next{0};
  auto worker = [&]() {
    for (int i = next++; i < n; i = next++) f(i);
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < nt; ++t) pool.emplace_back(worker);
  worker();
  for (auto &t : pool) t.join();
}

// Set up, shape-check and measure one request on the host.
int plan_request(const xg_device_options &dopt, const xg_netlist *nl, double tstop, Placed *R) {
  std::string err;
  int rc = build_plan(nl, &dopt, &R->P, &err);
  if (rc) {
    R->err = err;
    return rc;
  }
  R->bp = pulse_breakpoints(R->P, tstop);
  return XG_OK;
}

int check_fits(const SlotCaps &k, const Placed &R) {
  const Plan &P = R.P;
  if (P.n_unknowns + 1 > k.ucap || P.nnz > k.jcap || int64_t(R.bp.size()) > k.bpcap) return XG_ERR_ARG;
  for (int t = 0; t < kTypes; ++t)
    if (P.T[t].n > k.icap[t]) return XG_ERR_ARG;
  return XG_OK;
}

}  // namespace

// One iteration of a slotted batch: the solves, the pool's load, combine,
// control and vector.
int enqueue_pool_iteration(xg_batch *b) {
  SlotPool *p = b->pool;
  cudaStream_t s = b->stream;
  const int nc = b->nc;
  if (p->solve_smem) {
    if (p->precision == XG_LU_FP32) batch_solve_smem<float><<<nc, 32, p->solve_smem, s>>>(b->dev);
    else batch_solve_smem<double><<<nc, 32, p->solve_smem, s>>>(b->dev);
  } else {
    if (p->precision == XG_LU_FP32) batch_solve<float><<<(nc + 3) / 4, 128, 0, s>>>(b->dev);
    else batch_solve<double><<<(nc + 3) / 4, 128, 0, s>>>(b->dev);
  }
  count_launches(1);
  if (p->solve_lvl) {
    if (p->precision == XG_LU_FP32) batch_solve_lvl<float><<<nc, kLvlThreads, p->solve_lvl, s>>>(b->dev);
    else batch_solve_lvl<double><<<nc, kLvlThreads, p->solve_lvl, s>>>(b->dev);
    count_launches(1);
  }
  int rc = pool_eval(p, p->cid, b->dev.flags, s);
  if (rc) return rc;
  pool_reduce<<<dim3(nc, p->red_y), kPoolRedThreads, 0, s>>>(pool_red(p), b->dev.cs, nullptr, p->dopt.fma);
  batch_combine<<<nc, kBatchThreads, 0, s>>>(b->dev);
  batch_control<<<(nc + 31) / 32, 32, 0, s>>>(b->dev);
  batch_vector<<<nc, kVectorThreads, 0, s>>>(b->dev);
  count_launches(4);
  return cudaGetLastError() == cudaSuccess ? XG_OK : XG_ERR_CUDA;
}

}  // namespace xg

// ---- C ABI of slotted batches -------------------------------------------------

extern "C" int xg_slot_bytes(const xg_slot_shape *shape, const xg_batch_options *o, int64_t *bytes) {
  if (!shape || !o || !bytes || shape->max_unknowns <= 0 || o->max_points <= 0 || o->n_out < 0) {
    xg::set_error("xg_slot_bytes: bad argument");
    return XG_ERR_ARG;
  }
  *bytes = xg::slot_bytes(xg::slot_caps(*shape), o->lu_precision, o->n_out, o->max_points);
  return XG_OK;
}

extern "C" int xg_mem_info(xg_ctx *ctx, int64_t *free_bytes, int64_t *total_bytes) {
  int device = 0;
  void *stream = nullptr;
  if (!ctx || xg::ctx_info(ctx, &device, &stream)) {
    xg::set_error("xg_mem_info: bad argument");
    return XG_ERR_ARG;
  }
  int cur = 0;
  cudaGetDevice(&cur);
  if (cur != device) cudaSetDevice(device);
  size_t f = 0, t = 0;
  const cudaError_t e = cudaMemGetInfo(&f, &t);
  if (cur != device) cudaSetDevice(cur);
  if (e != cudaSuccess) {
    xg::set_error(std::string("xg_mem_info: ") + cudaGetErrorString(e));
    return XG_ERR_CUDA;
  }
  if (free_bytes) *free_bytes = int64_t(f);
  if (total_bytes) *total_bytes = int64_t(t);
  return XG_OK;
}

extern "C" int xg_slot_need(xg_ctx *ctx, const xg_netlist *nl, const double *x0, double tstop,
                            double tstep, xg_slot_shape *need) {
  using namespace xg;
  if (!ctx || !nl || !need || !(tstop > 0) || !(tstep > 0)) {
    set_error("xg_slot_need: bad argument");
    return XG_ERR_ARG;
  }
  xg_device_options dopt;
  ctx_options(ctx, &dopt);
  Placed R;
  int rc = plan_request(dopt, nl, tstop, &R);
  if (rc) {
    set_error("xg_slot_need: " + R.err);
    return rc;
  }
  const Plan &P = R.P;
  // the first Jacobian, from a circuit of its own
  xg_circuit *ck = nullptr;
  if ((rc = xg_circuit_create(ctx, nl, &ck))) return rc;
  std::vector<double> xu(size_t(P.n_unknowns) + 1, 0.0);
  if (x0) std::copy(x0, x0 + P.n_unknowns, xu.begin());
  std::vector<double> dfdx(size_t(std::max<int64_t>(P.nnz, 1))), dqdx(dfdx.size());
  for (int id : {XG_VEC_SOL_NEXT, XG_VEC_SOL_CURR, XG_VEC_SOL_LAST})
    if (!rc) rc = xg_vec_upload(ck, id, xu.data());
  xg_load_flags fl{};
  fl.transient = 1;
  fl.pdt = 1.0 / tstep;
  if (!rc) rc = xg_load(ck, &fl);
  if (!rc) rc = xg_vec_download(ck, XG_VEC_DFDX, dfdx.data());
  if (!rc) rc = xg_vec_download(ck, XG_VEC_DQDX, dqdx.data());
  xg_circuit_destroy(ck);
  if (rc) return rc;
  std::vector<double> val(size_t(P.nnz));
  for (int r = 0; r < P.n_unknowns; ++r)
    for (int e = P.rowptr[r]; e < P.rowptr[r + 1]; ++e) {
      double a = dfdx[e] + dqdx[e] / tstep;
      if (P.colidx[e] == r && a == 0.0) a = 1e-12;
      val[e] = a;
    }
  analyse_request(P.n_unknowns, P.rowptr, P.colidx, val, "xg_slot_need", &R.lu);
  if (R.lu.rc) {
    set_error(R.lu.err);
    return R.lu.rc;
  }
  std::memset(need, 0, sizeof(*need));
  need->max_unknowns = P.n_unknowns;
  for (int t = 0; t < kTypes; ++t) need->max_instances[t] = P.T[t].n;
  need->max_nnz = P.nnz;
  need->max_lu_nnz = R.lu.S.rp[P.n_unknowns];
  need->max_schedule = int64_t(R.lu.blob.size());
  need->max_breakpoints = int(R.bp.size());
  return XG_OK;
}

extern "C" int xg_batch_create_slots(xg_ctx *ctx, int n_slots, const xg_slot_shape *shape,
                                     const xg_batch_options *o, xg_batch **out) {
  using namespace xg;
  if (!ctx || n_slots <= 0 || !shape || shape->max_unknowns <= 0 || !o || !out || o->max_points <= 0 ||
      o->n_out < 0 || (o->lu_precision != XG_LU_FP64 && o->lu_precision != XG_LU_FP32) ||
      o->n_refine < 0 || n_slots > (1 << 20)) {
    set_error("xg_batch_create_slots: bad argument");
    return XG_ERR_ARG;
  }
  *out = nullptr;
  std::unique_ptr<xg_batch, void (*)(xg_batch *)> b(new xg_batch, [](xg_batch *q) {
    free_batch(q);
    delete q;
  });
  b->ctx = ctx;
  b->nc = n_slots;
  b->n_out = o->n_out;
  b->max_points = o->max_points;
  b->precision = o->lu_precision;
  SlotPool *p = new SlotPool;
  b->pool = p;
  p->shape = *shape;
  p->k = slot_caps(*shape);
  const SlotCaps &k = p->k;
  p->n_slots = n_slots;
  p->precision = o->lu_precision;
  p->n_out = o->n_out;
  p->max_points = o->max_points;
  p->n_refine = o->lu_precision == XG_LU_FP32 ? o->n_refine : 0;
  p->tstep = o->tstep > 0 ? o->tstep : 1e-12;
  p->maxstep = o->maxstep;
  p->reltol = o->reltol > 0 ? o->reltol : 1e-3;
  p->abstol = o->abstol > 0 ? o->abstol : 1e-6;
  ctx_options(ctx, &p->dopt);
  p->opt = DevOptions{p->dopt.gmin, p->dopt.voltlim};
  const int64_t ns = n_slots;
  if (ns * k.ucap >= (int64_t(1) << 31) - 1 || ns * k.jcap >= (int64_t(1) << 31) ||
      ns * k.lucap >= (int64_t(1) << 40)) {
    set_error("xg_batch_create_slots: too many slots for the shape");
    return XG_ERR_ARG;
  }
  p->NU = int(ns * k.ucap);
  p->NNZ = ns * k.jcap;
  int64_t sta = 0, sto = 0, term = 0;
  for (int t = 0; t < kTypes; ++t) {
    const TypeLayout &L = type_layout(t);
    p->NT[t] = int(ns * k.icap[t]);
    p->sta0[t] = sta;
    p->sto0[t] = sto;
    p->term0[t] = term;
    sta += int64_t(p->NT[t]) * L.nsta;
    sto += int64_t(p->NT[t]) * L.nsto;
    term += int64_t(p->NT[t]) * L.nterm;
  }
  p->n_state = sta;
  p->n_store = sto;
  p->n_terms = term;
  if (sta >= (int64_t(1) << 31) || sto >= (int64_t(1) << 31) || term >= (int64_t(1) << 32) - 1) {
    set_error("xg_batch_create_slots: too many slots for the shape");
    return XG_ERR_ARG;
  }
  const int64_t W = int64_t(p->NU) + 1;
  p->n_out_vals = 4 * W + 2 * p->NNZ;
  p->red_y = int(std::min<int64_t>(32, (k.ecap + kPoolRedThreads - 1) / kPoolRedThreads));
  const size_t tsz = o->lu_precision == XG_LU_FP32 ? sizeof(float) : sizeof(double);
  int device = 0;
  void *ctx_stream = nullptr;
  ctx_info(ctx, &device, &ctx_stream);
  if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&p->side, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&p->ready, cudaEventDisableTiming) != cudaSuccess) {
    set_error("xg_batch_create_slots: stream creation failed");
    return XG_ERR_CUDA;
  }
  auto oom = [&]() {
    set_error("xg_batch_create_slots: out of device memory");
    return XG_ERR_OOM;
  };
  // device arrays; circuits -1 (no instance), everything else zero
  for (int t = 0; t < kTypes; ++t) {
    const TypeLayout &L = type_layout(t);
    if (!p->NT[t]) continue;
    if (pool_alloc(p, &p->params[t], int64_t(L.np) * p->NT[t]) ||
        pool_alloc(p, &p->lid[t], int64_t(L.nlid) * p->NT[t]) ||
        pool_alloc(p, &p->cid[t], p->NT[t], 0xff) || pool_alloc(p, &p->cid_stage[t], p->NT[t], 0xff))
      return oom();
  }
  if (pool_alloc(p, &p->terms, p->n_terms) || pool_alloc(p, &p->out, p->n_out_vals) ||
      pool_alloc(p, &p->ref, ns * k.rcap) || pool_alloc(p, &p->ent, ns * k.ecap) ||
      pool_alloc(p, &p->ne, ns) || pool_alloc(p, &p->nl, ns) ||
      pool_alloc(p, &p->diode_vd, p->NT[XG_DEV_DIODE]) ||
      pool_alloc(p, &p->b3_mem, int64_t(kB3Mem) * p->NT[XG_DEV_BSIM3]) ||
      pool_alloc(p, &p->cs_next, ns) || pool_alloc(p, &p->fl_next, ns) || pool_alloc(p, &p->fl_stage, ns) ||
      pool_alloc(p, &p->d_list, ns))
    return oom();
  for (int v = 0; v < 3; ++v)
    if (pool_alloc(p, &p->sol[v], W) || pool_alloc(p, &p->sta[v], p->n_state) ||
        pool_alloc(p, &p->sto[v], p->n_store))
      return oom();
  BatchDev &d = b->dev;
  d.nc = n_slots;
  d.n_out = o->n_out;
  d.max_points = o->max_points;
  d.n_refine = p->n_refine;
  // fixed starts of each slot's regions
  std::vector<int> uptr(ns), sptr(ns), jptr(ns), lrp_off(ns), bp_ptr(ns), uidx(size_t(p->NU));
  std::vector<int64_t> lnz_off(ns), sched_off(ns);
  for (int c = 0; c < n_slots; ++c) {
    uptr[c] = c * k.ucap;
    sptr[c] = c * kTypes;
    jptr[c] = c;
    lrp_off[c] = c * (k.ucap + 1);
    bp_ptr[c] = c * k.bpcap;
    lnz_off[c] = int64_t(c) * k.lucap;
    sched_off[c] = int64_t(c) * k.blobcap;
  }
  for (int u = 0; u < p->NU; ++u) uidx[u] = u;
  if (pool_upload(p, &d.uptr, uptr) || pool_upload(p, &d.uidx, uidx) || pool_upload(p, &d.sptr, sptr) ||
      pool_upload(p, &d.optr, sptr) || pool_upload(p, &d.jptr, jptr) || pool_upload(p, &d.lrp_off, lrp_off) ||
      pool_upload(p, &d.lnz_off, lnz_off) || pool_upload(p, &d.sched_off, sched_off) ||
      pool_upload(p, &d.bp_ptr, bp_ptr))
    return oom();
  // the request's ends start equal to the starts (empty)
  if (pool_alloc(p, &p->uend, ns) || pool_alloc(p, &p->send, ns) || pool_alloc(p, &p->oend, ns) ||
      pool_alloc(p, &p->jend, ns) || pool_alloc(p, &p->bp_end, ns) || pool_alloc(p, &p->lnz_end, ns) ||
      pool_alloc(p, &p->sched_end, ns) || pool_alloc(p, &p->lvl, ns) ||
      pool_alloc(p, &p->sidx, 2 * kTypes * ns) || pool_alloc(p, &p->oidx, 2 * kTypes * ns) ||
      pool_alloc(p, &p->jidx, 2 * ns) || pool_alloc(p, &p->arp, W) || pool_alloc(p, &p->aci, p->NNZ) ||
      pool_alloc(p, &p->lrp, ns * (k.ucap + 1)) || pool_alloc(p, &p->lci, ns * k.lucap) ||
      pool_alloc(p, &p->ldiag, p->NU) || pool_alloc(p, &p->lP, p->NU) || pool_alloc(p, &p->lQ, p->NU) ||
      pool_alloc(p, &p->lu2a, ns * k.lucap) || pool_alloc(p, &p->sched, std::max<int64_t>(ns * k.blobcap, 1)) ||
      pool_alloc(p, &p->out_idx, ns * std::max(1, o->n_out)) || pool_alloc(p, &p->bp, ns * k.bpcap))
    return oom();
  if (cudaMemcpy(p->uend, uptr.data(), 4 * ns, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->send, sptr.data(), 4 * ns, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->oend, sptr.data(), 4 * ns, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->jend, jptr.data(), 4 * ns, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->bp_end, bp_ptr.data(), 4 * ns, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->lnz_end, lnz_off.data(), 8 * ns, cudaMemcpyHostToDevice) != cudaSuccess ||
      cudaMemcpy(p->sched_end, sched_off.data(), 8 * ns, cudaMemcpyHostToDevice) != cudaSuccess) {
    set_error("xg_batch_create_slots: copy failed");
    return XG_ERR_CUDA;
  }
  d.uend = p->uend; d.send = p->send; d.oend = p->oend; d.jend = p->jend; d.bp_end = p->bp_end;
  d.lnz_end = p->lnz_end; d.sched_end = p->sched_end;
  d.sidx = p->sidx; d.oidx = p->oidx; d.jidx = p->jidx; d.arp = p->arp; d.aci = p->aci;
  d.lrp = p->lrp; d.lci = p->lci; d.ldiag = p->ldiag; d.lu2a = p->lu2a; d.lP = p->lP; d.lQ = p->lQ;
  d.sched = p->sched; d.lvl = p->lvl; d.out_idx = p->out_idx; d.bp = p->bp;
  {
    void *pv = nullptr, *pr = nullptr;
    int *pm = nullptr;
    if (cudaMalloc(&pv, tsz * size_t(ns * k.lucap)) != cudaSuccess) return oom();
    p->allocs.push_back(pv);
    if (cudaMalloc(&pr, tsz * size_t(std::max(p->NU, 1))) != cudaSuccess) return oom();
    p->allocs.push_back(pr);
    if (pool_alloc(p, &pm, p->NU)) return oom();
    d.lval = pv;
    d.lrd = pr;
    d.map = pm;
  }
  double **wv[13] = {&d.y, &d.r, &d.dd, &d.rhs, &d.dx, &d.w, &d.xh0, &d.xh1, &d.xh2,
                     &d.qh0, &d.qh1, &d.qh2, &d.xn0};
  for (int q = 0; q < 13; ++q) {
    if (pool_alloc(p, wv[q], W)) return oom();
    p->work[q] = *wv[q];
  }
  if (pool_alloc(p, &d.jac, p->NNZ) || pool_alloc(p, &d.part, ns * Q_N) ||
      pool_alloc(p, &d.rec_t, ns * o->max_points) ||
      pool_alloc(p, &d.rec_v, ns * o->max_points * std::max(1, o->n_out)))
    return oom();
  p->jac = d.jac;
  p->part = d.part;
  d.x = p->sol[0]; d.xc = p->sol[1]; d.xl = p->sol[2];
  d.sta = p->sta[0]; d.stac = p->sta[1]; d.stal = p->sta[2];
  d.sto = p->sto[0]; d.stoc = p->sto[1]; d.stol = p->sto[2];
  d.f = p->out; d.q = p->out + W; d.fvp = p->out + 2 * W; d.qvp = p->out + 3 * W;
  d.dfdx = p->out + 4 * W; d.dqdx = p->out + 4 * W + p->NNZ;
  // request states: every slot free (phase done) and skipped by the load
  {
    std::vector<Flags> fl(ns);
    for (auto &f : fl) {
      f = Flags{};
      f.skip = 1;
    }
    CState *t_cs = nullptr;
    Flags *t_fl = nullptr;
    if (pool_alloc(p, &t_cs, ns) || pool_alloc(p, &t_fl, ns)) return oom();
    if (cudaMemcpy(t_fl, fl.data(), sizeof(Flags) * ns, cudaMemcpyHostToDevice) != cudaSuccess) {
      set_error("xg_batch_create_slots: copy failed");
      return XG_ERR_CUDA;
    }
    d.cs = t_cs;
    d.flags = t_fl;
  }
  if (cudaMallocHost((void **)&b->h_cs, sizeof(CState) * ns) != cudaSuccess) {
    set_error("xg_batch_create_slots: out of pinned host memory");
    return XG_ERR_OOM;
  }
  std::memset(b->h_cs, 0, sizeof(CState) * ns);
  // the solves: shared-memory paths sized for the shape
  {
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device);
    const size_t need_w = smem_bytes_request(k.ucap, k.lucap, tsz);
    if (need_w + 1024 <= size_t(optin) && !std::getenv("XG_BATCH_NO_SMEM")) {
      const void *fn = o->lu_precision == XG_LU_FP32 ? (const void *)batch_solve_smem<float>
                                                     : (const void *)batch_solve_smem<double>;
      if (allow_dynamic_smem(fn, need_w) == cudaSuccess) p->solve_smem = need_w;
    }
    const size_t need_l = smem_bytes_lvl(k.ucap, k.lucap, k.blobcap, tsz);
    if (k.blobcap > 0 && need_l + 1024 <= size_t(optin) && !std::getenv("XG_BATCH_NO_LVL")) {
      const void *fn = o->lu_precision == XG_LU_FP32 ? (const void *)batch_solve_lvl<float>
                                                     : (const void *)batch_solve_lvl<double>;
      if (allow_dynamic_smem(fn, need_l) == cudaSuccess) p->solve_lvl = need_l;
    }
  }
  if (cudaDeviceSynchronize() != cudaSuccess) {
    set_error("xg_batch_create_slots: set-up failed");
    return XG_ERR_CUDA;
  }
  p->used.assign(ns, 0);
  p->gen.assign(ns, 0);
  b->bytes = 0;
  {
    int64_t per = slot_bytes(k, o->lu_precision, o->n_out, o->max_points);
    b->bytes = per * ns + 8 * 4;  // the ground entries of the vectors
  }
  *out = b.release();
  return XG_OK;
}

extern "C" int xg_batch_submit(xg_batch *b, int n, const xg_netlist *const *nls, const double *const *x0,
                               const double *tstop, const int *const *out_idx, int *slots) {
  using namespace xg;
  if (!b || !b->pool || n < 0 || (n && (!nls || !tstop || !slots)) || (n && b->n_out && !out_idx)) {
    set_error("xg_batch_submit: bad argument");
    return XG_ERR_ARG;
  }
  SlotPool *p = b->pool;
  // one submit at a time per batch; the slot bookkeeping below is also read
  // by results / release / slots on other threads, under p->mu only briefly
  std::lock_guard<std::mutex> one(p->submit_mu);
  for (int i = 0; i < n; ++i) slots[i] = -1;
  std::vector<int> free_slots;
  {
    std::lock_guard<std::mutex> lock(p->mu);
    for (int c = 0; c < p->n_slots && int(free_slots.size()) < n; ++c)
      if (!p->used[c]) {
        free_slots.push_back(c);
        p->used[c] = 2;  // being set up
      }
  }
  const int m = int(free_slots.size());
  if (!m) return XG_OK;
  // on any failure the chosen slots go back to free (never activated)
  struct Unreserve {
    SlotPool *p;
    const std::vector<int> *slots;
    bool keep = false;
    ~Unreserve() {
      if (keep) return;
      std::lock_guard<std::mutex> lock(p->mu);
      for (int c : *slots) p->used[c] = 0;
    }
  } unreserve{p, &free_slots};
  std::vector<Placed> req(m);
  for (int i = 0; i < m; ++i) req[i].slot = free_slots[i];
  // set-up and relocation on the host
  for_each_parallel(m, [&](int i) {
    Placed &R = req[i];
    if (!(tstop[i] > 0) || !nls[i]) {
      R.rc = XG_ERR_ARG;
      R.err = "bad request";
      return;
    }
    R.rc = plan_request(p->dopt, nls[i], tstop[i], &R);
    if (!R.rc && check_fits(p->k, R)) {
      R.rc = XG_ERR_ARG;
      R.err = "larger than the batch's slot shape";
    }
    if (!R.rc && p->n_out)
      for (int j = 0; j < p->n_out; ++j)
        if (out_idx[i][j] < 0 || out_idx[i][j] >= R.P.n_unknowns) {
          R.rc = XG_ERR_ARG;
          R.err = "output index out of range";
        }
    if (!R.rc) stage_request(p, R, x0 ? x0[i] : nullptr, p->n_out ? out_idx[i] : nullptr);
  });
  for (int i = 0; i < m; ++i)
    if (req[i].rc) {
      set_error("xg_batch_submit: request " + std::to_string(i) + ": " + req[i].err);
      return req[i].rc;
    }
  // the slots' data, then their first Jacobian, on the set-up stream
  Staging st;
  for (auto &R : req) {
    st.append(R.st1);
    R.st1 = Staging{};
  }
  st.put(p->d_list, free_slots.data(), m);  // the slots of the restricted reduction
  int rc = XG_OK;
  {
    std::lock_guard<std::mutex> launch(launch_mutex());
    rc = run_staging(p, st);
    if (!rc) rc = pool_eval(p, p->cid_stage, p->fl_stage, p->side);
    if (!rc) {
      pool_reduce<<<dim3(m, p->red_y), kPoolRedThreads, 0, p->side>>>(pool_red(p), nullptr, p->d_list,
                                                                      p->dopt.fma);
      count_launches(1);
      if (cudaGetLastError() != cudaSuccess) rc = XG_ERR_CUDA;
    }
  }
  // read the slots' dF/dx and dQ/dx back
  int64_t tot = 0;
  for (auto &R : req) tot += 2 * R.P.nnz;
  if (!rc && size_t(tot) > p->h_jac_cap) {
    if (p->h_jac) cudaFreeHost(p->h_jac);
    p->h_jac = nullptr;
    p->h_jac_cap = 0;
    if (cudaMallocHost((void **)&p->h_jac, sizeof(double) * size_t(std::max<int64_t>(tot, 1))) != cudaSuccess)
      rc = XG_ERR_OOM;
    else
      p->h_jac_cap = size_t(std::max<int64_t>(tot, 1));
  }
  std::vector<int64_t> joff(m + 1, 0);
  for (int i = 0; i < m; ++i) joff[i + 1] = joff[i] + 2 * req[i].P.nnz;
  if (!rc) {
    const int64_t W = int64_t(p->NU) + 1;
    for (int i = 0; i < m && !rc; ++i) {
      const int64_t j0 = int64_t(req[i].slot) * p->k.jcap, nz = req[i].P.nnz;
      if (!nz) continue;
      if (cudaMemcpyAsync(p->h_jac + joff[i], p->out + 4 * W + j0, sizeof(double) * nz,
                          cudaMemcpyDeviceToHost, p->side) != cudaSuccess ||
          cudaMemcpyAsync(p->h_jac + joff[i] + nz, p->out + 4 * W + p->NNZ + j0, sizeof(double) * nz,
                          cudaMemcpyDeviceToHost, p->side) != cudaSuccess)
        rc = XG_ERR_CUDA;
    }
  }
  if (!rc && cudaStreamSynchronize(p->side) != cudaSuccess) rc = XG_ERR_CUDA;
  if (rc) {
    set_error("xg_batch_submit: set-up load failed");
    return rc;
  }
  // pivot analyses on the host
  for_each_parallel(m, [&](int i) {
    Placed &R = req[i];
    const Plan &P = R.P;
    const double *dfdx = p->h_jac + joff[i], *dqdx = dfdx + P.nnz;
    std::vector<double> val(size_t(P.nnz));
    for (int r = 0; r < P.n_unknowns; ++r)
      for (int e = P.rowptr[r]; e < P.rowptr[r + 1]; ++e) {
        double a = dfdx[e] + dqdx[e] / p->tstep;
        if (P.colidx[e] == r && a == 0.0) a = 1e-12;
        val[e] = a;
      }
    analyse_request(P.n_unknowns, P.rowptr, P.colidx, val, "xg_batch_submit: request " + std::to_string(i),
                    &R.lu);
    if (!R.lu.rc && int64_t(R.lu.S.rp[P.n_unknowns]) > p->k.lucap) {
      R.lu.rc = XG_ERR_ARG;
      R.lu.err = "xg_batch_submit: request " + std::to_string(i) + ": L\\U larger than the slot shape";
    }
  });
  for (int i = 0; i < m; ++i)
    if (req[i].lu.rc) {
      // the slots were written but never activated: they stay free
      set_error(req[i].lu.err);
      return req[i].lu.rc;
    }
  {
    std::lock_guard<std::mutex> lock(p->mu);
    for (int i = 0; i < m; ++i) req[i].gen = ++p->gen[req[i].slot];
  }
  for (int i = 0; i < m; ++i) stage_lu(p, req[i], tstop[i]);
  Staging st2;
  for (auto &R : req) st2.append(R.st2);
  {
    std::lock_guard<std::mutex> launch(launch_mutex());
    rc = run_staging(p, st2);
    if (!rc && cudaEventRecord(p->ready, p->side) != cudaSuccess) rc = XG_ERR_CUDA;
    // activation on the batch's stream: after the set-up stream's writes,
    // between two batch iterations
    if (!rc && cudaStreamWaitEvent(b->stream, p->ready, 0) != cudaSuccess) rc = XG_ERR_CUDA;
    for (int i0 = 0; i0 < m && !rc; i0 += kActivateMax) {
      SlotList l;
      l.n = std::min(kActivateMax, m - i0);
      for (int j = 0; j < l.n; ++j) l.slot[j] = req[i0 + j].slot;
      activate_slots<<<1, kActivateMax, 0, b->stream>>>(l, b->dev.cs, p->cs_next, b->dev.flags, p->fl_next);
      count_launches(1);
      if (cudaGetLastError() != cudaSuccess) rc = XG_ERR_CUDA;
    }
  }
  if (!rc && cudaStreamSynchronize(p->side) != cudaSuccess) rc = XG_ERR_CUDA;
  if (rc) {
    set_error("xg_batch_submit: activation failed");
    return rc;
  }
  {
    std::lock_guard<std::mutex> lock(p->mu);
    for (int i = 0; i < m; ++i) {
      p->used[req[i].slot] = 1;
      slots[i] = req[i].slot;
    }
  }
  unreserve.keep = true;
  return XG_OK;
}

extern "C" int xg_batch_release(xg_batch *b, int slot) {
  using namespace xg;
  if (!b || !b->pool || slot < 0 || slot >= b->nc) {
    set_error("xg_batch_release: bad argument");
    return XG_ERR_ARG;
  }
  SlotPool *p = b->pool;
  std::lock_guard<std::mutex> lock(p->mu);
  const CState &c = b->h_cs[slot];
  if (p->used[slot] == 2 || (p->used[slot] && !(c.gen == p->gen[slot] && c.phase == PH_DONE))) {
    set_error("xg_batch_release: the slot's request has not finished (poll first)");
    return XG_ERR_STATE;
  }
  p->used[slot] = 0;
  return XG_OK;
}

extern "C" int xg_batch_finished(const xg_batch *b, int max_slots, int *slots, int *n) {
  using namespace xg;
  if (!b || !b->pool || max_slots < 0 || (max_slots && !slots) || !n) {
    set_error("xg_batch_finished: bad argument");
    return XG_ERR_ARG;
  }
  SlotPool *p = b->pool;
  std::lock_guard<std::mutex> lock(p->mu);
  int k = 0;
  for (int c = 0; c < b->nc; ++c)
    if (p->used[c] == 1 && b->h_cs[c].gen == p->gen[c] && b->h_cs[c].phase == PH_DONE) {
      if (k < max_slots) slots[k] = c;
      ++k;
    }
  *n = k;
  return XG_OK;
}

extern "C" int xg_batch_slots(const xg_batch *b, int *n_free, int *n_running) {
  using namespace xg;
  if (!b || !b->pool) {
    set_error("xg_batch_slots: bad argument");
    return XG_ERR_ARG;
  }
  SlotPool *p = b->pool;
  std::lock_guard<std::mutex> lock(p->mu);
  int nf = 0, nr = 0;
  for (int c = 0; c < b->nc; ++c) {
    if (!p->used[c]) ++nf;
    else if (p->used[c] == 2 || !(b->h_cs[c].gen == p->gen[c] && b->h_cs[c].phase == PH_DONE)) ++nr;
  }
  if (n_free) *n_free = nf;
  if (n_running) *n_running = nr;
  return XG_OK;
}
