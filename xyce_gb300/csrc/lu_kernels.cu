// lu_kernels.cu — GPU numeric refactorisation and triangular solves of the
// Newton-solve LU, and the xg_lu_* C ABI.
//
// The reference refactors and solves with KLU on the host for every Newton
// iteration (N_LAS_AmesosSolver.C:405 NumericFactorization, :444 Solve).
// Here the pivot order and the filled L\U pattern come from the host analysis
// (lu_symbolic.cpp) and the numeric work runs on the GPU:
//
//  * refactor: row-wise ("up-looking") elimination of B = A(P, Q).  One warp
//    owns one row; rows are claimed in ascending order from a counter, and a
//    row waits (bounded polls of row k's U values and reciprocal pivot, which
//    hold a pending pattern until row k writes them) only for the rows k of
//    its L part, at the moment it reaches them.  Every row a warp waits for
//    was claimed earlier by a running warp, so the schedule always advances.
//    Rows far apart in the elimination order run concurrently; the row
//    pipeline needs no level barriers.  Each entry of a row is updated by one
//    lane in ascending k, so the result is the same on every run.  The
//    position in row i that each entry of U row k updates is precomputed on
//    the host (the update schedule, lu_build_updates), so an update is one
//    coalesced index load, one coalesced value load and one multiply-add.
//  * solves: the same claim/wait scheme by rows of L (forward) and of U
//    (backward, rows claimed in descending order), a fixed lane-strided
//    partial sum and a fixed shuffle tree per row; a row waits on the values
//    it needs themselves, which hold a pending pattern until written.  The
//    trailing rows of one or two per level go to the chain kernel, 32
//    columns at a time (lu_solve_chain, planned in lu_chain.h), and a long
//    row no other row waits for to a block of its own (lu_solve_long).
//  * precision: factors in FP64, or in FP32 with FP64 iterative refinement
//    (r = b - A x with the FP64 matrix, solve, x += d).
//
// Claim counters and pending patterns live in device memory and are reset by
// the kernel that precedes each phase, so a captured sequence can be replayed.
// Every spin has an iteration limit; a wait that gives up records bit 1 in the
// status word and the row is finished anyway, so a launch always ends.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <memory>
#include <string>

#include "xg.h"
#include "xg_internal.h"
#include "lu_chain.h"
#include "xg_lu.h"
#include "xg_smem.cuh"

namespace xg {
namespace {

enum Ctrl : int {
  C_CLAIM_F = 0, C_CLAIM_L, C_CLAIM_U, C_STATUS, C_BAD_ROW,
  // polls per wait before it gives up (kSpinLimit unless a caller lowers it);
  // 128 bytes past the counters, so their atomics do not evict it from L1
  C_SPIN = 32,
  C_N
};
enum Status : unsigned { ST_PIVOT = 1u, ST_TIMEOUT = 2u, ST_PATTERN = 4u };

constexpr int kSpinLimit = 1 << 20;  // default polls per wait (~0.1-0.5 s) before giving up

__device__ __forceinline__ unsigned ld_acquire(const unsigned *p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release(unsigned *p, unsigned v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

struct LuDev {
  int n;
  const int *rp, *ci, *diag;  // L\U pattern of B
  const int *lu2a;            // LU position -> A entry, -1 for fill
  const int *P, *Q;
  const int *arp, *aci;       // A pattern (CSR) for the residual
  const int64_t *urp;         // per row: start of its updates in upos
  const int *upos;            // per update: the position in the row it updates
  unsigned *ctrl;
  void *rdiag;                // 1 / U(k,k) per row, written by the refactor
  // grid solves: rows >= tail0 (a chain of one- or two-row levels) are
  // solved by the chain kernel (tail0 = n: none); per tail row {start,
  // first entry in a column >= tail0, diagonal, P}, and b(P(row)) less its
  // sum over columns < tail0
  int tail0;
  const int4 *tdesc;
  void *hpart;
  // per row: bit 0 its L part, bit 1 its U part, is longer than
  // kSolveLongRow and no other row of that solve reads its result (a supply
  // node's KCL row pivoted on its source's current): lu_solve_long sums it
  // with a block after the grid solve, which skips it
  const unsigned char *solo;
};

// The grid-wide kernels carry readiness in the value itself: before a
// refactor every reciprocal pivot, before a solve every entry of y and z,
// holds a signalling-NaN bit pattern, which no arithmetic produces (an
// invalid operation gives a quiet NaN); a row's result replaces it with one
// aligned store, and a row that needs it polls the value.  The solves need
// nothing else from the row, so relaxed accesses do; the refactor also reads
// the row's U part, so the pivot is stored with release after it and polled
// with acquire.
template <class T> struct Pending;
template <> struct Pending<double> {
  using U = unsigned long long;
  static constexpr U bits = 0x7FF4DEADBEEF0001ull;
};
template <> struct Pending<float> {
  using U = unsigned;
  static constexpr U bits = 0x7FA5DEADu;
};

__device__ __forceinline__ unsigned long long ld_relaxed(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_relaxed(const unsigned *p) {
  unsigned v;
  asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_relaxed(unsigned long long *p, unsigned long long v) {
  asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_relaxed(unsigned *p, unsigned v) {
  asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ double from_bits(unsigned long long v) { return __longlong_as_double((long long)v); }
__device__ __forceinline__ float from_bits(unsigned v) { return __uint_as_float(v); }
__device__ __forceinline__ unsigned long long to_bits(double v) {
  return (unsigned long long)__double_as_longlong(v);
}
__device__ __forceinline__ unsigned to_bits(float v) { return __float_as_uint(v); }

template <class T>
__device__ __forceinline__ void publish(T *p, T v) {
  st_relaxed(reinterpret_cast<typename Pending<T>::U *>(p), to_bits(v));
}

__device__ __forceinline__ unsigned long long ld_acq(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ unsigned ld_acq(const unsigned *p) { return ld_acquire(p); }
__device__ __forceinline__ void st_rel(unsigned long long *p, unsigned long long v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_rel(unsigned *p, unsigned v) { st_release(p, v); }

// The value at p once it is no longer pending, polled with acquire: what the
// writer stored before its release is visible after it.  Zero (and the
// timeout bit) if it never arrives.
template <class T>
__device__ T wait_value_acquire(const T *p, unsigned *ctrl) {
  using U = typename Pending<T>::U;
  const U *q = reinterpret_cast<const U *>(p);
  int it = 0;
  const int limit = int(__ldg(&ctrl[C_SPIN]));
  U v;
  while ((v = ld_acq(q)) == Pending<T>::bits) {
    ++it;
    if (it > limit ||
        ((it & 1023) == 0 && (*(volatile unsigned *)&ctrl[C_STATUS] & ST_TIMEOUT))) {
      atomicOr(&ctrl[C_STATUS], ST_TIMEOUT);
      return T(0);
    }
    if (it > 32) __nanosleep(64);
  }
  return from_bits(v);
}

template <class T>
__device__ __forceinline__ void publish_release(T *p, T v) {
  st_rel(reinterpret_cast<typename Pending<T>::U *>(p), to_bits(v));
}

// Scatter A into the L\U value array (fill entries zero), keep an FP64 copy of
// A for the residual, reset the claim counter and status, and mark every
// reciprocal pivot pending.  The positions set in `pending` (bit p % 32 of
// word p / 32: the U part right of the diagonal of every row the refactor
// stages) are marked pending too: those values carry their own readiness,
// and the row's warp takes its initial values from A.
template <class T>
__global__ void lu_assemble(LuDev d, const double *__restrict__ a, double *__restrict__ a_copy,
                            int64_t nnz_a, T *__restrict__ val, int64_t nnz_lu,
                            const unsigned *__restrict__ pending) {
  using U = typename Pending<T>::U;
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  const int64_t t0 = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t0 == 0) {
    d.ctrl[C_CLAIM_F] = 0;
    d.ctrl[C_STATUS] = 0;
    d.ctrl[C_BAD_ROW] = 0xffffffffu;
  }
  for (int64_t p = t0; p < nnz_lu; p += stride) {
    if ((__ldg(pending + (p >> 5)) >> (p & 31)) & 1u) {
      reinterpret_cast<U *>(val)[p] = Pending<T>::bits;
    } else {
      const int sa = d.lu2a[p];
      val[p] = sa >= 0 ? T(a[sa]) : T(0);
    }
  }
  if (a_copy != a)
    for (int64_t p = t0; p < nnz_a; p += stride) a_copy[p] = a[p];
  for (int64_t i = t0; i < d.n; i += stride) reinterpret_cast<U *>(d.rdiag)[i] = Pending<T>::bits;
}

// A warp's own row lives in shared memory while it is eliminated (rows up to
// `cap` entries, the matrix's longest row up to kStageBytes; longer ones stay
// in global memory): the multiplier of each L entry reads what the previous
// entries' updates wrote, and a shared-memory round trip is ~30 cycles where
// an L2 one is ~1 us.
constexpr int kStageBytes = 24 * 1024;
constexpr int kMinStageBytes = 4 * 1024;
constexpr int kUnstagedRows = 32;
constexpr int kFactorWarps = 8;

constexpr int kU = 4;  // pivot-row entries per lane in one chunk (128 a chunk)

// Readiness in the refactor.  The U part right of the diagonal of a staged
// row, and every reciprocal pivot, start pending and are each written once,
// final, with a relaxed store: a row that needs them polls the values
// themselves, so it has them one L2 round trip after they land and the
// writer needs no fence.  A row eliminated in place (longer than the stage)
// has A in its U part from the start: it stores its pivot with release after
// its U part, and a row that needs it polls the pivot with acquire before it
// loads the values.

// One L entry of the row being eliminated: its pivot row k, where k's U part
// right of the diagonal starts and how long it is, and whether those values
// carry their own readiness (k was staged).
struct PivotMeta {
  int k, q0, len, flagged;
};

__device__ __forceinline__ PivotMeta pivot_meta(const LuDev &d, int p, int dp, int cap) {
  PivotMeta m{0, 0, 0, 1};
  if (p < dp) {
    m.k = __ldg(d.ci + p);
    const int rs = __ldg(d.rp + m.k), dk = __ldg(d.diag + m.k), re = __ldg(d.rp + m.k + 1);
    m.q0 = dk + 1;
    m.len = re - m.q0;
    m.flagged = re - rs <= cap;
  }
  return m;
}

__device__ __forceinline__ PivotMeta shfl_meta(const PivotMeta &m, int src) {
  PivotMeta o;
  o.k = __shfl_sync(0xffffffffu, m.k, src);
  o.q0 = __shfl_sync(0xffffffffu, m.q0, src);
  o.len = __shfl_sync(0xffffffffu, m.len, src);
  o.flagged = __shfl_sync(0xffffffffu, m.flagged, src);
  return o;
}

// A chunk of a pivot row's U part: the positions in the row being eliminated
// that its entries update (-1: none) and, for a flagged row, the values as
// polled so far; lane 0 also holds the reciprocal pivot.
template <class T>
struct PivotChunk {
  int q[kU];
  typename Pending<T>::U v[kU];
  typename Pending<T>::U r;
};

// Loads (without waiting) the chunk of row m from entry j0 on; the pivot too
// when j0 is 0.  `up` points at the row's update positions.
template <class T>
__device__ __forceinline__ void pivot_fetch(const LuDev &d, const T *val, const PivotMeta &m,
                                            const int *up, int j0, int lane, PivotChunk<T> &c) {
  using U = typename Pending<T>::U;
  const U *vb = reinterpret_cast<const U *>(val) + m.q0;
#pragma unroll
  for (int r = 0; r < kU; ++r) {
    const int j = j0 + 32 * r + lane;
    c.q[r] = j < m.len ? __ldg(up + j) : -1;
    c.v[r] = m.flagged && j < m.len ? ld_relaxed(vb + j) : U(0);
  }
  c.r = m.flagged && j0 == 0 && lane == 0 ? ld_relaxed(reinterpret_cast<const U *>(d.rdiag) + m.k) : U(0);
}

// Polls a flagged chunk until none of its values (nor, with the pivot, lane
// 0's pivot) is pending; any that never arrive read as zero and set the
// timeout bit.  Every pending value is polled each time: they tend to land
// together, and one round trip then brings them all.
template <class T>
__device__ __forceinline__ void pivot_wait(const LuDev &d, const T *val, const PivotMeta &m, int j0,
                                           bool pivot, int lane, PivotChunk<T> &c) {
  using U = typename Pending<T>::U;
  const U *vb = reinterpret_cast<const U *>(val) + m.q0 + j0 + lane;
  const U *rp = reinterpret_cast<const U *>(d.rdiag) + m.k;
  const bool wp = pivot && lane == 0;
  const int limit = int(__ldg(&d.ctrl[C_SPIN]));
  for (int it = 1;; ++it) {
    bool pend = wp && c.r == Pending<T>::bits;
#pragma unroll
    for (int r = 0; r < kU; ++r) pend |= c.q[r] >= 0 && c.v[r] == Pending<T>::bits;
    if (!pend) break;
    if (it > limit ||
        ((it & 1023) == 0 && (*(volatile unsigned *)&d.ctrl[C_STATUS] & ST_TIMEOUT))) {
      atomicOr(&d.ctrl[C_STATUS], ST_TIMEOUT);
      if (wp && c.r == Pending<T>::bits) c.r = U(0);
#pragma unroll
      for (int r = 0; r < kU; ++r)
        if (c.v[r] == Pending<T>::bits) c.v[r] = U(0);
      break;
    }
    if (it > 32) __nanosleep(64);
    if (wp && c.r == Pending<T>::bits) c.r = ld_relaxed(rp);
#pragma unroll
    for (int r = 0; r < kU; ++r)
      if (c.q[r] >= 0 && c.v[r] == Pending<T>::bits) c.v[r] = ld_relaxed(vb + 32 * r);
  }
}

// row -= l * (U part of pivot row m), l = row[p] / U(k, k) stored at p; the
// first chunk comes from c (fetched an entry ahead), later ones (pivot rows
// with more than 256 entries right of the diagonal) are loaded here.  The
// target row and the pivot row are different rows: nothing aliases.
template <class T>
__device__ __forceinline__ void pivot_apply(const LuDev &d, const T *val, T *rb, int ro, int p,
                                            const PivotMeta &m, const int *up, int lane,
                                            PivotChunk<T> &c) {
  using U = typename Pending<T>::U;
  T rk = T(0);
  if (m.flagged) {
    pivot_wait(d, val, m, 0, true, lane, c);
    rk = from_bits(c.r);
  } else if (lane == 0) {
    rk = wait_value_acquire((const T *)d.rdiag + m.k, d.ctrl);
  }
  rk = __shfl_sync(0xffffffffu, rk, 0);
  if (!m.flagged) {
    // values of a row eliminated in place: after its pivot's acquire
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      const int j = 32 * r + lane;
      c.v[r] = j < m.len ? to_bits(__ldcg(val + m.q0 + j)) : U(0);
    }
  }
  const T l = rb[p - ro] * rk;
  __syncwarp();
  if (lane == 0) rb[p - ro] = l;
  // a step no lane has is skipped by the warp (m.len is the same in every
  // lane): an FP64 instruction costs its issue slot however few lanes it has
#pragma unroll
  for (int r = 0; r < kU; ++r) {
    if (32 * r >= m.len) break;
    if (c.q[r] >= 0) rb[c.q[r] - ro] -= l * from_bits(c.v[r]);
  }
  for (int j0 = 32 * kU; j0 < m.len; j0 += 32 * kU) {
    PivotChunk<T> e;
    pivot_fetch(d, val, m, up, j0, lane, e);
    if (m.flagged) {
      pivot_wait(d, val, m, j0, false, lane, e);
    } else {
#pragma unroll
      for (int r = 0; r < kU; ++r) {
        const int j = j0 + 32 * r + lane;
        e.v[r] = j < m.len ? to_bits(__ldcg(val + m.q0 + j)) : U(0);
      }
    }
#pragma unroll
    for (int r = 0; r < kU; ++r) {
      if (j0 + 32 * r >= m.len) break;
      if (e.q[r] >= 0) rb[e.q[r] - ro] -= l * from_bits(e.v[r]);
    }
  }
}

// Eliminate row `row` in rb (row entry p at rb[p - ro]).  The metadata of the
// row's L entries is loaded 32 at a time, one entry per lane, the next 32 in
// flight behind them; the next entry's first chunk is in flight while the
// current entry is applied.
template <class T>
__device__ __forceinline__ void eliminate(const LuDev &d, const T *val, T *rb, int ro, int s,
                                          int dp, const int *up, int cap, int lane) {
  const int nl = dp - s;
  if (nl <= 0) return;
  PivotMeta mc = pivot_meta(d, s + lane, dp, cap);
  PivotMeta mn = pivot_meta(d, s + 32 + lane, dp, cap);
  PivotMeta cur = shfl_meta(mc, 0);
  PivotChunk<T> cc, cn;
  pivot_fetch(d, val, cur, up, 0, lane, cc);
  for (int j = 0; j < nl; ++j) {
    const int *ucur = up;
    up += cur.len;
    PivotMeta nxt = cur;
    const bool more = j + 1 < nl;
    if (more) {
      const int jn = j + 1;
      if ((jn & 31) == 0) {
        mc = mn;
        mn = pivot_meta(d, s + jn + 32 + lane, dp, cap);
      }
      nxt = shfl_meta(mc, jn & 31);
      pivot_fetch(d, val, nxt, up, 0, lane, cn);
    }
    pivot_apply(d, val, rb, ro, s + j, cur, ucur, lane, cc);
    __syncwarp();
    if (more) {
      cur = nxt;
      cc = cn;
    }
  }
}

template <class T>
__global__ void __launch_bounds__(32 * kFactorWarps) lu_factor(LuDev d, T *val, const double *__restrict__ a,
                                                               int cap) {
  extern __shared__ __align__(16) unsigned char stage_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  T *stage = reinterpret_cast<T *>(stage_raw) + size_t(wid) * cap;
  T *rdiag = (T *)d.rdiag;
  while (true) {
    int row = 0;
    if (lane == 0) row = int(atomicAdd(&d.ctrl[C_CLAIM_F], 1u));
    row = __shfl_sync(0xffffffffu, row, 0);
    if (row >= d.n) break;
    const int s = __ldg(d.rp + row), dp = __ldg(d.diag + row), e = __ldg(d.rp + row + 1);
    const int *up = d.upos + __ldg(d.urp + row);
    const bool staged = e - s <= cap;
    T u;
    if (staged) {
      // the U part right of the diagonal is pending in val: its values come from A
      for (int p = s + lane; p < e; p += 32) {
        T v;
        if (p > dp) {
          const int sa = __ldg(d.lu2a + p);
          v = sa >= 0 ? T(a[sa]) : T(0);
        } else {
          v = val[p];
        }
        stage[p - s] = v;
      }
      __syncwarp();
      eliminate(d, val, stage, s, s, dp, up, cap, lane);
      for (int p = s + lane; p < e; p += 32) {
        if (p > dp)
          publish(val + p, stage[p - s]);
        else
          val[p] = stage[p - s];
      }
      __syncwarp();
      u = stage[dp - s];
    } else {
      eliminate(d, val, val, 0, s, dp, up, cap, lane);
      u = val[dp];
    }
    if (lane == 0) {
      if (!(fabs(double(u)) > 0.0) || !isfinite(double(u))) {
        atomicOr(&d.ctrl[C_STATUS], ST_PIVOT);
        atomicMin(&d.ctrl[C_BAD_ROW], unsigned(row));
      }
      if (staged) {
        publish(rdiag + row, T(1) / u);
      } else {
        __threadfence();
        publish_release(rdiag + row, T(1) / u);
      }
    }
  }
}

// Opens a solve: row claims restart, y and z become pending.
template <class T>
__global__ void lu_solve_open(LuDev d, T *y, T *z) {
  const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
  if (t0 == 0) {
    d.ctrl[C_CLAIM_L] = 0;
    d.ctrl[C_CLAIM_U] = 0;
  }
  using U = typename Pending<T>::U;
  for (int i = t0; i < d.n; i += gridDim.x * blockDim.x) {
    reinterpret_cast<U *>(y)[i] = Pending<T>::bits;
    reinterpret_cast<U *>(z)[i] = Pending<T>::bits;
  }
}

// The grid solves hold this many entries per lane of a row (128 a row) and
// wait for their inputs together: the loads of a row's entries, and the
// polls of the values they multiply, are all in flight at once, so a row
// costs about two L2 round trips after its last input lands, not two per
// 32 entries.
constexpr int kSolveHeld = 4;

// Waits for x[k[r]] (k[r] < 0: none, reads as zero) with every poll in
// flight together, polling again only those still pending; zero for any
// that never arrive (and the timeout bit).
template <class T, int K>
__device__ __forceinline__ void wait_values(const T *x, const int (&k)[K], T (&v)[K], unsigned *ctrl) {
  using U = typename Pending<T>::U;
  const U *q = reinterpret_cast<const U *>(x);
  U b[K];
#pragma unroll
  for (int r = 0; r < K; ++r) b[r] = k[r] >= 0 ? ld_relaxed(q + k[r]) : U(0);
  const int limit = int(__ldg(&ctrl[C_SPIN]));
  for (int it = 1;; ++it) {
    bool pend = false;
#pragma unroll
    for (int r = 0; r < K; ++r) pend |= b[r] == Pending<T>::bits;
    if (!pend) break;
    if (it > limit || ((it & 1023) == 0 && (*(volatile unsigned *)&ctrl[C_STATUS] & ST_TIMEOUT))) {
      atomicOr(&ctrl[C_STATUS], ST_TIMEOUT);
#pragma unroll
      for (int r = 0; r < K; ++r)
        if (b[r] == Pending<T>::bits) b[r] = U(0);
      break;
    }
    if (it > 32) __nanosleep(64);
#pragma unroll
    for (int r = 0; r < K; ++r)
      if (b[r] == Pending<T>::bits) b[r] = ld_relaxed(q + k[r]);
  }
#pragma unroll
  for (int r = 0; r < K; ++r) v[r] = from_bits(b[r]);
}

// Rows with more entries than this in a solve's part, that no other row of
// that solve waits for, are summed by a block of their own after it.
constexpr int kSolveLongRow = 4096;
constexpr int kLongThreads = 1024;

// A lane's share of sum over p in [p0, p1) of val[p] * x[ci[p]]: entries
// p0 + lane, p0 + lane + 32, ... in ascending order, kSolveHeld of them
// loaded and waited for at a time.  Lanes go at their own pace (no vote per
// step): a lane whose inputs have landed runs ahead to its next entries
// while others still wait.
template <class T>
__device__ __forceinline__ T lane_dot(const LuDev &d, const T *__restrict__ val, const T *x, int p0,
                                      int p1, int lane) {
  T acc = T(0);
  for (int p = p0 + lane; p < p1; p += 32 * kSolveHeld) {
    int k[kSolveHeld];
    T a[kSolveHeld], xv[kSolveHeld];
#pragma unroll
    for (int r = 0; r < kSolveHeld; ++r) {
      const int q = p + 32 * r;
      k[r] = q < p1 ? __ldg(d.ci + q) : -1;
      a[r] = q < p1 ? __ldcg(val + q) : T(0);
    }
    wait_values(x, k, xv, d.ctrl);
#pragma unroll
    for (int r = 0; r < kSolveHeld; ++r)
      if (k[r] >= 0) acc += a[r] * xv[r];
  }
  return acc;
}

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// y = L \ b(P)   (unit lower triangular, rows ascending)
template <class T>
__global__ void __launch_bounds__(256) lu_lsolve(LuDev d, const T *__restrict__ val,
                                                 const double *__restrict__ b, T *y) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int row = 0;
    if (lane == 0) row = int(atomicAdd(&d.ctrl[C_CLAIM_L], 1u));
    row = __shfl_sync(0xffffffffu, row, 0);
    if (row >= d.n) break;
    const int s = __ldg(d.rp + row), dp = __ldg(d.diag + row);
    if (row >= d.tail0) {
      // a row of the chain: b(P(row)) less its sum over the entries in
      // columns below tail0; the chain kernel starts from it
      const int sp = d.tdesc[row - d.tail0].y;
      const T bi = lane == 0 ? T(b[__ldg(d.P + row)]) : T(0);
      const T acc = warp_sum(lane_dot(d, val, y, s, sp, lane));
      if (lane == 0) reinterpret_cast<T *>(d.hpart)[row - d.tail0] = bi - acc;
      continue;
    }
    if (dp - s > kSolveLongRow && (__ldg(d.solo + row) & 1)) continue;  // lu_solve_long's
    const T bi = lane == 0 ? T(b[__ldg(d.P + row)]) : T(0);  // before any wait
    const T acc = warp_sum(lane_dot(d, val, y, s, dp, lane));
    if (lane == 0) publish(y + row, bi - acc);
  }
}

// z = U \ y, x(Q) = z   (rows descending)
template <class T>
__global__ void __launch_bounds__(256) lu_usolve(LuDev d, const T *__restrict__ val,
                                                 const T *__restrict__ y, T *z, double *x) {
  const int lane = threadIdx.x & 31;
  while (true) {
    int c = 0;
    if (lane == 0) c = int(atomicAdd(&d.ctrl[C_CLAIM_U], 1u));
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= d.tail0) break;
    const int row = d.tail0 - 1 - c;  // rows from tail0 on are solved already
    const int dp = __ldg(d.diag + row), e = __ldg(d.rp + row + 1);
    if (e - dp - 1 > kSolveLongRow && (__ldg(d.solo + row) & 2)) continue;  // lu_solve_long's
    const T yi = lane == 0 ? __ldcg(y + row) : T(0);
    const T ri = lane == 0 ? __ldcg((const T *)d.rdiag + row) : T(0);
    const int qi = lane == 0 ? __ldg(d.Q + row) : 0;
    const T acc = warp_sum(lane_dot(d, val, z, dp + 1, e, lane));
    if (lane == 0) {
      const T zi = (yi - acc) * ri;
      publish(z + row, zi);
      x[qi] = double(zi);
    }
  }
}

// The rows the grid solves skip (solo): a block per row, every input final
// (the grid solve before it has ended).  Each thread sums its entries
// p0 + t, p0 + t + kLongThreads, ... in order, then a fixed tree: the same
// result on every run.  upper = 0: y(row) = b(P(row)) - L(row,:) y;
// upper = 1: z(row) = (y(row) - U(row,:) z) / U(row,row), x(Q(row)) = z(row).
template <class T>
__global__ void __launch_bounds__(kLongThreads) lu_solve_long(LuDev d, const T *__restrict__ val,
                                                              const double *__restrict__ b, T *y, T *z,
                                                              double *x, const int *__restrict__ rows,
                                                              int upper) {
  __shared__ T part[kLongThreads / 32];
  const int row = rows[blockIdx.x];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int dp = __ldg(d.diag + row);
  const int p0 = upper ? dp + 1 : __ldg(d.rp + row);
  const int p1 = upper ? __ldg(d.rp + row + 1) : dp;
  const T *x_in = upper ? z : y;
  T acc = T(0);
  for (int p = p0 + t; p < p1; p += kLongThreads) acc += __ldcg(val + p) * __ldcg(x_in + __ldg(d.ci + p));
  acc = warp_sum(acc);
  if (lane == 0) part[w] = acc;
  __syncthreads();
  if (w == 0) {
    acc = lane < kLongThreads / 32 ? part[lane] : T(0);
    acc = warp_sum(acc);
    if (lane == 0) {
      if (upper) {
        const T zi = (__ldcg(y + row) - acc) * __ldcg((const T *)d.rdiag + row);
        z[row] = zi;
        x[__ldg(d.Q + row)] = double(zi);
      } else {
        y[row] = T(b[__ldg(d.P + row)]) - acc;
      }
    }
  }
}

// The chain at the end of a factor whose last rows each form their own
// level (a supply node and what hangs on it, or the dense block the order
// leaves last): grid-wide, every row would cost an L2 round trip for its
// dependencies.  Here one warp solves the chain 32 columns at a time, both
// ways, with the rows' running sums in shared memory (the plan is
// build_chain_plan in lu_chain.h):
//  * the block's own 32 x 32 triangle: lane i holds row i's sum and its
//    triangle row in registers; at step t lane t's value is final (times its
//    reciprocal pivot going backward) and goes to the other lanes by a
//    shuffle, each subtracting its multiple: a shuffle and a multiply-add
//    per column on the critical path;
//  * the block's entries in rows outside it, in rounds of 32 (a row per
//    lane, a lane's rows in turn), each row's sum read once and written once.
// Every row's sum takes its updates in the column order of a
// column-by-column solve, the same on every run.  Tiles and rounds are
// copied global -> shared by the bulk copy engine (cp.async.bulk, an
// mbarrier counting each copy's bytes) into rings, refilled as the warp
// passes them, so the warp does not wait on loads.
constexpr int kChainTileRing = 3;
constexpr int kChainChunks = 8;
constexpr int kChainEntChunk = 256;  // entries (8 rounds) per chunk

__host__ __device__ constexpr size_t chain_tile_bytes(size_t tsz) {
  return size_t(kChainTileValues) * tsz + kChainBlock * sizeof(int);
}

// Per refactor: each entry's value and each tile's triangle and reciprocal
// pivots from the factor.
template <class T>
__global__ void lu_chain_gather(LuDev d, const T *__restrict__ val, const int *__restrict__ ent_src,
                                T *__restrict__ ent_val, int64_t n_ent, const int *__restrict__ tile_src,
                                unsigned char *__restrict__ tiles, int n_blk) {
  const int64_t stride = int64_t(gridDim.x) * blockDim.x;
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  for (int64_t j = t; j < n_ent; j += stride) {
    const int p = __ldg(ent_src + j);
    ent_val[j] = p >= 0 ? __ldcg(val + p) : T(0);
  }
  const int64_t n_tv = int64_t(n_blk) * kChainTileValues;
  for (int64_t j = t; j < n_tv; j += stride) {
    const int p = __ldg(tile_src + j);
    const T v = p >= 0 ? __ldcg(val + p) : p == -1 ? T(0) : __ldcg((const T *)d.rdiag + (-2 - p));
    T *tv = reinterpret_cast<T *>(tiles + size_t(j / kChainTileValues) * chain_tile_bytes(sizeof(T)));
    tv[j % kChainTileValues] = v;
  }
}

struct ChainDev {
  const int4 *blk;             // ChainBlock per block: forward, then backward
  int n_blk;
  const unsigned char *tiles;  // per block chain_tile_bytes: triangle, pivots (T), x positions
  const int *ent_rowj;         // per entry (row << 5) | lane-column; whole chunks
  const void *ent_val;         // T per entry
  int64_t n_ent;               // entries, whole chunks
};

__device__ __forceinline__ unsigned smem_addr(const void *p) {
  return unsigned(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Polls the barrier's phase `parity` to completion, at most `limit` times.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, int limit) {
  for (int it = 0; it < limit; ++it)
    if (mbar_try(bar, parity)) return true;
  return false;
}
// One thread: `bytes` from global src to shared dst, counted on barrier mb
// (whose transaction count the caller has raised by them).
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, unsigned bytes, unsigned mb) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(mb)
               : "memory");
}
__device__ __forceinline__ void expect_bytes(unsigned mb, unsigned bytes) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(bytes) : "memory");
}

template <class T>
__global__ void __launch_bounds__(kChainLanes) lu_solve_chain(LuDev d, ChainDev c, T *y, T *z, double *x) {
  extern __shared__ __align__(128) unsigned char chain_raw[];
  constexpr int kE = kChainChunks * kChainEntChunk;
  constexpr int kRoundsPerChunk = kChainEntChunk / kChainLanes;
  constexpr unsigned kTile = unsigned(chain_tile_bytes(sizeof(T)));
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int t0 = d.tail0, nt = d.n - t0;
  // rings (tiles, entry rows, entry values), the block's values, barriers,
  // then the running sums (nt + scratch)
  unsigned char *ring_tile = chain_raw;
  int *ring_rowj = reinterpret_cast<int *>(ring_tile + kChainTileRing * kTile);
  T *ring_val = reinterpret_cast<T *>(ring_rowj + kE);
  T *vb = ring_val + kE;
  unsigned long long *bar_t = reinterpret_cast<unsigned long long *>(vb + kChainBlock);
  unsigned long long *bar_e = bar_t + kChainTileRing;
  T *acc = reinterpret_cast<T *>(bar_e + kChainChunks);
  const int limit = int(__ldg(&d.ctrl[C_SPIN]));
  const int n_ech = int(c.n_ent / kChainEntChunk);
  const T *cval = (const T *)c.ent_val;

  // thread 0 refills a ring slot with tile / entry chunk k
  auto issue_tile = [&](int k) {
    if (tid == 0 && k < c.n_blk) {
      const unsigned mb = smem_addr(bar_t + k % kChainTileRing);
      expect_bytes(mb, kTile);
      bulk_copy(ring_tile + (k % kChainTileRing) * kTile, c.tiles + size_t(k) * kTile, kTile, mb);
    }
  };
  auto issue_ent = [&](int k) {
    if (tid == 0 && k < n_ech) {
      const int s = k % kChainChunks;
      const unsigned mb = smem_addr(bar_e + s);
      expect_bytes(mb, unsigned(kChainEntChunk * (sizeof(int) + sizeof(T))));
      bulk_copy(ring_rowj + s * kChainEntChunk, c.ent_rowj + size_t(k) * kChainEntChunk,
                unsigned(kChainEntChunk * sizeof(int)), mb);
      bulk_copy(ring_val + s * kChainEntChunk, cval + size_t(k) * kChainEntChunk,
                unsigned(kChainEntChunk * sizeof(T)), mb);
    }
  };

  if (tid == 0) {
    for (int i = 0; i < kChainTileRing + kChainChunks; ++i)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar_t + i)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  for (int k = 0; k < kChainTileRing; ++k) issue_tile(k);
  for (int k = 0; k < kChainChunks; ++k) issue_ent(k);
  // the sums start from b(P(row)) minus the row's sum over columns < t0
  // (the grid lower solve's)
  const T *h = reinterpret_cast<const T *>(d.hpart);
#pragma unroll 8
  for (int r = tid; r < nt; r += kChainLanes) acc[r] = __ldcg(h + r);
  if (tid == 0) acc[nt] = T(0);
  __syncthreads();

  // block records: lane j of every warp holds block w + j's, and the next
  // window's
  int w = 0;
  int4 ba = lane < c.n_blk ? c.blk[lane] : make_int4(0, 0, 0, 0);
  int4 bb = 32 + lane < c.n_blk ? c.blk[32 + lane] : make_int4(0, 0, 0, 0);
  bool ok = true;    // the same in every thread: each decision is a block vote
  int gk = 0;        // rounds done, all blocks
  int ent_wait = 0;  // entry chunks waited for
  int ent_free = 0;  // entry chunks passed (and refilled)
  int blk = 0;
  for (; blk < c.n_blk; ++blk) {
    if (blk - w == 32) {
      w += 32;
      ba = bb;
      bb = w + 32 + lane < c.n_blk ? c.blk[w + 32 + lane] : make_int4(0, 0, 0, 0);
    }
    const int cbase = __shfl_sync(0xffffffffu, ba.x, blk - w);
    const int bs = __shfl_sync(0xffffffffu, ba.y, blk - w);
    const int rounds = __shfl_sync(0xffffffffu, ba.z, blk - w);
    const bool upper = __shfl_sync(0xffffffffu, ba.w, blk - w) != 0;
    // the triangle (warp 0): lane i is row i of the block
    bool fail = false;
    if (warp == 0) {
      fail = !mbar_wait(smem_addr(bar_t + blk % kChainTileRing), unsigned(blk / kChainTileRing) & 1u, limit);
      if (!__any_sync(0xffffffffu, fail)) {
        const T *tri = reinterpret_cast<const T *>(ring_tile + (blk % kChainTileRing) * kTile);
        const int col = upper ? cbase - lane : cbase + lane;
        T a = lane < bs ? acc[col] : T(0);
        T row[kChainBlock];
#pragma unroll
        for (int j = 0; j < kChainBlock; ++j) row[j] = tri[j * kChainBlock + lane];
        const T rdl = upper ? tri[kChainBlock * kChainBlock + lane] : T(1);
        const int ql = reinterpret_cast<const int *>(tri + kChainTileValues)[lane];
#pragma unroll
        for (int t = 0; t < kChainBlock; ++t) {
          if (t < bs) {
            if (upper && lane == t) a *= rdl;
            const T vt = __shfl_sync(0xffffffffu, a, t);
            if (lane > t) a -= row[t] * vt;
          }
        }
        if (lane < bs) {
          if (upper) {
            z[t0 + col] = a;
            x[ql] = double(a);
          } else {
            y[t0 + col] = a;
            acc[col] = a;
          }
        }
        vb[lane] = a;
      }
    }
    if (__syncthreads_or(fail)) {
      ok = false;
      break;
    }
    issue_tile(blk + kChainTileRing);
    // the block's entries in rows outside it, four rounds at a time with
    // their loads first (each thread's multiply-adds depend on one another)
    int cur = -1;
    T ar = T(0);
    for (int k0 = 0; k0 < rounds; k0 += 4) {
      const int nq = min(4, rounds - k0);
      const int need = (gk + nq - 1) / kRoundsPerChunk;
      bool bad = false;
      while (!bad && ent_wait <= need) {
        bad = !mbar_wait(smem_addr(bar_e + ent_wait % kChainChunks), unsigned(ent_wait / kChainChunks) & 1u, limit);
        ++ent_wait;
      }
      if (__syncthreads_or(bad)) {
        ok = false;
        break;
      }
      int rj[4];
      T wv[4], vv[4];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        rj[q] = nt << 5;
        wv[q] = T(0);
        if (q < nq) {
          const int e = ((gk + q) * kChainLanes + tid) & (kE - 1);
          rj[q] = ring_rowj[e];
          wv[q] = ring_val[e];
        }
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) vv[q] = vb[rj[q] & 31];
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        if (q < nq) {
          const int r = rj[q] >> 5;
          if (r != cur) {
            if (cur >= 0) acc[cur] = ar;
            ar = acc[r];
            cur = r;
          }
          ar -= wv[q] * vv[q];
        }
      }
      gk += nq;
      // refill the chunks these rounds finished (every thread past them)
      if (ent_free < gk / kRoundsPerChunk) {
        __syncthreads();
        while (ent_free < gk / kRoundsPerChunk) {
          issue_ent(ent_free + kChainChunks);
          ++ent_free;
        }
      }
    }
    if (cur >= 0) acc[cur] = ar;
    __syncthreads();
    if (!ok) break;
  }
  if (!ok) {
    // a copy that did not complete in time: report it, and let the copies
    // still in flight land before the block's shared memory is released
    if (tid == 0) {
      atomicOr(&d.ctrl[C_STATUS], ST_TIMEOUT);
      for (int k = blk; k < min(c.n_blk, blk + kChainTileRing + 1); ++k)
        mbar_wait(smem_addr(bar_t + k % kChainTileRing), unsigned(k / kChainTileRing) & 1u, 1 << 22);
      for (int k = max(ent_wait - 1, 0); k < min(n_ech, ent_free + kChainChunks); ++k)
        mbar_wait(smem_addr(bar_e + k % kChainChunks), unsigned(k / kChainChunks) & 1u, 1 << 22);
    }
    __syncthreads();
  }
}

// r = b - A x   (FP64, one thread per row, entries in CSR order)
__global__ void lu_residual(LuDev d, const double *__restrict__ a, const double *__restrict__ x,
                            const double *__restrict__ b, double *__restrict__ r) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < d.n; i += gridDim.x * blockDim.x) {
    const int p0 = __ldg(d.arp + i), p1 = __ldg(d.arp + i + 1);
    double acc = b[i];
    for (int p = p0; p < p1; ++p) acc -= a[p] * x[__ldg(d.aci + p)];
    r[i] = acc;
  }
}

__global__ void lu_axpy(int n, const double *__restrict__ dx, double *__restrict__ x) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    x[i] += dx[i];
}

template <class T>
struct SmemLU {
  T *val;
  volatile T *y;              // solve vector (forward result, then backward)
  T *rd;                      // reciprocal pivots (one-lane solve)
  int *ci, *rp, *diag;
  volatile int *flag, *flag_u;
};

// Shared-memory layout, the same for factor and solve:
// [val: T x nnz | y: T x n | rd: T x n | ci: nnz | rp: n+1 | diag: n | flag: n | flag_u: n]
// with the T arrays each padded to 16 bytes.
__host__ __device__ inline size_t smem_bytes(int n, int64_t nnz, size_t tsz) {
  auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
  return a16(tsz * size_t(nnz)) + 2 * a16(tsz * size_t(n)) +
         sizeof(int) * (size_t(nnz) + 4 * size_t(n) + 1);
}
template <class T>
__device__ SmemLU<T> smem_layout(char *base, int n, int64_t nnz) {
  auto a16 = [](size_t v) { return (v + 15) & ~size_t(15); };
  SmemLU<T> L;
  size_t off = 0;
  L.val = (T *)(base + off);
  off += a16(sizeof(T) * size_t(nnz));
  L.y = (volatile T *)(base + off);
  off += a16(sizeof(T) * size_t(n));
  L.rd = (T *)(base + off);
  off += a16(sizeof(T) * size_t(n));
  L.ci = (int *)(base + off);
  off += sizeof(int) * size_t(nnz);
  L.rp = (int *)(base + off);
  off += sizeof(int) * size_t(n + 1);
  L.diag = (int *)(base + off);
  off += sizeof(int) * size_t(n);
  L.flag = (volatile int *)(base + off);
  off += sizeof(int) * size_t(n);
  L.flag_u = (volatile int *)(base + off);
  return L;
}

// ---- narrow matrices: one lane walks the rows in order --------------------------
// When the elimination has little row parallelism (a chain of inverters, a
// ring: at most a few rows per level), handing rows between warps costs more
// than the rows themselves.  One warp loads the factor into shared memory and
// lane 0 factors, then solves, row after row with no flags at all.

// 1/u by Newton-Raphson on the reciprocal (x <- x (2 - u x), each step
// doubling the correct bits) from a single-precision seed; IEEE division
// outside the range where the seed is representable.  Within 1 ulp of 1/u.
template <class T>
__device__ __forceinline__ T recip(T u) {
  const double a = fabs(double(u));
  if (!(a > 1e-30 && a < 1e30)) return T(1) / u;
  double x = double(1.0f / float(u));
  x = x * (2.0 - double(u) * x);
  x = x * (2.0 - double(u) * x);
  return T(x);
}

constexpr int kSeqThreads = 512;  // for the copies in and out; thread 0 does the walk

template <class T>
__global__ void __launch_bounds__(kSeqThreads) lu_factor_seq(LuDev d, const double *__restrict__ a,
                                                    double *__restrict__ a_copy, int64_t nnz_a,
                                                    T *__restrict__ val_out, int64_t nnz) {
  extern __shared__ __align__(16) char smem[];
  SmemLU<T> L = smem_layout<T>(smem, d.n, nnz);
  const int n = d.n;
  if (threadIdx.x == 0) {
    d.ctrl[C_STATUS] = 0;
    d.ctrl[C_BAD_ROW] = 0xffffffffu;
  }
  for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) {
    const int s = d.lu2a[p];
    L.val[p] = s >= 0 ? T(a[s]) : T(0);
    L.ci[p] = d.ci[p];
  }
  for (int i = threadIdx.x; i <= n; i += blockDim.x) L.rp[i] = d.rp[i];
  for (int i = threadIdx.x; i < n; i += blockDim.x) L.diag[i] = d.diag[i];
  if (a_copy != a)
    for (int64_t p = threadIdx.x; p < nnz_a; p += blockDim.x) a_copy[p] = a[p];
  __syncthreads();
  if (threadIdx.x == 0) {
    T *rd = (T *)L.y;
    int bad = -1;
    const int *up = d.upos;
    for (int row = 0; row < n; ++row) {
      const int s = L.rp[row], dp = L.diag[row];
      for (int p = s; p < dp; ++p) {
        const int k = L.ci[p];
        const T l = L.val[p] * rd[k];
        L.val[p] = l;
        const int q0 = L.diag[k] + 1, len = L.rp[k + 1] - q0;
        for (int j = 0; j < len; ++j) L.val[__ldg(up + j)] -= l * L.val[q0 + j];
        up += len;
      }
      const T u = L.val[dp];
      if (!(fabs(double(u)) > 0.0) || !isfinite(double(u))) {
        if (bad == -1) bad = row;
      }
      rd[row] = recip(u);
    }
    if (bad >= 0) {
      atomicOr(&d.ctrl[C_STATUS], ST_PIVOT);
      d.ctrl[C_BAD_ROW] = unsigned(bad);
    }
  }
  __syncthreads();
  for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) val_out[p] = L.val[p];
  for (int i = threadIdx.x; i < n; i += blockDim.x) ((T *)d.rdiag)[i] = L.y[i];
}

template <class T>
__global__ void __launch_bounds__(kSeqThreads) lu_solve_seq(LuDev d, const T *__restrict__ val, int64_t nnz,
                                                   const double *__restrict__ b,
                                                   double *__restrict__ x) {
  extern __shared__ __align__(16) char smem[];
  SmemLU<T> L = smem_layout<T>(smem, d.n, nnz);
  const int n = d.n;
  T *y = (T *)L.y;
  for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) {
    L.val[p] = val[p];
    L.ci[p] = d.ci[p];
  }
  for (int i = threadIdx.x; i <= n; i += blockDim.x) L.rp[i] = d.rp[i];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    L.diag[i] = d.diag[i];
    y[i] = T(b[d.P[i]]);
    L.rd[i] = ((const T *)d.rdiag)[i];
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int row = 0; row < n; ++row) {
      T acc = y[row];
      for (int p = L.rp[row]; p < L.diag[row]; ++p) acc -= L.val[p] * y[L.ci[p]];
      y[row] = acc;
    }
    for (int row = n - 1; row >= 0; --row) {
      T acc = y[row];
      for (int p = L.diag[row] + 1; p < L.rp[row + 1]; ++p) acc -= L.val[p] * y[L.ci[p]];
      y[row] = acc * L.rd[row];
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[d.Q[i]] = double(y[i]);
}

// ---- small matrices: the whole factorisation or solve in one CTA ---------------
// When the L\U values, columns, row pointers and flags fit in shared memory,
// one CTA of 32 warps runs the same row-claim schedule with its flags in shared
// memory: a dependency costs a shared-memory poll instead of an L2 round trip
// between SMs.  Chains of dependent rows (an inverter chain is one) are the
// case this serves.

constexpr int kCtaThreads = 1024;

// Spin on a shared-memory flag; after a few polls back off with a short
// sleep so waiting warps leave the issue slots to the warp they wait for.
__device__ __forceinline__ bool wait_flag_smem(volatile int *flag, unsigned *ctrl) {
  int it = 0;
  const int limit = int(__ldg(&ctrl[C_SPIN]));
  while (*flag == 0) {
    if (++it > limit) {
      atomicOr(&ctrl[C_STATUS], ST_TIMEOUT);
      return false;
    }
    if (it > 4) __nanosleep(20);
  }
  __threadfence_block();
  return true;
}

template <class T>
__global__ void __launch_bounds__(kCtaThreads) lu_factor_cta(LuDev d, const double *__restrict__ a,
                                                             double *__restrict__ a_copy, int64_t nnz_a,
                                                             T *__restrict__ val_out, int64_t nnz) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int claim;
  SmemLU<T> L = smem_layout<T>(smem, d.n, nnz);
  const int n = d.n;
  if (threadIdx.x == 0) {
    claim = 0;
    d.ctrl[C_STATUS] = 0;
    d.ctrl[C_BAD_ROW] = 0xffffffffu;
  }
  for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) {
    const int s = d.lu2a[p];
    L.val[p] = s >= 0 ? T(a[s]) : T(0);
    L.ci[p] = d.ci[p];
  }
  for (int i = threadIdx.x; i <= n; i += blockDim.x) L.rp[i] = d.rp[i];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    L.diag[i] = d.diag[i];
    L.flag[i] = 0;
  }
  if (a_copy != a)
    for (int64_t p = threadIdx.x; p < nnz_a; p += blockDim.x) a_copy[p] = a[p];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  while (true) {
    int row = 0;
    if (lane == 0) row = atomicAdd(&claim, 1);
    row = __shfl_sync(0xffffffffu, row, 0);
    if (row >= n) break;
    const int s = L.rp[row], dp = L.diag[row];
    const int *up = d.upos + __ldg(d.urp + row);
    for (int p = s; p < dp; ++p) {
      const int k = L.ci[p];
      if (lane == 0) wait_flag_smem(L.flag + k, d.ctrl);
      __syncwarp();
      __threadfence_block();
      const int q0 = L.diag[k] + 1, len = L.rp[k + 1] - q0;
      const T l = L.val[p] * L.y[k];
      __syncwarp();
      if (lane == 0) L.val[p] = l;
      for (int j = lane; j < len; j += 32) L.val[__ldg(up + j)] -= l * L.val[q0 + j];
      up += len;
      __syncwarp();
    }
    if (lane == 0) {
      const T u = L.val[dp];
      if (!(fabs(double(u)) > 0.0) || !isfinite(double(u))) {
        atomicOr(&d.ctrl[C_STATUS], ST_PIVOT);
        atomicMin(&d.ctrl[C_BAD_ROW], unsigned(row));
      }
      L.y[row] = T(1) / u;  // the reciprocal pivot, used by later rows and the solves
      __threadfence_block();
      L.flag[row] = 1;
    }
  }
  __syncthreads();
  for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) val_out[p] = L.val[p];
  for (int i = threadIdx.x; i < n; i += blockDim.x) ((T *)d.rdiag)[i] = L.y[i];
}

// x(Q) = U \ (L \ b(P)) in one CTA; y and z share one shared-memory vector.
template <class T>
__global__ void __launch_bounds__(kCtaThreads) lu_solve_cta(LuDev d, const T *__restrict__ val,
                                                            int64_t nnz, const double *__restrict__ b,
                                                            double *__restrict__ x) {
  extern __shared__ __align__(16) char smem[];
  __shared__ int claim_l, claim_u;
  SmemLU<T> L = smem_layout<T>(smem, d.n, nnz);
  const int n = d.n;
  volatile T *y = L.y;
  volatile int *flag_u = L.flag_u;
  if (threadIdx.x == 0) {
    claim_l = 0;
    claim_u = 0;
  }
  for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) {
    L.val[p] = val[p];
    L.ci[p] = d.ci[p];
  }
  for (int i = threadIdx.x; i <= n; i += blockDim.x) L.rp[i] = d.rp[i];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    L.diag[i] = d.diag[i];
    L.flag[i] = 0;
    flag_u[i] = 0;
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  // forward: y = L \ b(P)
  while (true) {
    int row = 0;
    if (lane == 0) row = atomicAdd(&claim_l, 1);
    row = __shfl_sync(0xffffffffu, row, 0);
    if (row >= n) break;
    const int s = L.rp[row], dp = L.diag[row];
    const T bi = lane == 0 ? T(b[d.P[row]]) : T(0);  // before any wait
    T acc = T(0);
    for (int p = s + lane; p < dp; p += 32) {
      const int k = L.ci[p];
      wait_flag_smem(L.flag + k, d.ctrl);
      acc += L.val[p] * y[k];
    }
    acc = warp_sum(acc);
    if (lane == 0) {
      y[row] = bi - acc;
      __threadfence_block();
      L.flag[row] = 1;
    }
  }
  __syncthreads();
  // backward: z = U \ y (z overwrites y row by row: row i reads only z of rows > i)
  while (true) {
    int c = 0;
    if (lane == 0) c = atomicAdd(&claim_u, 1);
    c = __shfl_sync(0xffffffffu, c, 0);
    if (c >= n) break;
    const int row = n - 1 - c;
    const int dp = L.diag[row], e = L.rp[row + 1];
    const T ri = lane == 0 ? ((const T *)d.rdiag)[row] : T(0);
    const int qi = lane == 0 ? d.Q[row] : 0;
    T acc = T(0);
    for (int p = dp + 1 + lane; p < e; p += 32) {
      const int k = L.ci[p];
      wait_flag_smem(flag_u + k, d.ctrl);
      acc += L.val[p] * y[k];
    }
    acc = warp_sum(acc);
    if (lane == 0) {
      const T zi = (y[row] - acc) * ri;
      y[row] = zi;
      x[qi] = double(zi);
      __threadfence_block();
      flag_u[row] = 1;
    }
  }
}

// ---- small matrices, level by level: one thread per row -------------------------
// GB300 issues FP64 at two lanes per clock per SM, so an FP64 instruction
// costs about the same whether one lane of the warp uses it or all 32.  The
// warp-per-row kernels above leave most lanes idle on the short rows of
// circuit matrices.  Here the rows of one dependency level (independent of
// each other) go to different threads, the levels follow one another with a
// block barrier, and everything the kernel reads sits in shared memory: the
// values, the pattern, the update schedule and the level lists.  With a
// nested-dissection order a chain of 1,000 inverters has ~22 levels.  The
// trailing rows with long L parts (the tail, see LuSymbolic) are done after
// the levels, one row at a time with all threads.  A Newton step refactors
// and then solves: lu_factor_solve_lvl does both from one staging of the
// shared-memory working set.

struct LvlDev {
  const int *lrow, *lptr, *urow, *uptr;  // rows by L level / by U level
  const int *lheavy;                     // per L level: where its heavy rows start
  const int *urp32;                      // update-schedule row starts (int)
  const int *tail_rowg, *tail_gptr, *tail_glong, *tail_pos, *tail_pp, *tail_pm, *tail_q;
  int levels, ulevels, nup;
  int tail0, ntail, ngroups, npos, npairs;
};

enum LvlOff { O_VAL, O_RD, O_Y, O_RED, O_CI, O_RP, O_DIAG, O_URP, O_UPOS, O_LROW, O_LPTR, O_UROW,
              O_UPTR, O_TROWG, O_TGPTR, O_TGLONG, O_TPOS, O_TPP, O_TPM, O_TQ, O_LHEAVY, O_END };
enum LvlMode { LVL_FACTOR = 1, LVL_SOLVE = 2, LVL_BOTH = 3 };

// Shared-memory layout of the level kernels (the same function on host and
// device).  The factor uses val, rd, the schedule and the tail; the solve
// uses val, rd, y, the reduction scratch (one T per thread) and both level
// lists.  The T arrays come first, each padded to 16 bytes.
__host__ __device__ inline size_t lvl_layout(int n, int64_t nnz, const LvlDev &v, int threads,
                                             size_t tsz, int mode, size_t *off) {
  auto a16 = [](size_t x) { return (x + 15) & ~size_t(15); };
  const size_t I = sizeof(int);
  const bool f = mode & LVL_FACTOR, sv = mode & LVL_SOLVE;
  size_t o = 0;
  off[O_VAL] = o; o += a16(tsz * size_t(nnz));
  off[O_RD] = o; o += a16(tsz * size_t(n));
  off[O_Y] = o; o += sv ? a16(tsz * size_t(n)) : 0;
  off[O_RED] = o; o += sv ? a16(tsz * size_t(threads)) : 0;
  off[O_CI] = o; o += I * size_t(nnz);
  off[O_RP] = o; o += I * size_t(n + 1);
  off[O_DIAG] = o; o += I * size_t(n);
  off[O_URP] = o; o += f ? I * size_t(n + 1) : 0;
  off[O_UPOS] = o; o += f ? I * size_t(v.nup) : 0;
  off[O_LROW] = o; o += I * size_t(v.tail0);
  off[O_LPTR] = o; o += I * size_t(v.levels + 1);
  off[O_UROW] = o; o += sv ? I * size_t(n) : 0;
  off[O_UPTR] = o; o += sv ? I * size_t(v.ulevels + 1) : 0;
  off[O_TROWG] = o; o += f ? I * size_t(v.ntail + 1) : 0;
  off[O_TGPTR] = o; o += f ? I * size_t(v.ngroups + 1) : 0;
  off[O_TGLONG] = o; o += f ? I * size_t(v.ngroups) : 0;
  off[O_TPOS] = o; o += f ? I * size_t(v.npos) : 0;
  off[O_TPP] = o; o += f ? I * size_t(v.npos + 1) : 0;
  off[O_TPM] = o; o += f ? I * size_t(v.npairs) : 0;
  off[O_TQ] = o; o += f ? I * size_t(v.npairs) : 0;
  off[O_LHEAVY] = o; o += f ? I * size_t(v.levels) : 0;
  off[O_END] = o;
  return o;
}

// A zero, infinite or NaN pivot, from the bits (no FP64 instruction).
__device__ __forceinline__ bool bad_pivot(double u) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(u);
  return (b << 1) == 0 || ((b >> 52) & 0x7ff) == 0x7ff;
}
__device__ __forceinline__ bool bad_pivot(float u) {
  const unsigned b = __float_as_uint(u);
  return (b << 1) == 0 || ((b >> 23) & 0xff) == 0xff;
}

// Copies count ints into shared memory, four loads in flight per thread.
__device__ __forceinline__ void stage_ints(int *dst, const int *__restrict__ src, int count) {
  const int T = blockDim.x;
  int i = threadIdx.x;
  for (; i + 3 * T < count; i += 4 * T) {
    const int a0 = __ldg(src + i), a1 = __ldg(src + i + T), a2 = __ldg(src + i + 2 * T),
              a3 = __ldg(src + i + 3 * T);
    dst[i] = a0;
    dst[i + T] = a1;
    dst[i + 2 * T] = a2;
    dst[i + 3 * T] = a3;
  }
  for (; i < count; i += T) dst[i] = __ldg(src + i);
}

template <class T>
struct LvlSmem {
  T *val, *rd, *y, *red;
  int *ci, *rp, *diag, *urp, *upos, *lrow, *lptr, *urow, *uptr;
  int *trowg, *tgptr, *tglong, *tpos, *tpp, *tpm, *tq, *lheavy;
};

template <class T>
__device__ LvlSmem<T> lvl_smem(char *smem, int n, int64_t nnz, const LvlDev &v, int mode) {
  size_t off[O_END + 1];
  lvl_layout(n, nnz, v, blockDim.x, sizeof(T), mode, off);
  LvlSmem<T> m;
  m.val = (T *)(smem + off[O_VAL]);
  m.rd = (T *)(smem + off[O_RD]);
  m.y = (T *)(smem + off[O_Y]);
  m.red = (T *)(smem + off[O_RED]);
  m.ci = (int *)(smem + off[O_CI]);
  m.rp = (int *)(smem + off[O_RP]);
  m.diag = (int *)(smem + off[O_DIAG]);
  m.urp = (int *)(smem + off[O_URP]);
  m.upos = (int *)(smem + off[O_UPOS]);
  m.lrow = (int *)(smem + off[O_LROW]);
  m.lptr = (int *)(smem + off[O_LPTR]);
  m.urow = (int *)(smem + off[O_UROW]);
  m.uptr = (int *)(smem + off[O_UPTR]);
  m.trowg = (int *)(smem + off[O_TROWG]);
  m.tgptr = (int *)(smem + off[O_TGPTR]);
  m.tglong = (int *)(smem + off[O_TGLONG]);
  m.tpos = (int *)(smem + off[O_TPOS]);
  m.tpp = (int *)(smem + off[O_TPP]);
  m.tpm = (int *)(smem + off[O_TPM]);
  m.tq = (int *)(smem + off[O_TQ]);
  m.lheavy = (int *)(smem + off[O_LHEAVY]);
  return m;
}

// Stage what `mode` needs.  The factor scatters A into the L\U positions and
// keeps the FP64 copy of A the refinement uses; the solve takes the factor's
// values, or (LVL_BOTH) keeps them in place.
template <class T>
__device__ void lvl_stage(const LuDev &d, const LvlDev &v, const LvlSmem<T> &m, int mode,
                          const double *__restrict__ a, double *__restrict__ a_copy, int64_t nnz_a,
                          const T *__restrict__ val_in, int64_t nnz, const double *__restrict__ b) {
  const int n = d.n;
  if (mode & LVL_FACTOR) {
    for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) {
      const int s = __ldg(d.lu2a + p);
      m.val[p] = s >= 0 ? T(a[s]) : T(0);
    }
    if (a_copy != a)
      for (int64_t p = threadIdx.x; p < nnz_a; p += blockDim.x) a_copy[p] = a[p];
    stage_ints(m.urp, v.urp32, n + 1);
    stage_ints(m.upos, d.upos, v.nup);
    stage_ints(m.trowg, v.tail_rowg, v.ntail + 1);
    stage_ints(m.tgptr, v.tail_gptr, v.ngroups + 1);
    stage_ints(m.tglong, v.tail_glong, v.ngroups);
    stage_ints(m.tpos, v.tail_pos, v.npos);
    stage_ints(m.tpp, v.tail_pp, v.npos + 1);
    stage_ints(m.tpm, v.tail_pm, v.npairs);
    stage_ints(m.tq, v.tail_q, v.npairs);
    stage_ints(m.lheavy, v.lheavy, v.levels);
  } else {
    for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) m.val[p] = val_in[p];
    for (int i = threadIdx.x; i < n; i += blockDim.x) m.rd[i] = ((const T *)d.rdiag)[i];
  }
  stage_ints(m.ci, d.ci, int(nnz));
  stage_ints(m.rp, d.rp, n + 1);
  stage_ints(m.diag, d.diag, n);
  stage_ints(m.lrow, v.lrow, v.tail0);
  stage_ints(m.lptr, v.lptr, v.levels + 1);
  if (mode & LVL_SOLVE) {
    stage_ints(m.urow, v.urow, n);
    stage_ints(m.uptr, v.uptr, v.ulevels + 1);
    for (int i = threadIdx.x; i < n; i += blockDim.x) m.y[i] = T(b[__ldg(d.P + i)]);
  }
}

// The factorisation in shared memory; ends with a barrier.
template <class T>
__device__ void lvl_factor(const LuDev &d, const LvlDev &v, const LvlSmem<T> &m) {
  T *val = m.val, *rd = m.rd;
  const int *ci = m.ci, *rp = m.rp, *diag = m.diag, *urp = m.urp, *upos = m.upos;
  unsigned bad = 0xffffffffu;
  const int lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  for (int lv = 0; lv < v.levels; ++lv) {
    // heavy rows: a warp each, the updates of one L entry spread over the
    // lanes, the L entries in order (the same sequence per entry as below)
    for (int t = m.lheavy[lv] + (threadIdx.x >> 5); t < m.lptr[lv + 1]; t += nw) {
      const int i = m.lrow[t];
      const int dp = diag[i];
      int u = urp[i];
      for (int p = rp[i]; p < dp; ++p) {
        const int k = ci[p];
        const T l = val[p] * rd[k];
        const int q0 = diag[k] + 1, len = rp[k + 1] - q0;
        for (int j = lane; j < len; j += 32) val[upos[u + j]] -= l * val[q0 + j];
        u += len;
        __syncwarp();
        if (lane == 0) val[p] = l;
      }
      __syncwarp();
      if (lane == 0) {
        const T piv = val[dp];
        if (bad_pivot(piv)) bad = min(bad, unsigned(i));
        rd[i] = recip(piv);
      }
    }
    for (int t = m.lptr[lv] + threadIdx.x; t < m.lheavy[lv]; t += blockDim.x) {
      const int i = m.lrow[t];
      const int dp = diag[i];
      int u = urp[i];
      for (int p = rp[i]; p < dp; ++p) {
        const int k = ci[p];
        const T l = val[p] * rd[k];
        val[p] = l;
        const int q0 = diag[k] + 1, len = rp[k + 1] - q0;
        // four updates at a time, all loads before the stores: the targets are
        // distinct positions of row i, the sources lie in row k
        int j = 0;
        for (; j + 4 <= len; j += 4) {
          const int t0 = upos[u + j], t1 = upos[u + j + 1], t2 = upos[u + j + 2],
                    t3 = upos[u + j + 3];
          const T s0 = val[q0 + j], s1 = val[q0 + j + 1], s2 = val[q0 + j + 2],
                  s3 = val[q0 + j + 3];
          const T v0 = val[t0], v1 = val[t1], v2 = val[t2], v3 = val[t3];
          val[t0] = v0 - l * s0;
          val[t1] = v1 - l * s1;
          val[t2] = v2 - l * s2;
          val[t3] = v3 - l * s3;
        }
        for (; j < len; ++j) val[upos[u + j]] -= l * val[q0 + j];
        u += len;
      }
      const T piv = val[dp];
      if (bad_pivot(piv)) bad = min(bad, unsigned(i));
      rd[i] = recip(piv);
    }
    __syncthreads();
  }
  // the tail: each position pulls its updates, group after group
  for (int r = 0; r < v.ntail; ++r) {
    const int i = v.tail0 + r, dp = diag[i];
    for (int g = m.trowg[r]; g < m.trowg[r + 1]; ++g) {
      for (int t = m.tgptr[g] + threadIdx.x; t < m.tglong[g]; t += blockDim.x) {
        const int p = m.tpos[t];
        T acc = val[p];
        for (int j = m.tpp[t]; j < m.tpp[t + 1]; ++j) acc -= val[m.tpm[j]] * val[m.tq[j]];
        val[p] = p < dp ? acc * rd[ci[p]] : acc;
      }
      // long pulls: a warp each, lane-strided partial sums added in a fixed
      // butterfly
      for (int t = m.tglong[g] + (threadIdx.x >> 5); t < m.tgptr[g + 1]; t += nw) {
        const int p = m.tpos[t];
        T part = T(0);
        for (int j = m.tpp[t] + lane; j < m.tpp[t + 1]; j += 32) part += val[m.tpm[j]] * val[m.tq[j]];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == 0) {
          const T acc = val[p] - part;
          val[p] = p < dp ? acc * rd[ci[p]] : acc;
        }
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const T piv = val[dp];
      if (bad_pivot(piv)) bad = min(bad, unsigned(i));
      rd[i] = recip(piv);
    }
    __syncthreads();
  }
  if (bad != 0xffffffffu) {
    atomicOr(&d.ctrl[C_STATUS], ST_PIVOT);
    atomicMin(&d.ctrl[C_BAD_ROW], bad);
  }
}

// x(Q) = U \ (L \ b(P)) in shared memory (y staged from b).
template <class T>
__device__ void lvl_solve(const LuDev &d, const LvlDev &v, const LvlSmem<T> &m,
                          double *__restrict__ x) {
  const int n = d.n;
  const T *val = m.val, *rd = m.rd;
  T *y = m.y, *red = m.red;
  const int *ci = m.ci, *rp = m.rp, *diag = m.diag;
  // y = L \ b(P): the levels, then the tail rows as block-wide dot products
  for (int lv = 0; lv < v.levels; ++lv) {
    for (int t = m.lptr[lv] + threadIdx.x; t < m.lptr[lv + 1]; t += blockDim.x) {
      const int i = m.lrow[t];
      T acc = y[i];
      for (int p = rp[i]; p < diag[i]; ++p) acc -= val[p] * y[ci[p]];
      y[i] = acc;
    }
    __syncthreads();
  }
  for (int i = v.tail0; i < n; ++i) {
    T part = T(0);
    for (int p = rp[i] + threadIdx.x; p < diag[i]; p += blockDim.x) part += val[p] * y[ci[p]];
    red[threadIdx.x] = part;
    __syncthreads();
    // fixed pairing: the same sum on every run (blockDim is a power of two)
    for (int h = blockDim.x >> 1; h > 0; h >>= 1) {
      if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
      __syncthreads();
    }
    if (threadIdx.x == 0) y[i] -= red[0];
    __syncthreads();
  }
  // z = U \ y in place: a row reads only rows of lower U levels
  for (int lv = 0; lv < v.ulevels; ++lv) {
    for (int t = m.uptr[lv] + threadIdx.x; t < m.uptr[lv + 1]; t += blockDim.x) {
      const int i = m.urow[t];
      T acc = y[i];
      for (int p = diag[i] + 1; p < rp[i + 1]; ++p) acc -= val[p] * y[ci[p]];
      y[i] = acc * rd[i];
    }
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[__ldg(d.Q + i)] = double(y[i]);
}

template <class T>
__device__ void lvl_open(const LuDev &d) {
  if (threadIdx.x == 0) {
    d.ctrl[C_STATUS] = 0;
    d.ctrl[C_BAD_ROW] = 0xffffffffu;
  }
}

template <class T>
__device__ void lvl_store_factor(const LuDev &d, const LvlSmem<T> &m, T *__restrict__ val_out,
                                 int64_t nnz) {
  for (int64_t p = threadIdx.x; p < nnz; p += blockDim.x) val_out[p] = m.val[p];
  for (int i = threadIdx.x; i < d.n; i += blockDim.x) ((T *)d.rdiag)[i] = m.rd[i];
}

template <class T>
__global__ void __launch_bounds__(1024) lu_factor_lvl(LuDev d, LvlDev v, const double *__restrict__ a,
                                                      double *__restrict__ a_copy, int64_t nnz_a,
                                                      T *__restrict__ val_out, int64_t nnz) {
  extern __shared__ __align__(16) char smem[];
  const LvlSmem<T> m = lvl_smem<T>(smem, d.n, nnz, v, LVL_FACTOR);
  lvl_open<T>(d);
  lvl_stage<T>(d, v, m, LVL_FACTOR, a, a_copy, nnz_a, nullptr, nnz, nullptr);
  __syncthreads();
  lvl_factor<T>(d, v, m);
  lvl_store_factor<T>(d, m, val_out, nnz);
}

template <class T>
__global__ void __launch_bounds__(1024) lu_solve_lvl(LuDev d, LvlDev v, const T *__restrict__ val_in,
                                                     int64_t nnz, const double *__restrict__ b,
                                                     double *__restrict__ x) {
  extern __shared__ __align__(16) char smem[];
  const LvlSmem<T> m = lvl_smem<T>(smem, d.n, nnz, v, LVL_SOLVE);
  lvl_stage<T>(d, v, m, LVL_SOLVE, nullptr, nullptr, 0, val_in, nnz, b);
  __syncthreads();
  lvl_solve<T>(d, v, m, x);
}

// Refactor, keep the factor, then solve with it while it is in shared memory.
template <class T>
__global__ void __launch_bounds__(1024) lu_factor_solve_lvl(LuDev d, LvlDev v,
                                                            const double *__restrict__ a,
                                                            double *__restrict__ a_copy,
                                                            int64_t nnz_a, T *__restrict__ val_out,
                                                            int64_t nnz, const double *__restrict__ b,
                                                            double *__restrict__ x) {
  extern __shared__ __align__(16) char smem[];
  const LvlSmem<T> m = lvl_smem<T>(smem, d.n, nnz, v, LVL_BOTH);
  lvl_open<T>(d);
  lvl_stage<T>(d, v, m, LVL_BOTH, a, a_copy, nnz_a, nullptr, nnz, b);
  __syncthreads();
  lvl_factor<T>(d, v, m);
  lvl_store_factor<T>(d, m, val_out, nnz);
  lvl_solve<T>(d, v, m, x);
}

// Shared memory of lu_solve_chain: the tile and entry rings, the block's
// values, the barriers, and the running sums of nt rows plus the scratch row.
size_t chain_smem_bytes(int nt, size_t tsz) {
  return size_t(kChainTileRing) * chain_tile_bytes(tsz) + size_t(kChainChunks) * kChainEntChunk * (sizeof(int) + tsz) +
         kChainBlock * tsz + size_t(kChainTileRing + kChainChunks) * 8 + size_t(nt + 1) * tsz;
}

// Where the grid solves hand the trailing rows to the chain kernel.  A
// level of the grid solves costs L2 round trips and a publish (~2.2 us per
// solve, measured on random logic); in the chain a column costs a step of
// its block's triangle (~0.075 us per solve: a shuffle and an FP64
// multiply-add, which one warp issues at 64 cycles) and an entry ~3 ns (its
// round's share: 32 lanes, each a multiply-add on its row's sum).
// Candidates are the last 256, 512, ... rows, as many as shared memory
// holds the running sums of; the tail that saves the most modelled time over
// both solves wins, none when nothing is saved.
constexpr double kGridLevelSeconds = 2.2e-6;
constexpr double kChainColSeconds = 0.075e-6;
constexpr double kChainEntrySeconds = 3e-9;
constexpr size_t kChainSmem = 226 * 1024;

int chain_start(const LuSymbolic &S, size_t tsz) {
  const int n = S.n;
  if (n < 4096) return n;
  const int max_rows = int((kChainSmem - chain_smem_bytes(0, tsz)) / tsz) - 1;
  // L level of each row, the levels of the rows before r, and per column the
  // L entries below the diagonal (a tail from r holds those of columns >= r)
  std::vector<int> lev(n), head(n + 1, 0), col_cnt(n, 0);
  for (int i = 0; i < n; ++i) {
    int m = -1;
    for (int p = S.rp[i]; p < S.diag[i]; ++p) {
      m = std::max(m, lev[S.ci[p]]);
      ++col_cnt[S.ci[p]];
    }
    lev[i] = m + 1;
    head[i + 1] = std::max(head[i], lev[i] + 1);
  }
  const int total = head[n];
  int best = n;
  double best_gain = 0.0;
  int64_t entries = 0;
  for (int r = n - 1; r >= std::max(1, n - max_rows); --r) {
    // row r joins: the L entries of column r (all in rows below it, in the
    // tail) and its own U entries
    entries += col_cnt[r] + (S.rp[r + 1] - S.diag[r] - 1);
    if ((n - r) % 256) continue;
    const double saved = 2.0 * (total - head[r]) * kGridLevelSeconds;
    const double cost = 2.0 * (n - r) * kChainColSeconds + entries * kChainEntrySeconds;
    if (saved - cost > best_gain) {
      best_gain = saved - cost;
      best = r;
    }
  }
  return best;
}

}  // namespace
}  // namespace xg

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------

struct xg_lu {
  int device = 0;
  cudaStream_t stream = nullptr;
  int precision = XG_LU_FP64;
  xg::LuSymbolic S;
  int64_t nnz_lu = 0;
  int *d_rp = nullptr, *d_ci = nullptr, *d_diag = nullptr, *d_lu2a = nullptr;
  int *d_P = nullptr, *d_Q = nullptr, *d_arp = nullptr, *d_aci = nullptr;
  int64_t *d_urp = nullptr;
  int *d_upos = nullptr;
  unsigned *d_ctrl = nullptr;                     // claim counters, status, bad row
  void *d_val = nullptr;                          // nnz_lu of T
  void *d_y = nullptr, *d_z = nullptr;            // n of T
  void *d_rdiag = nullptr;                        // n of T: 1 / U(k,k)
  double *d_a = nullptr;                          // FP64 copy of A
  double *d_r = nullptr, *d_dx = nullptr;         // refinement work
  double *d_hv = nullptr, *d_hb = nullptr, *d_hx = nullptr;  // xg_lu_solve_host staging
  int grid_factor = 0, grid_solve = 0;
  int stage_cap = 0;                       // grid refactor: staged row entries per warp
  unsigned *d_pending = nullptr;           // its positions that start pending (one bit each)
  size_t smem_grid = 0;                    // its dynamic shared memory
  int grid_tri = 0;                        // grid solves: blocks
  int solve_tail0 = 0;                     // grid solves: first row of the chain (n: none)
  int4 *d_tdesc = nullptr;                 // its row descriptors
  void *d_hpart = nullptr;                 // its rows' sums over earlier columns (T)
  int4 *d_chain_blk = nullptr;             // its blocks (ChainBlock)
  unsigned char *d_chain_tiles = nullptr;  // per block: triangle and pivots (T, per refactor), x positions
  int *d_chain_tsrc = nullptr;             // per tile value: its source (ChainPlan::tile_src)
  int *d_chain_rowj = nullptr, *d_chain_esrc = nullptr;  // per entry: row and lane-column, value source
  void *d_chain_val = nullptr;             // per entry: value (T), gathered per refactor
  int n_chain_blk = 0;
  int64_t n_chain_ent = 0;                 // entries, whole chunks
  size_t smem_chain = 0;                   // its y and z in shared memory
  unsigned char *d_solo = nullptr;         // grid solves: rows lu_solve_long sums (LuDev::solo)
  int *d_long = nullptr;                   // those rows: the lower solve's, then the upper's
  int n_long_l = 0, n_long_u = 0;
  size_t smem_factor = 0, smem_solve = 0;  // > 0: the one-CTA path
  int cta_threads = 0;                     // its block size (warps ~ level width)
  bool narrow = false;                     // one lane walks the rows (<= 2 rows per level)
  bool lvl = false;                        // level by level, one thread per row, in one CTA
  size_t smem_lvl_factor = 0, smem_lvl_solve = 0;
  size_t smem_lvl_both = 0;                // > 0: the fused refactor + solve fits
  int lvl_threads = 0;
  int *d_lvl = nullptr;                    // level lists, row starts and tail, one buffer
  xg::LvlDev lvl_dev{};
  bool factored = false;
  xg::LuDev dev() const {
    return xg::LuDev{S.n, d_rp, d_ci, d_diag, d_lu2a, d_P, d_Q, d_arp, d_aci, d_urp, d_upos,
                     d_ctrl, d_rdiag, solve_tail0, d_tdesc, d_hpart, d_solo};
  }
};

namespace {

int cuda_fail(cudaError_t e, const char *what) {
  xg::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return XG_ERR_CUDA;
}

#define XG_CU(call)                                      \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return cuda_fail(e_, #call);  \
  } while (0)

template <class V>
int upload(V **dst, const std::vector<V> &src) {
  XG_CU(cudaMalloc((void **)dst, sizeof(V) * std::max<size_t>(src.size(), 1)));
  if (!src.empty()) XG_CU(cudaMemcpy(*dst, src.data(), sizeof(V) * src.size(), cudaMemcpyHostToDevice));
  return XG_OK;
}

void free_lu(xg_lu *lu) {
  void *ptrs[] = {lu->d_rp, lu->d_ci, lu->d_diag, lu->d_lu2a, lu->d_P, lu->d_Q, lu->d_arp,
                  lu->d_urp, lu->d_upos, lu->d_lvl,
                  lu->d_aci, lu->d_ctrl, lu->d_tdesc, lu->d_hpart, lu->d_solo, lu->d_long, lu->d_pending, lu->d_chain_blk, lu->d_chain_tiles, lu->d_chain_tsrc,
                  lu->d_chain_rowj, lu->d_chain_esrc, lu->d_chain_val, lu->d_val, lu->d_y, lu->d_z, lu->d_rdiag, lu->d_a,
                  lu->d_r, lu->d_dx, lu->d_hv, lu->d_hb, lu->d_hx};
  for (void *p : ptrs)
    if (p) cudaFree(p);
}

template <class T>
int refactor_t(xg_lu *lu, const double *dev_values) {
  xg::LuDev d = lu->dev();
  if (lu->lvl) {
    xg::lu_factor_lvl<T><<<1, lu->lvl_threads, lu->smem_lvl_factor, lu->stream>>>(
        d, lu->lvl_dev, dev_values, lu->d_a, lu->S.nnz_a, (T *)lu->d_val, lu->nnz_lu);
    xg::count_launches(1);
    XG_CU(cudaGetLastError());
    return XG_OK;
  }
  if (lu->narrow) {
    xg::lu_factor_seq<T><<<1, xg::kSeqThreads, lu->smem_factor, lu->stream>>>(
        d, dev_values, lu->d_a, lu->S.nnz_a, (T *)lu->d_val, lu->nnz_lu); xg::count_launches(1);
    XG_CU(cudaGetLastError());
    return XG_OK;
  }
  if (lu->smem_factor) {
    xg::lu_factor_cta<T><<<1, lu->cta_threads, lu->smem_factor, lu->stream>>>(
        d, dev_values, lu->d_a, lu->S.nnz_a, (T *)lu->d_val, lu->nnz_lu); xg::count_launches(1);
    XG_CU(cudaGetLastError());
    return XG_OK;
  }
  xg::lu_assemble<T><<<lu->grid_solve, 256, 0, lu->stream>>>(
      d, dev_values, lu->d_a, lu->S.nnz_a, (T *)lu->d_val, lu->nnz_lu, lu->d_pending); xg::count_launches(1);
  xg::lu_factor<T><<<lu->grid_factor, 32 * xg::kFactorWarps, lu->smem_grid, lu->stream>>>(
      d, (T *)lu->d_val, lu->d_a, lu->stage_cap); xg::count_launches(1);
  if (lu->n_chain_blk) {
    const int blocks = int(std::min<int64_t>(1024, (lu->n_chain_ent + 255) / 256));
    xg::lu_chain_gather<T><<<blocks, 256, 0, lu->stream>>>(d, (const T *)lu->d_val, lu->d_chain_esrc,
                                                          (T *)lu->d_chain_val, lu->n_chain_ent, lu->d_chain_tsrc,
                                                          lu->d_chain_tiles, lu->n_chain_blk);
    xg::count_launches(1);
  }
  XG_CU(cudaGetLastError());
  return XG_OK;
}

template <class T>
int solve_once(xg_lu *lu, const double *b, double *x) {
  xg::LuDev d = lu->dev();
  if (lu->lvl) {
    xg::lu_solve_lvl<T><<<1, lu->lvl_threads, lu->smem_lvl_solve, lu->stream>>>(
        d, lu->lvl_dev, (const T *)lu->d_val, lu->nnz_lu, b, x);
    xg::count_launches(1);
    XG_CU(cudaGetLastError());
    return XG_OK;
  }
  if (lu->narrow) {
    xg::lu_solve_seq<T><<<1, xg::kSeqThreads, lu->smem_solve, lu->stream>>>(d, (const T *)lu->d_val, lu->nnz_lu,
                                                               b, x); xg::count_launches(1);
    XG_CU(cudaGetLastError());
    return XG_OK;
  }
  if (lu->smem_solve) {
    xg::lu_solve_cta<T><<<1, lu->cta_threads, lu->smem_solve, lu->stream>>>(
        d, (const T *)lu->d_val, lu->nnz_lu, b, x); xg::count_launches(1);
    XG_CU(cudaGetLastError());
    return XG_OK;
  }
  xg::lu_solve_open<T><<<std::min(1024, (lu->S.n + 255) / 256), 256, 0, lu->stream>>>(
      d, (T *)lu->d_y, (T *)lu->d_z);
  xg::count_launches(1);
  xg::lu_lsolve<T><<<lu->grid_tri, 256, 0, lu->stream>>>(d, (const T *)lu->d_val, b, (T *)lu->d_y); xg::count_launches(1);
  if (lu->n_long_l) {
    xg::lu_solve_long<T><<<lu->n_long_l, xg::kLongThreads, 0, lu->stream>>>(
        d, (const T *)lu->d_val, b, (T *)lu->d_y, (T *)lu->d_z, x, lu->d_long, 0);
    xg::count_launches(1);
  }
  if (lu->solve_tail0 < lu->S.n) {
    const xg::ChainDev c{lu->d_chain_blk, lu->n_chain_blk, lu->d_chain_tiles, lu->d_chain_rowj,
                         lu->d_chain_val, lu->n_chain_ent};
    xg::lu_solve_chain<T><<<1, xg::kChainLanes, lu->smem_chain, lu->stream>>>(d, c, (T *)lu->d_y, (T *)lu->d_z,
                                                                              x);
    xg::count_launches(1);
  }
  xg::lu_usolve<T><<<lu->grid_tri, 256, 0, lu->stream>>>(d, (const T *)lu->d_val, (const T *)lu->d_y,
                                                         (T *)lu->d_z, x); xg::count_launches(1);
  if (lu->n_long_u) {
    xg::lu_solve_long<T><<<lu->n_long_u, xg::kLongThreads, 0, lu->stream>>>(
        d, (const T *)lu->d_val, b, (T *)lu->d_y, (T *)lu->d_z, x, lu->d_long + lu->n_long_l, 1);
    xg::count_launches(1);
  }
  XG_CU(cudaGetLastError());
  return XG_OK;
}

// Refactor and solve; one fused launch on the level path when it fits.
template <class T>
int refactor_solve_t(xg_lu *lu, const double *dev_values, const double *b, double *x,
                     int n_refine);

template <class T>
int solve_t(xg_lu *lu, const double *b, double *x, int n_refine) {
  int rc = solve_once<T>(lu, b, x);
  if (rc) return rc;
  xg::LuDev d = lu->dev();
  const int nb = std::min(1024, (lu->S.n + 255) / 256);
  for (int it = 0; it < n_refine; ++it) {
    xg::lu_residual<<<nb, 256, 0, lu->stream>>>(d, lu->d_a, x, b, lu->d_r); xg::count_launches(1);
    rc = solve_once<T>(lu, lu->d_r, lu->d_dx);
    if (rc) return rc;
    xg::lu_axpy<<<nb, 256, 0, lu->stream>>>(lu->S.n, lu->d_dx, x); xg::count_launches(1);
  }
  XG_CU(cudaGetLastError());
  return XG_OK;
}

template <class T>
int refactor_solve_t(xg_lu *lu, const double *dev_values, const double *b, double *x,
                     int n_refine) {
  if (!lu->lvl || !lu->smem_lvl_both) {
    int rc = refactor_t<T>(lu, dev_values);
    return rc ? rc : solve_t<T>(lu, b, x, n_refine);
  }
  xg::LuDev d = lu->dev();
  xg::lu_factor_solve_lvl<T><<<1, lu->lvl_threads, lu->smem_lvl_both, lu->stream>>>(
      d, lu->lvl_dev, dev_values, lu->d_a, lu->S.nnz_a, (T *)lu->d_val, lu->nnz_lu, b, x);
  xg::count_launches(1);
  XG_CU(cudaGetLastError());
  for (int it = 0; it < n_refine; ++it) {
    const int nb = std::min(1024, (lu->S.n + 255) / 256);
    xg::lu_residual<<<nb, 256, 0, lu->stream>>>(d, lu->d_a, x, b, lu->d_r); xg::count_launches(1);
    int rc = solve_once<T>(lu, lu->d_r, lu->d_dx);
    if (rc) return rc;
    xg::lu_axpy<<<nb, 256, 0, lu->stream>>>(lu->S.n, lu->d_dx, x); xg::count_launches(1);
  }
  XG_CU(cudaGetLastError());
  return XG_OK;
}

}  // namespace

extern "C" int xg_lu_analyze(xg_ctx *ctx, int n, const int *host_rowptr, const int *host_colidx,
                             const double *host_values, int precision, xg_lu **out) {
  if (!ctx || !out || n <= 0 || !host_rowptr || !host_colidx || !host_values ||
      (precision != XG_LU_FP64 && precision != XG_LU_FP32)) {
    xg::set_error("xg_lu_analyze: bad argument");
    return XG_ERR_ARG;
  }
  *out = nullptr;
  std::unique_ptr<xg_lu> lu(new xg_lu);
  void *stream = nullptr;
  xg::ctx_info(ctx, &lu->device, &stream);
  lu->stream = (cudaStream_t)stream;
  lu->precision = precision;
  std::string err;
  if (xg::lu_analyze(n, host_rowptr, host_colidx, host_values, 1e-3, &lu->S, &err)) {
    xg::set_error(err);
    return XG_ERR_SINGULAR;
  }
  if (!xg::lu_build_updates(lu->S)) {
    xg::set_error("xg_lu_analyze: internal error, an update falls outside the L\\U pattern");
    return XG_ERR_ARG;
  }
  XG_CU(cudaSetDevice(lu->device));
  const xg::LuSymbolic &S = lu->S;
  lu->nnz_lu = S.rp[n];
  lu->solve_tail0 = n;  // no chain unless the grid path below picks one
  std::vector<int> arp(host_rowptr, host_rowptr + n + 1);
  std::vector<int> aci(host_colidx, host_colidx + S.nnz_a);
  int rc = 0;
  auto fail = [&](int r) {
    free_lu(lu.get());
    return r;
  };
  if ((rc = upload(&lu->d_rp, S.rp)) || (rc = upload(&lu->d_ci, S.ci)) ||
      (rc = upload(&lu->d_diag, S.diag)) || (rc = upload(&lu->d_lu2a, S.lu2a)) ||
      (rc = upload(&lu->d_P, S.P)) || (rc = upload(&lu->d_Q, S.Q)) ||
      (rc = upload(&lu->d_arp, arp)) || (rc = upload(&lu->d_aci, aci)) ||
      (rc = upload(&lu->d_urp, S.urp)) || (rc = upload(&lu->d_upos, S.upos)))
    return fail(rc);
  const int64_t nup = S.urp[n];
  std::vector<int> urp32;  // the row starts as int, for the level path
  if (nup < (int64_t(1) << 31)) urp32.assign(S.urp.begin(), S.urp.end());
  // the schedule lives on the device only
  std::vector<int64_t>().swap(lu->S.urp);
  std::vector<int>().swap(lu->S.upos);
  const size_t tsz = precision == XG_LU_FP32 ? sizeof(float) : sizeof(double);
  cudaError_t e = cudaSuccess;
  if ((e = cudaMalloc((void **)&lu->d_ctrl, sizeof(unsigned) * xg::C_N)) ||
      (e = cudaMalloc(&lu->d_val, tsz * size_t(lu->nnz_lu))) ||
      (e = cudaMalloc(&lu->d_y, tsz * size_t(n))) || (e = cudaMalloc(&lu->d_z, tsz * size_t(n))) ||
      (e = cudaMalloc(&lu->d_rdiag, tsz * size_t(n))) ||
      (e = cudaMalloc((void **)&lu->d_a, sizeof(double) * size_t(S.nnz_a))) ||
      (e = cudaMalloc((void **)&lu->d_r, sizeof(double) * size_t(n))) ||
      (e = cudaMalloc((void **)&lu->d_dx, sizeof(double) * size_t(n)))) {
    free_lu(lu.get());
    return e == cudaErrorMemoryAllocation ? (xg::set_error("xg_lu_analyze: out of device memory"),
                                             XG_ERR_OOM)
                                          : cuda_fail(e, "xg_lu_analyze");
  }
  {
    unsigned init[xg::C_N] = {};
    init[xg::C_SPIN] = unsigned(xg::kSpinLimit);
    if ((e = cudaMemcpy(lu->d_ctrl, init, sizeof(init), cudaMemcpyHostToDevice))) {
      free_lu(lu.get());
      return cuda_fail(e, "xg_lu_analyze: cudaMemcpy");
    }
  }
  int sms = 0, occ = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, lu->device);
  {
    // Stage every row when the longest fits kStageBytes per warp (the long
    // rows of a dense trailing block are the critical path).  Otherwise (a
    // supply node's row) every row that fits kStageBytes when that costs no
    // resident warps, else all but the kUnstagedRows longest, with at least
    // kMinStageBytes (a stage that small costs no occupancy: registers bound
    // it first): the longest rows stay in global memory rather than cut the
    // number of resident warps.
    std::vector<int> len(n);
    for (int i = 0; i < n; ++i) len[i] = S.rp[i + 1] - S.rp[i];
    const int max_row = *std::max_element(len.begin(), len.end());
    const int cap_max = xg::kStageBytes / int(tsz);
    const void *fn = precision == XG_LU_FP32 ? (const void *)xg::lu_factor<float>
                                             : (const void *)xg::lu_factor<double>;
    auto round_cap = [](int c) { return (c + 31) / 32 * 32; };
    auto occupancy = [&](int c, int *o) -> cudaError_t {
      const size_t b = size_t(xg::kFactorWarps) * size_t(round_cap(c)) * tsz;
      cudaError_t e2 = xg::allow_dynamic_smem(fn, b);
      if (e2 == cudaSuccess) e2 = cudaOccupancyMaxActiveBlocksPerMultiprocessor(o, fn, 32 * xg::kFactorWarps, b);
      return e2;
    };
    int cap = max_row;
    if (max_row > cap_max) {
      int fit = 0;
      for (int l : len)
        if (l <= cap_max) fit = std::max(fit, l);
      const int k = std::min(n - 1, xg::kUnstagedRows);
      std::nth_element(len.begin(), len.begin() + k, len.end(), std::greater<int>());
      cap = std::min(cap_max, std::max(len[k], xg::kMinStageBytes / int(tsz)));
      int occ_fit = 0, occ_cap = 0;
      if (fit > cap) {
        if ((e = occupancy(fit, &occ_fit)) || (e = occupancy(cap, &occ_cap))) {
          free_lu(lu.get());
          return cuda_fail(e, "xg_lu_analyze: shared-memory limit");
        }
        if (occ_fit >= occ_cap) cap = fit;
      }
    }
    lu->stage_cap = round_cap(cap);
    lu->smem_grid = size_t(xg::kFactorWarps) * size_t(lu->stage_cap) * tsz;
    if ((e = occupancy(lu->stage_cap, &occ))) {
      free_lu(lu.get());
      return cuda_fail(e, "xg_lu_analyze: shared-memory limit");
    }
    // the U part right of the diagonal of every staged row starts pending
    std::vector<unsigned> pending((size_t(lu->nnz_lu) + 31) / 32, 0u);
    for (int i = 0; i < n; ++i)
      if (S.rp[i + 1] - S.rp[i] <= lu->stage_cap)
        for (int p = S.diag[i] + 1; p < S.rp[i + 1]; ++p) pending[size_t(p) >> 5] |= 1u << (p & 31);
    if ((rc = upload(&lu->d_pending, pending))) {
      free_lu(lu.get());
      return rc;
    }
  }
  // one warp per row: never more warps than rows
  lu->grid_factor = std::max(1, std::min(sms * std::max(occ, 1), (n + xg::kFactorWarps - 1) / xg::kFactorWarps));
  lu->grid_solve = std::max(1, std::min(sms * 4, int((lu->nnz_lu + 255) / 256)));
  {
    int occ_tri = 0;
    if (precision == XG_LU_FP32)
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_tri, xg::lu_lsolve<float>, 256, 0);
    else
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ_tri, xg::lu_lsolve<double>, 256, 0);
    lu->grid_tri = std::max(1, std::min(sms * std::max(occ_tri, 1), (n + 7) / 8));
    lu->solve_tail0 = std::getenv("XG_LU_NO_CHAIN") ? n : xg::chain_start(S, tsz);
    const int t0 = lu->solve_tail0, nt = n - t0;
    if (nt > 0) {
      // per chain row {start, first entry in a column >= t0, diagonal, P}
      std::vector<int4> desc(nt);
      for (int r = t0; r < n; ++r) {
        const int *c0 = S.ci.data() + S.rp[r], *c1 = S.ci.data() + S.diag[r];
        desc[r - t0] = make_int4(S.rp[r], S.rp[r] + int(std::lower_bound(c0, c1, t0) - c0), S.diag[r],
                                 S.P[r]);
      }
      // the blocked chain's plan: block records, tiles (value sources and x
      // positions) and rounds (rows and value sources), the entries padded
      // to whole chunks
      xg::ChainPlan plan = xg::build_chain_plan(S, t0);
      while (plan.ent_rowj.size() % xg::kChainEntChunk) {
        plan.ent_rowj.push_back(nt << 5);
        plan.ent_src.push_back(-1);
      }
      lu->n_chain_blk = int(plan.blocks.size());
      lu->n_chain_ent = int64_t(plan.ent_rowj.size());
      const size_t tb = xg::chain_tile_bytes(tsz);
      std::vector<unsigned char> tiles(plan.blocks.size() * tb, 0);
      for (size_t k = 0; k < plan.blocks.size(); ++k)
        std::memcpy(tiles.data() + k * tb + xg::kChainTileValues * tsz, plan.tile_q.data() + k * xg::kChainBlock,
                    xg::kChainBlock * sizeof(int));
      lu->smem_chain = xg::chain_smem_bytes(nt, tsz);
      const void *fn = precision == XG_LU_FP32 ? (const void *)xg::lu_solve_chain<float>
                                               : (const void *)xg::lu_solve_chain<double>;
      std::vector<int4> blk(plan.blocks.size());
      for (size_t k = 0; k < blk.size(); ++k)
        blk[k] = make_int4(plan.blocks[k].cbase, plan.blocks[k].bs, plan.blocks[k].rounds, plan.blocks[k].upper);
      if ((rc = upload(&lu->d_tdesc, desc)) || (rc = upload(&lu->d_chain_blk, blk)) ||
          (rc = upload(&lu->d_chain_tiles, tiles)) || (rc = upload(&lu->d_chain_tsrc, plan.tile_src)) ||
          (rc = upload(&lu->d_chain_rowj, plan.ent_rowj)) || (rc = upload(&lu->d_chain_esrc, plan.ent_src)) ||
          (e = cudaMalloc(&lu->d_chain_val, std::max<size_t>(plan.ent_rowj.size(), 1) * tsz)) ||
          (e = cudaMalloc(&lu->d_hpart, size_t(nt) * tsz)) ||
          (e = xg::allow_dynamic_smem((const void *)fn, lu->smem_chain))) {
        free_lu(lu.get());
        return rc ? rc : cuda_fail(e, "xg_lu_analyze");
      }
    }
    // rows of the grid solves (below the chain) that lu_solve_long sums
    std::vector<unsigned char> solo;
    std::vector<int> long_l, long_u;
    xg::solo_rows(S, t0, xg::kSolveLongRow, &solo, &long_l, &long_u);
    lu->n_long_l = int(long_l.size());
    lu->n_long_u = int(long_u.size());
    long_l.insert(long_l.end(), long_u.begin(), long_u.end());
    if ((rc = upload(&lu->d_solo, solo)) || (rc = upload(&lu->d_long, long_l))) {
      free_lu(lu.get());
      return rc;
    }
  }
  // one-CTA path when the factor (and the solve's extra vectors) fit in shared memory
  {
    const size_t factor_b = xg::smem_bytes(n, lu->nnz_lu, tsz);
    const size_t solve_b = factor_b;
    int max_optin = 0;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, lu->device);
    const size_t limit = size_t(max_optin) > 8192 ? size_t(max_optin) - 4096 : 0;
    if (solve_b <= limit && factor_b <= limit && !std::getenv("XG_LU_NO_CTA")) {
      cudaError_t e1, e2, e3, e4;
      if (precision == XG_LU_FP32) {
        e1 = xg::allow_dynamic_smem((const void *)xg::lu_factor_cta<float>, factor_b);
        e2 = xg::allow_dynamic_smem((const void *)xg::lu_solve_cta<float>, solve_b);
        e3 = xg::allow_dynamic_smem((const void *)xg::lu_factor_seq<float>, factor_b);
        e4 = xg::allow_dynamic_smem((const void *)xg::lu_solve_seq<float>, solve_b);
      } else {
        e1 = xg::allow_dynamic_smem((const void *)xg::lu_factor_cta<double>, factor_b);
        e2 = xg::allow_dynamic_smem((const void *)xg::lu_solve_cta<double>, solve_b);
        e3 = xg::allow_dynamic_smem((const void *)xg::lu_factor_seq<double>, factor_b);
        e4 = xg::allow_dynamic_smem((const void *)xg::lu_solve_seq<double>, solve_b);
      }
      if (e3 != cudaSuccess || e4 != cudaSuccess) e1 = e3 != cudaSuccess ? e3 : e4;
      if (e1 == cudaSuccess && e2 == cudaSuccess) {
        lu->smem_factor = factor_b;
        lu->smem_solve = solve_b;
        // as many warps as rows can be in flight, 2 to 32
        const int warps = std::max(2, std::min(32, lu->S.max_width));
        lu->cta_threads = 32 * warps;
        // average rows per level: little parallelism -> the one-lane walk
        lu->narrow = double(n) / std::max(1, lu->S.levels) < 3.0 && !std::getenv("XG_LU_NO_SEQ");
      } else {
        cudaGetLastError();
      }
    }
  }
  // level-by-level path when its whole working set fits in shared memory and
  // the levels hold several rows each (a chain of single rows is walked faster
  // by the one lane of the narrow path)
  if (!std::getenv("XG_LU_NO_LVL") && !lu->narrow && !urp32.empty() &&
      lu->nnz_lu < (int64_t(1) << 31)) {
    // lrow | lptr | urow | uptr | urp32 | tail_rowg | tail_gptr | tail_pos | tail_pp | tail_pm |
    // tail_q | tail_glong | lheavy
    const std::vector<int> *parts[] = {&S.lrow, &S.lptr, &S.urow, &S.uptr, &urp32, &S.tail_rowg,
                                       &S.tail_gptr, &S.tail_pos, &S.tail_pp, &S.tail_pm, &S.tail_q,
                                       &S.tail_glong, &S.lheavy};
    size_t start[13], total = 0;
    for (int k = 0; k < 13; ++k) { start[k] = total; total += parts[k]->size(); }
    xg::LvlDev v{};
    v.levels = int(S.lptr.size()) - 1;
    v.ulevels = int(S.uptr.size()) - 1;
    v.nup = int(nup);
    v.tail0 = S.tail0;
    v.ntail = int(S.tail_rowg.size()) - 1;
    v.ngroups = int(S.tail_gptr.size()) - 1;
    v.npos = int(S.tail_pos.size());
    v.npairs = int(S.tail_pm.size());
    // threads: the widest level or tail group, in warps, 1 to 32
    int maxw = 1;
    for (int l = 0; l < v.levels; ++l) maxw = std::max(maxw, S.lptr[l + 1] - S.lptr[l]);
    for (int l = 0; l < v.ulevels; ++l) maxw = std::max(maxw, S.uptr[l + 1] - S.uptr[l]);
    for (int g = 0; g < v.ngroups; ++g) maxw = std::max(maxw, S.tail_gptr[g + 1] - S.tail_gptr[g]);
    // a power of two (the tail reduction); 1,024 threads when there are heavy
    // rows (a warp each) or the widest level needs them, else 256, so the
    // staging keeps many loads in flight
    int threads = 256;
    for (int l = 0; l < v.levels; ++l)
      if (S.lheavy[l] < S.lptr[l + 1]) maxw = std::max(maxw, 1024);
    while (threads < maxw && threads < 1024) threads *= 2;
    size_t off[xg::O_END + 1];
    const size_t fb = xg::lvl_layout(n, lu->nnz_lu, v, threads, tsz, xg::LVL_FACTOR, off);
    const size_t sb = xg::lvl_layout(n, lu->nnz_lu, v, threads, tsz, xg::LVL_SOLVE, off);
    const size_t bb = xg::lvl_layout(n, lu->nnz_lu, v, threads, tsz, xg::LVL_BOTH, off);
    int max_optin = 0;
    cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, lu->device);
    const size_t limit = size_t(max_optin) > 8192 ? size_t(max_optin) - 4096 : 0;
    if (fb <= limit && sb <= limit) {
      cudaError_t e1, e2;
      if (precision == XG_LU_FP32) {
        e1 = xg::allow_dynamic_smem((const void *)xg::lu_factor_lvl<float>, fb);
        e2 = xg::allow_dynamic_smem((const void *)xg::lu_solve_lvl<float>, sb);
      } else {
        e1 = xg::allow_dynamic_smem((const void *)xg::lu_factor_lvl<double>, fb);
        e2 = xg::allow_dynamic_smem((const void *)xg::lu_solve_lvl<double>, sb);
      }
      if (e1 == cudaSuccess && e2 == cudaSuccess) {
        std::vector<int> buf;
        buf.reserve(total);
        for (auto *pv : parts) buf.insert(buf.end(), pv->begin(), pv->end());
        if ((rc = upload(&lu->d_lvl, buf))) return fail(rc);
        const int *b0 = lu->d_lvl;
        v.lrow = b0 + start[0];
        v.lptr = b0 + start[1];
        v.urow = b0 + start[2];
        v.uptr = b0 + start[3];
        v.urp32 = b0 + start[4];
        v.tail_rowg = b0 + start[5];
        v.tail_gptr = b0 + start[6];
        v.tail_pos = b0 + start[7];
        v.tail_pp = b0 + start[8];
        v.tail_pm = b0 + start[9];
        v.tail_q = b0 + start[10];
        v.tail_glong = b0 + start[11];
        v.lheavy = b0 + start[12];
        lu->lvl_dev = v;
        lu->lvl_threads = threads;
        lu->smem_lvl_factor = fb;
        lu->smem_lvl_solve = sb;
        lu->lvl = true;
        // the fused refactor + solve when both working sets fit together
        if (bb <= limit) {
          const void *fn = precision == XG_LU_FP32 ? (const void *)xg::lu_factor_solve_lvl<float>
                                                   : (const void *)xg::lu_factor_solve_lvl<double>;
          if (xg::allow_dynamic_smem(fn, bb) == cudaSuccess) lu->smem_lvl_both = bb;
        }
      } else {
        cudaGetLastError();
      }
    }
  }
  *out = lu.release();
  return XG_OK;
}

extern "C" int xg_lu_refactor(xg_lu *lu, const double *dev_values) {
  if (!lu || !dev_values) {
    xg::set_error("xg_lu_refactor: bad argument");
    return XG_ERR_ARG;
  }
  XG_CU(cudaSetDevice(lu->device));
  int rc = lu->precision == XG_LU_FP32 ? refactor_t<float>(lu, dev_values)
                                       : refactor_t<double>(lu, dev_values);
  if (!rc) lu->factored = true;
  return rc;
}

extern "C" int xg_lu_refactor_solve(xg_lu *lu, const double *dev_values, const double *dev_b,
                                    double *dev_x, int n_refine) {
  if (!lu || !dev_values || !dev_b || !dev_x || n_refine < 0 || dev_b == dev_x) {
    xg::set_error("xg_lu_refactor_solve: bad argument (b and x must be distinct device buffers)");
    return XG_ERR_ARG;
  }
  XG_CU(cudaSetDevice(lu->device));
  int rc = lu->precision == XG_LU_FP32
               ? refactor_solve_t<float>(lu, dev_values, dev_b, dev_x, n_refine)
               : refactor_solve_t<double>(lu, dev_values, dev_b, dev_x, n_refine);
  if (!rc) lu->factored = true;
  return rc;
}

extern "C" int xg_lu_solve(xg_lu *lu, const double *dev_b, double *dev_x, int n_refine) {
  if (!lu || !dev_b || !dev_x || n_refine < 0 || dev_b == dev_x) {
    xg::set_error("xg_lu_solve: bad argument (b and x must be distinct device buffers)");
    return XG_ERR_ARG;
  }
  if (!lu->factored) {
    xg::set_error("xg_lu_solve: no factorisation yet (call xg_lu_refactor)");
    return XG_ERR_STATE;
  }
  XG_CU(cudaSetDevice(lu->device));
  return lu->precision == XG_LU_FP32 ? solve_t<float>(lu, dev_b, dev_x, n_refine)
                                     : solve_t<double>(lu, dev_b, dev_x, n_refine);
}

extern "C" int xg_lu_solve_host(xg_lu *lu, const double *host_values, const double *host_b,
                                double *host_x, int n_refine, int reuse_factors, int *status) {
  if (!lu || !host_b || !host_x || !status || n_refine < 0 || (!reuse_factors && !host_values)) {
    xg::set_error("xg_lu_solve_host: bad argument");
    return XG_ERR_ARG;
  }
  if (reuse_factors && !lu->factored) {
    xg::set_error("xg_lu_solve_host: no factorisation to reuse");
    return XG_ERR_STATE;
  }
  XG_CU(cudaSetDevice(lu->device));
  const size_t n = size_t(lu->S.n), nnz = size_t(lu->S.nnz_a);
  if (!lu->d_hv) {  // staging for host callers, made on first use
    cudaError_t e;
    if ((e = cudaMalloc((void **)&lu->d_hv, sizeof(double) * nnz)) ||
        (e = cudaMalloc((void **)&lu->d_hb, sizeof(double) * n)) ||
        (e = cudaMalloc((void **)&lu->d_hx, sizeof(double) * n))) {
      cudaFree(lu->d_hv);
      cudaFree(lu->d_hb);
      lu->d_hv = lu->d_hb = lu->d_hx = nullptr;
      return e == cudaErrorMemoryAllocation
                 ? (xg::set_error("xg_lu_solve_host: out of device memory"), XG_ERR_OOM)
                 : cuda_fail(e, "xg_lu_solve_host");
    }
  }
  if (!reuse_factors)
    XG_CU(cudaMemcpyAsync(lu->d_hv, host_values, sizeof(double) * nnz, cudaMemcpyHostToDevice,
                          lu->stream));
  XG_CU(cudaMemcpyAsync(lu->d_hb, host_b, sizeof(double) * n, cudaMemcpyHostToDevice, lu->stream));
  const int rc = reuse_factors ? xg_lu_solve(lu, lu->d_hb, lu->d_hx, n_refine)
                               : xg_lu_refactor_solve(lu, lu->d_hv, lu->d_hb, lu->d_hx, n_refine);
  if (rc) return rc;
  XG_CU(cudaMemcpyAsync(host_x, lu->d_hx, sizeof(double) * n, cudaMemcpyDeviceToHost, lu->stream));
  int bad = -1;
  return xg_lu_status(lu, status, &bad);  // synchronises the stream
}

namespace xg {
const unsigned *lu_status_device(const xg_lu *lu) { return lu->d_ctrl + C_STATUS; }
}  // namespace xg

extern "C" int xg_lu_status(xg_lu *lu, int *status, int *bad_row) {
  if (!lu || !status) {
    xg::set_error("xg_lu_status: bad argument");
    return XG_ERR_ARG;
  }
  XG_CU(cudaSetDevice(lu->device));
  unsigned h[xg::C_N];
  XG_CU(cudaMemcpyAsync(h, lu->d_ctrl, sizeof(h), cudaMemcpyDeviceToHost, lu->stream));
  XG_CU(cudaStreamSynchronize(lu->stream));
  *status = int(h[xg::C_STATUS]);
  if (bad_row) *bad_row = h[xg::C_BAD_ROW] == 0xffffffffu ? -1 : int(h[xg::C_BAD_ROW]);
  return XG_OK;
}

extern "C" int xg_lu_set_wait_limit(xg_lu *lu, int polls) {
  if (!lu || polls < 1) {
    xg::set_error("xg_lu_set_wait_limit: bad argument");
    return XG_ERR_ARG;
  }
  XG_CU(cudaSetDevice(lu->device));
  // after the work already queued, so a launch in flight keeps the limit it began with
  XG_CU(cudaStreamSynchronize(lu->stream));
  const unsigned v = unsigned(polls);
  XG_CU(cudaMemcpy(lu->d_ctrl + xg::C_SPIN, &v, sizeof(v), cudaMemcpyHostToDevice));
  return XG_OK;
}

// with_chain: model the chain of the grid solves (the host-only analysis;
// an analysed xg_lu reports the one it chose)
static void fill_info(const xg::LuSymbolic &S, int precision, xg_lu_info *info, bool with_chain) {
  std::memset(info, 0, sizeof(*info));
  info->n = S.n;
  info->nnz_a = S.nnz_a;
  info->nnz_lu = S.rp.empty() ? 0 : S.rp[S.n];
  info->precision = precision;
  info->levels = S.levels;
  info->n_dense = S.n_dense;
  info->refactor_flops = S.refactor_flops;
  info->solve_flops = S.solve_flops;
  info->min_pivot = S.min_pivot;
  info->max_pivot = S.max_pivot;
  info->ordering = S.ordering;
  const size_t tsz = precision == XG_LU_FP32 ? sizeof(float) : sizeof(double);
  info->solve_chain = with_chain && !S.rp.empty() ? S.n - xg::chain_start(S, tsz) : 0;
}

extern "C" int xg_lu_get_info(const xg_lu *lu, xg_lu_info *info) {
  if (!lu || !info) {
    xg::set_error("xg_lu_get_info: bad argument");
    return XG_ERR_ARG;
  }
  fill_info(lu->S, lu->precision, info, false);
  const bool grid = !lu->lvl && !lu->narrow && !lu->smem_solve;
  info->solve_chain = grid ? lu->S.n - lu->solve_tail0 : 0;
  return XG_OK;
}

extern "C" int xg_lu_get_symbolic(const xg_lu *lu, int *P, int *Q, int *lu_rowptr, int *lu_colidx) {
  if (!lu) {
    xg::set_error("xg_lu_get_symbolic: bad argument");
    return XG_ERR_ARG;
  }
  const xg::LuSymbolic &S = lu->S;
  if (P) std::memcpy(P, S.P.data(), sizeof(int) * S.n);
  if (Q) std::memcpy(Q, S.Q.data(), sizeof(int) * S.n);
  if (lu_rowptr) std::memcpy(lu_rowptr, S.rp.data(), sizeof(int) * (S.n + 1));
  if (lu_colidx) std::memcpy(lu_colidx, S.ci.data(), sizeof(int) * S.ci.size());
  return XG_OK;
}

extern "C" int xg_lu_destroy(xg_lu *lu) {
  if (!lu) return XG_OK;
  cudaSetDevice(lu->device);
  cudaStreamSynchronize(lu->stream);
  free_lu(lu);
  delete lu;
  return XG_OK;
}

extern "C" int xg_lu_order(int n, const int *host_rowptr, const int *host_colidx, int *order,
                           int *n_dense) {
  if (n <= 0 || !host_rowptr || !host_colidx || !order) {
    xg::set_error("xg_lu_order: bad argument");
    return XG_ERR_ARG;
  }
  std::vector<int> o = xg::amd_order(n, host_rowptr, host_colidx, n_dense);
  std::memcpy(order, o.data(), sizeof(int) * n);
  return XG_OK;
}

extern "C" int xg_lu_analyze_host(int n, const int *host_rowptr, const int *host_colidx,
                                  const double *host_values, int *P, int *Q, int64_t *nnz_lu,
                                  xg_lu_info *info) {
  if (n <= 0 || !host_rowptr || !host_colidx || !host_values) {
    xg::set_error("xg_lu_analyze_host: bad argument");
    return XG_ERR_ARG;
  }
  xg::LuSymbolic S;
  std::string err;
  if (xg::lu_analyze(n, host_rowptr, host_colidx, host_values, 1e-3, &S, &err)) {
    xg::set_error(err);
    return XG_ERR_SINGULAR;
  }
  if (P) std::memcpy(P, S.P.data(), sizeof(int) * n);
  if (Q) std::memcpy(Q, S.Q.data(), sizeof(int) * n);
  if (nnz_lu) *nnz_lu = S.rp[n];
  if (info) fill_info(S, XG_LU_FP64, info, true);
  return XG_OK;
}
