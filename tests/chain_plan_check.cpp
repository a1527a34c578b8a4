// chain_plan_check.cpp — test program for build_chain_plan (lu_chain.h).
//
// Reads a CSR matrix (int64 n, nnz; int32 rowptr[n+1], colidx[nnz]; double
// values[nnz]), analyses it (lu_analyze), plans the chain of its last
// `rows` rows and checks the plan:
//  * every L and U entry of the chain lands exactly once, in its block's
//    triangle or in a round of that block, in a row outside the block;
//  * a block's rounds give each row to one thread and keep its entries in
//    the solve's column order; padding is the scratch row with no value;
//  * the blocked solve, emulated on the host with fused multiply-adds in the
//    order the device kernel issues them, gives the same bits as a
//    column-by-column solve, and agrees with a row-by-row solve to rounding.
// Prints "ok" and exits 0, or prints the first failure and exits 1.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <string>
#include <vector>

#include "lu_chain.h"
#include "xg_lu.h"

using namespace xg;

static int fail(const char *what, long a = 0, long b = 0) {
  std::printf("FAIL %s (%ld, %ld)\n", what, a, b);
  return 1;
}

int main(int argc, char **argv) {
  if (argc < 3) return 2;
  FILE *f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int64_t hdr[2];
  if (std::fread(hdr, 8, 2, f) != 2) return 2;
  const int n = int(hdr[0]);
  const int64_t nz = hdr[1];
  std::vector<int> rp(n + 1), ci(nz);
  std::vector<double> av(nz);
  if (std::fread(rp.data(), 4, n + 1, f) != size_t(n + 1) || std::fread(ci.data(), 4, nz, f) != size_t(nz) ||
      std::fread(av.data(), 8, nz, f) != size_t(nz))
    return 2;
  std::fclose(f);
  LuSymbolic S;
  std::string err;
  if (lu_analyze(n, rp.data(), ci.data(), av.data(), 0.001, &S, &err)) return fail("analysis");
  const int nt = std::atoi(argv[2]), t0 = n - nt;
  if (nt < 1 || nt >= n) return fail("chain rows out of range", nt, n);
  const ChainPlan P = build_chain_plan(S, t0);

  // every chain entry exactly once
  std::vector<int> seen(S.ci.size(), 0);
  size_t e = 0;
  for (size_t b = 0; b < P.blocks.size(); ++b) {
    const ChainBlock &B = P.blocks[b];
    if (B.bs < 1 || B.bs > kChainBlock) return fail("block size", long(b), B.bs);
    const int *src = P.tile_src.data() + b * kChainTileValues;
    for (int j = 0; j < kChainBlock; ++j)
      for (int i = 0; i < kChainBlock; ++i) {
        const int s = src[j * kChainBlock + i];
        if (s < 0) continue;
        if (i <= j || i >= B.bs) return fail("triangle slot", long(b), j * kChainBlock + i);
        ++seen[s];
      }
    for (int l = 0; l < kChainLanes; ++l) {
      int prev_row = -1, prev_j = -1;
      for (int k = 0; k < B.rounds; ++k) {
        const int rj = P.ent_rowj[e + size_t(k) * kChainLanes + l], s = P.ent_src[e + size_t(k) * kChainLanes + l];
        const int r = rj >> 5, j = rj & 31;
        if (s < 0) {
          if (r != nt) return fail("padding row", long(b), r);
          continue;
        }
        const int lane_of_row = B.upper ? B.cbase - r : r - B.cbase;
        if (lane_of_row >= 0 && lane_of_row < B.bs) return fail("round row inside block", long(b), r);
        if (j >= B.bs) return fail("round column", long(b), j);
        if (r == prev_row && j <= prev_j) return fail("column order", long(b), r);
        prev_row = r;
        prev_j = j;
        ++seen[s];
      }
    }
    e += size_t(B.rounds) * kChainLanes;
  }
  if (e != P.ent_rowj.size()) return fail("round count", long(e), long(P.ent_rowj.size()));
  for (int r = t0; r < n; ++r)
    for (int p = S.rp[r]; p < S.rp[r + 1]; ++p) {
      const bool chain = p > S.diag[r] || (p < S.diag[r] && S.ci[p] >= t0);
      if (seen[p] != (chain ? 1 : 0)) return fail("entry placement", r, p);
    }
  // each row's rounds belong to one thread per block
  e = 0;
  for (size_t b = 0; b < P.blocks.size(); ++b) {
    std::vector<int> owner(nt + 1, -1);
    for (int k = 0; k < P.blocks[b].rounds; ++k)
      for (int l = 0; l < kChainLanes; ++l) {
        const int r = P.ent_rowj[e + size_t(k) * kChainLanes + l] >> 5;
        if (r == nt) continue;
        if (owner[r] >= 0 && owner[r] != l) return fail("row on two threads", long(b), r);
        owner[r] = l;
      }
    e += size_t(P.blocks[b].rounds) * kChainLanes;
  }

  // numbers: random L\U values and pivots, random starting sums
  std::mt19937_64 rng(11);
  std::uniform_real_distribution<double> U(-0.05, 0.05), D(0.5, 1.5);
  std::vector<double> val(S.ci.size()), rdiag(n), acc0(nt);
  for (double &x : val) x = U(rng);
  for (double &x : rdiag) x = D(rng);
  for (double &x : acc0) x = 20 * U(rng);
  // column by column
  std::vector<std::vector<std::pair<int, int>>> lcol(nt), ucol(nt);
  for (int r = t0; r < n; ++r) {
    for (int p = S.rp[r]; p < S.diag[r]; ++p)
      if (S.ci[p] >= t0) lcol[S.ci[p] - t0].push_back({r - t0, p});
    for (int p = S.diag[r] + 1; p < S.rp[r + 1]; ++p) ucol[S.ci[p] - t0].push_back({r - t0, p});
  }
  std::vector<double> a(acc0), zc(nt);
  for (int c = 0; c < nt; ++c)
    for (const auto &q : lcol[c]) a[q.first] = std::fma(-val[q.second], a[c], a[q.first]);
  for (int c = nt - 1; c >= 0; --c) {
    zc[c] = a[c] * rdiag[t0 + c];
    for (const auto &q : ucol[c]) a[q.first] = std::fma(-val[q.second], zc[c], a[q.first]);
  }
  // row by row
  std::vector<double> yr(nt), zr(nt);
  for (int r = 0; r < nt; ++r) {
    double s = acc0[r];
    for (int p = S.rp[t0 + r]; p < S.diag[t0 + r]; ++p)
      if (S.ci[p] >= t0) s -= val[p] * yr[S.ci[p] - t0];
    yr[r] = s;
  }
  for (int r = nt - 1; r >= 0; --r) {
    double s = yr[r];
    for (int p = S.diag[t0 + r] + 1; p < S.rp[t0 + r + 1]; ++p) s -= val[p] * zr[S.ci[p] - t0];
    zr[r] = s * rdiag[t0 + r];
  }
  // blocked, as the device kernel orders it
  std::vector<double> acc(nt + 1, 0.0), zb(nt, 0.0);
  for (int c = 0; c < nt; ++c) acc[c] = acc0[c];
  e = 0;
  for (size_t b = 0; b < P.blocks.size(); ++b) {
    const ChainBlock &B = P.blocks[b];
    const int *src = P.tile_src.data() + b * kChainTileValues;
    auto tv = [&](int k) {
      const int s = src[k];
      return s >= 0 ? val[s] : s == -1 ? 0.0 : rdiag[-2 - s];
    };
    double lane[kChainBlock];
    for (int i = 0; i < kChainBlock; ++i)
      lane[i] = i < B.bs ? acc[B.upper ? B.cbase - i : B.cbase + i] : 0.0;
    for (int t = 0; t < B.bs; ++t) {
      if (B.upper) lane[t] *= tv(kChainBlock * kChainBlock + t);
      for (int i = t + 1; i < kChainBlock; ++i) lane[i] = std::fma(-tv(t * kChainBlock + i), lane[t], lane[i]);
    }
    for (int i = 0; i < B.bs; ++i) {
      const int col = B.upper ? B.cbase - i : B.cbase + i;
      if (B.upper) zb[col] = lane[i];
      else acc[col] = lane[i];
    }
    std::vector<int> cur(kChainLanes, -1);
    std::vector<double> ar(kChainLanes, 0.0);
    for (int k = 0; k < B.rounds; ++k)
      for (int l = 0; l < kChainLanes; ++l) {
        const int rj = P.ent_rowj[e + size_t(k) * kChainLanes + l], s = P.ent_src[e + size_t(k) * kChainLanes + l];
        const int r = rj >> 5;
        if (r != cur[l]) {
          if (cur[l] >= 0) acc[cur[l]] = ar[l];
          ar[l] = acc[r];
          cur[l] = r;
        }
        ar[l] = std::fma(-(s >= 0 ? val[s] : 0.0), lane[rj & 31], ar[l]);
      }
    for (int l = 0; l < kChainLanes; ++l)
      if (cur[l] >= 0) acc[cur[l]] = ar[l];
    e += size_t(B.rounds) * kChainLanes;
  }
  double scale = 0, diff = 0;
  for (int c = 0; c < nt; ++c) {
    if (zb[c] != zc[c]) return fail("blocked differs from column order", c);
    scale = std::fmax(scale, std::fabs(zr[c]));
    diff = std::fmax(diff, std::fabs(zb[c] - zr[c]));
  }
  if (!(diff <= 1e-12 * scale)) return fail("blocked differs from row order", long(diff * 1e15), long(scale));
  // the rows a block sums after the grid solves (solo_rows), with a low
  // length bar so the small matrix has some: a solve that leaves them to the
  // end never reads one of them before it is computed, and gives the same
  // values as the plain row order
  {
    const int bar = argc > 3 ? std::atoi(argv[3]) : 2;
    std::vector<unsigned char> solo;
    std::vector<int> long_l, long_u;
    solo_rows(S, t0, bar, &solo, &long_l, &long_u);
    size_t nl = 0, nu = 0;
    for (int i = 0; i < n; ++i) {
      if ((solo[i] & 1) && (i >= t0 || S.diag[i] - S.rp[i] <= bar)) return fail("solo L row", i);
      if ((solo[i] & 2) && (i >= t0 || S.rp[i + 1] - S.diag[i] - 1 <= bar)) return fail("solo U row", i);
      if (solo[i] & 1) {
        if (nl >= long_l.size() || long_l[nl] != i) return fail("long_l list", i);
        ++nl;
      }
      if (solo[i] & 2) {
        if (nu >= long_u.size() || long_u[nu] != i) return fail("long_u list", i);
        ++nu;
      }
    }
    if (nl != long_l.size() || nu != long_u.size()) return fail("list lengths");
    std::vector<double> b(n), yp(n), zp(n), yd(n, 0.0), zd(n, 0.0);
    std::vector<char> done(n, 0);
    for (double &x : b) x = U(rng);
    for (int i = 0; i < n; ++i) {
      double s = b[i];
      for (int p = S.rp[i]; p < S.diag[i]; ++p) s -= val[p] * yp[S.ci[p]];
      yp[i] = s;
    }
    auto lower_row = [&](int i) {
      double s = b[i];
      for (int p = S.rp[i]; p < S.diag[i]; ++p) {
        if (!done[S.ci[p]]) return false;
        s -= val[p] * yd[S.ci[p]];
      }
      yd[i] = s;
      done[i] = 1;
      return true;
    };
    for (int i = 0; i < n; ++i)
      if (!(solo[i] & 1) && !lower_row(i)) return fail("lower solve read a deferred row", i);
    for (int i : long_l)
      if (!lower_row(i)) return fail("deferred lower row not ready", i);
    for (int i = n - 1; i >= 0; --i) {
      double s = yp[i];
      for (int p = S.diag[i] + 1; p < S.rp[i + 1]; ++p) s -= val[p] * zp[S.ci[p]];
      zp[i] = s * rdiag[i];
    }
    std::fill(done.begin(), done.end(), 0);
    auto upper_row = [&](int i) {
      double s = yd[i];
      for (int p = S.diag[i] + 1; p < S.rp[i + 1]; ++p) {
        if (!done[S.ci[p]]) return false;
        s -= val[p] * zd[S.ci[p]];
      }
      zd[i] = s * rdiag[i];
      done[i] = 1;
      return true;
    };
    for (int i = n - 1; i >= 0; --i)
      if (!(solo[i] & 2) && !upper_row(i)) return fail("upper solve read a deferred row", i);
    for (int i : long_u)
      if (!upper_row(i)) return fail("deferred upper row not ready", i);
    for (int i = 0; i < n; ++i)
      if (zd[i] != zp[i]) return fail("deferred rows change the solution", i);
    std::printf("solo rows: %zu lower, %zu upper\n", long_l.size(), long_u.size());
  }
  std::printf("ok blocks %zu entries %zu\n", P.blocks.size(), P.ent_rowj.size());
  return 0;
}
