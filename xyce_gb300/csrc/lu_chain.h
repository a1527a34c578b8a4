// lu_chain.h — host plans of the grid solves' special rows (lu_kernels.cu):
// the blocked chain (lu_solve_chain), the trailing rows of a factor that the
// grid-wide solves hand to one CTA, and the long rows no other row waits
// for (lu_solve_long, solo_rows below).
//
// The chain is solved 32 columns at a time, both ways (forward over L,
// columns ascending; backward over U, columns descending).  For a block:
//  * its tile: the 32 x 32 triangle of the block's own rows and columns,
//    column-major (tile value j * 32 + i: lane-row i, lane-column j), then
//    the 32 reciprocal pivots (backward solve) and the 32 x positions;
//  * its rounds: the block's entries in rows outside it (below it forward,
//    above it backward), each row given to one of kChainLanes threads
//    (longest rows first, to the least loaded), a thread's rows one after
//    another and each row's entries in the solve's column order; round k
//    holds every thread's k-th entry (the scratch row nt, value 0, where a
//    thread has run out).
// A row's running sum so takes its updates in the column order of a
// column-by-column solve, the same on every run.
#pragma once
#include <algorithm>
#include <cstdint>
#include <utility>
#include <vector>

#include "xg_lu.h"

namespace xg {

constexpr int kChainBlock = 32;
constexpr int kChainLanes = 128;  // threads sharing a block's rounds
constexpr int kChainTileValues = kChainBlock * kChainBlock + kChainBlock;  // triangle, reciprocal pivots

struct ChainBlock {
  int cbase;   // the column of lane 0 (chain-local); lane i has cbase + i forward, cbase - i backward
  int bs;      // columns in the block (<= 32)
  int rounds;  // rounds of the block's entries outside it
  int upper;   // 1: backward solve
};

struct ChainPlan {
  int t0 = 0, nt = 0;
  std::vector<ChainBlock> blocks;  // forward blocks, then backward blocks
  // per block, kChainTileValues value sources: >= 0 a position of the L\U
  // values, -1 zero, <= -2 the reciprocal pivot of row -2 - src
  std::vector<int> tile_src;
  std::vector<int> tile_q;         // per block 32 x positions (backward), 0 otherwise
  // per entry (kChainLanes per round): (chain-local row << 5) |
  // lane-column, and the position of its value (-1: padding)
  std::vector<int> ent_rowj, ent_src;
};

// Plan of the chain of rows [t0, n) of the analysed factor S.
inline ChainPlan build_chain_plan(const LuSymbolic &S, int t0) {
  ChainPlan P;
  const int n = S.n, nt = n - t0;
  P.t0 = t0;
  P.nt = nt;
  if (nt <= 0) return P;
  // per chain column: its L entries (rows below) and U entries (rows above)
  // in chain rows, as (chain-local row, position)
  std::vector<std::vector<std::pair<int, int>>> lcol(nt), ucol(nt);
  for (int r = t0; r < n; ++r) {
    for (int p = S.rp[r]; p < S.diag[r]; ++p)
      if (S.ci[p] >= t0) lcol[S.ci[p] - t0].push_back({r - t0, p});
    for (int p = S.diag[r] + 1; p < S.rp[r + 1]; ++p) ucol[S.ci[p] - t0].push_back({r - t0, p});
  }
  std::vector<int> row_slot(nt, -1);  // scratch: a row's index in the block's row list
  auto add_block = [&](int cbase, int bs, int upper) {
    const int b = int(P.blocks.size());
    P.tile_src.resize(size_t(b + 1) * kChainTileValues, -1);
    P.tile_q.resize(size_t(b + 1) * kChainBlock, 0);
    int *src = P.tile_src.data() + size_t(b) * kChainTileValues;
    int *q = P.tile_q.data() + size_t(b) * kChainBlock;
    auto lane_of = [&](int col) { return upper ? cbase - col : col - cbase; };  // -1.. or >= bs: outside
    // rows outside the block and their entries (lane-column, position)
    std::vector<int> rows;
    std::vector<std::vector<std::pair<int, int>>> ents;
    for (int j = 0; j < bs; ++j) {
      const int col = upper ? cbase - j : cbase + j;
      for (const auto &e : upper ? ucol[col] : lcol[col]) {
        const int i = lane_of(e.first);
        if (i >= 0 && i < bs) {
          src[j * kChainBlock + i] = e.second;  // inside: the triangle (i > j)
          continue;
        }
        if (row_slot[e.first] < 0) {
          row_slot[e.first] = int(rows.size());
          rows.push_back(e.first);
          ents.emplace_back();
        }
        ents[row_slot[e.first]].push_back({j, e.second});  // j ascending: the solve's column order
      }
    }
    for (int r : rows) row_slot[r] = -1;
    if (upper)
      for (int i = 0; i < bs; ++i) {
        src[kChainBlock * kChainBlock + i] = -2 - (t0 + cbase - i);
        q[i] = S.Q[t0 + cbase - i];
      }
    // rows to lanes, longest first to the least loaded
    std::vector<int> order(rows.size());
    for (size_t k = 0; k < order.size(); ++k) order[k] = int(k);
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int c) { return ents[a].size() > ents[c].size(); });
    std::vector<std::vector<int>> lane_rows(kChainLanes);
    std::vector<size_t> load(kChainLanes, 0);
    for (int k : order) {
      int best = 0;
      for (int l = 1; l < kChainLanes; ++l)
        if (load[l] < load[best]) best = l;
      lane_rows[best].push_back(k);
      load[best] += ents[k].size();
    }
    size_t rounds = 0;
    for (size_t l : load) rounds = std::max(rounds, l);
    const size_t e0 = P.ent_rowj.size();
    P.ent_rowj.resize(e0 + rounds * kChainLanes, nt << 5);
    P.ent_src.resize(e0 + rounds * kChainLanes, -1);
    for (int l = 0; l < kChainLanes; ++l) {
      size_t k = 0;
      for (int ri : lane_rows[l])
        for (const auto &e : ents[ri]) {
          P.ent_rowj[e0 + k * kChainLanes + l] = (rows[ri] << 5) | e.first;
          P.ent_src[e0 + k * kChainLanes + l] = e.second;
          ++k;
        }
    }
    P.blocks.push_back(ChainBlock{cbase, bs, int(rounds), upper});
  };
  for (int c0 = 0; c0 < nt; c0 += kChainBlock) add_block(c0, std::min(kChainBlock, nt - c0), 0);
  for (int c1 = nt - 1; c1 >= 0; c1 -= kChainBlock) add_block(c1, std::min(kChainBlock, c1 + 1), 1);
  return P;
}

// Rows of the grid solves (below the chain, rows < t0) that a block sums on
// its own after the grid solve instead of a warp inside it: bit 0 of
// (*solo)[i] when row i's L part is longer than min_len and its column has
// no L entry below it (no later row of the lower solve reads its y), bit 1
// when its U part is longer than min_len and its column has no U entry
// above it (no earlier row of the upper solve reads its z).  *long_l and
// *long_u list those rows, ascending.
inline void solo_rows(const LuSymbolic &S, int t0, int min_len, std::vector<unsigned char> *solo,
                      std::vector<int> *long_l, std::vector<int> *long_u) {
  const int n = S.n;
  solo->assign(n, 0);
  long_l->clear();
  long_u->clear();
  std::vector<unsigned char> l_read(n, 0), u_read(n, 0);
  for (int i = 0; i < n; ++i) {
    for (int p = S.rp[i]; p < S.diag[i]; ++p) l_read[S.ci[p]] = 1;
    for (int p = S.diag[i] + 1; p < S.rp[i + 1]; ++p) u_read[S.ci[p]] = 1;
  }
  for (int i = 0; i < t0; ++i) {
    if (S.diag[i] - S.rp[i] > min_len && !l_read[i]) {
      (*solo)[i] |= 1;
      long_l->push_back(i);
    }
    if (S.rp[i + 1] - S.diag[i] - 1 > min_len && !u_read[i]) {
      (*solo)[i] |= 2;
      long_u->push_back(i);
    }
  }
}

}  // namespace xg
