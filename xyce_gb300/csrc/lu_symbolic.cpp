// lu_symbolic.cpp — host symbolic analysis of the Newton-solve LU.
//
// The reference's KLU analysis (Amesos_Klu SymbolicFactorization and the
// first NumericFactorization, N_LAS_AmesosSolver.C:388-405) orders the
// matrix with AMD and then factors it left-looking with threshold partial
// pivoting (Gilbert-Peierls).  Both steps are restated here from the
// published methods:
//   * approximate minimum degree on a quotient graph (Amestoy, Davis and
//     Duff, "An approximate minimum degree ordering algorithm", SIAM J.
//     Matrix Anal. Appl. 17(4), 1996): element absorption, the approximate
//     external degree bound, aggressive absorption, dense rows ordered last;
//     supervariable detection is left out;
//   * left-looking sparse LU with a depth-first search for the nonzero
//     pattern of each column (Gilbert and Peierls, "Sparse partial pivoting
//     in time proportional to arithmetic operations", SIAM J. Sci. Stat.
//     Comput. 9(5), 1988), diagonal preference with a relative threshold as
//     KLU uses (tol 0.001).
// The pivot order found on the first matrix is kept for every later
// factorisation, which the GPU performs (lu_kernels.cu).

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include "xg_lu.h"

namespace xg {

namespace {

// Degree buckets: doubly linked lists of variables by approximate degree.
struct Buckets {
  std::vector<int> head, next, prev;
  int mindeg = 0;
  explicit Buckets(int n) : head(n + 1, -1), next(n, -1), prev(n, -1) {}
  void insert(int i, int d) {
    prev[i] = -1;
    next[i] = head[d];
    if (head[d] >= 0) prev[head[d]] = i;
    head[d] = i;
    if (d < mindeg) mindeg = d;
  }
  void remove(int i, int d) {
    if (prev[i] >= 0) next[prev[i]] = next[i]; else head[d] = next[i];
    if (next[i] >= 0) prev[next[i]] = prev[i];
    next[i] = prev[i] = -1;
  }
  int pop_min(int maxd) {
    while (mindeg <= maxd && head[mindeg] < 0) ++mindeg;
    if (mindeg > maxd) return -1;
    int i = head[mindeg];
    remove(i, mindeg);
    return i;
  }
};

}  // namespace

std::vector<int> amd_order(int n, const int *rp, const int *ci, int *n_dense_out) {
  // symmetric adjacency without the diagonal
  std::vector<std::vector<int>> adj(n);
  for (int i = 0; i < n; ++i)
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
      int j = ci[p];
      if (j == i) continue;
      adj[i].push_back(j);
      adj[j].push_back(i);
    }
  for (auto &a : adj) {
    std::sort(a.begin(), a.end());
    a.erase(std::unique(a.begin(), a.end()), a.end());
  }
  // dense rows go last, in their original order
  const int dense = std::max(16, int(10.0 * std::sqrt(double(n))));
  enum : char { VAR = 0, ELEM = 1, DEAD = 2, DENSE = 3 };
  std::vector<char> state(n, VAR);
  std::vector<int> dense_list;
  for (int i = 0; i < n; ++i)
    if (int(adj[i].size()) > dense) {
      state[i] = DENSE;
      dense_list.push_back(i);
    }
  if (!dense_list.empty())
    for (int i = 0; i < n; ++i) {
      if (state[i] == DENSE) { adj[i].clear(); continue; }
      auto &a = adj[i];
      a.erase(std::remove_if(a.begin(), a.end(), [&](int j) { return state[j] == DENSE; }), a.end());
    }
  const int nv = n - int(dense_list.size());
  std::vector<std::vector<int>> elems(n), members(n);
  std::vector<int> deg(n, 0), mark(n, 0), wstamp(n, 0), w(n, 0);
  int stamp = 0, wst = 0;
  Buckets B(n);
  for (int i = 0; i < n; ++i)
    if (state[i] == VAR) {
      deg[i] = int(adj[i].size());
      B.insert(i, deg[i]);
    }
  B.mindeg = 0;
  std::vector<int> order;
  order.reserve(n);
  std::vector<int> Lp;
  int alive = nv;
  while (int(order.size()) < nv) {
    const int p = B.pop_min(n);
    if (p < 0) break;
    ++stamp;
    mark[p] = stamp;
    Lp.clear();
    // new element: union of p's elements and p's variable neighbours
    for (int e : elems[p]) {
      if (state[e] != ELEM) continue;
      for (int v : members[e])
        if (state[v] == VAR && mark[v] != stamp) { mark[v] = stamp; Lp.push_back(v); }
      state[e] = DEAD;  // absorbed into p
      std::vector<int>().swap(members[e]);
    }
    for (int v : adj[p])
      if (state[v] == VAR && mark[v] != stamp) { mark[v] = stamp; Lp.push_back(v); }
    state[p] = ELEM;
    std::vector<int>().swap(adj[p]);
    std::vector<int>().swap(elems[p]);
    order.push_back(p);
    --alive;
    // prune the neighbours' lists; p now stands for the absorbed elements
    for (int i : Lp) {
      B.remove(i, deg[i]);
      auto &E = elems[i];
      E.erase(std::remove_if(E.begin(), E.end(), [&](int e) { return state[e] != ELEM; }), E.end());
      E.push_back(p);
      auto &A = adj[i];
      A.erase(std::remove_if(A.begin(), A.end(),
                             [&](int v) { return state[v] != VAR || mark[v] == stamp; }),
              A.end());
    }
    // |Le \ Lp| for every element next to Lp
    ++wst;
    for (int i : Lp)
      for (int e : elems[i]) {
        if (e == p) continue;
        if (wstamp[e] != wst) { wstamp[e] = wst; w[e] = int(members[e].size()); }
        --w[e];
      }
    const int lp_ext = int(Lp.size()) - 1;
    for (int i : Lp) {
      int d = int(adj[i].size()) + lp_ext;
      auto &E = elems[i];
      for (int e : E) {
        if (e == p || state[e] != ELEM) continue;
        if (w[e] <= 0) {
          state[e] = DEAD;  // aggressive absorption: Le is inside Lp
          std::vector<int>().swap(members[e]);
        } else {
          d += w[e];
        }
      }
      E.erase(std::remove_if(E.begin(), E.end(), [&](int e) { return state[e] != ELEM; }), E.end());
      d = std::min(d, deg[i] + lp_ext);
      d = std::min(d, alive - 1);
      deg[i] = std::max(d, 0);
      B.insert(i, deg[i]);
    }
    members[p] = Lp;
  }
  for (int i : dense_list) order.push_back(i);
  if (n_dense_out) *n_dense_out = int(dense_list.size());
  return order;
}

// Nested dissection by level-structure separators (A. George, "Nested
// dissection of a regular finite element mesh", SIAM J. Numer. Anal. 10(2),
// 1973; the automatic form of George and Liu, "Computer Solution of Large
// Sparse Positive Definite Systems", 1981, ch. 8): a breadth-first level
// structure from a pseudo-peripheral vertex, the smallest level near the
// middle as separator (only its vertices with a neighbour in the next level),
// the two sides ordered first, recursively, the separator after them.  Parts
// of at most `leaf` vertices are ordered by minimum degree; disconnected
// parts are split without a separator; dense vertices go last as in
// amd_order.  The elimination tree is then about log2(n / leaf) separators
// deep instead of following the long chains minimum degree leaves in
// path-like circuits.
std::vector<int> nd_order(int n, const int *rp, const int *ci, int leaf, int *n_dense_out) {
  std::vector<int> ap(n + 1, 0), aj;
  {
    std::vector<std::vector<int>> adj(n);
    for (int i = 0; i < n; ++i)
      for (int p = rp[i]; p < rp[i + 1]; ++p) {
        int j = ci[p];
        if (j == i) continue;
        adj[i].push_back(j);
        adj[j].push_back(i);
      }
    for (int i = 0; i < n; ++i) {
      auto &a = adj[i];
      std::sort(a.begin(), a.end());
      a.erase(std::unique(a.begin(), a.end()), a.end());
      ap[i + 1] = ap[i] + int(a.size());
    }
    aj.reserve(ap[n]);
    for (auto &a : adj) aj.insert(aj.end(), a.begin(), a.end());
  }
  const int dense = std::max(16, int(10.0 * std::sqrt(double(n))));
  std::vector<char> is_dense(n, 0);
  std::vector<int> dense_list, all;
  for (int i = 0; i < n; ++i) {
    if (ap[i + 1] - ap[i] > dense) { is_dense[i] = 1; dense_list.push_back(i); }
    else all.push_back(i);
  }
  std::vector<int> order;
  order.reserve(n);
  std::vector<int> in_set(n, 0), level(n, -1), local(n, -1);
  int stamp = 0;
  // Work items: a vertex set to dissect, or a separator to emit.  Popping
  // A's subtree before B's and the separator last gives a post-order.
  struct Item { bool emit; std::vector<int> v; };
  std::vector<Item> work;
  work.push_back({false, std::move(all)});
  std::vector<int> queue, counts;
  auto bfs = [&](int root, int st, std::vector<int> &q) {
    q.clear();
    q.push_back(root);
    level[root] = 0;
    in_set[root] = -st;  // visited in this search
    for (size_t h = 0; h < q.size(); ++h) {
      int u = q[h];
      for (int p = ap[u]; p < ap[u + 1]; ++p) {
        int v = aj[p];
        if (in_set[v] != st) continue;
        in_set[v] = -st;
        level[v] = level[u] + 1;
        q.push_back(v);
      }
    }
    for (int u : q) in_set[u] = st;  // restore membership
  };
  auto order_leaf = [&](const std::vector<int> &V) {
    // minimum degree on the induced subgraph
    const int m = int(V.size());
    for (int k = 0; k < m; ++k) local[V[k]] = k;
    std::vector<int> lp(m + 1, 0), lj;
    for (int k = 0; k < m; ++k) {
      int u = V[k];
      for (int p = ap[u]; p < ap[u + 1]; ++p)
        if (local[aj[p]] >= 0 && !is_dense[aj[p]]) lj.push_back(local[aj[p]]);
      lp[k + 1] = int(lj.size());
    }
    std::vector<int> o = amd_order(m, lp.data(), lj.data(), nullptr);
    for (int k : o) order.push_back(V[k]);
    for (int u : V) local[u] = -1;
  };
  while (!work.empty()) {
    Item it = std::move(work.back());
    work.pop_back();
    std::vector<int> &V = it.v;
    if (it.emit) {
      order.insert(order.end(), V.begin(), V.end());
      continue;
    }
    if (int(V.size()) <= leaf) {
      order_leaf(V);
      continue;
    }
    const int st = ++stamp;
    for (int u : V) in_set[u] = st;
    // pseudo-peripheral root: restart from a least-degree vertex of the last
    // level while the eccentricity grows
    int root = V[0], ecc = -1;
    for (int tries = 0; tries < 6; ++tries) {
      bfs(root, st, queue);
      int e = level[queue.back()];
      if (e <= ecc) break;
      ecc = e;
      int best = queue.back(), bd = n + 1;
      for (int k = int(queue.size()) - 1; k >= 0 && level[queue[k]] == e; --k) {
        int d = ap[queue[k] + 1] - ap[queue[k]];
        if (d < bd) { bd = d; best = queue[k]; }
      }
      if (tries < 5) root = best;
    }
    bfs(root, st, queue);
    if (queue.size() < V.size()) {
      // disconnected: this component and the rest are independent parts
      std::vector<int> rest;
      for (int u : V)
        if (level[u] < 0) rest.push_back(u);
      for (int u : V) level[u] = -1;
      work.push_back({false, std::move(rest)});
      work.push_back({false, queue});
      continue;
    }
    const int h = level[queue.back()] + 1;
    if (h < 3) {  // too shallow to split: a near-clique
      for (int u : V) level[u] = -1;
      order_leaf(V);
      continue;
    }
    counts.assign(h, 0);
    for (int u : V) counts[level[u]]++;
    int mid = 0;
    for (int c = 0, acc = 0; c < h; ++c) {
      acc += counts[c];
      if (2 * acc >= int(V.size())) { mid = c; break; }
    }
    int m = std::min(std::max(mid, 1), h - 2);
    for (int c = std::max(1, mid - 2); c <= std::min(h - 2, mid + 2); ++c)
      if (counts[c] < counts[m] || (counts[c] == counts[m] && std::abs(c - mid) < std::abs(m - mid)))
        m = c;
    std::vector<int> A, B, sep;
    for (int u : V) {
      int lu = level[u];
      if (lu < m) { A.push_back(u); continue; }
      if (lu > m) { B.push_back(u); continue; }
      bool touches = false;
      for (int p = ap[u]; p < ap[u + 1] && !touches; ++p)
        touches = in_set[aj[p]] == st && level[aj[p]] == m + 1;
      (touches ? sep : A).push_back(u);
    }
    for (int u : V) level[u] = -1;
    work.push_back({true, std::move(sep)});
    work.push_back({false, std::move(B)});
    work.push_back({false, std::move(A)});
  }
  for (int i : dense_list) order.push_back(i);
  if (n_dense_out) *n_dense_out = int(dense_list.size());
  return order;
}

namespace {

// The pivoting factorisation for a given column order.
int analyze_ordered(int n, const int *rp, const int *ci, const double *val, double pivot_tol,
                    std::vector<int> order, int n_dense, LuSymbolic *out, std::string *err) {
  LuSymbolic &S = *out;
  S = LuSymbolic();
  S.n = n;
  S.nnz_a = rp[n];
  S.Q = std::move(order);
  S.n_dense = n_dense;
  std::vector<int> qinv(n);
  for (int j = 0; j < n; ++j) qinv[S.Q[j]] = j;
  // A by columns, remembering each entry's CSR index
  std::vector<int> cp(n + 1, 0), cr(S.nnz_a), cpos(S.nnz_a);
  for (int64_t p = 0; p < S.nnz_a; ++p) cp[ci[p] + 1]++;
  for (int j = 0; j < n; ++j) cp[j + 1] += cp[j];
  {
    std::vector<int> fill(cp.begin(), cp.end() - 1);
    for (int i = 0; i < n; ++i)
      for (int p = rp[i]; p < rp[i + 1]; ++p) {
        int q = fill[ci[p]]++;
        cr[q] = i;
        cpos[q] = p;
      }
  }
  // left-looking factorisation with partial pivoting
  std::vector<int> pinv(n, -1);
  std::vector<int> Lcp(1, 0), Li;
  std::vector<double> Lx;
  std::vector<int> Ucp(1, 0), Ui;
  std::vector<double> Ux;
  std::vector<double> x(n, 0.0);
  std::vector<int> visited(n, -1), xi(n), stack(n), pstack(n);
  S.P.assign(n, -1);
  S.min_pivot = INFINITY;
  S.max_pivot = 0;
  for (int k = 0; k < n; ++k) {
    const int col = S.Q[k];
    int top = n;
    // depth-first search from each nonzero of A(:, col) through the graph of L
    for (int q = cp[col]; q < cp[col + 1]; ++q) {
      int r0 = cr[q];
      if (visited[r0] == k) continue;
      int head = 0;
      stack[0] = r0;
      while (head >= 0) {
        int r = stack[head];
        int jc = pinv[r];
        if (visited[r] != k) {
          visited[r] = k;
          pstack[head] = jc < 0 ? 0 : Lcp[jc];
        }
        int pend = jc < 0 ? 0 : Lcp[jc + 1];
        bool leaf = true;
        for (int p = pstack[head]; p < pend; ++p) {
          int child = Li[p];
          if (visited[child] == k) continue;
          pstack[head] = p + 1;
          stack[++head] = child;
          leaf = false;
          break;
        }
        if (leaf) {
          --head;
          xi[--top] = r;
        }
      }
    }
    for (int q = top; q < n; ++q) x[xi[q]] = 0.0;
    for (int q = cp[col]; q < cp[col + 1]; ++q) x[cr[q]] = val[cpos[q]];
    // x = L \ A(:, col) in topological order
    for (int q = top; q < n; ++q) {
      int r = xi[q];
      int j = pinv[r];
      if (j < 0) continue;
      double xj = x[r];
      for (int p = Lcp[j]; p < Lcp[j + 1]; ++p) x[Li[p]] -= Lx[p] * xj;
    }
    // pivot: largest candidate, or the diagonal when within the threshold
    int best = -1;
    double amax = 0.0;
    for (int q = top; q < n; ++q) {
      int r = xi[q];
      if (pinv[r] >= 0) continue;
      double a = std::fabs(x[r]);
      if (best < 0 || a > amax) { amax = a; best = r; }
    }
    if (best < 0 || !(amax > 0.0) || !std::isfinite(amax)) {
      *err = "lu_analyze: matrix is singular at pivot step " + std::to_string(k) +
             " (column " + std::to_string(col) + ")";
      return -1;
    }
    int piv = best;
    const int drow = col;
    if (visited[drow] == k && pinv[drow] < 0 && std::fabs(x[drow]) >= pivot_tol * amax) piv = drow;
    const double pivot = x[piv];
    // U(:, k): rows already pivotal, then the diagonal
    for (int q = top; q < n; ++q) {
      int r = xi[q];
      if (pinv[r] >= 0) {
        Ui.push_back(pinv[r]);
        Ux.push_back(x[r]);
      }
    }
    Ui.push_back(k);
    Ux.push_back(pivot);
    Ucp.push_back(int(Ui.size()));
    // L(:, k): the other candidates, scaled
    for (int q = top; q < n; ++q) {
      int r = xi[q];
      if (pinv[r] < 0 && r != piv) {
        Li.push_back(r);
        Lx.push_back(x[r] / pivot);
      }
    }
    Lcp.push_back(int(Li.size()));
    pinv[piv] = k;
    S.P[k] = piv;
    S.min_pivot = std::min(S.min_pivot, std::fabs(pivot));
    S.max_pivot = std::max(S.max_pivot, std::fabs(pivot));
  }
  // row-wise L\U pattern of B = A(P, Q)
  std::vector<int> cnt(n + 1, 0);
  for (size_t p = 0; p < Li.size(); ++p) cnt[pinv[Li[p]] + 1]++;
  for (size_t p = 0; p < Ui.size(); ++p) cnt[Ui[p] + 1]++;
  S.rp.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) S.rp[i + 1] = S.rp[i] + cnt[i + 1];
  S.ci.assign(S.rp[n], 0);
  S.diag.assign(n, -1);
  {
    std::vector<int> fill(S.rp.begin(), S.rp.end() - 1);
    for (int j = 0; j < n; ++j) {
      for (int p = Ucp[j]; p < Ucp[j + 1]; ++p) {
        int r = Ui[p];
        int q = fill[r]++;
        S.ci[q] = j;
        if (r == j) S.diag[r] = q;
      }
      for (int p = Lcp[j]; p < Lcp[j + 1]; ++p) {
        int r = pinv[Li[p]];
        S.ci[fill[r]++] = j;
      }
    }
  }
  // the columns of a row arrive in ascending order, U entries of a row come
  // from later columns than its L entries: rows are sorted.
  S.lu2a.assign(S.rp[n], -1);
  for (int i = 0; i < n; ++i)
    for (int p = rp[i]; p < rp[i + 1]; ++p) {
      int bi = pinv[i], bj = qinv[ci[p]];
      auto b = S.ci.begin() + S.rp[bi], e = S.ci.begin() + S.rp[bi + 1];
      auto it = std::lower_bound(b, e, bj);
      if (it == e || *it != bj) {
        *err = "lu_analyze: internal error, A entry missing from the L\\U pattern";
        return -1;
      }
      S.lu2a[it - S.ci.begin()] = p;
    }
  // work and dependency depth of one refactorisation
  std::vector<int> level(n, 0);
  double fl = 0, sfl = 0;
  for (int i = 0; i < n; ++i) {
    int lv = 0;
    for (int p = S.rp[i]; p < S.diag[i]; ++p) {
      int k = S.ci[p];
      lv = std::max(lv, level[k]);
      fl += 1 + (S.rp[k + 1] - S.diag[k] - 1);
    }
    level[i] = lv + 1;
    S.levels = std::max(S.levels, level[i]);
    sfl += S.rp[i + 1] - S.rp[i];
  }
  S.refactor_flops = fl;
  S.solve_flops = sfl;
  // rows per level at the widest level: how many rows can be in flight
  std::vector<int> width(S.levels + 1, 0);
  for (int i = 0; i < n; ++i) S.max_width = std::max(S.max_width, ++width[level[i]]);
  return 0;
}

}  // namespace

int lu_analyze(int n, const int *rp, const int *ci, const double *val, double pivot_tol,
               LuSymbolic *out, std::string *err, int ordering) {
  const char *force = ordering >= 0 ? nullptr : std::getenv("XG_LU_ORDER");
  const int forced = !force ? ordering
                            : std::string(force) == "nd" ? 1 : std::string(force) == "amd" ? 0 : -1;
  // (each order is computed before the call: its dense count is an argument)
  auto with_nd = [&](LuSymbolic *dst, std::string *e) {
    int nd_dense = 0;
    std::vector<int> q = nd_order(n, rp, ci, kNdLeaf, &nd_dense);
    if (analyze_ordered(n, rp, ci, val, pivot_tol, std::move(q), nd_dense, dst, e)) return -1;
    dst->ordering = 1;
    return 0;
  };
  if (forced == 1) return with_nd(out, err);
  int amd_dense = 0;
  std::vector<int> q = amd_order(n, rp, ci, &amd_dense);
  if (analyze_ordered(n, rp, ci, val, pivot_tol, std::move(q), amd_dense, out, err)) return -1;
  out->ordering = 0;
  // nested dissection pays where minimum degree leaves chains (few rows per
  // level); on wide matrices it only adds fill, and its analysis costs more
  // than the minimum-degree one
  if (forced == 0 || out->levels <= kNdMinLevels || double(n) / out->levels >= kNdMaxRowsPerLevel)
    return 0;
  // A long dependency chain: try nested dissection and keep it when the
  // modelled refactorisation time is lower.
  LuSymbolic nd;
  std::string nd_err;
  if (with_nd(&nd, &nd_err)) return 0;
  if (lu_model_seconds(nd) < 0.8 * lu_model_seconds(*out)) *out = std::move(nd);
  return 0;
}

bool lu_build_updates(LuSymbolic &S) {
  const int n = S.n;
  S.urp.assign(n + 1, 0);
  for (int i = 0; i < n; ++i) {
    int64_t c = 0;
    for (int p = S.rp[i]; p < S.diag[i]; ++p) {
      const int k = S.ci[p];
      c += S.rp[k + 1] - S.diag[k] - 1;
    }
    S.urp[i + 1] = S.urp[i] + c;
  }
  S.upos.assign(size_t(S.urp[n]), 0);
  std::vector<int> map(n, -1);
  for (int i = 0; i < n; ++i) {
    const int s = S.rp[i], e = S.rp[i + 1];
    for (int p = s; p < e; ++p) map[S.ci[p]] = p;
    int64_t u = S.urp[i];
    for (int p = s; p < S.diag[i]; ++p) {
      const int k = S.ci[p];
      for (int q = S.diag[k] + 1; q < S.rp[k + 1]; ++q) {
        const int pos = map[S.ci[q]];
        if (pos <= p || pos >= e || S.ci[pos] != S.ci[q]) return false;
        S.upos[size_t(u++)] = pos;
      }
    }
    for (int p = s; p < e; ++p) map[S.ci[p]] = -1;
  }
  // the tail: from the first row with a long L part among the last
  // kTailMaxRows rows to the end
  S.tail0 = n;
  for (int i = std::max(0, n - kTailMaxRows); i < n; ++i)
    if (S.diag[i] - S.rp[i] > kTailMinL) { S.tail0 = i; break; }
  S.tail_rowg.assign(1, 0);
  S.tail_gptr.assign(1, 0);
  S.tail_glong.clear();
  S.tail_pos.clear();
  S.tail_pp.assign(1, 0);
  S.tail_pm.clear();
  S.tail_q.clear();
  for (int i = S.tail0; i < n; ++i) {
    const int s = S.rp[i], e = S.rp[i + 1], len = e - s;
    std::vector<std::vector<std::pair<int, int>>> pulls(len);  // by target, pm ascending
    int64_t u = S.urp[i];
    for (int p = s; p < S.diag[i]; ++p) {
      const int k = S.ci[p];
      for (int q = S.diag[k] + 1; q < S.rp[k + 1]; ++q)
        pulls[S.upos[size_t(u++)] - s].push_back({p, q});
    }
    std::vector<int> plev(len, 0);
    int ng = 1;
    for (int t = 0; t < len; ++t) {
      int l = 0;
      for (auto &pq : pulls[t]) l = std::max(l, plev[pq.first - s] + 1);
      plev[t] = l;
      ng = std::max(ng, l + 1);
    }
    std::vector<int> cnt(ng + 1, 0);
    for (int t = 0; t < len; ++t) cnt[plev[t] + 1]++;
    for (int g = 0; g < ng; ++g) cnt[g + 1] += cnt[g];
    const int base = int(S.tail_pos.size());
    S.tail_pos.resize(size_t(base + len));
    // within a group, positions with few pulls first, then the long ones
    // (a warp each)
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    std::vector<int> nshort(ng, 0);
    for (int t = 0; t < len; ++t)
      if (int(pulls[t].size()) <= kTailLongPulls) nshort[plev[t]]++;
    std::vector<int> lfill(ng);
    for (int g = 0; g < ng; ++g) lfill[g] = cnt[g] + nshort[g];
    for (int t = 0; t < len; ++t) {
      const bool lng = int(pulls[t].size()) > kTailLongPulls;
      S.tail_pos[size_t(base + (lng ? lfill[plev[t]]++ : fill[plev[t]]++))] = s + t;
    }
    for (int g = 0; g < ng; ++g) {
      S.tail_glong.push_back(base + cnt[g] + nshort[g]);
      S.tail_gptr.push_back(base + cnt[g + 1]);
    }
    S.tail_rowg.push_back(int(S.tail_gptr.size()) - 1);
    for (int t = base; t < base + len; ++t) {
      for (auto &pq : pulls[S.tail_pos[size_t(t)] - s]) {
        S.tail_pm.push_back(pq.first);
        S.tail_q.push_back(pq.second);
      }
      S.tail_pp.push_back(int(S.tail_pm.size()));
    }
  }
  // rows by level, ascending row within a level
  auto group = [](const std::vector<int> &lev, int nlev, int nrows, std::vector<int> &rows,
                  std::vector<int> &ptr) {
    ptr.assign(nlev + 1, 0);
    for (int i = 0; i < nrows; ++i) ptr[lev[i] + 1]++;
    for (int l = 0; l < nlev; ++l) ptr[l + 1] += ptr[l];
    rows.assign(nrows, 0);
    std::vector<int> fill(ptr.begin(), ptr.end() - 1);
    for (int i = 0; i < nrows; ++i) rows[fill[lev[i]]++] = i;
  };
  std::vector<int> lev(n, 0);
  int nlev = 0;
  for (int i = 0; i < S.tail0; ++i) {
    int l = 0;
    for (int p = S.rp[i]; p < S.diag[i]; ++p) l = std::max(l, lev[S.ci[p]] + 1);
    lev[i] = l;
    nlev = std::max(nlev, l + 1);
  }
  group(lev, nlev, S.tail0, S.lrow, S.lptr);
  // within a level, the rows with many updates last, from lheavy[l] on
  S.lheavy.assign(nlev, 0);
  for (int l = 0; l < nlev; ++l) {
    auto b = S.lrow.begin() + S.lptr[l], e = S.lrow.begin() + S.lptr[l + 1];
    auto light = [&](int i) { return S.urp[i + 1] - S.urp[i] <= kHeavyRowUpdates; };
    // a warp per row only while few rows need it: a warp's FP64 instruction
    // costs the same with 4 lanes busy as with 32, so many heavy rows run
    // better one per lane
    if (e - b - std::count_if(b, e, light) > kMaxHeavyRows) {
      S.lheavy[l] = S.lptr[l + 1];
      continue;
    }
    auto mid = std::stable_partition(b, e, light);
    S.lheavy[l] = int(mid - S.lrow.begin());
  }
  // U levels, from the last row up: a row's U part names later rows only
  nlev = 0;
  for (int i = n - 1; i >= 0; --i) {
    int l = 0;
    for (int p = S.diag[i] + 1; p < S.rp[i + 1]; ++p) l = std::max(l, lev[S.ci[p]] + 1);
    lev[i] = l;
    nlev = std::max(nlev, l + 1);
  }
  group(lev, nlev, n, S.urow, S.uptr);
  return true;
}

double lu_model_seconds(const LuSymbolic &S) {
  // dependent steps cost a fixed latency each, independent work a rate
  return S.levels * kLuLevelSeconds + S.refactor_flops * kLuFlopSeconds;
}

}  // namespace xg
