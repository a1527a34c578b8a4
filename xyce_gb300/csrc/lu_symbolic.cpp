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

int lu_analyze(int n, const int *rp, const int *ci, const double *val, double pivot_tol,
               LuSymbolic *out, std::string *err) {
  LuSymbolic &S = *out;
  S = LuSymbolic();
  S.n = n;
  S.nnz_a = rp[n];
  // column order
  S.Q = amd_order(n, rp, ci, &S.n_dense);
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

}  // namespace xg
