/*
 * xgo_order.c — column order for the oracle's sparse LU (TEST INFRASTRUCTURE
 * ONLY; see xgo.h).
 *
 * The reference's default linear solver, KLU through Amesos
 * (src/LinearAlgebraServicesPKG/src/N_LAS_AmesosSolver.C:298-444), orders
 * the columns by approximate minimum degree on the pattern of A + A^T.  KLU is
 * not in the reference tree, so this restates the published minimum-degree
 * method itself: eliminate, one at a time, a vertex of least degree in the
 * elimination graph of A + A^T, joining its neighbours into a clique
 * (Tinney & Walker's scheme 2; George & Liu, "The evolution of the minimum
 * degree ordering algorithm", SIAM Review 31, 1989).  As in approximate
 * minimum degree (Amestoy, Davis & Duff, SIAM J. Matrix Anal. Appl. 17,
 * 1996), rows denser than 10 sqrt(n) (supply rails) are taken out first and
 * ordered last.  Degrees here are exact rather than approximate, and
 * vertices are not merged, so the order can differ from AMD's in ties.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "xgo_internal.h"

typedef struct {
  int *v;
  int len, cap;
} ivec;

static int push(ivec *a, int x) {
  if (a->len == a->cap) {
    int c = a->cap ? 2 * a->cap : 4;
    int *p = (int *)realloc(a->v, sizeof(int) * (size_t)c);
    if (!p) return -1;
    a->v = p;
    a->cap = c;
  }
  a->v[a->len++] = x;
  return 0;
}

static void drop(ivec *a, int x) {
  for (int k = 0; k < a->len; ++k)
    if (a->v[k] == x) {
      a->v[k] = a->v[--a->len];
      return;
    }
}

/* degree buckets: doubly linked lists, head[d] */
typedef struct {
  int *head, *next, *prev, *deg;
  int n, mind;
} buckets;

static void b_insert(buckets *B, int v, int d) {
  if (d > B->n) d = B->n;
  B->deg[v] = d;
  B->prev[v] = -1;
  B->next[v] = B->head[d];
  if (B->head[d] >= 0) B->prev[B->head[d]] = v;
  B->head[d] = v;
  if (d < B->mind) B->mind = d;
}

static void b_remove(buckets *B, int v) {
  const int d = B->deg[v];
  if (B->prev[v] >= 0) B->next[B->prev[v]] = B->next[v];
  else B->head[d] = B->next[v];
  if (B->next[v] >= 0) B->prev[B->next[v]] = B->prev[v];
}

int xgo_min_degree(int n, const int *rowptr, const int *col, int *order) {
  if (n <= 0 || !rowptr || !col || !order) return XG_ERR_ARG;
  ivec *adj = (ivec *)calloc((size_t)n, sizeof(ivec));
  int *mark = (int *)calloc((size_t)n, sizeof(int));
  char *gone = (char *)calloc((size_t)n, 1);
  buckets B;
  B.n = n;
  B.mind = n;
  B.head = (int *)malloc(sizeof(int) * (size_t)(n + 1));
  B.next = (int *)malloc(sizeof(int) * (size_t)n);
  B.prev = (int *)malloc(sizeof(int) * (size_t)n);
  B.deg = (int *)malloc(sizeof(int) * (size_t)n);
  int rc = XG_OK;
  if (!adj || !mark || !gone || !B.head || !B.next || !B.prev || !B.deg) {
    rc = XG_ERR_OOM;
    goto done;
  }
  for (int d = 0; d <= n; ++d) B.head[d] = -1;
  /* the pattern of A + A^T without the diagonal, each edge once per end */
  int stamp = 0;
  for (int i = 0; i < n; ++i)
    for (int p = rowptr[i]; p < rowptr[i + 1]; ++p) {
      const int j = col[p];
      if (j == i || j < 0 || j >= n) continue;
      if (push(&adj[i], j) || push(&adj[j], i)) { rc = XG_ERR_OOM; goto done; }
    }
  for (int i = 0; i < n; ++i) { /* remove duplicate edges */
    ++stamp;
    int w = 0;
    for (int k = 0; k < adj[i].len; ++k) {
      const int j = adj[i].v[k];
      if (mark[j] != stamp) {
        mark[j] = stamp;
        adj[i].v[w++] = j;
      }
    }
    adj[i].len = w;
  }
  /* dense rows last, in order of increasing degree */
  const int dense = (int)fmax(16.0, 10.0 * sqrt((double)n));
  int n_dense = 0;
  int *dense_list = (int *)malloc(sizeof(int) * (size_t)n);
  if (!dense_list) { rc = XG_ERR_OOM; goto done; }
  for (int i = 0; i < n; ++i)
    if (adj[i].len > dense) {
      gone[i] = 2;
      dense_list[n_dense++] = i;
    }
  for (int a = 1; a < n_dense; ++a) { /* insertion sort by degree, then index */
    const int v = dense_list[a];
    int b = a - 1;
    while (b >= 0 && adj[dense_list[b]].len > adj[v].len) {
      dense_list[b + 1] = dense_list[b];
      --b;
    }
    dense_list[b + 1] = v;
  }
  for (int i = 0; i < n; ++i) {
    if (gone[i]) continue;
    int w = 0;
    for (int k = 0; k < adj[i].len; ++k)
      if (!gone[adj[i].v[k]]) adj[i].v[w++] = adj[i].v[k];
    adj[i].len = w;
  }
  for (int i = n - 1; i >= 0; --i)
    if (!gone[i]) b_insert(&B, i, adj[i].len);
  int k = 0;
  while (k < n - n_dense) {
    while (B.mind <= n && B.head[B.mind] < 0) ++B.mind;
    const int v = B.head[B.mind];
    b_remove(&B, v);
    gone[v] = 1;
    order[k++] = v;
    /* join v's neighbours into a clique */
    for (int a = 0; a < adj[v].len; ++a) {
      const int u = adj[v].v[a];
      drop(&adj[u], v);
      ++stamp;
      mark[u] = stamp;
      for (int c = 0; c < adj[u].len; ++c) mark[adj[u].v[c]] = stamp;
      for (int c = 0; c < adj[v].len; ++c) {
        const int w = adj[v].v[c];
        if (mark[w] != stamp) {
          mark[w] = stamp;
          if (push(&adj[u], w)) { free(dense_list); rc = XG_ERR_OOM; goto done; }
        }
      }
      b_remove(&B, u);
      b_insert(&B, u, adj[u].len);
    }
    free(adj[v].v);
    adj[v].v = NULL;
    adj[v].len = adj[v].cap = 0;
  }
  for (int a = 0; a < n_dense; ++a) order[k++] = dense_list[a];
  free(dense_list);
done:
  if (adj)
    for (int i = 0; i < n; ++i) free(adj[i].v);
  free(adj);
  free(mark);
  free(gone);
  free(B.head);
  free(B.next);
  free(B.prev);
  free(B.deg);
  return rc;
}
