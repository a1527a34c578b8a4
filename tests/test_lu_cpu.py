"""Host side of the Newton-solve LU (no GPU): the approximate-minimum-degree
order and the pivoting analysis that fixes the pivot order and the L\\U
pattern the GPU refactorisation reuses."""
import heapq

import numpy as np
import pytest
import scipy.sparse as sp

from helpers import circuit_jacobian
from xyce_gb300 import engine, netlists


def _structural_fill(B):
    """Non-zeros of the L\\U of B with diagonal pivots (row-wise symbolic)."""
    n = B.shape[0]
    upper = [None] * n
    total = 0
    for i in range(n):
        S = set(B.indices[B.indptr[i]:B.indptr[i + 1]].tolist())
        S.add(i)
        h = [k for k in S if k < i]
        heapq.heapify(h)
        seen = set(h)
        while h:
            k = heapq.heappop(h)
            for m in upper[k]:
                if m not in S:
                    S.add(m)
                    if m < i and m not in seen:
                        heapq.heappush(h, m)
                        seen.add(m)
        upper[i] = [m for m in S if m > i]
        total += len(S)
    return total


def _grid_laplacian(k):
    n = k * k
    rows, cols = [], []
    for i in range(k):
        for j in range(k):
            a = i * k + j
            rows.append(a), cols.append(a)
            for di, dj in ((1, 0), (0, 1)):
                if i + di < k and j + dj < k:
                    b = (i + di) * k + j + dj
                    rows += [a, b]
                    cols += [b, a]
    vals = np.where(np.array(rows) == np.array(cols), 4.0, -1.0)
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A.sort_indices()
    return A


@pytest.mark.parametrize("case", ["inverter_chain_24", "power_grid_20x20", "random_mos_3000"])
def test_analysis_pattern_and_pivots(case, engine_lib, oracle_lib):
    nl = {"inverter_chain_24": lambda: netlists.inverter_chain(24),
          "power_grid_20x20": lambda: netlists.power_grid(20, 20, 60, seed=1),
          "random_mos_3000": lambda: netlists.random_mos_netlist(3000, 800, seed=3)}[case]()
    A = circuit_jacobian(nl, seed=4)
    n = A.shape[0]
    P, Q, nnz_lu = engine.lu_analyze_host(A.indptr, A.indices, A.data)
    assert sorted(P.tolist()) == list(range(n)) and sorted(Q.tolist()) == list(range(n))
    B = A[P][:, Q].tocsr()
    B.sort_indices()
    # the reported pattern is exactly the structural fill of B = A(P, Q)
    assert nnz_lu == _structural_fill(B)
    # the pivot order works without further pivoting: dense Doolittle on B
    D = B.toarray()
    for k in range(n):
        assert D[k, k] != 0.0
        D[k + 1:, k] /= D[k, k]
        D[k + 1:, k + 1:] -= np.outer(D[k + 1:, k], D[k, k + 1:])
    # and solves the system
    L = np.tril(D, -1) + np.eye(n)
    U = np.triu(D)
    b = np.random.default_rng(1).standard_normal(n)
    z = np.linalg.solve(U, np.linalg.solve(L, b[P]))
    x = np.empty(n)
    x[Q] = z
    # backward error of the solution (the matrices are badly scaled: random
    # node voltages forward-bias junctions, so entries span ~17 decades)
    Ad = A.toarray()
    r = b - Ad @ x
    assert np.abs(r).max() <= 1e-13 * (np.abs(Ad).sum(1).max() * np.abs(x).max() + np.abs(b).max())


def test_amd_reduces_fill_on_a_mesh(engine_lib):
    A = _grid_laplacian(30)
    order, n_dense = engine.amd_order(A.indptr, A.indices)
    assert sorted(order.tolist()) == list(range(A.shape[0])) and n_dense == 0
    natural = _structural_fill(A)
    B = A[order][:, order].tocsr()
    B.sort_indices()
    amd = _structural_fill(B)
    assert amd < 0.5 * natural, (amd, natural)


def test_dense_rows_are_ordered_last(engine_lib):
    # a star: node 0 touches every other node
    n = 400
    rows = list(range(n)) + [0] * (n - 1) + list(range(1, n))
    cols = list(range(n)) + list(range(1, n)) + [0] * (n - 1)
    A = sp.csr_matrix((np.ones(len(rows)), (rows, cols)), shape=(n, n))
    A.sort_indices()
    order, n_dense = engine.amd_order(A.indptr, A.indices)
    assert n_dense == 1 and order[-1] == 0


def test_singular_matrix_is_reported(engine_lib):
    A = sp.csr_matrix(np.array([[1.0, 2.0], [2.0, 4.0]]))
    with pytest.raises(engine.XgError) as e:
        engine.lu_analyze_host(A.indptr, A.indices, A.data)
    assert e.value.status == -4


@pytest.mark.parametrize("case", ["inverter_chain_200", "power_grid_20x20", "ring_oscillator_51",
                                  "random_logic_2000"])
def test_oracle_solve_matches_the_reference_sparse_solver(case, oracle_lib):
    """The oracle's sparse direct solve (minimum-degree order, threshold
    partial pivoting) against the reference's own bundled Kundert sparse
    solver (its KSparse linear-solver option) on circuit Jacobians: the same
    solution to 1e-10 relative, and both backward-stable."""
    from oracle import ref
    from oracle.oracle import sparse_solve
    if not ref.ksparse_available():
        pytest.skip("oracle/_ref/libksparse.so is built only where the reference sources are")
    nl = {"inverter_chain_200": lambda: netlists.inverter_chain(200),
          "power_grid_20x20": lambda: netlists.power_grid(20, 20, 60, seed=1),
          "ring_oscillator_51": lambda: netlists.ring_oscillator(51, seed=2),
          "random_logic_2000": lambda: netlists.random_logic(2000, seed=1)}[case]()
    A = circuit_jacobian(nl, seed=6)
    b = np.random.default_rng(13).standard_normal(A.shape[0])
    xk = ref.ksparse_solve(A.indptr, A.indices, A.data, b)
    order, _ = engine.amd_order(A.indptr, A.indices)
    xo = sparse_solve(A.indptr, A.indices, A.data, b, col_order=order)
    scale = np.abs(xk).max()
    assert np.abs(xo - xk).max() <= 1e-10 * scale, np.abs(xo - xk).max() / scale
    for x in (xk, xo):
        r = b - A @ x
        assert np.abs(r).max() / (abs(A).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max()) <= 1e-13


def test_chain_tail_is_modelled_where_rows_are_levels(engine_lib, oracle_lib):
    """The grid solves hand a factor's trailing run of one-row levels to one
    warp when the time model says it pays: on the 60x60 power grid the last
    768 rows (its dense block and the levels above it), never on factors
    below 4,096 rows."""
    from helpers import circuit_jacobian
    A = circuit_jacobian(netlists.power_grid(60, 60, 1200, seed=1), seed=5)
    info = engine.lu_analyze_host(A.indptr, A.indices, A.data, with_info=True)[3]
    assert info.solve_chain == 768
    small = circuit_jacobian(netlists.inverter_chain(200), seed=5)
    assert engine.lu_analyze_host(small.indptr, small.indices, small.data, with_info=True)[3].solve_chain == 0
