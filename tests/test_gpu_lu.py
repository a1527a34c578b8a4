"""GPU refactorisation and solves of the Newton-solve LU, through the C ABI.

The host analysis fixes the pivot order on one matrix; the GPU refactors a
second matrix of the same pattern (another load of the same circuit) with
that order, then solves.  Checked against scipy's SuperLU in FP64 and by the
backward error |b - A x| / (|A| |x| + |b|) (infinity norms), which a
backward-stable FP64 solve keeps near 1e-16 whatever the conditioning:
  * FP64 factors: backward error <= 1e-13;
  * FP32 factors: ~1e-7 unrefined; <= 1e-13 after FP64 iterative refinement.
"""
import numpy as np
import pytest
import scipy.sparse.linalg as sla

from helpers import circuit_jacobian
from xyce_gb300 import abi, engine, netlists

pytestmark = pytest.mark.gpu

CASES = {
    "inverter_chain_1000": lambda: netlists.inverter_chain(1000),
    "power_grid_60x60": lambda: netlists.power_grid(60, 60, 1200, seed=1),
    "ring_oscillator_101": lambda: netlists.ring_oscillator(101, seed=2),
    "random_mos_3000": lambda: netlists.random_mos_netlist(3000, 800, seed=3),
    "random_bsim3_3000": lambda: netlists.random_mos_netlist(
        3000, 700, dev_type=abi.DEV_BSIM3, seed=5,
        models=(abi.Model(abi.DEV_BSIM3, 1), abi.Model(abi.DEV_BSIM3, -1))),
}


def _backward_error(A, x, b):
    r = b - A @ x
    return np.abs(r).max() / (abs(A).sum(axis=1).max() * np.abs(x).max() + np.abs(b).max())


def _solve(ctx, A_analyse, A, b, precision, n_refine):
    import torch
    lu = engine.LU(ctx, A_analyse.indptr, A_analyse.indices, A_analyse.data, precision)
    dev_vals = torch.from_numpy(A.data.copy()).cuda()
    dev_b = torch.from_numpy(b).cuda()
    dev_x = torch.zeros_like(dev_b)
    lu.refactor(dev_vals.data_ptr())
    lu.solve(dev_b.data_ptr(), dev_x.data_ptr(), n_refine)
    status, _ = lu.status()
    x = dev_x.cpu().numpy()
    info = lu.info
    lu.close()
    return x, status, info


@pytest.mark.parametrize("case", sorted(CASES))
def test_fp64_refactor_and_solve(case, gpu_ctx, oracle_lib):
    nl = CASES[case]()
    A0 = circuit_jacobian(nl, seed=4)
    A = circuit_jacobian(nl, seed=5)
    assert np.array_equal(A0.indices, A.indices)
    b = np.random.default_rng(7).standard_normal(A.shape[0])
    x, status, info = _solve(gpu_ctx, A0, A, b, abi.LU_FP64, 0)
    assert status == 0
    assert _backward_error(A, x, b) <= 1e-13
    ref = sla.spsolve(A.tocsc(), b)
    assert _backward_error(A, ref, b) <= 1e-13
    if case in ("inverter_chain_1000", "power_grid_60x60", "ring_oscillator_101"):
        assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("case", ["inverter_chain_1000", "power_grid_60x60", "ring_oscillator_101"])
def test_fp32_factors_with_fp64_refinement(case, gpu_ctx, oracle_lib):
    nl = CASES[case]()
    A0 = circuit_jacobian(nl, seed=4)
    A = circuit_jacobian(nl, seed=5)
    b = np.random.default_rng(8).standard_normal(A.shape[0])
    x0, st0, _ = _solve(gpu_ctx, A0, A, b, abi.LU_FP32, 0)
    x3, st3, _ = _solve(gpu_ctx, A0, A, b, abi.LU_FP32, 3)
    assert st0 == 0 and st3 == 0
    e0, e3 = _backward_error(A, x0, b), _backward_error(A, x3, b)
    assert e0 <= 1e-5
    assert e3 <= 1e-13, (e0, e3)


def test_refactor_and_solve_are_deterministic(gpu_ctx, oracle_lib):
    nl = CASES["power_grid_60x60"]()
    A = circuit_jacobian(nl, seed=5)
    b = np.random.default_rng(9).standard_normal(A.shape[0])
    xs = [_solve(gpu_ctx, A, A, b, abi.LU_FP64, 0)[0] for _ in range(2)]
    assert np.array_equal(xs[0], xs[1])


def test_zero_pivot_is_reported(gpu_ctx, oracle_lib):
    """All-zero values: the refactor meets a zero pivot, finishes, and says so."""
    import torch
    nl = CASES["inverter_chain_1000"]()
    A = circuit_jacobian(nl, seed=5)
    lu = engine.LU(gpu_ctx, A.indptr, A.indices, A.data, abi.LU_FP64)
    zeros = torch.zeros(A.nnz, dtype=torch.float64, device="cuda:0")
    lu.refactor(zeros.data_ptr())
    status, bad_row = lu.status()
    assert status & 1 and bad_row == 0
    # a good matrix afterwards factors cleanly again
    vals = torch.from_numpy(A.data.copy()).cuda()
    lu.refactor(vals.data_ptr())
    assert lu.status() == (0, -1)
    lu.close()


def test_full_size_power_grid_solve(gpu_ctx, oracle_lib):
    """200x200 mesh with 40,000 MOSFET sinks (120,002 unknowns)."""
    nl = netlists.power_grid(200, 200, 40000, seed=0)
    A0 = circuit_jacobian(nl, seed=4)
    A = circuit_jacobian(nl, seed=5)
    b = np.random.default_rng(10).standard_normal(A.shape[0])
    x, status, info = _solve(gpu_ctx, A0, A, b, abi.LU_FP64, 0)
    assert status == 0 and info.n == 120002
    assert _backward_error(A, x, b) <= 1e-13
    x32, status, _ = _solve(gpu_ctx, A0, A, b, abi.LU_FP32, 3)
    assert status == 0
    assert _backward_error(A, x32, b) <= 1e-13


@pytest.mark.parametrize("order", ["amd", "nd"])
@pytest.mark.parametrize("case", ["inverter_chain_1000", "ring_oscillator_101", "random_mos_3000"])
def test_level_sequential_cta_and_grid_paths_agree(case, order, gpu_ctx, oracle_lib, monkeypatch):
    """Small factors run level by level in one CTA (long trailing rows with
    all threads); with that path off, narrow ones are walked by one lane,
    other small ones run warp-per-row in one CTA, the rest grid-wide.
    Forcing each path, under either column order, on the same matrix gives
    the same solution."""
    nl = CASES[case]()
    A = circuit_jacobian(nl, seed=5)
    b = np.random.default_rng(11).standard_normal(A.shape[0])
    xs = []
    monkeypatch.setenv("XG_LU_ORDER", order)
    for env in ({}, {"XG_LU_NO_LVL": "1"}, {"XG_LU_NO_LVL": "1", "XG_LU_NO_SEQ": "1"},
                {"XG_LU_NO_LVL": "1", "XG_LU_NO_SEQ": "1", "XG_LU_NO_CTA": "1"}):
        for k in ("XG_LU_NO_LVL", "XG_LU_NO_SEQ", "XG_LU_NO_CTA"):
            monkeypatch.delenv(k, raising=False)
        for k, v in env.items():
            monkeypatch.setenv(k, v)
        x, st, _ = _solve(gpu_ctx, A, A, b, abi.LU_FP64, 0)
        assert st == 0
        assert _backward_error(A, x, b) <= 1e-13
        xs.append(x)
    for x in xs[1:]:
        assert np.abs(x - xs[0]).max() <= 1e-12 * np.abs(xs[0]).max()


@pytest.mark.parametrize("case", ["inverter_chain_1000", "ring_oscillator_101", "power_grid_60x60"])
def test_fused_refactor_solve_matches_separate_calls(case, gpu_ctx, oracle_lib):
    """xg_lu_refactor_solve (one launch for small factors) gives the same
    factor and solution as xg_lu_refactor then xg_lu_solve."""
    import torch
    nl = CASES[case]()
    A0 = circuit_jacobian(nl, seed=4)
    A = circuit_jacobian(nl, seed=5)
    b = torch.from_numpy(np.random.default_rng(12).standard_normal(A.shape[0])).cuda()
    vals = torch.from_numpy(A.data.copy()).cuda()
    xs = []
    for fused in (False, True):
        lu = engine.LU(gpu_ctx, A0.indptr, A0.indices, A0.data, abi.LU_FP64)
        x = torch.zeros_like(b)
        if fused:
            lu.refactor_solve(vals.data_ptr(), b.data_ptr(), x.data_ptr())
        else:
            lu.refactor(vals.data_ptr())
            lu.solve(b.data_ptr(), x.data_ptr(), 0)
        assert lu.status() == (0, -1)
        xs.append(x.cpu().numpy())
        lu.close()
    assert np.array_equal(xs[0], xs[1])
    assert _backward_error(A, xs[1], b.cpu().numpy()) <= 1e-13


@pytest.mark.parametrize("precision,n_refine", [(abi.LU_FP64, 0), (abi.LU_FP32, 3)])
def test_grid_refactor_of_a_row_too_long_to_stage(precision, n_refine, gpu_ctx):
    """An arrowhead (a supply node coupled to 20,000 others): the last row of
    the factor is longer than any shared-memory stage, so the grid refactor
    eliminates it in global memory while the short rows are staged."""
    import scipy.sparse as sp
    n = 20001
    rng = np.random.default_rng(14)
    k = np.arange(n - 1)
    rows = np.r_[np.arange(n), k, np.full(n - 1, n - 1)]
    cols = np.r_[np.arange(n), np.full(n - 1, n - 1), k]
    vals = np.r_[rng.uniform(4.0, 5.0, n - 1), float(n), rng.uniform(-1, 1, n - 1), rng.uniform(-1, 1, n - 1)]
    A = sp.csr_matrix((vals, (rows, cols)), shape=(n, n))
    A.sort_indices()
    b = rng.standard_normal(n)
    x, st, info = _solve(gpu_ctx, A, A, b, precision, n_refine)
    assert st == 0 and info.nnz_lu >= 3 * (n - 1)
    assert _backward_error(A, x, b) <= 1e-13
    ref = sla.spsolve(A.tocsc(), b)
    assert np.abs(x - ref).max() <= 1e-9 * np.abs(ref).max()


@pytest.mark.parametrize("precision", [abi.LU_FP64, abi.LU_FP32])
def test_chain_tail_matches_grid_solves(precision, gpu_ctx, oracle_lib, monkeypatch):
    """The trailing rows of one row per level (the 60x60 grid's dense block)
    are solved by one warp column by column, their entries brought into
    shared memory by bulk copies.  The solution agrees with the one where
    every row is solved grid-wide (XG_LU_NO_CHAIN) to rounding, both meet
    the backward-error bound, and the chain's sums (each row's in column
    order) give the same bits on every run."""
    A = circuit_jacobian(CASES["power_grid_60x60"](), seed=5)
    b = np.random.default_rng(15).standard_normal(A.shape[0])
    x, st, info = _solve(gpu_ctx, A, A, b, precision, 0)
    x_again, st_again, _ = _solve(gpu_ctx, A, A, b, precision, 0)
    monkeypatch.setenv("XG_LU_NO_CHAIN", "1")
    x_grid, st_grid, info_grid = _solve(gpu_ctx, A, A, b, precision, 0)
    assert st == 0 and st_again == 0 and st_grid == 0
    assert info.solve_chain > 0 and info_grid.solve_chain == 0
    assert np.array_equal(x, x_again)
    tol = 1e-10 if precision == abi.LU_FP64 else 1e-3
    assert np.max(np.abs(x - x_grid)) <= tol * np.max(np.abs(x_grid))
    bound = 1e-13 if precision == abi.LU_FP64 else 1e-5
    assert _backward_error(A, x, b) <= bound and _backward_error(A, x_grid, b) <= bound


def test_wait_that_runs_out_reports_timeout(gpu_ctx, oracle_lib):
    """The grid refactor's rows wait, bounded, for the pivots of the rows
    their L part names.  With the limit lowered to one poll those waits give
    up: the launch still ends, xg_lu_status reports bit 2 (a wait gave up),
    and the context stays usable, as the next refactor at the default limit
    shows."""
    import torch
    A = circuit_jacobian(CASES["power_grid_60x60"](), seed=5)
    b = np.random.default_rng(16).standard_normal(A.shape[0])
    lu = engine.LU(gpu_ctx, A.indptr, A.indices, A.data, abi.LU_FP64)
    try:
        vals = torch.from_numpy(A.data.copy()).cuda()
        db = torch.from_numpy(b).cuda()
        dx = torch.zeros_like(db)
        lu.set_wait_limit(1)
        lu.refactor(vals.data_ptr())
        lu.solve(db.data_ptr(), dx.data_ptr(), 0)
        status, _ = lu.status()
        assert status & 2, status
        lu.set_wait_limit(1 << 20)
        lu.refactor(vals.data_ptr())
        lu.solve(db.data_ptr(), dx.data_ptr(), 0)
        assert lu.status() == (0, -1)
        assert _backward_error(A, dx.cpu().numpy(), b) <= 1e-13
    finally:
        lu.close()
    with pytest.raises(engine.XgError):
        lu2 = engine.LU(gpu_ctx, A.indptr, A.indices, A.data, abi.LU_FP64)
        try:
            lu2.set_wait_limit(0)
        finally:
            lu2.close()
