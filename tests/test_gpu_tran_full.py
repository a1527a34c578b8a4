"""Waveform parity at the exact transient workloads that bench.py times:

* the 1,000-stage CMOS inverter chain, .TRAN 1ps 20ns (2,000 level-1 MOSFETs);
* the 200x200 power grid with 40,000 diode-clamped level-1 sinks, its
  .TRAN 1ps 3ps window (120,002 unknowns);
* 500,000 BSIM3 MOSFETs of seeded random logic, its .TRAN 2ps 10ps window.

Each runs on the GPU in the benchmark's own build (the FMA load build) with
FP64 factors and with FP32 factors plus two FP64 refinement steps per solve,
and once through the oracle's CPU transient driver.  The CPU runs start in
spawned processes before the first GPU call, so they overlap the GPU work.

Bar: the same number of accepted time points within 2% (+2), and every
recorded node within reltol 1e-3 of the 1.8 V swing of the oracle at the
oracle's time points.  With XG_PARITY_REPORT=<path> each case appends its
largest waveform error and point counts to that JSON-lines file.
"""
import concurrent.futures as cf
import multiprocessing as mp

import numpy as np
import pytest

from helpers import report
from xyce_gb300 import abi

pytestmark = pytest.mark.gpu

VTOL = 1e-3 * 1.8
WORKLOADS = ("tran_inverter_chain_1000", "tran_power_grid_200x200", "tran_random_logic_500k")
FORMS = ((abi.LU_FP64, 0), (abi.LU_FP32, 2))


@pytest.fixture(scope="module")
def oracle_runs():
    from helpers import oracle_transient_workload
    ex = cf.ProcessPoolExecutor(max_workers=len(WORKLOADS), mp_context=mp.get_context("spawn"))
    futs = {w: ex.submit(oracle_transient_workload, w) for w in WORKLOADS}
    yield futs
    ex.shutdown(cancel_futures=True)


@pytest.mark.parametrize("name", WORKLOADS)
def test_benchmarked_transient_matches_oracle(name, oracle_runs, gpu_ctx, oracle_lib):
    import bench
    from xyce_gb300 import engine
    nl, guess, tstop, tstep, uic, out = bench.build_tran(name)
    x0 = bench._x0(nl, guess)
    gpu_ctx.set_options(abi.device_options(fma=1))
    c = engine.Circuit(gpu_ctx, nl)
    gpu = {}
    try:
        for prec, nref in FORMS:
            gpu[(prec, nref)] = engine.transient(c, tstop, tstep, out, x0=x0, uic=uic,
                                                 precision=prec, n_refine=nref)
    finally:
        c.close()
    tc, vc, sc = oracle_runs[name].result(timeout=1800)
    assert sc["status"] == 0
    for (prec, nref), (tg, vg, sg) in gpu.items():
        assert sg["status"] == 0, sg
        assert tg[-1] == pytest.approx(tstop, rel=1e-12)
        assert abs(len(tg) - len(tc)) <= 0.02 * len(tc) + 2, (len(tg), len(tc))
        vi = np.stack([np.interp(tc, tg, vg[:, k]) for k in range(vg.shape[1])], 1)
        err = float(np.abs(vi - vc).max())
        report({"workload": name, "lu": "fp64" if prec == abi.LU_FP64 else f"fp32+{nref}",
                 "max_waveform_err_v": err, "points_gpu": int(len(tg)), "points_cpu": int(len(tc)),
                 "newton_gpu": sg["newton_iters"], "newton_cpu": sc["newton_iters"]})
        assert err <= VTOL, (prec, nref, err)
