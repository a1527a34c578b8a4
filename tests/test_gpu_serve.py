"""The continuous-batching server end to end: a Poisson stream of seeded
Monte-Carlo rings is admitted into batches as it arrives, several batches in
flight, and every request's waveform matches the same request solved alone,
to within the simulation's own tolerance (reltol 1e-3 of the 1.8 V swing).
Mixed precision (FP32 factors corrected by Newton) matches FP64 the same way;
every request finishes after it arrives and the summary counts them all."""
import numpy as np
import pytest

from xyce_gb300 import abi, engine, serve

pytestmark = pytest.mark.gpu

VTOL = 1e-3 * 1.8
TSTOP = 1e-9


def _agree(a, b):
    (ta, va, sa), (tb, vb, sb) = a, b
    assert sa["status"] == 0 and sb["status"] == 0
    vi = np.stack([np.interp(tb, ta, va[:, k]) for k in range(va.shape[1])], 1)
    err = np.abs(vi - vb).max()
    assert err <= VTOL, err


def _stream(n=24, seed=7):
    return serve.ring_mc_requests(n, seed=seed, stages=(5, 61), tstop=TSTOP)


@pytest.mark.parametrize("precision", [abi.LU_FP64, abi.LU_FP32])
def test_served_stream_matches_each_request_alone(precision, gpu_ctx):
    gpu_ctx.set_options(abi.device_options(fma=1))
    reqs = _stream()
    arrivals = serve.poisson_arrivals(len(reqs), 400.0, seed=3)
    srv = serve.Server(gpu_ctx, precision=precision, max_batch=6, max_concurrent=3, chunk=16)
    out = srv.run(reqs, arrivals)
    assert out["requests"] == len(reqs) and out["failed"] == 0
    assert out["p99_ms"] >= out["p50_ms"] > 0
    for r in reqs:
        assert r.done is not None and r.done >= r.arrival
    # the same requests (the same seeds) one at a time, FP64 factors
    for served, r in zip(reqs, _stream()):
        b = engine.Batch(gpu_ctx, [r.netlist], [r.x0], [r.tstop], [r.out_idx], max_points=8192)
        engine.run_batch(b)
        alone = b.results(0)
        b.close()
        _agree(served.result, alone)
