"""Slotted batches: continuous batching at request granularity.

Requests of uneven length are submitted into a slotted batch while it runs:
as each one finishes its slot is released and the next waiting request joins
the running batch in that slot.  Every request's waveform and counters are
bit-identical to the same request run alone in a slotted batch of its own
(its arithmetic depends on it alone) and to the same request in a fixed batch
of its own (the slotted load sums every output in the fixed batch's order,
and the pivot order comes from the same first Jacobian).  The
slot bookkeeping refuses what it must: a request larger than the slot shape,
releasing a slot whose request still runs; a full batch takes nothing."""
import numpy as np
import pytest

from xyce_gb300 import abi, engine, serve

pytestmark = pytest.mark.gpu

TSTOP = 0.6e-9
VTOL = 1e-3 * 1.8


def _requests(n=10, seed=11):
    reqs = serve.ring_mc_requests(n, seed=seed, stages=(5, 41), tstop=TSTOP)
    for k, r in enumerate(reqs):
        r.tstop = TSTOP * (0.25 + 0.375 * (k % 3))  # three lengths
    return reqs


def _shape(ctx, reqs):
    return serve.merge_shapes([engine.slot_need(ctx, r.netlist, r.x0, r.tstop) for r in reqs])


def _batch(ctx, n_slots, shape, fp32):
    return engine.SlotBatch(ctx, n_slots, shape, 2, precision=abi.LU_FP32 if fp32 else abi.LU_FP64,
                            n_refine=2 if fp32 else 0, max_points=4096)


def _drain(b, held, out, chunk=16):
    b.run(chunk)
    b.poll(wait=True)
    for s, k in list(held.items()):
        if b.stats(s)["finished"]:
            out[k] = b.results(s)
            b.release(s)
            del held[s]


def _alone(ctx, shape, r, fp32):
    b = _batch(ctx, 1, shape, fp32)
    assert b.submit([r.netlist], [r.x0], [r.tstop], [r.out_idx]) == [0]
    out, held = {}, {0: 0}
    for _ in range(100000):
        if not held:
            break
        _drain(b, held, out)
    b.close()
    return out[0]


@pytest.mark.parametrize("fp32", [0, 1])
def test_requests_join_a_running_batch_and_match_alone(fp32, gpu_ctx):
    gpu_ctx.set_options(abi.device_options(fma=1))
    reqs = _requests()
    shape = _shape(gpu_ctx, reqs)
    b = _batch(gpu_ctx, 3, shape, fp32)
    waiting = list(range(len(reqs)))
    held, out = {}, {}
    joined_while_others_ran = 0
    for _ in range(100000):
        free = b.n - len(held)
        if waiting and free:
            take, waiting = waiting[:free], waiting[free:]
            slots = b.submit([reqs[k].netlist for k in take], [reqs[k].x0 for k in take],
                             [reqs[k].tstop for k in take], [reqs[k].out_idx for k in take])
            assert all(s >= 0 for s in slots)
            if held:
                joined_while_others_ran += len(take)
            held.update(zip(slots, take))
        if not held and not waiting:
            break
        _drain(b, held, out)
    b.close()
    assert len(out) == len(reqs) and joined_while_others_ran >= 5
    for k, r in enumerate(reqs):
        t, v, st = out[k]
        assert st["status"] == 0 and abs(t[-1] - r.tstop) <= 1e-12 * r.tstop
        ta, va, sa = _alone(gpu_ctx, shape, r, fp32)
        # the same bits as alone, point for point
        assert np.array_equal(t, ta) and np.array_equal(v, va), k
        assert {x: st[x] for x in ("steps", "rejected", "newton_iters")} == \
               {x: sa[x] for x in ("steps", "rejected", "newton_iters")}
        # and the same bits as a fixed batch of its own
        fb = engine.Batch(gpu_ctx, [r.netlist], [r.x0], [r.tstop], [r.out_idx], max_points=4096,
                          precision=abi.LU_FP32 if fp32 else abi.LU_FP64, n_refine=2 if fp32 else 0)
        engine.run_batch(fb, chunk=16)
        tf, vf, sf = fb.results(0)
        fb.close()
        assert np.array_equal(t, tf) and np.array_equal(v, vf), k


def test_slot_bookkeeping_refuses_what_it_must(gpu_ctx):
    gpu_ctx.set_options(abi.device_options(fma=1))
    small = serve.ring_mc_requests(3, seed=5, stages=(5, 9), tstop=0.2e-9)
    shape = _shape(gpu_ctx, small)
    b = _batch(gpu_ctx, 2, shape, 0)
    assert b.slots() == (2, 0)
    # a request larger than the shape: refused, nothing admitted
    big = serve.ring_mc_requests(1, seed=6, stages=(41, 41), tstop=0.2e-9)[0]
    with pytest.raises(engine.XgError) as e:
        b.submit([small[0].netlist, big.netlist], [small[0].x0, big.x0], [0.2e-9] * 2,
                 [small[0].out_idx, big.out_idx])
    assert e.value.status == -1
    assert b.slots() == (2, 0)
    # two fit, the third finds no free slot
    s = b.submit([r.netlist for r in small], [r.x0 for r in small], [r.tstop for r in small],
                 [r.out_idx for r in small])
    assert sorted(s[:2]) == [0, 1] and s[2] == -1
    assert b.slots() == (0, 2)
    # a running request's slot cannot be released
    with pytest.raises(engine.XgError) as e:
        b.release(s[0])
    assert e.value.status == -7
    held, out = {s[0]: 0, s[1]: 1}, {}
    for _ in range(100000):
        if not held:
            break
        _drain(b, held, out)
    assert b.slots() == (2, 0) and set(out) == {0, 1}
    # the device memory of the batch is what the shape says per slot
    assert b.device_bytes() >= 2 * engine.slot_bytes(shape, engine.batch_options(n_out=2, max_points=4096))
    b.close()


def test_slot_server_serves_a_stream(gpu_ctx):
    gpu_ctx.set_options(abi.device_options(fma=1))
    reqs = serve.ring_mc_requests(24, seed=7, stages=(5, 61), tstop=1e-9)
    shapes = serve.ring_class_shapes(gpu_ctx, stages=(5, 61), tstop=1e-9)
    arrivals = serve.poisson_arrivals(len(reqs), 400.0, seed=3)
    srv = serve.SlotServer(gpu_ctx, shapes, slots=4, chunk=16, max_points=8192)
    out = srv.run(reqs, arrivals)
    assert out["requests"] == len(reqs) and out["failed"] == 0 and out["oversize"] == 0
    assert out["p99_ms"] >= out["p50_ms"] > 0
    # a second stream on the same server reuses its batches: the same results
    again = serve.ring_mc_requests(24, seed=7, stages=(5, 61), tstop=1e-9)
    held = sum(len(v) for v in srv.pools.values())
    assert srv.run(again, arrivals)["failed"] == 0
    assert sum(len(v) for v in srv.pools.values()) == held
    for a, b in zip(reqs, again):
        assert np.array_equal(a.result[0], b.result[0]) and np.array_equal(a.result[1], b.result[1])
    srv.close()
    for served, r in zip(reqs, serve.ring_mc_requests(24, seed=7, stages=(5, 61), tstop=1e-9)):
        assert served.done >= served.arrival
        b = engine.Batch(gpu_ctx, [r.netlist], [r.x0], [r.tstop], [r.out_idx], max_points=8192)
        engine.run_batch(b)
        tb, vb, sb = b.results(0)
        b.close()
        t, v, st = served.result
        assert st["status"] == 0 and sb["status"] == 0
        vi = np.stack([np.interp(tb, t, v[:, j]) for j in range(v.shape[1])], 1)
        assert np.abs(vi - vb).max() <= VTOL


def test_batches_of_other_shapes_do_not_lower_each_others_limits(gpu_ctx):
    # a batch of large slots, then one of small slots (its shared-memory
    # needs are smaller), then the large one runs: its solves still launch
    gpu_ctx.set_options(abi.device_options(fma=1))
    big = serve.ring_mc_requests(2, seed=8, stages=(201, 201), tstop=0.1e-9)
    small = serve.ring_mc_requests(2, seed=9, stages=(5, 5), tstop=0.1e-9)
    b_big = _batch(gpu_ctx, 2, _shape(gpu_ctx, big), 0)
    b_small = _batch(gpu_ctx, 2, _shape(gpu_ctx, small), 0)
    for b, reqs in ((b_big, big), (b_small, small)):
        s = b.submit([r.netlist for r in reqs], [r.x0 for r in reqs], [r.tstop for r in reqs],
                     [r.out_idx for r in reqs])
        held, out = dict(zip(s, range(len(reqs)))), {}
        for _ in range(100000):
            if not held:
                break
            _drain(b, held, out)
        assert all(out[k][2]["status"] == 0 for k in range(len(reqs)))
    b_big.close()
    b_small.close()
