"""The serving path's host logic on CPU: the schedule autotuner against a
fake server whose throughput peaks at a known schedule, and its cache."""
import json

from xyce_gb300.serve import Autotuner


def _fake(peak):
    calls = []

    def serve(params, reqs, arr):
        calls.append(dict(params))
        score = 1000.0
        for k, v in peak.items():
            score -= abs(params[k] - v) / v * 100.0
        return {"solves_per_s": score}
    return serve, calls


def test_autotuner_finds_the_fastest_schedule():
    peak = {"max_batch": 256, "chunk": 16, "max_concurrent": 4}
    serve, calls = _fake(peak)
    t = Autotuner(serve, lambda: ([], []))
    assert t.tune() == peak
    # each schedule is measured once: at most the start plus one per grid value
    assert len(calls) <= 1 + sum(len(v) for v in Autotuner.GRID.values())
    assert len({tuple(sorted(c.items())) for c in calls}) == len(calls)


def test_autotuner_cache_round_trip(tmp_path):
    peak = {"max_batch": 1024, "chunk": 256, "max_concurrent": 2}
    path = tmp_path / "tune.json"
    serve, calls = _fake(peak)
    assert Autotuner(serve, lambda: ([], []), cache_path=str(path), key="gb300/rings").tune() == peak
    n = len(calls)
    # a second tuner with the same key reads the cache and measures nothing
    again = Autotuner(serve, lambda: ([], []), cache_path=str(path), key="gb300/rings")
    assert again.tune() == peak and len(calls) == n
    assert json.loads(path.read_text())["gb300/rings"] == peak


# ---- admission arithmetic of the slot server -------------------------------------

def _shape(u=100, mos=200, cap=50, nnz=900, lu=1500, sched=3000, bp=4):
    from xyce_gb300 import abi
    d = {"max_unknowns": u, "max_instances": [0] * abi.NUM_DEV_TYPES, "max_nnz": nnz,
         "max_lu_nnz": lu, "max_schedule": sched, "max_breakpoints": bp}
    d["max_instances"][abi.DEV_MOS1] = mos
    d["max_instances"][abi.DEV_CAP] = cap
    d["max_instances"][abi.DEV_VSRC] = 1
    return abi.XgSlotShape.from_dict(d)


def test_slot_bytes_grow_with_every_dimension(engine_lib):
    from xyce_gb300 import abi, engine
    o = engine.batch_options(n_out=2, max_points=1000)
    base = engine.slot_bytes(_shape(), o)
    assert base > 0
    for kw in ({"u": 101}, {"mos": 201}, {"cap": 51}, {"nnz": 901}, {"lu": 1501}, {"sched": 3001}, {"bp": 5}):
        assert engine.slot_bytes(_shape(**kw), o) > base, kw
    # the recorded history: (1 + n_out) doubles per point
    more = engine.slot_bytes(_shape(), engine.batch_options(n_out=2, max_points=1001))
    assert more - base == 8 * 3
    # FP32 factors take less than FP64 ones
    assert engine.slot_bytes(_shape(), engine.batch_options(n_out=2, max_points=1000,
                                                            precision=abi.LU_FP32)) < base


def test_slot_bytes_reject_a_bad_shape(engine_lib):
    import pytest as _pt
    from xyce_gb300 import engine
    with _pt.raises(engine.XgError):
        engine.slot_bytes(_shape(u=0), engine.batch_options())


def test_plan_slots_admits_within_free_memory_less_reserve():
    from xyce_gb300.serve import plan_slots
    per = 2 << 20
    assert plan_slots(512, per, free_bytes=10 << 30, reserve_bytes=4 << 30) == 512
    # only 3 slots' worth above the reserve
    assert plan_slots(512, per, free_bytes=(4 << 30) + 3 * per + 5, reserve_bytes=4 << 30) == 3
    assert plan_slots(512, per, free_bytes=(4 << 30) - 1, reserve_bytes=4 << 30) == 0
    # a cap on what the server holds counts what it already holds
    assert plan_slots(512, per, 100 << 30, 4 << 30, in_use_bytes=10 * per, cap_bytes=14 * per) == 4
    assert plan_slots(512, per, 100 << 30, 4 << 30, in_use_bytes=14 * per, cap_bytes=14 * per) == 0


def test_size_classes_and_merged_shapes():
    from xyce_gb300 import abi
    from xyce_gb300.serve import merge_shapes, size_class
    assert [size_class(u) for u in (7, 8, 15, 16, 503, 512)] == [2, 3, 3, 4, 8, 9]
    a, b = _shape(u=100, mos=200, lu=1000, sched=100), _shape(u=90, mos=240, lu=2000, sched=50, nnz=1000)
    m = merge_shapes([a, b], margin=1.25)
    assert m.max_unknowns == 100 and m.max_instances[abi.DEV_MOS1] == 240 and m.max_nnz == 1000
    assert m.max_lu_nnz == int(2000 * 1.25) + 16 and m.max_schedule == int(100 * 1.25) + 64
