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
