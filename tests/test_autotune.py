"""The autotuner's search on the host: a greedy pass over one knob at a time
from the defaults, combinations that `valid` rules out never run, and the
result cache keyed by device and workload signature."""
from raccoongpurender_gb300 import autotune as at


def _cost(p):
    # sorting halves the time; staging helps a little; refill 16 is best
    t = 1.0 - 0.5 * p["trace_reorder"] - 0.01 * (p["trace_stage"] > 0)
    return t + 0.001 * abs(p["trace_refill"] - 16) + 0.0001 * abs(p["trace_search"] - 12)


def test_greedy_search_and_valid(tmp_path):
    runs = []

    def run(p):
        runs.append(dict(p))
        return _cost(p)

    t = at.Autotuner(0, cache_path=str(tmp_path / "tuned.json"), log=lambda *_: None)
    best = t.tune("trace|1", run, use_cache=False, defaults=at.TRACE_DEFAULTS, candidates=at.TRACE_CANDIDATES,
                  valid=lambda p: not (p["trace_reorder"] and p["trace_stage"]))
    assert best == dict(trace_reorder=1, trace_refill=16, trace_search=12, trace_stage=0)
    assert not any(p["trace_reorder"] and p["trace_stage"] for p in runs)
    assert runs[0] == at.TRACE_DEFAULTS
    assert [tr["params"] for tr in t.trials] == runs


def test_cache(tmp_path):
    path = str(tmp_path / "tuned.json")
    first = at.Autotuner(0, cache_path=path, log=lambda *_: None).tune(
        "trace|2", _cost, use_cache=True, defaults=at.TRACE_DEFAULTS, candidates=at.TRACE_CANDIDATES)
    runs = []
    again = at.Autotuner(0, cache_path=path, log=lambda *_: None).tune(
        "trace|2", lambda p: runs.append(p) or 0.0, use_cache=True, defaults=at.TRACE_DEFAULTS,
        candidates=at.TRACE_CANDIDATES)
    assert again == first and runs == []
    other = at.Autotuner(0, cache_path=path, log=lambda *_: None).tune(
        "trace|3", lambda p: runs.append(p) or 1.0, use_cache=True, defaults=at.TRACE_DEFAULTS,
        candidates=at.TRACE_CANDIDATES)
    assert runs and other == at.TRACE_DEFAULTS  # a new signature is tuned; ties keep the defaults
