"""The launch-shape autotuner's selection logic (att_gb300.autotune.Tuner),
with an injected timer instead of CUDA events: no GPU needed."""
import pytest
import torch

from att_gb300 import autotune


def _fake_timer(times):
    calls = []

    def timer(run, warmup, reps):
        run()
        calls.append(timer.current)
        return times[timer.current]
    timer.current = None
    timer.calls = calls
    return timer


def test_picks_fastest_and_applies_it():
    times = {"a": 3.0, "b": 1.5, "c": 2.0}
    timer = _fake_timer(times)
    applied = []
    t = autotune.Tuner(timer=timer)

    def setup(c):
        timer.current = c
        applied.append(c)
    choice, table = t.best("k", ["a", "b", "c"], setup, lambda: None)
    assert choice == "b" and table == times
    assert applied[-1] == "b"                  # the winner is left applied
    assert timer.calls == ["a", "b", "c"]      # each candidate timed once


def test_ties_keep_candidate_order_and_cache_skips_timing():
    timer = _fake_timer({1: 2.0, 2: 2.0, 4: 5.0})
    t = autotune.Tuner(timer=timer)

    def setup(c):
        timer.current = c
    assert t.best("g", [1, 2, 4], setup, lambda: None)[0] == 1
    n = len(timer.calls)
    applied = []
    choice, _ = t.best("g", [1, 2, 4], lambda c: applied.append(c), lambda: None)
    assert choice == 1 and applied == [1] and len(timer.calls) == n   # cached: not re-timed
    with pytest.raises(ValueError):
        t.best("empty", [], setup, lambda: None)


def test_spmm_candidates():
    c16 = autotune.spmm_candidates(torch.float16, 128)
    assert ("spmm", 64, 3) in c16 and ("spmm", 128, 2) in c16 and len(c16) == 6
    assert all(c[1] == 64 for c in autotune.spmm_candidates(torch.bfloat16, 64))
    assert autotune.spmm_candidates(torch.float8_e4m3fn, 128) == [("fp8", 1), ("fp8", 0)]
    assert autotune.spmm_candidates(torch.float32, 128) == [("tf32", k) for k in range(4)]
    assert autotune.spmm_candidates(torch.float32, 32) == []
