"""bench.py's serving-sweep summary on CPU: which swept rates each mode
sustains, and the latencies both modes show at the highest rate both sustain."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def _mode(p50, p99, late_over_early, offered, completed):
    m = {"p50_ms": p50, "p99_ms": p99, "late_over_early_p50": late_over_early, "offered_queries_per_s": offered,
         "completed_queries_per_s": completed, "Grays_per_s": 0.5}
    m["sustained"] = bench.sustained(m)
    return m


def test_sustained_rule():
    assert bench.sustained(_mode(2.0, 5.0, 1.1, 1000, 950))
    assert not bench.sustained(_mode(20.0, 60.0, 4.0, 1000, 950))   # the queue builds up
    assert not bench.sustained(_mode(2.0, 5.0, 1.0, 1000, 500))      # completions fall behind
    assert bench.sustained(_mode(0.5, 1.0, 5.0, 1000, 990))          # short waits: +2 ms slack


def test_summary_picks_highest_rates():
    runs = []
    for rate, seq_ok in ((250, True), (500, True), (1000, True), (2000, False), (4000, False)):
        runs.append({"rate_per_s": rate,
                     "batched": _mode(1.0, 3.0, 1.0, rate, rate),
                     "sequential": _mode(1.5, 5.0, 1.0 if seq_ok else 6.0, rate, rate if seq_ok else rate / 3)})
    runs[-1]["batched"] = _mode(9.0, 40.0, 5.0, 4000, 1000)
    s = bench.serving_summary(runs)
    assert s["batched_max_sustained_req_per_s"] == 2000
    assert s["sequential_max_sustained_req_per_s"] == 1000
    assert s["at_rate_both_sustain"]["rate_per_s"] == 1000
    assert s["at_rate_both_sustain"]["batched_p50_p99_ms"] == [1.0, 3.0]
    assert set(s["p99_ms_by_rate"]) == {"250", "500", "1000", "2000", "4000"}
