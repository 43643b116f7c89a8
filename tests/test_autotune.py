"""Autotuner: picks the fastest candidate, caches per key, persists to JSON."""
import json

from ghostlight_gb300.autotune import Tuner


def test_picks_fastest_and_caches(tmp_path):
    cost = {(0, 0): 3.0, (1, 0): 1.5, (4, 0): 2.0}
    calls = []

    def timer(run, c):
        run(c)
        return cost[c]

    path = tmp_path / "tune.json"
    t = Tuner(cache_path=str(path), reps=3, warm=1)
    got = t.best(("ghost", "dev", 10), list(cost), lambda c: calls.append(c), timer=timer)
    assert got == (1, 0)
    assert len(calls) == 3 * 4                      # warm + reps per candidate
    # cached: no more runs, same answer, also from a fresh tuner reading the file
    assert t.best(("ghost", "dev", 10), list(cost), lambda c: calls.append(c), timer=timer) == (1, 0)
    assert len(calls) == 12
    assert json.loads(path.read_text())["ghost|dev|10"] == [1, 0]
    t2 = Tuner(cache_path=str(path))
    assert t2.best(("ghost", "dev", 10), list(cost), lambda c: None, timer=timer) == (1, 0)
    # another key is tuned separately
    assert t2.best(("ghost", "dev", 11), [2, 5], lambda c: None, timer=lambda r, c: float(c)) == 2
