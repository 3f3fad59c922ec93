"""Host logic of the accuracy helpers: the tolerance selection of match_p99,
with the walk evaluation replaced by a fake (no GPU)."""
import pytest

from gravity_gb300 import accuracy


def _fake(monkeypatch, p99_of, inter_of):
    calls = []

    def evaluate(sim, ref_sample, params):
        calls.append(params)
        return {"p99": p99_of(params), "interactions": inter_of(params)}

    monkeypatch.setattr(accuracy, "evaluate", evaluate)
    return calls


def test_match_p99_picks_fewest_interactions_at_target(monkeypatch):
    # p99 grows and interactions fall along the grid (accurate -> aggressive)
    _fake(monkeypatch, lambda v: 10 ** v, lambda v: int(1e6 * 10 ** (-v)))
    grid = [-3.0, -2.5, -2.0, -1.5]
    best, res = accuracy.match_p99(None, None, lambda v: v, grid, target_p99=10 ** -2.2)
    assert best[0] == -2.5
    assert [r["setting"] for r in res] == grid


def test_match_p99_refines_between_passing_and_failing(monkeypatch):
    calls = _fake(monkeypatch, lambda v: 10 ** v, lambda v: int(1e6 * 10 ** (-v)))
    grid = [-3.0, -2.5, -2.0, -1.5]
    target = 10 ** -2.2
    best, res = accuracy.match_p99(None, None, lambda v: v, grid, target_p99=target, refine=3)
    assert len(calls) == len(grid) + 3
    # bisection between -2.5 (passes) and -2.0 (fails): -2.25 passes, -2.125
    # fails, -2.1875 fails
    assert [r["setting"] for r in res[len(grid):]] == [-2.25, -2.125, -2.1875]
    assert best[0] == pytest.approx(-2.25)
    assert best[1]["p99"] <= target


def test_match_p99_no_refinement_when_nothing_fails_after_best(monkeypatch):
    calls = _fake(monkeypatch, lambda v: 0.0, lambda v: int(1e6 * 10 ** (-v)))
    grid = [-3.0, -2.0]
    best, _ = accuracy.match_p99(None, None, lambda v: v, grid, target_p99=1.0, refine=3)
    assert best[0] == -2.0 and len(calls) == 2


def test_match_p99_none_when_no_setting_reaches_target(monkeypatch):
    _fake(monkeypatch, lambda v: 1.0, lambda v: 1)
    best, res = accuracy.match_p99(None, None, lambda v: v, [-3.0, -2.0], target_p99=0.5, refine=3)
    assert best is None and len(res) == 2
