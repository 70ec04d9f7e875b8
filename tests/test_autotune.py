"""The launch autotuner's selection logic (galax_gb300/autotune.py), on the CPU:
the library setters and the timer are replaced by fakes, so no device is needed.
It must keep the candidate whose slowest run is fastest, tune the team SM count
and then the split fraction only for adaptive Dopri5, and leave the library set
to the winners."""

from __future__ import annotations

import pytest


@pytest.fixture()
def fake(monkeypatch):
    import galax_gb300.autotune as A

    state = {"launch": None, "team": None, "split": None, "calls": []}
    # step time as a function of the current settings (ms); two runs each, the second slower
    launch_ms = {(128, 1, 2): 1200.0, (64, 2, 2): 1190.0, (128, 0, 0): 1300.0}
    team_ms = {6: 70.0, 8: 90.0, 10: 55.0, 12: 30.0, 16: 80.0, 20: 50.0, 24: 40.0, 28: 0.0, 32: 10.0,
               40: 60.0}
    split_ms = {0.08: -15.0, 0.1: 0.0, 0.12: 20.0}

    def set_launch(method, adaptive, block, per_sm, variant):
        state["launch"] = (block, per_sm, variant)
        state["calls"].append(("launch", method, adaptive))

    def set_team(blocks):
        state["team"] = blocks
        state["calls"].append(("team", blocks))

    def set_split_fraction(frac):
        state["split"] = frac
        state["calls"].append(("split", frac))

    def worst_ms(run, repeats):
        assert repeats == 2
        base = launch_ms[state["launch"]]
        base += team_ms.get(state["team"], 0.0) + split_ms.get(state["split"], 0.0)
        return max(base, base + 0.5)

    monkeypatch.setattr(A, "set_launch", set_launch)
    monkeypatch.setattr(A, "set_team", set_team)
    monkeypatch.setattr(A, "set_split_fraction", set_split_fraction)
    monkeypatch.setattr(A, "_worst_ms", worst_ms)
    return A, state, list(launch_ms)


def test_adaptive_dopri5_tunes_shape_then_teams_then_split(fake):
    A, state, cands = fake
    out = A.tune(lambda: None, 5, True, candidates=cands)
    assert out["best"] == {"block_threads": 64, "blocks_per_sm": 2, "variant": 2, "team_blocks": 28,
                           "split_fraction": 0.08}
    assert state["launch"] == (64, 2, 2) and state["team"] == 28 and state["split"] == 0.08
    assert set(out["team_ms"]) == {str(t) for t in A.DEFAULT_TEAMS[5]}
    assert set(out["split_ms"]) == {str(f) for f in A.DEFAULT_SPLITS}
    # the split fraction is tuned with the chosen team count in place
    kinds = [c[0] for c in state["calls"]]
    last_team = max(i for i, k in enumerate(kinds) if k == "team")
    assert state["calls"][last_team] == ("team", 28) and kinds.index("split") > last_team


def test_fixed_step_batches_tune_the_launch_shape_only(fake):
    A, state, cands = fake
    for method in (5, 8):
        state["calls"].clear()
        out = A.tune(lambda: None, method, False, candidates=cands)
        assert set(out["best"]) == {"block_threads", "blocks_per_sm", "variant"}
        assert "team_ms" not in out and "split_ms" not in out
        assert all(c[0] == "launch" for c in state["calls"])


def test_adaptive_dopri8_teams_without_shape_candidates(fake):
    A, state, _ = fake
    state["launch"] = (128, 1, 2)  # left as it is
    out = A.tune(lambda: None, 8, True, candidates=())
    assert out["ms"] == {} and "block_threads" not in out["best"]
    assert set(out["team_ms"]) == {str(t) for t in A.DEFAULT_TEAMS[8]}
    assert out["best"]["team_blocks"] == 12 and state["team"] == 12 and state["launch"] == (128, 1, 2)
    assert all(c[0] != "launch" for c in state["calls"])
