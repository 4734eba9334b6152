"""The autotuner's host logic on the CPU, with the timed step replaced by a
fake: coordinate descent finds the fastest setting of a separable cost, the
split form's candidates collapse onto one cell_block, the result is applied
to the solver with every setting, and a candidate that changes the results
is refused."""
import pytest


class _FakeSolver:
    mech = "fullchem"

    def __init__(self):
        self.calls = []

    def set(self, **kw):
        self.calls.append(kw)


def _cost(cfg):
    # separable: each axis has its own best value
    c = 1.0
    c += {32: 0.4, 64: 0.1, 128: 0.0, 256: 0.2}[cfg["block"]]
    c += {"fast": 0.0, "fast2": 0.3}[cfg["arith"]]
    c += {1: 0.0, 2: 0.2, 4: 0.5, 8: 0.9}[cfg["queue_chunk"]]
    c += 0.0 if cfg["block_split"] else 0.05 + {32: 0.3, 128: 0.0, 256: 0.1}[cfg["cell_block"]]
    c += {0: 0.6, 2: 0.2, 4: 0.0, 8: 0.1, 16: 0.3}[cfg["evict_after"]]
    return c


def _fake_time_step(seen, bad=None):
    import torch

    def f(solver, cfg, case, hs0, order=None, nblock=0):
        seen.append(dict(cfg))
        c = torch.full((4, 3), 1.0e6, dtype=torch.float64)  # species above 1e4 molec/cm3
        if bad is not None and all(cfg.get(k) == v for k, v in bad.items()):
            c = c * 2.0
        return _cost(cfg), (c, torch.zeros(3, dtype=torch.int32))

    return f


def test_coordinate_descent_finds_the_fastest_setting(monkeypatch):
    import gcchem.autotune as autotune

    seen = []
    monkeypatch.setattr(autotune, "time_step", _fake_time_step(seen))
    solver = _FakeSolver()
    best, t, table = autotune.tune(solver, {}, None, sweeps=2, reps=1)
    assert best == {"block": 128, "arith": "fast", "queue_chunk": 1, "cell_block": 256, "block_split": True,
                    "evict_after": 4}
    assert t == pytest.approx(1.0)
    # the split form always runs 256 threads: no split candidate with another cell_block
    assert all(row["cell_block"] == 256 for row in table if row["block_split"])
    assert {row["cell_block"] for row in table if not row["block_split"]} == {256}
    keys = [tuple(sorted(row.items())) for row in table]
    assert len(keys) == len(set(keys))  # each candidate timed once
    assert {row["queue_chunk"] for row in table} == set(autotune.AXES["queue_chunk"])
    # the result is applied with every setting the step uses
    assert solver.calls[-1] == {k: best[k] for k in autotune.SETTINGS}


def test_level_form_axis_and_warp_per_cell(monkeypatch):
    import gcchem.autotune as autotune

    seen = []
    monkeypatch.setattr(autotune, "time_step", _fake_time_step(seen))
    axes = {"block_split": [False], "cell_block": [32, 128, 256], "evict_after": [0, 4]}
    best, t, table = autotune.tune(_FakeSolver(), {}, None, sweeps=1, reps=1, axes=axes)
    assert best["block_split"] is False and best["cell_block"] == 128
    assert {row["cell_block"] for row in table} == {32, 128, 256}


def test_candidate_that_changes_results_is_refused(monkeypatch):
    import gcchem.autotune as autotune

    monkeypatch.setattr(autotune, "time_step", _fake_time_step([], bad={"queue_chunk": 4}))
    with pytest.raises(RuntimeError, match="changed the results"):
        autotune.tune(_FakeSolver(), {}, None, sweeps=1, reps=1)
