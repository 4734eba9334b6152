"""The autotuner's candidates all give the default configuration's results
(bit for bit, or to rounding where the split block-per-cell form takes
cells), and it returns the fastest one it timed."""
import numpy as np
import pytest


@pytest.mark.gpu
def test_autotune_small_grid():
    import torch
    import gcchem.autotune as autotune
    import gcchem.capi as capi
    import gcchem.inputs as inputs

    cells = inputs.grid_cells(20, 10, 12, seed=5)
    dev = torch.device("cuda", 0)
    T = lambda a: torch.tensor(a, device=dev).contiguous()
    n = cells["c"].shape[1]
    atol, rtol = inputs.tolerances()
    ic, rc = inputs.default_controls()
    case = {"met": T(cells["met"]), "ph": T(cells["photol"]), "c": T(cells["c"]), "at": T(atol), "rt": T(rtol),
            "ic": ic, "rc": rc, "dt": 600.0, "ist": torch.zeros((20, n), dtype=torch.int32, device=dev),
            "rst": torch.zeros((20, n), dtype=torch.float64, device=dev),
            "ierr": torch.zeros(n, dtype=torch.int32, device=dev)}
    solver = capi.Solver(0, arith="fast", schedule="queue")
    axes = {"block": [64, 128], "arith": ["fast", "fast2"], "queue_chunk": [1, 4], "cell_block": [32, 128],
            "block_split": [False], "evict_after": [0, 3]}
    best, t, table = autotune.tune(solver, case, torch.zeros(n, dtype=torch.float64, device=dev), sweeps=1,
                                   reps=1, axes=axes)
    assert all(best[k] in axes[k] for k in axes)
    assert {row["queue_chunk"] for row in table} == {1, 4} and {row["cell_block"] for row in table} == {32, 128}
    assert len(table) >= 4 and np.isclose(table[0]["ms"], t * 1e3)
