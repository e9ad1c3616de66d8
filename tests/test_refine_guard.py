"""Host logic of iterative refinement's divergence stop (no GPU): which residual histories stop the
outer loop and which iterate the solver keeps."""

import math

from warp_gb300.optim.linear import _DivergenceGuard


def _run(r0, seq, bnorm=1.0):
    g = _DivergenceGuard(r0, bnorm)
    return [g.step(r) for r in seq]


def test_converging_history_never_stops():
    assert _run(1.0, [1e-2, 1e-4, 1e-6, 1e-8]) == ["ok"] * 4


def test_moderate_steady_growth_stops_after_two_steps_and_restores():
    # ~4x per step (the bf16-inner history on a rough field): no single step trips the 100x test
    assert _run(1.0, [4.0, 16.0]) == ["save", "restore"]
    # growth from a warm start far below ||b||
    assert _run(1e-6, [3e-6, 9e-6]) == ["save", "restore"]


def test_single_growth_followed_by_progress_continues():
    assert _run(1.0, [2.0, 0.1, 1e-3]) == ["save", "ok", "ok"]
    # a later growth needs a fresh second growth to stop
    assert _run(1.0, [2.0, 0.1, 0.2, 0.05]) == ["save", "ok", "save", "ok"]


def test_blow_up_is_undone_at_once():
    assert _run(1.0, [500.0]) == ["undo"]
    assert _run(1.0, [math.nan]) == ["undo"]
    assert _run(1.0, [math.inf]) == ["undo"]
    # over 1e3 x max(||b||, r0) without a 100x step
    g = _DivergenceGuard(1.0, 1.0)
    assert [g.step(r) for r in (0.5, 0.4)] == ["ok", "ok"]
    g.prev = 20.0
    assert g.step(1500.0) == "undo"


def test_blow_up_after_a_growth_restores_the_saved_iterate():
    assert _run(1.0, [2.0, 400.0]) == ["save", "restore"]
