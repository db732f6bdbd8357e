"""Cell-tile autotuner.

The fine-cell size is the one free tiling parameter of the particle step:
a bucket of the reference grid (edge 8 h0) is cut into `subcells`^3 fine
cells, and every sweep walks the fine cells that overlap its search box.
Small cells test fewer far candidates but split rows into more segments
(more list windows, more cell-start reads); large cells do the opposite.
The best size depends on h / bucket edge and on the particle count, so it is
measured: each candidate runs a few steps of the workload (or of a
representative member of an ensemble) and the fastest device time wins.

The choice changes the order in which neighbours are summed (rows of fine
cells), hence results at rounding level; a run is reproducible for a given
choice, and an ensemble member equals its single run with the same choice.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .solver import Solver

SUBCELL_CANDIDATES = (2, 3, 4, 5, 6)


def with_subcells(case, s: int):
    """the case with its bucket grid cut into s^3 fine cells per bucket"""
    return dataclasses.replace(case, grid=dataclasses.replace(case.grid, subcells=int(s)))


def time_case(case, steps: int = 3, warmup: int = 2) -> float:
    """device ms per step of `case` (after `warmup` untimed steps)"""
    sol = Solver(case)
    try:
        if case.pre_adaptive:
            sol.adaptive_sml()
        sol.steps(warmup)
        sol.steps(steps)
        return sol.phase_times()["total"] / steps
    finally:
        sol.close()


def tune_subcells(case, candidates=SUBCELL_CANDIDATES, steps: int = 3, warmup: int = 2):
    """(best subcells, {subcells: ms per step}) for a 3D case; 1D cases have
    one cell per bucket and are returned unchanged"""
    if case.options.dim != 3:
        return case.grid.subcells, {}
    table = {}
    for s in candidates:
        table[int(s)] = time_case(with_subcells(case, s), steps, warmup)
    best = min(table, key=table.get)
    return best, table


def tune_ensemble(cases, candidates=SUBCELL_CANDIDATES, classes: int = 3, steps: int = 3,
                  warmup: int = 2):
    """Per-member cell tiles for an ensemble: members are split into
    `classes` size classes (quantiles of the particle count); the median
    member of each class is tuned alone and its choice applies to the class.
    Returns (tuned cases, report)."""
    cases = list(cases)
    if not cases or cases[0].options.dim != 3:
        return cases, {"classes": []}
    n = np.array([c.particles.n for c in cases])
    order = np.argsort(n, kind="stable")
    groups = [g for g in np.array_split(order, max(1, min(classes, len(cases)))) if len(g)]
    out = list(cases)
    report = []
    for g in groups:
        rep = int(g[len(g) // 2])
        best, table = tune_subcells(cases[rep], candidates, steps, warmup)
        for k in g:
            out[int(k)] = with_subcells(cases[int(k)], best)
        report.append({"members": int(len(g)), "representative": rep,
                       "particles": int(cases[rep].particles.n), "subcells": int(best),
                       "ms_per_step": {str(k): round(v, 3) for k, v in table.items()}})
    return out, {"classes": report}
