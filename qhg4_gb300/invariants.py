"""Integer invariants of a run's state, checked on the host after a step.

The reference relies on per-thread lists and sorting for its consistency
(actions/RandomPair.cpp:192-196) and has no checker; these are the
invariants every committed table of this implementation keeps, so a test (or
a user debugging a configuration) can assert them step by step:

- the table is ordered by cell (the device's layout), every cell index lies
  in the grid, every row is alive (state ALIVE or FERTILE);
- agent IDs are unique and below the run's next ID;
- the per-cell counts are the table's cell histogram and sum to its size;
- the statistics add up: live(t) = live(t-1) + births(t) - deaths(t).

Each check returns a list of messages, empty when the state is consistent.
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np

from .workload import Agents

LS_ALIVE = 1
LS_FERTILE = 5


def check_table(a: Agents, counts: np.ndarray, next_id: Optional[int] = None) -> List[str]:
    """The table in device order (cell-sorted) against its per-cell counts."""
    bad = []
    C = len(counts)
    cell = np.asarray(a.cell, dtype=np.int64)
    if len(cell) and (cell.min() < 0 or cell.max() >= C):
        bad.append(f"cell index outside [0, {C})")
    if len(cell) > 1 and np.any(np.diff(cell) < 0):
        bad.append("table not ordered by cell")
    st = np.asarray(a.state)
    if np.any((st != LS_ALIVE) & (st != LS_FERTILE)):
        bad.append("a row that is not alive")
    ids = np.asarray(a.id, dtype=np.int64)
    if len(np.unique(ids)) != len(ids):
        bad.append("agent IDs not unique")
    if next_id is not None and len(ids) and ids.max() >= next_id:
        bad.append("an agent ID at or above the next ID")
    if not bad:
        hist = np.bincount(cell, minlength=C)
        if not np.array_equal(hist, np.asarray(counts, dtype=np.int64)):
            bad.append("per-cell counts differ from the table")
    if int(np.asarray(counts, dtype=np.int64).sum()) != len(ids):
        bad.append("per-cell counts do not sum to the table size")
    return bad


def check_stats(stats: np.ndarray, live_before: int) -> List[str]:
    """Per-step statistics rows (live, births, deaths, moves) after a table
    of `live_before` agents."""
    bad = []
    prev = int(live_before)
    for k, (live, births, deaths, _moves) in enumerate(np.asarray(stats, dtype=np.int64)):
        if live != prev + births - deaths:
            bad.append(f"step {k}: live {live} != {prev} + {births} - {deaths}")
        prev = int(live)
    return bad


def check_run(run, live_before: Optional[int] = None, nsteps: int = 0) -> List[str]:
    """A GpuRun's current table and counts, and its last `nsteps` rows of
    statistics when `live_before` (the live count before them) is given."""
    bad = check_table(run.agents(sort_by_id=False), run.counts(), run.next_id())
    if live_before is not None and nsteps > 0:
        bad += check_stats(run.stats(nsteps), live_before)
    return bad
