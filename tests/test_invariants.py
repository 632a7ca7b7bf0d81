"""The host-side invariant checks (qhg4_gb300/invariants.py) on tables of
the oracle, and on copies with a mistake planted on the CPU."""
import numpy as np

from oracle import port
from qhg4_gb300.invariants import check_stats, check_table
from qhg4_gb300.workload import Agents

from helpers import case_config2

FIELDS = ("id", "cell", "birth", "age", "lastb", "gender", "state")


def cell_order(a: Agents) -> Agents:
    o = np.argsort(a.cell, kind="stable")
    return Agents(*(getattr(a, k)[o] for k in FIELDS))


def test_invariants_hold_and_catch_planted_mistakes():
    grid, agents, acts = case_config2(n=10, N=12000, seed=3)
    r = port.OracleRun(grid, acts, 17)
    r.load(agents)
    live = len(agents)
    st = r.step(12)
    a = cell_order(r.agents())
    counts = r.counts()
    assert check_table(a, counts, r.next_id()) == []
    assert check_stats(st, live) == []

    b = cell_order(r.agents())
    b.id[5] = b.id[6]
    assert any("unique" in m for m in check_table(b, counts))
    b = cell_order(r.agents())
    b.cell[[0, -1]] = b.cell[[-1, 0]]
    assert any("ordered" in m for m in check_table(b, counts))
    b = cell_order(r.agents())
    b.state[3] = 0
    assert any("alive" in m for m in check_table(b, counts))
    c = counts.copy()
    c[a.cell[0]] += 1
    assert check_table(a, c) != []
    assert any("next ID" in m for m in check_table(a, counts, int(a.id.max())))
    bad = st.copy()
    bad[4, 1] += 1
    assert check_stats(bad, live) != []
