"""Occupation history of the cells (QHG_FLAG_TRACK_OCCUPANCY), the
reference's OccTracker / OccHistory for one population: per cell, the first
step whose agent table holds an agent there (the uploaded table counts as
its step), -1 for cells never occupied.  Checked against the oracle's
per-step cell counts."""
import numpy as np
import pytest

from oracle import port
from qhg4_gb300.gpu import GpuRun, QhgError

from helpers import case_config1, case_config2

pytestmark = pytest.mark.gpu


def expected_first_steps(grid, agents, acts, steps, seed):
    o = port.OracleRun(grid, acts, seed)
    o.load(agents)
    first = np.full(grid.num_cells, -1, dtype=np.int32)
    first[o.counts() > 0] = 0
    for t in range(1, steps + 1):
        o.step(1)
        first[(o.counts() > 0) & (first < 0)] = t
    return first


@pytest.mark.parametrize("case", ["config1", "config2"])
def test_first_occupation_matches_oracle(gpu_lib, case):
    if case == "config1":
        grid, agents, acts = case_config1(n=8, N=500, seed=4)
    else:
        grid, agents, acts = case_config2(n=12, N=1500, seed=6)
    exp = expected_first_steps(grid, agents, acts, 25, 9)
    g = GpuRun(grid, acts, 9, track_occupancy=True)
    g.load(agents)
    assert np.array_equal(g.occupancy(), np.where(exp == 0, 0, -1))
    g.step(10)
    g.step(15)
    got = g.occupancy()
    assert np.array_equal(got, exp)
    assert (got > 0).any()   # cells were reached during the run
    g.close()


def test_occupancy_needs_the_flag(gpu_lib):
    grid, agents, acts = case_config1(n=6, N=1000, seed=2)
    g = GpuRun(grid, acts, 1)
    g.load(agents)
    with pytest.raises(QhgError):
        g.occupancy()
    g.close()
