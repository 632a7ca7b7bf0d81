"""MoveStats (qhg_gpu_move_stats_enable / qhg_gpu_move_stats) against the
oracle, bit for bit: per cell hops, distance and arrival time.

The oracle's MoveStats is pinned against the reference's own class in
tests/test_oracle_pinning.py (MIN mode; FIRST and LAST depend on the order
of the moves, which the reference takes by slot and this build by agent ID).
The large run's actions put OldAgeDeath after WeightedMove, so agents that
move and then die in the same step are part of every case.
"""
import numpy as np
import pytest

from oracle import port
from qhg4_gb300.gpu import GpuRun, QhgError
from qhg4_gb300.spec import config1_actions, config2_actions
from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid

from helpers import cell_lonlat, table_diff

pytestmark = pytest.mark.gpu


def spreading_case(form):
    """Agents that start in a part of the grid and spread out."""
    if form == "sparse":        # cell-aligned tiles
        grid = terrain_grid(12, seed=41)
        agents = make_agents(grid, 6000, seed=42, age_max=70.0, proportional_to_K=True)
        top = np.argsort(-grid.K)[:60]
        agents.cell[:] = top[agents.id % 60]
        return grid, agents, config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    if form == "dense":         # ~35 agents per cell: one warp per pair of cells
        grid = uniform_grid(8, 60.0)
        cap = np.nonzero(grid.xyz[:, 2] > 0.6)[0]
        agents = make_agents(grid, 35 * len(cap), seed=43, age_max=70.0)
        agents.cell[:] = cap[agents.id % len(cap)]
        return grid, agents, config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    grid = uniform_grid(3, 900.0)  # ~600 agents per cell: the big-cell kernels
    cap = np.nonzero(grid.xyz[:, 2] > 0.3)[0]
    agents = make_agents(grid, 600 * len(cap), seed=44, age_max=50.0)
    agents.cell[:] = cap[agents.id % len(cap)]
    return grid, agents, config1_actions(K=900.0, move_p=0.3)


def compare(o, g):
    d = table_diff(o.agents(), g.agents())
    assert d is None, d
    oh, od, ot = o.move_stats()
    gh, gd, gt = g.move_stats()
    assert np.array_equal(oh, gh), f"hops differ in {(oh != gh).sum()} cells"
    assert np.array_equal(od.view(np.uint64), gd.view(np.uint64)), "distances differ"
    assert np.array_equal(ot.view(np.uint64), gt.view(np.uint64)), "times differ"
    return gh


@pytest.mark.parametrize("form", ["sparse", "dense", "big"])
@pytest.mark.parametrize("mode", [0, 1, 2], ids=["first", "min", "last"])
def test_move_stats(gpu_lib, form, mode):
    grid, agents, acts = spreading_case(form)
    lon, lat = cell_lonlat(grid)
    o = port.OracleRun(grid, acts, 91)
    o.load(agents)
    o.move_stats_enable(mode, lon, lat, 6371.0)
    g = GpuRun(grid, acts, 91)
    g.load(agents)
    g.move_stats_enable(mode, lon, lat, 6371.0)
    o.step(3)
    g.step(3)
    compare(o, g)
    o.step(17)
    g.step(17)
    h = compare(o, g)
    assert (h > 1).sum() > 5


def test_move_stats_enabled_late_and_after_upload(gpu_lib):
    """Enabling after some steps starts from the current table; a new upload
    starts again; plane coordinates (cartdist)."""
    grid, agents, acts = spreading_case("sparse")
    rng = np.random.default_rng(5)
    x, y = rng.uniform(0, 100, grid.num_cells), rng.uniform(0, 100, grid.num_cells)
    o = port.OracleRun(grid, acts, 92)
    g = GpuRun(grid, acts, 92)
    o.load(agents)
    g.load(agents)
    o.step(4)
    g.step(4)
    o.move_stats_enable(1, x, y, 1.0, cartesian=True)
    g.move_stats_enable(1, x, y, 1.0, cartesian=True)
    o.step(8)
    g.step(8)
    compare(o, g)
    a = g.agents()
    o.load(a, first_step=12)
    g.load(a, first_step=12)
    o.step(6)
    g.step(6)
    compare(o, g)


def test_move_stats_errors(gpu_lib):
    grid, agents, acts = spreading_case("dense")
    g = GpuRun(grid, acts, 93)
    g.load(agents)
    with pytest.raises(QhgError):
        g.move_stats()
    lon, lat = cell_lonlat(grid)
    with pytest.raises(QhgError):
        g.move_stats_enable(3, lon, lat, 1.0)
