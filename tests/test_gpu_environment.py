"""Environment updates between steps (qhg_gpu_set_capacity,
qhg_gpu_set_move_weights, qhg_gpu_set_ice) against the oracle, bit for bit.

FlatExpPop (populations/FlatExpPop.cpp:43-56) takes VerhulstVarK's K from
NPPCapacity and WeightedMove's cumulative weights from a MultiEvaluator;
both change when the environment does.  The oracle's handling of both is
pinned against the reference's own classes in tests/test_oracle_pinning.py.
"""
import numpy as np
import pytest

from oracle import port
from qhg4_gb300.gpu import GpuRun, QhgError
from qhg4_gb300.spec import config2_actions
from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid

from helpers import move_weights, table_diff

pytestmark = pytest.mark.gpu


def env_case(form):
    if form == "sparse":      # mostly empty cells: cell-aligned tiles
        grid = terrain_grid(12, seed=21)
        return grid, make_agents(grid, 30000, seed=22, age_max=70.0, proportional_to_K=True)
    grid = uniform_grid(6, 40.0)   # ~35 agents per cell: one warp per pair of cells
    return grid, make_agents(grid, 35 * grid.num_cells, seed=23, age_max=70.0)


def run_with_updates(grid, agents, acts, steps, seed, weights=None, updates=(), ice=None):
    """updates: (step, kind, array) with kind "K", "W" or "ice", applied before that step."""
    o = port.OracleRun(grid, acts, seed)
    g = GpuRun(grid, acts, seed, log_births=True)
    if ice is not None:           # before the upload
        o.set_ice(ice)
        g.set_ice(ice)
    if weights is not None:
        o.set_move_weights(weights)
        g.set_move_weights(weights)
    o.load(agents)
    g.load(agents)
    done, ost = 0, []
    for step, kind, arr in list(updates) + [(steps, None, None)]:
        if step > done:
            ost.append(o.step(step - done))
            g.step(step - done)
            done = step
        if kind == "K":
            o.set_capacity(arr)
            g.set_capacity(arr)
        elif kind == "W":
            o.set_move_weights(arr)
            g.set_move_weights(arr)
        elif kind == "ice":
            o.set_ice(arr)
            g.set_ice(arr)
    ost = np.concatenate(ost)
    d = table_diff(o.agents(), g.agents())
    assert d is None, d
    assert np.array_equal(o.counts(), g.counts())
    assert np.array_equal(ost, g.stats(steps))
    assert np.array_equal(o.birth_log(), g.birth_log())
    return ost


@pytest.mark.parametrize("form", ["sparse", "dense"])
def test_given_move_weights(gpu_lib, form):
    """Cumulative weights given from outside, with rows that are not
    monotone and rows of equal weights, set before the upload and replaced
    after 6 steps."""
    grid, agents = env_case(form)
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    st = run_with_updates(grid, agents, acts, 16, 301, weights=move_weights(grid, 302),
                          updates=[(6, "W", move_weights(grid, 303, nonmonotone=0.3, equal=0.2))])
    assert st[:, 3].sum() > 0


@pytest.mark.parametrize("form", ["sparse", "dense"])
def test_capacity_changes(gpu_lib, form):
    """K changed after 4 and after 11 steps (some cells to K = 0): the rates
    of the next step use the new K, and the move weights follow it."""
    grid, agents = env_case(form)
    rng = np.random.default_rng(311)
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    K1 = grid.K * rng.uniform(0.3, 1.5, grid.num_cells)
    K2 = np.where(rng.random(grid.num_cells) < 0.2, 0.0, grid.K * 1.2)
    st = run_with_updates(grid, agents, acts, 18, 312, updates=[(4, "K", K1), (11, "K", K2)])
    assert st[:, 2].sum() > 0


def test_capacity_changes_with_given_weights(gpu_lib):
    """With weights given, a K change leaves the weights as they are."""
    grid, agents = env_case("sparse")
    rng = np.random.default_rng(321)
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    K1 = grid.K * rng.uniform(0.5, 2.0, grid.num_cells)
    run_with_updates(grid, agents, acts, 14, 322, weights=move_weights(grid, 323), updates=[(5, "K", K1)])


def test_bad_move_weights_rejected(gpu_lib):
    grid, agents = env_case("dense")
    g = GpuRun(grid, config2_actions(), 5)
    g.load(agents)
    W = move_weights(grid, 331, nonmonotone=0.0, equal=0.0)
    W[3] = 0.0
    W[3, 0] = 1.0           # W[0] != W[n] and W[n] <= 0
    with pytest.raises(QhgError):
        g.set_move_weights(W)
    W = move_weights(grid, 332, nonmonotone=0.0, equal=0.0)
    W[5, 1] = np.nan
    with pytest.raises(QhgError):
        g.set_move_weights(W)
    g.step(2)               # the run is unaffected
    assert g.num_agents() > 0


@pytest.mark.parametrize("form", ["sparse", "dense"])
@pytest.mark.parametrize("weights", [False, True])
def test_ice_refuses_weighted_moves(gpu_lib, form, weights):
    """The Geography's ice (actions/WeightedMove.cpp:91): no move into an ice
    cell, weights from K give ice cells weight 0; ice set before the upload,
    changed after 5 steps and removed after 10 (then K changes, and weights
    that follow K follow the ice as well)."""
    grid, agents = env_case(form)
    rng = np.random.default_rng(341)
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.4)
    C = grid.num_cells
    ice0 = (rng.random(C) < 0.3).astype(np.uint8)
    ice1 = (rng.random(C) < 0.15).astype(np.uint8)
    W = move_weights(grid, 342) if weights else None
    st = run_with_updates(grid, agents, acts, 18, 343, weights=W, ice=ice0,
                          updates=[(5, "ice", ice1), (10, "ice", None), (13, "ice", ice0),
                                   (15, "K", grid.K * rng.uniform(0.5, 1.5, C))])
    assert st[:, 3].sum() > 0
