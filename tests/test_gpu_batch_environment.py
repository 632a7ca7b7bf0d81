"""Environment updates and occupation history of runs inside a batch
(qhg_batch_set_capacity, qhg_batch_set_move_weights, qhg_batch_set_ice,
qhg_batch_enable_occupancy, qhg_batch_occupancy): every run must give, bit
for bit, what the same run gives alone through the single-run path with the
same updates at the same steps (tests/test_gpu_environment.py and
tests/test_gpu_occupancy.py pin the single-run path against the oracle).

FlatExpPop (populations/FlatExpPop.cpp:43-56) takes VerhulstVarK's K from
NPPCapacity and WeightedMove's weights from a MultiEvaluator; both change
with the environment, and WeightedMove refuses moves into ice cells
(actions/WeightedMove.cpp:91).  OccTracker records when each cell is first
occupied (core/OccTracker.cpp)."""
import numpy as np
import pytest

from qhg4_gb300.batch import GpuBatch
from qhg4_gb300.gpu import GpuRun, QhgError
from qhg4_gb300.spec import config1_actions, config2_actions
from qhg4_gb300.workload import Agents, make_agents, terrain_grid, uniform_grid

from helpers import move_weights, table_diff

pytestmark = pytest.mark.gpu


def env_cases(form):
    cases = []
    for k in range(3):
        if form == "sparse":   # mostly empty cells: cell-aligned tiles
            g = terrain_grid(8 + 2 * k, seed=60 + k)
            a = make_agents(g, 12_000 + 4_000 * k, seed=600 + k, age_max=70.0, proportional_to_K=True)
        else:                  # ~35 agents per cell: the warp-per-cell form
            g = uniform_grid(5 + k, 40.0)
            a = make_agents(g, 35 * g.num_cells, seed=610 + k, age_max=70.0)
        cases.append((g, a, config2_actions(b0=0.4 + 0.05 * k, move_p=0.15 + 0.05 * k), 80 + k))
    return cases


def updates_for(k, grid):
    """(steps done, kind, array): K changes, given weights and ice flags."""
    rng = np.random.default_rng(900 + k)
    C = grid.num_cells

    def newK():
        return grid.K * rng.uniform(0.5, 1.5, size=C)

    ice = (rng.random(C) < 0.2).astype(np.uint8)
    if k == 0:
        return [(4, "K", newK()), (9, "K", newK())]
    if k == 1:
        return [(3, "W", move_weights(grid, 70 + k)), (7, "K", newK()), (11, "W", move_weights(grid, 90 + k))]
    return [(2, "ice", ice), (6, "K", newK()), (10, "ice", None)]


def apply_alone(r, kind, arr):
    {"K": r.set_capacity, "W": r.set_move_weights, "ice": r.set_ice}[kind](arr)


def apply_batch(b, run, kind, arr):
    {"K": b.set_capacity, "W": b.set_move_weights, "ice": b.set_ice}[kind](run, arr)


@pytest.mark.parametrize("form", ["sparse", "dense"])
def test_batch_environment_updates_equal_alone(gpu_lib, form):
    cases = env_cases(form)
    steps = 14
    b = GpuBatch(config2_actions(), agent_capacity=600_000, cell_capacity=6_000, max_runs=3)
    ids = [b.add_run(g, acts, seed, a) for g, a, acts, seed in cases]
    sched = {k: updates_for(k, cases[k][0]) for k in range(3)}
    # the batch: updates of every run at its own steps done
    b.step(1)   # the runs' agents enter (step 0)
    done = 0
    while done < steps:
        for k, r in enumerate(ids):
            for s, kind, arr in sched[k]:
                if s == done:
                    apply_batch(b, r, kind, arr)
        b.step(1)
        done += 1
    for k, r in enumerate(ids):
        g, a, acts, seed = cases[k]
        assert b.steps_done(r) == steps
        alone = GpuRun(g, acts, seed)
        alone.load(a)
        d0 = 0
        for s, kind, arr in sched[k]:
            if s > d0:
                alone.step(s - d0)
                d0 = s
            apply_alone(alone, kind, arr)
        alone.step(steps - d0)
        d = table_diff(b.agents(r), alone.agents())
        assert d is None, f"run {k}: {d}"
        assert np.array_equal(b.counts(r), alone.counts())
        assert np.array_equal(b.stats(r, steps), alone.stats(steps))
        alone.close()
    b.close()


def test_batch_environment_update_of_a_leaving_run_is_refused(gpu_lib):
    g, a, acts, seed = env_cases("sparse")[0]
    b = GpuBatch(config2_actions(), agent_capacity=200_000, cell_capacity=2_000, max_runs=2)
    r = b.add_run(g, acts, seed, a)
    b.step(3)
    b.remove_run(r)
    with pytest.raises(QhgError):
        b.set_capacity(r, g.K)
    b.close()


def clustered(grid, n, seed, ncells):
    """Agents placed in the first `ncells` cells only, so that the occupation
    spreads over the grid as they move."""
    a = make_agents(grid, n, seed=seed, age_max=50.0)
    return Agents(a.id, (a.cell % ncells).astype(np.int32), a.birth, a.age, a.lastb, a.gender, a.state)


def test_batch_occupancy_equal_alone(gpu_lib):
    acts = [config1_actions(b0=0.5, d0=0.02, move_p=0.3 + 0.1 * k) for k in range(4)]
    grids = [uniform_grid(6 + k, 30.0) for k in range(4)]
    # near K in the first cells (far above K, the Verhulst rates kill them all)
    agents = [clustered(grids[k], 25 * (20 + 10 * k), 700 + k, 20 + 10 * k) for k in range(4)]
    b = GpuBatch(config1_actions(), agent_capacity=400_000, cell_capacity=5_000, max_runs=3)
    b.enable_occupancy()
    ids = {k: b.add_run(grids[k], acts[k], 40 + k, agents[k]) for k in range(2)}
    b.step(6)
    ids[2] = b.add_run(grids[2], acts[2], 42, agents[2])
    b.step(5)
    b.remove_run(ids[0])
    b.step(2)
    ids[3] = b.add_run(grids[3], acts[3], 43, agents[3])   # reuses the first run's slot (and cells)
    b.step(9)
    for k in (1, 2, 3):
        r = ids[k]
        done = b.steps_done(r)
        alone = GpuRun(grids[k], acts[k], 40 + k, track_occupancy=True)
        alone.load(agents[k])
        alone.step(done)
        occ = b.occupancy(r)
        assert np.array_equal(occ, alone.occupancy()), f"run {k}"
        assert (occ >= 0).sum() > (occ == 0).sum()   # cells were first occupied after step 0
        d = table_diff(b.agents(r), alone.agents())
        assert d is None, f"run {k}: {d}"
        alone.close()
    b.close()


def test_batch_occupancy_needs_enabling_first(gpu_lib):
    g = uniform_grid(6, 30.0)
    b = GpuBatch(config1_actions(), agent_capacity=100_000, cell_capacity=3_000, max_runs=2)
    r = b.add_run(g, config1_actions(), 5, make_agents(g, 2_000, seed=5, age_max=50.0))
    with pytest.raises(QhgError):
        b.occupancy(r)        # not enabled
    with pytest.raises(QhgError):
        b.enable_occupancy()  # a run is in the batch already
    b.close()


def spreading_runs(form):
    """Runs whose agents start in part of their grid and spread out (the
    large run's actions: OldAgeDeath after WeightedMove, so some movers die
    in the step of their move)."""
    cases = []
    for k in range(3):
        if form == "sparse":
            g = terrain_grid(8 + 2 * k, seed=70 + k)
            a = make_agents(g, 4_000 + 1_000 * k, seed=710 + k, age_max=70.0, proportional_to_K=True)
            top = np.argsort(-g.K)[:40]
            a.cell[:] = top[a.id % 40]
        else:
            g = uniform_grid(6 + k, 60.0)
            cap = np.nonzero(g.xyz[:, 2] > 0.6)[0]
            a = make_agents(g, 35 * len(cap), seed=720 + k, age_max=70.0)
            a.cell[:] = cap[a.id % len(cap)]
        cases.append((g, a, config2_actions(b0=0.3, d0=0.03, move_p=0.25 + 0.05 * k), 95 + k))
    return cases


@pytest.mark.parametrize("form", ["sparse", "dense"])
@pytest.mark.parametrize("mode", [0, 1, 2], ids=["first", "min", "last"])
def test_batch_move_stats_equal_alone(gpu_lib, form, mode):
    from helpers import cell_lonlat
    cases = spreading_runs(form)
    b = GpuBatch(config2_actions(), agent_capacity=400_000, cell_capacity=4_000, max_runs=3)
    b.move_stats_enable(mode)
    ids = []
    for g, a, acts, seed in cases:
        r = b.add_run(g, acts, seed, a)
        b.move_stats_coords(r, *cell_lonlat(g))
        ids.append(r)
    b.step(13)
    for k, r in enumerate(ids):
        g, a, acts, seed = cases[k]
        alone = GpuRun(g, acts, seed)
        alone.load(a)
        alone.move_stats_enable(mode, *cell_lonlat(g))
        alone.step(b.steps_done(r))
        d = table_diff(b.agents(r), alone.agents())
        assert d is None, f"run {k}: {d}"
        bh, bd, bt = b.move_stats(r)
        ah, ad, at = alone.move_stats()
        assert np.array_equal(bh, ah), f"run {k}: hops differ in {(bh != ah).sum()} cells"
        assert np.array_equal(bd.view(np.uint64), ad.view(np.uint64)), f"run {k}: distances differ"
        assert np.array_equal(bt.view(np.uint64), at.view(np.uint64)), f"run {k}: times differ"
        assert (bh > 0).sum() > 0   # arrivals were recorded
        alone.close()
    b.close()


def test_batch_move_stats_needs_enabling_first(gpu_lib):
    g = uniform_grid(6, 30.0)
    b = GpuBatch(config1_actions(), agent_capacity=100_000, cell_capacity=3_000, max_runs=2)
    r = b.add_run(g, config1_actions(), 5, make_agents(g, 2_000, seed=5, age_max=50.0))
    with pytest.raises(QhgError):
        b.move_stats(r)            # not enabled
    with pytest.raises(QhgError):
        b.move_stats_enable(1)     # a run is in the batch already
    b.close()
