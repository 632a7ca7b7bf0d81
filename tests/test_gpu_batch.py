"""Batches (qhg_batch_*): every run of a batch must give, bit for bit, what
the same run gives alone through the single-run path -- agent tables sorted
by ID, per-cell counts and per-step statistics -- however the runs join and
leave and whatever launch shape the batch uses.

A run admitted between two batch steps enters the table during the next
batch step and does its step 0 in the one after: after k batch steps it has
done k - 1 steps."""
import numpy as np
import pytest

from qhg4_gb300.batch import Autotuner, GpuBatch
from qhg4_gb300.gpu import GpuRun
from qhg4_gb300.spec import config1_actions, config2_actions
from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid

from helpers import table_diff

pytestmark = pytest.mark.gpu


def plain_case(k):
    rng = np.random.default_rng(100 + k)
    g = uniform_grid(int(rng.choice([6, 8, 10, 12])), 30.0)
    n = int(rng.integers(2000, 12000))
    acts = config1_actions(b0=float(rng.uniform(0.1, 0.6)), d0=float(rng.uniform(0.02, 0.08)),
                           move_p=float(rng.uniform(0.05, 0.3)))
    return g, make_agents(g, n, seed=200 + k, age_max=50.0), acts, 1000 + k


def alone(grid, agents, acts, seed, steps):
    r = GpuRun(grid, acts, seed)
    r.load(agents)
    r.step(steps)
    return r


def same_as_alone(batch, run, case, steps):
    grid, agents, acts, seed = case
    assert batch.steps_done(run) == steps
    r = alone(grid, agents, acts, seed, steps)
    d = table_diff(batch.agents(run), r.agents())
    assert d is None, f"run {run}: {d}"
    assert np.array_equal(batch.counts(run), r.counts())
    k = min(steps, 64)
    if k > 0:
        assert np.array_equal(batch.stats(run, k), r.stats(k))
    r.close()


def test_batch_runs_equal_alone_with_joins_and_leaves(gpu_lib):
    cases = [plain_case(k) for k in range(6)]
    b = GpuBatch(config1_actions(), agent_capacity=400_000, cell_capacity=8_000, max_runs=4)
    ids = {}
    for k in range(3):
        g, a, acts, seed = cases[k]
        ids[k] = b.add_run(g, acts, seed, a)
    b.step(7)
    for k in (3,):
        g, a, acts, seed = cases[k]
        ids[k] = b.add_run(g, acts, seed, a)
    b.step(5)
    same_as_alone(b, ids[1], cases[1], 11)
    b.remove_run(ids[1])
    b.step(3)
    # the freed slot and cells go to a new run
    g, a, acts, seed = cases[4]
    ids[4] = b.add_run(g, acts, seed, a)
    b.step(20)
    for k, steps in ((0, 34), (2, 34), (3, 27), (4, 19)):
        same_as_alone(b, ids[k], cases[k], steps)


def test_batch_shape_does_not_change_results(gpu_lib):
    cases = [plain_case(k) for k in range(3)]
    b = GpuBatch(config1_actions(), agent_capacity=200_000, cell_capacity=5_000, max_runs=3)
    ids = [b.add_run(g, acts, seed, a) for g, a, acts, seed in cases]
    b.step(2)
    _, _, ma, ms = b.shape()
    for k, (sa, ss) in enumerate(((1, 1), (ma, 1), (1, ms), (ma, ms))):
        b.set_shape(sa, ss)
        b.step(3)
    b.set_launch(ma, ms, 2, 200)   # wide scan tiles; warp-per-cell form only above 200 per cell
    b.step(3)
    b.set_launch(1, 1, 1, 2)       # narrow scan tiles; warp-per-cell form from 2 per cell
    b.step(3)
    tuner = Autotuner(trial_steps=1, span=2)
    tuner.tune(b)
    # CTA stage: 4 shapes, the incumbent among them; scan stage: the
    # incumbent + 2 widths; form stage: the incumbent + 3 thresholds
    assert tuner.table and len(tuner.trials[next(iter(tuner.trials))]) == 4 + 3 + 4
    b.step(2)
    for k, r in enumerate(ids):
        same_as_alone(b, r, cases[k], b.steps_done(r))


def test_batch_large_run_actions(gpu_lib):
    """VerhulstVarK, OldAgeDeath and WeightedMove through the batch's
    interpreted action program."""
    cases = []
    for k in range(3):
        g = terrain_grid(8 + 2 * k, seed=30 + k)
        a = make_agents(g, 15_000 + 5_000 * k, seed=300 + k, age_max=60.0, proportional_to_K=True)
        cases.append((g, a, config2_actions(b0=0.4 + 0.05 * k, move_p=0.1 + 0.05 * k), 50 + k))
    b = GpuBatch(config2_actions(), agent_capacity=400_000, cell_capacity=6_000, max_runs=3)
    ids = [b.add_run(g, acts, seed, a) for g, a, acts, seed in cases]
    b.step(25)
    for k, r in enumerate(ids):
        same_as_alone(b, r, cases[k], 24)


def test_batch_with_a_dense_run(gpu_lib):
    """One run with cells of more than 512 agents puts the batch's steps into
    the big-cell kernels; the other runs are unaffected."""
    cases = [plain_case(k) for k in range(2)]
    g = uniform_grid(4, 1000.0)
    cases.append((g, make_agents(g, 100_000, seed=77, age_max=50.0), config1_actions(K=1000.0), 5))
    b = GpuBatch(config1_actions(), agent_capacity=600_000, cell_capacity=4_000, max_runs=3)
    ids = [b.add_run(gg, acts, seed, a) for gg, a, acts, seed in cases]
    b.step(12)
    for k, r in enumerate(ids):
        same_as_alone(b, r, cases[k], 11)


def test_batch_dense_cells_cell_form(gpu_lib):
    """Runs whose cells hold ~60 agents: the batch steps in the warp-per-cell
    form with the specialised program; a run leaves and another joins."""
    cases = []
    for k in range(3):
        g = uniform_grid(6 + k, 80.0)
        acts = config1_actions(K=80.0, b0=0.3 + 0.1 * k)
        cases.append((g, make_agents(g, 60 * g.num_cells, seed=400 + k, age_max=50.0), acts, 70 + k))
    b = GpuBatch(config1_actions(K=80.0), agent_capacity=600_000, cell_capacity=6_000, max_runs=3)
    ids = {k: b.add_run(g, acts, seed, a) for k, (g, a, acts, seed) in enumerate(cases[:2])}
    b.step(6)
    b.remove_run(ids[1])
    b.step(2)
    g, a, acts, seed = cases[2]
    ids[2] = b.add_run(g, acts, seed, a)
    b.step(8)
    same_as_alone(b, ids[0], cases[0], 15)
    same_as_alone(b, ids[2], cases[2], 7)


def test_batch_atan_death(gpu_lib):
    """ATanDeath through the batch's interpreted action program, with each
    run's own curve (per-run max age, range and slope)."""
    from qhg4_gb300.spec import (ACT_ATANDEATH, ACT_FERTILITY, ACT_GETOLD, ACT_RANDOMPAIR, ACT_VERHULSTVARK,
                                 ACT_WEIGHTEDMOVE, Action)

    def acts(params):
        return [Action(ACT_GETOLD, 1), Action(ACT_FERTILITY, 2, (15.0, 45.0, 2.0)), Action(ACT_RANDOMPAIR, 3),
                Action(ACT_ATANDEATH, 4, params), Action(ACT_VERHULSTVARK, 6, (0.25, 0.04, 0.01)),
                Action(ACT_WEIGHTEDMOVE, 8, (0.15,))]

    curves = [(55.0, 12.0, 0.35), (50.0, 8.0, -0.4), (60.0, 300.0, 5.0)]
    cases = []
    for k, prm in enumerate(curves):
        g = terrain_grid(8 + k, seed=60 + k)
        a = make_agents(g, 10_000 + 4_000 * k, seed=600 + k, age_max=80.0, proportional_to_K=True)
        cases.append((g, a, acts(prm), 90 + k))
    b = GpuBatch(acts(curves[0]), agent_capacity=300_000, cell_capacity=6_000, max_runs=3)
    ids = [b.add_run(g, ac, seed, a) for g, a, ac, seed in cases]
    b.step(16)
    for k, r in enumerate(ids):
        same_as_alone(b, r, cases[k], 15)
