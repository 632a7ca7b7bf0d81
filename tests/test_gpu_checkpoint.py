"""Checkpoint and resume: a run saved after some steps and resumed in a new
handle must continue exactly as the uninterrupted run (tables, statistics,
birth log), also with genomes."""
import numpy as np
import pytest

from qhg4_gb300 import checkpoint
from qhg4_gb300.gpu import GpuRun
from qhg4_gb300.spec import CROSSOVER_POISSON1, Genetics, config2_actions, config3_actions
from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid

from helpers import table_diff

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind", ["large_actions", "genetics"])
def test_resume_equals_uninterrupted(gpu_lib, tmp_path, kind):
    if kind == "genetics":
        grid = uniform_grid(5, 40.0)
        gen = Genetics(512, CROSSOVER_POISSON1, 1e-3)
        agents = make_agents(grid, 3000, seed=8, age_max=50.0, genome_blocks=gen.num_blocks)
        acts = config3_actions()
    else:
        grid = terrain_grid(12, seed=4)
        gen = Genetics()
        agents = make_agents(grid, 20000, seed=8, age_max=60.0, proportional_to_K=True)
        acts = config2_actions()
    whole = GpuRun(grid, acts, 99, gen, log_births=True)
    whole.load(agents)
    whole.step(30)
    part = GpuRun(grid, acts, 99, gen, log_births=True)
    part.load(agents)
    part.step(12)
    path = str(tmp_path / "ck.npz")
    checkpoint.save(part, path)
    part_log = part.birth_log()
    part.close()
    res = checkpoint.resume(grid, acts, 99, path, gen, log_births=True)
    assert res.current_step() == 12
    res.step(18)
    d = table_diff(res.agents(), whole.agents())
    assert d is None, d
    assert np.array_equal(res.stats(18), whole.stats(18))
    assert np.array_equal(np.concatenate([part_log, res.birth_log()]), whole.birth_log())
    res.close()
    whole.close()


def test_resume_with_environment_and_statistics(gpu_lib, tmp_path):
    """A run with K and move weights changed between steps, its occupation
    history and MoveStats: the checkpoint carries all of it, and the resumed
    run continues exactly as the uninterrupted one."""
    from helpers import cell_lonlat, move_weights
    grid = terrain_grid(12, seed=14)
    agents = make_agents(grid, 8000, seed=15, age_max=60.0, proportional_to_K=True)
    top = np.argsort(-grid.K)[:80]
    agents.cell[:] = top[agents.id % 80]
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    lon, lat = cell_lonlat(grid)
    K1 = grid.K * np.random.default_rng(16).uniform(0.5, 1.5, grid.num_cells)
    W = move_weights(grid, 17)

    def started():
        r = GpuRun(grid, acts, 55, track_occupancy=True)
        r.set_move_weights(W)
        r.load(agents)
        r.move_stats_enable(1, lon, lat, 6371.0)
        r.step(5)
        r.set_capacity(K1)
        r.step(5)
        return r

    whole = started()
    whole.step(15)
    part = started()
    path = str(tmp_path / "ck_env.npz")
    checkpoint.save(part, path)
    part.close()
    res = checkpoint.resume(grid, acts, 55, path)
    assert res.current_step() == 10
    res.step(15)
    d = table_diff(res.agents(), whole.agents())
    assert d is None, d
    assert np.array_equal(res.occupancy(), whole.occupancy())
    for x, y in zip(res.move_stats(), whole.move_stats()):
        assert np.array_equal(x.view(np.uint8), y.view(np.uint8))
    assert (whole.move_stats()[0] > 0).sum() > 10
    res.close()
    whole.close()
