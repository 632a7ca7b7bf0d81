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
