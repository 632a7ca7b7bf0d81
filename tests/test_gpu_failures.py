"""Failure detection without a GPU fault.  Every device-side wait of the step
is bounded (about one second); a test makes one run out -- the next step's
cell scan withholds a tile's status -- and checks that the failure is
reported as QHG_ERR_TIMEOUT, that the run keeps its last step, and that
stepping on gives exactly the results of a run that never failed.  Capacity
and cell-size errors are reported the same way."""
import numpy as np
import pytest

from qhg4_gb300.gpu import GpuRun, QhgError
from qhg4_gb300.spec import config1_actions, config2_actions
from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid

from helpers import table_diff

pytestmark = pytest.mark.gpu

QHG_ERR_CAPACITY = -7
QHG_ERR_TIMEOUT = -6
QHG_ERR_CELL_TOO_LARGE = -5


@pytest.mark.parametrize("tile", [0, 1])
def test_bounded_wait_runs_out_and_the_run_recovers(gpu_lib, tile):
    grid = terrain_grid(12, seed=4)          # 1442 cells: 3 scan tiles
    agents = make_agents(grid, 30000, seed=3, age_max=60.0, proportional_to_K=True)
    acts = config2_actions()
    whole = GpuRun(grid, acts, 17, log_births=True)
    whole.load(agents)
    whole.step(10)
    run = GpuRun(grid, acts, 17, log_births=True)
    run.load(agents)
    run.step(5)
    run.sync()
    run.test_stall_scan(tile)
    run.step(1)
    with pytest.raises(QhgError) as e:
        run.sync()
    assert e.value.code == QHG_ERR_TIMEOUT
    assert run.current_step() == 5
    run.step(5)
    d = table_diff(run.agents(), whole.agents())
    assert d is None, d
    assert np.array_equal(run.stats(5), whole.stats(5))
    assert np.array_equal(run.birth_log(), whole.birth_log())
    run.close()
    whole.close()


def test_capacity_error_keeps_the_step(gpu_lib):
    grid = uniform_grid(6, 30.0)
    agents = make_agents(grid, 5000, seed=2, age_max=50.0)
    acts = config1_actions(b0=0.9, d0=0.0, theta=0.0)   # a growing population: no deaths below K
    run = GpuRun(grid, acts, 5, capacity=5100)
    run.load(agents)
    with pytest.raises(QhgError) as e:
        for _ in range(40):
            run.step(1)
            run.sync()
    assert e.value.code == QHG_ERR_CAPACITY
    s = run.current_step()
    assert run.num_agents() <= 5100
    run.close()
    assert s >= 0


def test_cell_too_large_is_rejected_at_upload(gpu_lib):
    grid = uniform_grid(1, 30.0)               # 12 cells
    agents = make_agents(grid, 12 * 5000, seed=2, age_max=50.0)
    run = GpuRun(grid, config1_actions(), 5)
    with pytest.raises(QhgError) as e:
        run.load(agents)
    assert e.value.code == QHG_ERR_CELL_TOO_LARGE
    run.close()
