"""The integer invariants of the committed table (qhg4_gb300/invariants.py)
after every step of the CUDA path: cell order, valid cells and states,
unique IDs below the next ID, counts equal to the table's histogram, and
statistics that add up -- in the tile and the warp-per-cell forms."""
import pytest

from qhg4_gb300.gpu import GpuRun
from qhg4_gb300.invariants import check_run

from helpers import case_config1, case_config2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["sparse", "dense"])
def test_invariants_every_step(gpu_lib, case):
    if case == "sparse":
        grid, agents, acts = case_config2(n=12, N=20000, seed=21)
    else:
        grid, agents, acts = case_config1(n=6, N=12000, seed=22)
    g = GpuRun(grid, acts, 23)
    g.load(agents)
    live = len(agents)
    for _ in range(8):
        g.step(1)
        bad = check_run(g, live, 1)
        assert bad == [], bad
        live = g.num_agents()
    g.close()
