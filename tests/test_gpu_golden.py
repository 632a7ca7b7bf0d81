"""The CUDA path (through the C ABI) against the golden fixtures made by the
reference's own action code: every agent field bit for bit, the per-step
statistics and the birth log."""
import numpy as np
import pytest

from qhg4_gb300.gpu import GpuRun

from golden_util import Golden, golden_names
from helpers import table_diff

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_names())
def test_gpu_reproduces_golden(gpu_lib, name):
    g = Golden(name)
    run = GpuRun(g.grid, g.actions, g.seed, g.genetics, log_births=True)
    run.load(g.agents)
    run.step(g.steps)
    d = table_diff(run.agents(), g.expected)
    assert d is None, d
    assert np.array_equal(run.stats(g.steps), g.stats)
    assert np.array_equal(run.birth_log(), g.births)
    run.close()
