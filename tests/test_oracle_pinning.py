"""The C port oracle against the reference's own action code.

The golden fixtures were produced by the Philox test build of the reference
(oracle/_ref/qhg_ref_philox: the reference's action classes and SPopulation
compiled from its sources, draws keyed by seed, step, agent ID and action).
The port oracle must reproduce every fixture bit for bit: agent tables sorted
by ID, genomes, per-step statistics and the birth log.  When the reference
build is present (it is built from the reference sources, so only where they
are available), a fresh random case is also run through both.
"""
import os

import numpy as np
import pytest

from oracle import port
from oracle.refsim_io import ref_program, run_reference

from golden_util import Golden, golden_names
from helpers import table_diff


@pytest.mark.parametrize("name", golden_names())
def test_port_oracle_reproduces_reference_build(name):
    g = Golden(name)
    r = port.OracleRun(g.grid, g.actions, g.seed, g.genetics)
    r.load(g.agents)
    st = r.step(g.steps)
    d = table_diff(r.agents(), g.expected)
    assert d is None, d
    assert np.array_equal(st, g.stats)
    assert np.array_equal(r.birth_log(), g.births)


@pytest.mark.skipif(not os.path.exists(ref_program("philox")), reason="reference build not present")
def test_port_oracle_random_case_against_reference_build(tmp_path):
    from qhg4_gb300.spec import config2_actions
    from qhg4_gb300.workload import make_agents, terrain_grid
    grid = terrain_grid(9, seed=77)
    agents = make_agents(grid, 9000, seed=78, age_max=70.0, proportional_to_K=True)
    acts = config2_actions(b0=0.3, d0=0.03)
    ref = run_reference("philox", str(tmp_path), grid, agents, acts, 20, 31337, threads=2)
    r, st = port.run(grid, agents, acts, 20, 31337)
    assert ref.draw_errors == 0
    d = table_diff(r.agents(), ref.agents)
    assert d is None, d
    assert np.array_equal(st, ref.stats)
