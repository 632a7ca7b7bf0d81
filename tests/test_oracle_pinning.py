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


@pytest.mark.skipif(not os.path.exists(ref_program("philox")), reason="reference build not present")
@pytest.mark.parametrize("atan_params", [(50.0, 8.0, -0.4), (60.0, 300.0, 5.0), (45.0, 20.0, 0.1)])
def test_port_oracle_atan_death_against_reference_build(tmp_path, atan_params):
    """ATanDeath (actions/ATanDeath.cpp) with a negative slope, a slope so
    steep that the death probability never reaches 0 or 1 (scale < 1), and a
    shallow one, against the reference's own class."""
    from qhg4_gb300.spec import (ACT_ATANDEATH, ACT_FERTILITY, ACT_GETOLD, ACT_RANDOMMOVE, ACT_RANDOMPAIR,
                                 ACT_VERHULSTVARK, Action)
    from qhg4_gb300.workload import make_agents, terrain_grid
    grid = terrain_grid(8, seed=81)
    agents = make_agents(grid, 6000, seed=82, age_max=80.0, proportional_to_K=True)
    acts = [Action(ACT_FERTILITY, 2, (15.0, 45.0, 2.0)), Action(ACT_RANDOMPAIR, 3),
            Action(ACT_ATANDEATH, 5, atan_params), Action(ACT_VERHULSTVARK, 6, (0.3, 0.03, 0.01)),
            Action(ACT_RANDOMMOVE, 7, (0.1,)), Action(ACT_GETOLD, 8)]
    ref = run_reference("philox", str(tmp_path), grid, agents, acts, 15, 4242, threads=2)
    r, st = port.run(grid, agents, acts, 15, 4242)
    assert ref.draw_errors == 0
    assert st[:, 2].sum() > 0
    d = table_diff(r.agents(), ref.agents)
    assert d is None, d
    assert np.array_equal(st, ref.stats)


@pytest.mark.skipif(not os.path.exists(ref_program("philox")), reason="reference build not present")
@pytest.mark.parametrize("given_weights,k_changes", [(True, False), (False, True), (True, True)],
                         ids=["weights", "capacity", "both"])
def test_port_oracle_environment_updates_against_reference_build(tmp_path, given_weights, k_changes):
    """WeightedMove on cumulative weights given from outside (what
    FlatExpPop's MultiEvaluator leaves, populations/FlatExpPop.cpp:43-56),
    including rows that are not monotone and rows of equal weights, and K
    changed between steps (NPPCapacity's output after an environment event),
    against the reference's classes."""
    from qhg4_gb300.spec import config2_actions
    from qhg4_gb300.workload import make_agents, terrain_grid
    from helpers import move_weights
    grid = terrain_grid(9, seed=91)
    agents = make_agents(grid, 9000, seed=92, age_max=70.0, proportional_to_K=True)
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    W = move_weights(grid, 93) if given_weights else None
    rng = np.random.default_rng(94)
    changes = []
    if k_changes:
        changes = [(5, grid.K * rng.uniform(0.3, 1.5, grid.num_cells)),
                   (12, np.where(rng.random(grid.num_cells) < 0.2, 0.0, grid.K * 1.2))]
    ref = run_reference("philox", str(tmp_path), grid, agents, acts, 18, 2718, threads=2, weights=W,
                        k_changes=changes)
    r = port.OracleRun(grid, acts, 2718)
    r.load(agents)
    if W is not None:
        r.set_move_weights(W)
    done, st = 0, []
    for step, K in changes + [(18, None)]:
        st.append(r.step(step - done))
        done = step
        if K is not None:
            r.set_capacity(K)
    st = np.concatenate(st)
    assert ref.draw_errors == 0
    d = table_diff(r.agents(), ref.agents)
    assert d is None, d
    assert np.array_equal(st, ref.stats)
    assert st[:, 3].sum() > 0


@pytest.mark.skipif(not os.path.exists(ref_program("philox")), reason="reference build not present")
@pytest.mark.parametrize("moves", ["random", "weighted"])
def test_port_oracle_move_stats_against_reference_build(tmp_path, moves):
    """MoveStats in its MIN mode (actions/MoveStats.cpp): per cell the
    fewest hops, the shortest distance and the first time agents reached
    it, against the reference's class on one thread (its per-thread merge
    makes more threads order-dependent); distances on a sphere of radius
    6371 from the cell centres' longitudes and latitudes."""
    from qhg4_gb300.spec import config1_actions, config2_actions
    from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid
    from helpers import cell_lonlat
    if moves == "random":
        grid = uniform_grid(10, 30.0)
        agents = make_agents(grid, 400, seed=101, age_max=50.0)
        agents.cell[:] = grid.nbr[0, agents.id % 5]   # start around one cell and spread out
        acts = config1_actions(b0=0.4, d0=0.02, move_p=0.4)
    else:
        grid = terrain_grid(10, seed=102)
        agents = make_agents(grid, 2000, seed=103, age_max=60.0, proportional_to_K=True)
        top = np.argsort(-grid.K)[:40]
        agents.cell[:] = top[agents.id % 40]      # start in the 40 best cells and spread out
        acts = config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    lon, lat = cell_lonlat(grid)
    ref = run_reference("philox", str(tmp_path), grid, agents, acts, 30, 777, threads=1,
                        move_stats=(1, lon, lat, 6371.0))
    r = port.OracleRun(grid, acts, 777)
    r.load(agents)
    r.move_stats_enable(1, lon, lat, 6371.0)
    st = r.step(30)
    assert ref.draw_errors == 0
    assert table_diff(r.agents(), ref.agents) is None
    assert np.array_equal(st, ref.stats)
    h, d, t = r.move_stats()
    rh, rd, rt = ref.move_stats
    assert (h > 0).sum() > 20
    assert np.array_equal(h, rh)
    assert np.array_equal(d.view(np.uint64), rd.view(np.uint64))
    assert np.array_equal(t.view(np.uint64), rt.view(np.uint64))


@pytest.mark.skipif(not os.path.exists(ref_program("philox")), reason="reference build not present")
@pytest.mark.parametrize("case", range(int(os.environ.get("QHG_PIN_CASES", "8"))))
def test_port_oracle_random_programs_against_reference_build(tmp_path, case):
    """Random action lists -- which actions, their priorities (ties broken by
    name), their parameters -- through the oracle and the reference's own
    classes: the oracle's action chain, draw windows and ordering rules hold
    for any program, not only the ones the other cases fix."""
    from qhg4_gb300.spec import (ACT_ATANDEATH, ACT_FERTILITY, ACT_GETOLD, ACT_OLDAGEDEATH, ACT_RANDOMMOVE,
                                 ACT_RANDOMPAIR, ACT_VERHULST, ACT_VERHULSTVARK, ACT_WEIGHTEDMOVE, Action)
    from qhg4_gb300.workload import make_agents, terrain_grid
    rng = np.random.default_rng(500 + case)

    def prio():
        return int(rng.integers(1, 6))

    acts = [Action(ACT_FERTILITY, prio(), (float(rng.uniform(10, 20)), float(rng.uniform(35, 50)),
                                           float(rng.uniform(0, 3)))),
            Action(ACT_RANDOMPAIR, prio())]
    if rng.random() < 0.5:
        acts.append(Action(ACT_VERHULST, prio(), (float(rng.uniform(0.1, 0.5)), float(rng.uniform(0.01, 0.08)),
                                                  0.01, float(rng.uniform(20, 80)))))
    else:
        acts.append(Action(ACT_VERHULSTVARK, prio(), (float(rng.uniform(0.1, 0.5)), float(rng.uniform(0.01, 0.08)),
                                                      0.01)))
    if rng.random() < 0.6:
        acts.append(Action(ACT_RANDOMMOVE, prio(), (float(rng.uniform(0.05, 0.5)),)))
    if rng.random() < 0.6:
        acts.append(Action(ACT_WEIGHTEDMOVE, prio(), (float(rng.uniform(0.05, 0.5)),)))
    if rng.random() < 0.6:
        acts.append(Action(ACT_OLDAGEDEATH, prio(), (float(rng.uniform(50, 70)), float(rng.uniform(0.01, 0.15)))))
    if rng.random() < 0.5:
        acts.append(Action(ACT_ATANDEATH, prio(), (float(rng.uniform(45, 65)), float(rng.uniform(5, 20)),
                                                   float(rng.uniform(-0.6, 0.6)))))
    if rng.random() < 0.8:
        acts.append(Action(ACT_GETOLD, prio()))
    grid = terrain_grid(8, seed=600 + case)
    agents = make_agents(grid, 5000, seed=700 + case, age_max=75.0, proportional_to_K=True)
    ref = run_reference("philox", str(tmp_path), grid, agents, acts, 15, 800 + case, threads=2)
    r, st = port.run(grid, agents, acts, 15, 800 + case)
    assert ref.draw_errors == 0
    d = table_diff(r.agents(), ref.agents)
    assert d is None, (d, [(a.type, a.prio) for a in acts])
    assert np.array_equal(st, ref.stats)


@pytest.mark.skipif(not os.path.exists(ref_program("philox")), reason="reference build not present")
def test_port_oracle_geography_kills_against_reference_build(tmp_path):
    """After a geography event FlatExpPop kills every agent in water or ice
    (populations/FlatExpPop.cpp:187-214); the plugin does it by taking the
    table out, leaving those cells' agents out and loading it back at the
    run's step with its next ID.  The oracle run that way equals the
    reference's registerDeath / recycleDeadSpaceNew path."""
    from qhg4_gb300.spec import config2_actions
    from qhg4_gb300.workload import Agents, make_agents, terrain_grid
    grid = terrain_grid(9, seed=950)
    agents = make_agents(grid, 9000, seed=951, age_max=70.0, proportional_to_K=True)
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    rng = np.random.default_rng(952)
    kills = [(5, (rng.random(grid.num_cells) < 0.15).astype(np.uint8)),
             (11, (rng.random(grid.num_cells) < 0.3).astype(np.uint8))]
    ref = run_reference("philox", str(tmp_path), grid, agents, acts, 16, 953, threads=2, kills=kills)
    r = port.OracleRun(grid, acts, 953)
    r.load(agents)
    done = 0
    for step, flags in kills + [(16, None)]:
        r.step(step - done)
        done = step
        if flags is None:
            continue
        a, nid, st = r.agents(), r.next_id(), r.current_step()
        keep = flags[a.cell] == 0
        r.load(Agents(*(getattr(a, k)[keep] for k in ("id", "cell", "birth", "age", "lastb", "gender", "state"))),
               first_step=st)
        r.set_next_id(nid)
    assert ref.draw_errors == 0
    d = table_diff(r.agents(), ref.agents)
    assert d is None, d


@pytest.mark.skipif(not os.path.exists(ref_program("philox")), reason="reference build not present")
@pytest.mark.parametrize("weights", [False, True])
def test_port_oracle_ice_refusal_against_reference_build(tmp_path, weights):
    """WeightedMove does not register a move into an ice cell of the grid's
    Geography (actions/WeightedMove.cpp:91); its draws are taken all the
    same.  A quarter of the cells is ice, with the weights from K and with
    given weights (rows of equal weights draw with wrandi)."""
    from helpers import move_weights
    from qhg4_gb300.spec import config2_actions
    from qhg4_gb300.workload import make_agents, terrain_grid
    grid = terrain_grid(8, seed=960)
    agents = make_agents(grid, 8000, seed=961, age_max=70.0, proportional_to_K=True)
    acts = config2_actions(b0=0.35, d0=0.03, move_p=0.4)
    ice = (np.random.default_rng(962).random(grid.num_cells) < 0.25).astype(np.uint8)
    W = move_weights(grid, 963) if weights else None
    ref = run_reference("philox", str(tmp_path), grid, agents, acts, 14, 964, threads=2, ice=ice, weights=W)
    r = port.OracleRun(grid, acts, 964)
    r.set_ice(ice)
    if W is not None:
        r.set_move_weights(W)
    r.load(agents)
    st = r.step(14)
    assert ref.draw_errors == 0
    d = table_diff(r.agents(), ref.agents)
    assert d is None, d
    assert np.array_equal(st, ref.stats)
    # the ice made a difference: without it the oracle registers more moves
    r2 = port.OracleRun(grid, acts, 964)
    if W is not None:
        r2.set_move_weights(W)
    r2.load(agents)
    st2 = r2.step(14)
    assert st2[:, 3].sum() > st[:, 3].sum()
