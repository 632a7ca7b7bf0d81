"""Bit-exact parity of the CUDA path (through the C ABI) with the oracle.

The oracle is the C port in oracle/qhg_oracle.c, itself pinned against the
reference's own action code (tests/test_oracle_pinning.py).  Every field of
every agent, sorted by ID, must match bit for bit, as must the per-step
statistics, the per-cell counts and the (baby, mother, father) birth log.
"""
import numpy as np
import pytest

from oracle import port
from qhg4_gb300.gpu import GpuRun
from qhg4_gb300.spec import (ACT_ATANDEATH, ACT_FERTILITY, ACT_GETOLD, ACT_OLDAGEDEATH, ACT_RANDOMMOVE, ACT_RANDOMPAIR,
                             ACT_VERHULST, ACT_VERHULSTVARK, ACT_WEIGHTEDMOVE, CROSSOVER_POISSON1, Action,
                             Genetics, config1_actions, config3_actions)
from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid

from helpers import case_config1, case_config2, table_diff

pytestmark = pytest.mark.gpu


def run_both(grid, agents, actions, steps, seed, chunks=(None,), genetics=Genetics()):
    o = port.OracleRun(grid, actions, seed, genetics)
    o.load(agents)
    g = GpuRun(grid, actions, seed, genetics, log_births=True)
    g.load(agents)
    done = 0
    ost = []
    for ch in chunks:
        k = steps - done if ch is None else ch
        ost.append(o.step(k))
        g.step(k)
        done += k
    ost = np.concatenate(ost, axis=0)
    return o, g, ost


def assert_same(o, g, ost, steps):
    d = table_diff(o.agents(), g.agents())
    assert d is None, d
    assert np.array_equal(o.counts(), g.counts())
    assert np.array_equal(ost[-min(steps, 1024):], g.stats(min(steps, 1024)))
    ob, gb = o.birth_log(), g.birth_log()
    assert np.array_equal(ob, gb), f"birth logs differ ({len(ob)} vs {len(gb)})"


def test_config1_small(gpu_lib):
    grid, agents, acts = case_config1()
    o, g, st = run_both(grid, agents, acts, 60, 42)
    assert_same(o, g, st, 60)


def test_config1_stepwise(gpu_lib):
    grid, agents, acts = case_config1(n=6, N=6000, seed=5)
    o, g, st = run_both(grid, agents, acts, 25, 7, chunks=(1, 1, 3, 20))
    assert_same(o, g, st, 25)


def test_config2_small(gpu_lib):
    grid, agents, acts = case_config2()
    o, g, st = run_both(grid, agents, acts, 40, 5)
    assert_same(o, g, st, 40)


def test_interpreted_program_order(gpu_lib):
    """An action order that matches no specialised kernel program runs the
    run-time interpreter; GetOld first, OldAgeDeath before Verhulst and both
    move actions."""
    grid, agents, _ = case_config2(n=12, N=20000, seed=11)
    acts = [Action(ACT_GETOLD, 1), Action(ACT_FERTILITY, 2, (15.0, 45.0, 2.0)), Action(ACT_RANDOMPAIR, 3),
            Action(ACT_OLDAGEDEATH, 4, (64.0, 5.0 / 64.0)), Action(ACT_VERHULSTVARK, 6, (0.25, 0.04, 0.01)),
            Action(ACT_RANDOMMOVE, 7, (0.05,)), Action(ACT_WEIGHTEDMOVE, 8, (0.15,))]
    o, g, st = run_both(grid, agents, acts, 30, 123)
    assert_same(o, g, st, 30)


def atan_actions(params):
    """GetOld, Fertility, RandomPair, ATanDeath, VerhulstVarK, WeightedMove."""
    return [Action(ACT_GETOLD, 1), Action(ACT_FERTILITY, 2, (15.0, 45.0, 2.0)), Action(ACT_RANDOMPAIR, 3),
            Action(ACT_ATANDEATH, 4, params), Action(ACT_VERHULSTVARK, 6, (0.25, 0.04, 0.01)),
            Action(ACT_WEIGHTEDMOVE, 8, (0.15,))]


def atan_case(form):
    if form == "sparse":      # mostly empty cells: cell-aligned tiles
        grid = terrain_grid(10, seed=5)
        return grid, make_agents(grid, 15000, seed=51, age_max=80.0, proportional_to_K=True)
    if form == "dense":       # ~35 agents per cell: one warp per pair of cells
        grid = uniform_grid(5, 40.0)
        return grid, make_agents(grid, 35 * grid.num_cells, seed=52, age_max=80.0)
    grid = uniform_grid(3, 700.0)  # ~600 agents per cell: the big-cell kernels
    return grid, make_agents(grid, 600 * grid.num_cells, seed=53, age_max=80.0)


@pytest.mark.parametrize("form", ["sparse", "dense", "big"])
def test_atan_death(gpu_lib, form):
    """ATanDeath (actions/ATanDeath.cpp): the death probability 0.5 + scale *
    atan(slope * (age - M)) / pi against each draw, in all three kernel
    forms; ages far from M decide without evaluating the arctangent."""
    grid, agents = atan_case(form)
    o, g, st = run_both(grid, agents, atan_actions((55.0, 12.0, 0.35)), 20, 61, chunks=(1, 19))
    assert_same(o, g, st, 20)
    assert st[:, 2].sum() > 0


@pytest.mark.parametrize("params", [(50.0, 8.0, -0.4), (60.0, 300.0, 5.0), (45.0, 20.0, 0.1)],
                         ids=["negative_slope", "steep_no_window", "shallow"])
def test_atan_death_curves(gpu_lib, params):
    """A negative slope (the curve still rises: scale changes sign with it),
    a slope so steep that the probability never reaches 0 or 1 (every age
    evaluates the arctangent), and a shallow curve."""
    grid, agents = atan_case("dense")
    o, g, st = run_both(grid, agents, atan_actions(params), 15, 62)
    assert_same(o, g, st, 15)
    assert st[:, 2].sum() > 0


def test_no_pairing_no_moves(gpu_lib):
    """Without RandomPair no female has a mate: no births; no move actions."""
    grid, agents, _ = case_config1(n=6, N=8000, seed=2)
    acts = [Action(ACT_FERTILITY, 2, (15.0, 45.0, 2.0)), Action(ACT_VERHULST, 6, (0.2, 0.05, 0.01, 30.0)),
            Action(ACT_GETOLD, 8)]
    o, g, st = run_both(grid, agents, acts, 15, 5)
    assert_same(o, g, st, 15)
    assert st[:, 1].sum() == 0


@pytest.mark.parametrize("genetics", [Genetics(4096, CROSSOVER_POISSON1, 1e-4), Genetics(1000, 3, 1e-3),
                                      Genetics(100, 0, 0.0), Genetics(64, 1, 0.0)],
                         ids=["poisson_4096", "fixed3_1000", "nocross_100", "fixed1_64"])
def test_genetics(gpu_lib, genetics):
    """Genetics::makeOffspring: crossover (Poisson(1) or fixed counts, none),
    mutation counts from the binomial table, genomes whose size is not a
    multiple of 64 loci; genome slots of the dead reused by later births."""
    grid = uniform_grid(5, 40.0)
    agents = make_agents(grid, 3000, seed=31, age_max=50.0, genome_blocks=genetics.num_blocks)
    o, g, st = run_both(grid, agents, config3_actions(), 20, 77, chunks=(3, 17), genetics=genetics)
    assert_same(o, g, st, 20)
    assert st[:, 1].sum() > 0 and st[:, 2].sum() > 0


@pytest.mark.parametrize("K,N", [(1000.0, 120_000), (300.0, 90_000)], ids=["dense", "dense_to_sparse"])
def test_big_cells(gpu_lib, K, N):
    """Cells of more than 512 agents run the big-cell kernels (1024 threads
    per tile); the step after the largest cell drops to 512 or fewer, the
    normal ones again."""
    grid = uniform_grid(4, K)
    agents = make_agents(grid, N, seed=41, age_max=50.0)
    acts = config1_actions(K=K)
    o, g, st = run_both(grid, agents, acts, 30, 9, chunks=(1, 29))
    assert_same(o, g, st, 30)
    assert o.counts().max() > 0


def test_ids_past_32_bits(gpu_lib):
    """Agent IDs around 2^32 (and newborn IDs above it): pairing ranks IDs by
    their full 64 bits, and draws are keyed by the full ID."""
    grid, agents, acts = case_config2(n=12, N=30000, seed=17)
    agents.id = agents.id + np.int64(2**32 - 15000)
    o, g, st = run_both(grid, agents, acts, 12, 3)
    assert_same(o, g, st, 12)
    assert st[:, 1].sum() > 0


@pytest.mark.parametrize("K,N", [(200.0, 18000), (400.0, 25000)], ids=["cell_form", "tile_form"])
def test_dense_cells_multi_warp_lists(gpu_lib, K, N):
    """Cells of a few hundred agents: FERTILE lists longer than a warp, more
    than 32 picks per cell (warp-per-cell form up to 256 agents per cell,
    tile form above)."""
    grid = uniform_grid(3, K)
    agents = make_agents(grid, N, seed=8, age_max=50.0)
    o, g, st = run_both(grid, agents, config1_actions(K=K), 20, 21)
    assert_same(o, g, st, 20)
    assert 64 < o.counts().max() <= 512
