#!/usr/bin/env python3
"""Generates the golden fixtures of tests/golden/ from the reference's own
action code.

Each case runs oracle/_ref/qhg_ref_philox -- the reference's GetOld,
Fertility, VerhulstVarK/LinearBirth/LinearDeath, OldAgeDeath, ATanDeath, RandomMove,
WeightedMove/SingleEvaluator, Genetics/BitGeneUtils/BinomialDist and
SPopulation code, compiled from the reference sources by oracle/ref/Makefile,
with Philox draws keyed by (seed, step, agent ID, action) -- on a small seeded
input and stores input and output in <case>.npz:

  inputs   nbr, nnbr, K, agent columns (+ genome), actions, genetics, steps, seed
  outputs  final agents sorted by ID (+ genome), per-step stats (live,
           births, deaths, moves), birth log (baby, mother, father)

Run from the repository root after `make -C oracle/ref`:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.refsim_io import run_reference  # noqa: E402
from qhg4_gb300.spec import (ACT_ATANDEATH, ACT_FERTILITY, ACT_GETOLD, ACT_OLDAGEDEATH, ACT_RANDOMMOVE,  # noqa: E402
                             ACT_RANDOMPAIR, ACT_VERHULSTVARK, ACT_WEIGHTEDMOVE, CROSSOVER_POISSON1,
                             Action, Genetics, config1_actions, config2_actions, config3_actions)
from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid  # noqa: E402


def cases():
    g1 = uniform_grid(6, 30.0)
    yield "plain_small", g1, make_agents(g1, 5000, seed=11, age_max=50.0), config1_actions(), Genetics(), 40, 42
    g2 = terrain_grid(10, seed=5)
    yield ("large_small", g2, make_agents(g2, 15000, seed=12, age_max=60.0, proportional_to_K=True),
           config2_actions(), Genetics(), 30, 7)
    g3 = uniform_grid(3, 40.0)
    gen3 = Genetics(4096, CROSSOVER_POISSON1, 1e-4)
    yield ("genetics_poisson", g3, make_agents(g3, 600, seed=13, age_max=50.0, genome_blocks=gen3.num_blocks),
           config3_actions(), gen3, 12, 9)
    gen4 = Genetics(256, 2, 2e-3)
    yield ("genetics_fixed2", g3, make_agents(g3, 1500, seed=14, age_max=50.0, genome_blocks=gen4.num_blocks),
           config3_actions(), gen4, 15, 21)
    g5 = terrain_grid(8, seed=3)
    acts5 = [Action(ACT_GETOLD, 1), Action(ACT_FERTILITY, 2, (15.0, 45.0, 2.0)), Action(ACT_RANDOMPAIR, 3),
             Action(ACT_OLDAGEDEATH, 4, (64.0, 5.0 / 64.0)), Action(ACT_VERHULSTVARK, 6, (0.25, 0.04, 0.01)),
             Action(ACT_RANDOMMOVE, 7, (0.05,)), Action(ACT_WEIGHTEDMOVE, 8, (0.15,))]
    yield ("mixed_order", g5, make_agents(g5, 8000, seed=15, age_max=70.0, proportional_to_K=True), acts5,
           Genetics(), 25, 123)
    # ATanDeath in place of OldAgeDeath: the arctangent death curve around
    # age 55 (range 12, slope 0.35), ages up to 80
    g7 = terrain_grid(8, seed=8)
    acts7 = [Action(ACT_GETOLD, 1), Action(ACT_FERTILITY, 2, (15.0, 45.0, 2.0)), Action(ACT_RANDOMPAIR, 3),
             Action(ACT_ATANDEATH, 4, (55.0, 12.0, 0.35)), Action(ACT_VERHULSTVARK, 6, (0.25, 0.04, 0.01)),
             Action(ACT_WEIGHTEDMOVE, 8, (0.15,))]
    yield ("atan_death", g7, make_agents(g7, 8000, seed=17, age_max=80.0, proportional_to_K=True), acts7,
           Genetics(), 25, 77)
    # cells of more than 512 agents (the big-cell kernels), thinning out below it
    g6 = uniform_grid(3, 400.0)
    yield ("dense_cells", g6, make_agents(g6, 60000, seed=16, age_max=50.0), config1_actions(K=400.0),
           Genetics(), 12, 31)


def main():
    only = set(sys.argv[1:])
    with tempfile.TemporaryDirectory() as work:
        for name, grid, agents, acts, gen, steps, seed in cases():
            if only and name not in only:
                continue
            out = run_reference("philox", work, grid, agents, acts, steps, seed, gen, threads=4)
            if out.draw_errors != 0:
                raise RuntimeError(f"{name}: {out.draw_errors} draws outside a keyed stream")
            a = out.agents
            arrays = dict(
                nbr=grid.nbr, nnbr=grid.nnbr, K=grid.K,
                in_id=agents.id, in_cell=agents.cell, in_birth=agents.birth, in_age=agents.age,
                in_lastb=agents.lastb, in_gender=agents.gender, in_state=agents.state,
                act_type=np.array([x.type for x in acts], np.int32),
                act_prio=np.array([x.prio for x in acts], np.int32),
                act_param=np.array([x.params4() for x in acts], np.float64),
                genetics=np.array([gen.genome_size, gen.num_crossover], np.int64),
                mutation_rate=np.array([gen.mutation_rate]), steps=np.array([steps]), seed=np.array([seed]),
                out_id=a.id, out_cell=a.cell, out_birth=a.birth, out_age=a.age, out_lastb=a.lastb,
                out_gender=a.gender, out_state=a.state, stats=out.stats, births=out.births)
            if gen.genome_size > 0:
                arrays["in_genome"] = agents.genome
                arrays["out_genome"] = a.genome
            np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrays)
            print(f"{name}: {len(agents)} -> {len(a)} agents after {steps} steps, {len(out.births)} births")


if __name__ == "__main__":
    main()
