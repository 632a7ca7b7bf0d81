"""The named workloads: seeded synthetic inputs with the shapes, sizes and
distributions of the configurations the path is measured and checked on.

Each function returns a Workload (grid, initial agents, actions, genetics,
simulation seed, steps).  bench.py times them and the configuration-size
parity tests compare the CUDA path with the oracle on exactly these inputs.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List

from .spec import CROSSOVER_POISSON1, Action, Genetics, config1_actions, config2_actions, config3_actions
from .workload import Agents, Grid, make_agents, terrain_grid, uniform_grid


@dataclass
class Workload:
    name: str
    grid: Grid
    agents: Agents
    actions: List[Action]
    genetics: Genetics = field(default_factory=Genetics)
    seed: int = 42
    steps: int = 0
    cell_bytes: int = 53          # algorithmic bytes per cell-step (53, +56 with WeightedMove)
    desc: str = ""


def plain_method(seed: int = 42, agents: int = 100_000) -> Workload:
    """Plain method: grid n=32 (10,242 cells), K=30 in every cell, 100,000
    agents uniform over the cells, ages U[0,50), GetOld + Fertility (15-45)
    + RandomPair + Verhulst (b0 0.2, d0 0.05, theta 0.01) + RandomMove
    (p 0.1); 1,000 steps, seed 42."""
    g = uniform_grid(32, 30.0)
    a = make_agents(g, agents, seed=seed, age_max=50.0)
    return Workload("plain", g, a, config1_actions(), Genetics(), seed, 1000, 53,
                    "plain method: grid n=32 (10,242 cells), K=30, 100k agents, "
                    "GetOld+Fertility+RandomPair+Verhulst+RandomMove(p=0.1)")


def single_large_run(seed: int = 42, grid_seed: int = 2024, agents: int = 20_000_000, n: int = 256) -> Workload:
    """Single large run: grid n=256 (655,362 cells), altitude from 16 random
    sinusoids, K = 0 below sea level else 100 max(0, 1 - alt/3000); 20M
    agents placed in proportion to K, ages U[0,60); GetOld + Fertility +
    RandomPair + VerhulstVarK + OldAgeDeath (onset U[60,70)) + WeightedMove
    (p 0.2); 200 steps."""
    g = terrain_grid(n, seed=grid_seed)
    a = make_agents(g, agents, seed=seed, age_max=60.0, proportional_to_K=True)
    return Workload("large" if (n, agents) == (256, 20_000_000) else f"large_n{n}_{agents}", g, a,
                    config2_actions(), Genetics(), seed, 200, 53 + 56,
                    f"single large run: grid n={n} ({g.num_cells:,} cells), altitude K, {agents:,} agents, "
                    "GetOld+Fertility+RandomPair+VerhulstVarK+OldAgeDeath+WeightedMove(p=0.2)")


GENETICS = Genetics(4096, CROSSOVER_POISSON1, 1e-4)


def genetics_run(seed: int = 42, agents: int = 5_000_000, n: int = 128) -> Workload:
    """Genetics run: grid n=128 (163,842 cells), K=40 in every cell; 5M
    agents, each with a diploid genome of 2 x 4,096 loci (1 bit per locus in
    uint64 words, bits Bernoulli(0.5)); Poisson(1) crossovers per parent,
    mutation rate 1e-4 per locus; GetOld + Fertility + RandomPair +
    Verhulst + RandomMove (p 0.1); 100 steps."""
    g = uniform_grid(n, 40.0)
    a = make_agents(g, agents, seed=seed, age_max=50.0, genome_blocks=GENETICS.num_blocks)
    return Workload("genetics" if (n, agents) == (128, 5_000_000) else f"genetics_n{n}_{agents}", g, a,
                    config3_actions(), GENETICS, seed, 100, 53,
                    f"genetics run: grid n={n} ({g.num_cells:,} cells), K=40, {agents:,} agents with 2x4096-locus "
                    "genomes, Poisson(1) crossover, mutation 1e-4; GetOld+Fertility+RandomPair+Verhulst+"
                    "RandomMove(p=0.1)")
