"""Ensembles of independent runs: the batched configuration and the served
stream's job mix, as seeded synthetic inputs.

Batched ensemble: 256 runs; grid subdivision n uniform in {32, 64, 128}
(K = 30 in every cell); initial agents log-uniform in [1e4, 2e6], placed
uniformly; ages U[0, 50); the plain method's action set (GetOld, Fertility,
RandomPair, Verhulst, RandomMove) with Verhulst b0 ~ U[0.1, 0.3],
d0 ~ U[0.02, 0.08], theta = 0.01, K = 30 and RandomMove p ~ U[0.05, 0.3];
run r has Philox seed r; 500 steps each.
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Dict, List, Sequence

import numpy as np

from .spec import Action, config1_actions
from .workload import Agents, Grid, make_agents, uniform_grid

_GRIDS: Dict[int, Grid] = {}


def grid_n(n: int) -> Grid:
    """The uniform-K icosahedral grid of subdivision n (cached)."""
    if n not in _GRIDS:
        _GRIDS[n] = uniform_grid(n, 30.0)
    return _GRIDS[n]


@dataclass
class RunSpec:
    index: int
    grid: Grid
    agents: Agents
    actions: List[Action]
    seed: int
    steps: int


def ensemble_specs(n_runs: int = 256, steps: int = 500, seed: int = 2024, grid_ns: Sequence[int] = (32, 64, 128),
                   n_min: float = 1e4, n_max: float = 2e6) -> List[RunSpec]:
    rng = np.random.default_rng(seed)
    out = []
    for r in range(n_runs):
        n = int(rng.choice(grid_ns))
        N = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
        b0 = float(rng.uniform(0.1, 0.3))
        d0 = float(rng.uniform(0.02, 0.08))
        p = float(rng.uniform(0.05, 0.3))
        g = grid_n(n)
        a = make_agents(g, N, seed=seed * 1000 + r, age_max=50.0)
        out.append(RunSpec(r, g, a, config1_actions(b0=b0, d0=d0, move_p=p), r, steps))
    return out
