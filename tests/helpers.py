"""Shared helpers of the tests: table comparison and standard small cases."""
import numpy as np

from qhg4_gb300.spec import (ACT_FERTILITY, ACT_GETOLD, ACT_OLDAGEDEATH, ACT_RANDOMMOVE, ACT_RANDOMPAIR,
                             ACT_VERHULST, ACT_VERHULSTVARK, ACT_WEIGHTEDMOVE, Action, Genetics,
                             config1_actions, config2_actions, config3_actions)
from qhg4_gb300.workload import Agents, make_agents, terrain_grid, uniform_grid

FIELDS = ("id", "cell", "birth", "age", "lastb", "gender", "state")


def table_diff(a: Agents, b: Agents):
    """None if the two ID-sorted tables are bit-identical, else a message."""
    if len(a) != len(b):
        return f"agent counts differ: {len(a)} vs {len(b)}"
    for k in FIELDS:
        x, y = getattr(a, k), getattr(b, k)
        xv = x.view(np.uint32) if x.dtype == np.float32 else x
        yv = y.view(np.uint32) if y.dtype == np.float32 else y
        bad = np.nonzero(xv != yv)[0]
        if bad.size:
            i = bad[0]
            return f"field {k} differs in {bad.size} rows, first at id {a.id[i]}: {x[i]} vs {y[i]}"
    if (a.genome is None) != (b.genome is None):
        return "genome present in only one table"
    if a.genome is not None and not np.array_equal(a.genome, b.genome):
        rows = np.nonzero((a.genome != b.genome).any(axis=1))[0]
        return f"genomes differ in {rows.size} agents, first id {a.id[rows[0]]}"
    return None


def case_config1(n=8, N=15000, seed=1):
    g = uniform_grid(n, 30.0)
    return g, make_agents(g, N, seed=seed, age_max=50.0), config1_actions()


def case_config2(n=16, N=40000, seed=3, grid_seed=7):
    g = terrain_grid(n, seed=grid_seed)
    return g, make_agents(g, N, seed=seed, age_max=60.0, proportional_to_K=True), config2_actions()


def move_weights(grid, seed, nonmonotone=0.1, equal=0.05):
    """Cumulative WeightedMove weights (C x 7) like a MultiEvaluator leaves
    them: W[c][0] the cell's own weight, W[c][i+1] = W[c][i] + the weight of
    neighbour i.  A fraction of the cells has a negative contribution (the
    cumulated row is not monotone; a combination weight can be negative),
    another fraction all contributions zero (all weights equal); the total
    W[c][n] stays positive elsewhere."""
    rng = np.random.default_rng(seed)
    C = grid.num_cells
    inc = rng.uniform(0.0, 1.0, size=(C, 7))
    inc[rng.random((C, 7)) < 0.15] = 0.0
    neg = rng.random(C) < nonmonotone
    inc[neg, 1 + rng.integers(0, 5, size=int(neg.sum()))] = -rng.uniform(0.1, 0.6, size=int(neg.sum()))
    W = np.cumsum(inc, axis=1)
    eq = rng.random(C) < equal
    W[eq] = W[eq, :1]
    nn = grid.nnbr.astype(np.int64)
    tot = W[np.arange(C), nn]
    low = (~eq) & (tot <= 0.05)
    W[low] += 1.0
    return W


def cell_lonlat(grid):
    """Longitude and latitude (degrees) of the grid's cell centres."""
    x, y, z = grid.xyz[:, 0], grid.xyz[:, 1], grid.xyz[:, 2]
    return np.degrees(np.arctan2(y, x)), np.degrees(np.arcsin(np.clip(z, -1.0, 1.0)))
