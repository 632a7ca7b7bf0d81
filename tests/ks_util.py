"""Statistical comparison with the unmodified reference (two-sample KS tests).

The unmodified reference (WELL512 generators, slot-ordered pairing, the
reference's own slot recycling and ID generators; built from its sources by
oracle/ref/Makefile as oracle/_ref/qhg_ref_well) and this library draw from
different random streams, so their runs can only agree in distribution. For
each case, 64 seeds are run on each side and, per seed, a few summary values
are taken from the population-size trajectory and from the per-cell
occupancy at fixed steps. Each summary is compared across the two samples of
64 with a two-sample Kolmogorov-Smirnov test at alpha = 0.01.

Summaries (SUMMARY_NAMES): live agents after steps 50, 100 and 200; fraction
of empty cells and coefficient of variation of the per-cell counts after
steps 100 and 200.
"""
from __future__ import annotations

import numpy as np

from qhg4_gb300.spec import config1_actions, config2_actions
from qhg4_gb300.workload import make_agents, terrain_grid, uniform_grid

KS_ALPHA = 0.01
N_SEEDS = 64
LIVE_AT = (50, 100, 200)
OCC_AT = (100, 200)
SUMMARY_NAMES = ([f"live@{t}" for t in LIVE_AT] + [f"empty_frac@{t}" for t in OCC_AT] +
                 [f"occupancy_cv@{t}" for t in OCC_AT])

# name: (grid maker, agents, age max, K-proportional placement, actions, steps)
CASES = {
    # the plain method's action set with rates at which the population persists
    "plain_stationary": (lambda: uniform_grid(32, 30.0), 100_000, 50.0, False,
                         lambda: config1_actions(b0=0.5, d0=0.02), 200),
    # the plain method exactly as configured (b0 0.2, d0 0.05): the population
    # shrinks to a few dozen agents by step 200 and dies out soon after, so
    # its summaries cover the decline (running on to step 1,000 adds nothing)
    "plain_configured": (lambda: uniform_grid(32, 30.0), 100_000, 50.0, False, config1_actions, 200),
    # the large run's action set (VerhulstVarK, OldAgeDeath, WeightedMove) on a
    # smaller altitude grid
    "large_actions": (lambda: terrain_grid(32, seed=5), 100_000, 60.0, True, config2_actions, 200),
    # a small case for the CPU test of the Philox-keyed oracle
    "small": (lambda: uniform_grid(12, 30.0), 12_000, 50.0, False,
              lambda: config1_actions(b0=0.5, d0=0.02), 200),
}


def case_inputs(name: str, seed: int):
    make_grid, n, age_max, prop, acts, steps = CASES[name]
    grid = make_grid()
    agents = make_agents(grid, n, seed=seed, age_max=age_max, proportional_to_K=prop)
    return grid, agents, acts(), steps


def summaries(live: np.ndarray, counts_at: dict) -> np.ndarray:
    """live[t-1] = agents after step t; counts_at[t] = per-cell counts after step t."""
    out = [float(live[t - 1]) for t in LIVE_AT]
    for t in OCC_AT:
        c = counts_at[t].astype(np.float64)
        out.append(float((c == 0).mean()))
    for t in OCC_AT:
        c = counts_at[t].astype(np.float64)
        m = c.mean()
        out.append(float(c.std() / m) if m > 0 else 0.0)
    return np.array(out)


def ks_pvalues(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Two-sample KS p-value per summary column (exact distribution)."""
    from scipy.stats import ks_2samp
    return np.array([ks_2samp(a[:, k], b[:, k], method="exact").pvalue for k in range(a.shape[1])])


def run_summaries(runner, name: str, seeds) -> np.ndarray:
    """runner(grid, agents, actions, seed) -> object with step(k) -> stats
    rows and counts(); returns the summaries of every seed."""
    rows = []
    for s in seeds:
        grid, agents, acts, steps = case_inputs(name, s)
        r = runner(grid, agents, acts, s)
        live = []
        counts_at = {}
        done = 0
        for t in sorted(set(OCC_AT) | {steps}):
            st = r.step(t - done)
            live.extend(int(x) for x in np.asarray(st)[:, 0])
            done = t
            if t in OCC_AT:
                counts_at[t] = np.asarray(r.counts()).copy()
        rows.append(summaries(np.array(live), counts_at))
        if hasattr(r, "close"):
            r.close()
    return np.array(rows)
