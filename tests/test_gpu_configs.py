"""Bit-exact parity at the sizes of the configurations themselves.

The CUDA path (through the C ABI) against the oracle on exactly the inputs
bench.py times (qhg4_gb300/configs.py): ID-sorted agent tables (every field,
floats as bits, genome words), per-cell counts, per-step statistics and the
(baby, mother, father) birth log.  At these sizes the warp-per-cell kernels
run with ~76 agents per cell, the cell scan with its wide tiles (grids above
4M cells are not in these configurations; 655,362 cells give 2,560 look-back
tiles) and the genome kernel with thousands of newborns per step.  The
oracle uses every host core.
"""
import numpy as np
import pytest

from oracle import port
from qhg4_gb300.configs import genetics_run, plain_method, single_large_run
from qhg4_gb300.gpu import GpuRun

from helpers import table_diff

pytestmark = pytest.mark.gpu


def _compare(o, g, ost, steps, log=True):
    d = table_diff(o.agents(), g.agents())
    assert d is None, d
    assert np.array_equal(o.counts(), g.counts())
    assert np.array_equal(ost[-min(steps, 1024):], g.stats(min(steps, 1024)))
    if log:
        ob, gb = o.birth_log(), g.birth_log()
        assert np.array_equal(ob, gb), f"birth logs differ ({len(ob)} vs {len(gb)})"


def _run(w, chunks, capacity=0):
    port.set_threads(port.max_threads())
    o = port.OracleRun(w.grid, w.actions, w.seed, w.genetics)
    o.load(w.agents)
    g = GpuRun(w.grid, w.actions, w.seed, w.genetics, log_births=True, capacity=capacity)
    g.load(w.agents)
    ost = []
    for k in chunks:
        ost.append(o.step(k))
        g.step(k)
    return o, g, np.concatenate(ost, axis=0)


def test_plain_method_as_configured(gpu_lib):
    """n=32, K=30, 100,000 agents, seed 42, all 1,000 steps."""
    w = plain_method()
    o, g, ost = _run(w, (w.steps,))
    assert ost.shape == (1000, 4)
    _compare(o, g, ost, w.steps)
    g.close()
    o.close()


def test_single_large_run_full_size(gpu_lib):
    """n=256, 20M agents, the bench's seed and rates; five steps launched one
    at a time (each relaunches the step graph), then three more together."""
    w = single_large_run()
    o, g, ost = _run(w, (1, 1, 1, 1, 1, 3), capacity=int(len(w.agents) * 2.5) + 65536)
    assert int(ost[-1, 0]) > 15_000_000
    _compare(o, g, ost, 8)
    g.close()
    o.close()


def test_genetics_run_full_size(gpu_lib):
    """n=128, K=40, 5M agents with 2 x 4,096-locus genomes, Poisson(1)
    crossover, mutation 1e-4 per locus: genome words compared bit for bit."""
    w = genetics_run()
    o, g, ost = _run(w, (1, 1, 1), capacity=int(len(w.agents) * 1.6) + 65536)
    assert int(ost[:, 1].sum()) > 10_000   # newborns with genomes were made
    _compare(o, g, ost, 3)
    g.close()
    o.close()
