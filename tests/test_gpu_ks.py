"""The CUDA path against the unmodified reference, in distribution.

Sample 1: the unmodified reference (WELL512 generators, slot-ordered pairing,
its own slot recycling) for seeds 1000..1063, stored by
tests/golden/make_ks_reference.py. Sample 2: this library through the C ABI
for seeds 5000..5063. Population-size and per-cell-occupancy summaries
(tests/ks_util.py) must each pass a two-sample KS test at alpha = 0.01.
"""
import os

import numpy as np
import pytest

from qhg4_gb300.gpu import GpuRun

from ks_util import KS_ALPHA, N_SEEDS, SUMMARY_NAMES, ks_pvalues, run_summaries

pytestmark = pytest.mark.gpu
pytest.importorskip("scipy")
HERE = os.path.dirname(os.path.abspath(__file__))


class _GpuRunner:
    def __init__(self, grid, agents, acts, seed):
        self.r = GpuRun(grid, acts, seed)
        self.r.load(agents)

    def step(self, k):
        self.r.step(k)
        return self.r.stats(k)

    def counts(self):
        return self.r.counts()

    def close(self):
        self.r.close()


@pytest.mark.parametrize("case", ["plain_stationary", "plain_configured", "large_actions"])
def test_gpu_matches_unmodified_reference_in_distribution(gpu_lib, case):
    ref = np.load(os.path.join(HERE, "golden", f"ks_{case}.npz"))["summaries"]
    ours = run_summaries(_GpuRunner, case, range(5000, 5000 + N_SEEDS))
    p = ks_pvalues(ref, ours)
    report = ", ".join(f"{n} p={v:.3f}" for n, v in zip(SUMMARY_NAMES, p))
    print(case, report)
    assert (p >= KS_ALPHA).all(), report
