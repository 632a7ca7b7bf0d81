"""The Philox-keyed oracle against the unmodified reference, in distribution.

Sample 1: the unmodified reference (WELL512, the reference's pairing and slot
recycling) for seeds 1000..1063, stored by tests/golden/make_ks_reference.py.
Sample 2: the C port oracle for seeds 5000..5063. Each per-seed summary
(tests/ks_util.py) must pass a two-sample KS test at alpha = 0.01. This
checks that keying the draws by (seed, step, agent ID, action) and pairing in
ID order leave the model's behaviour unchanged.
"""
import os

import numpy as np
import pytest

from oracle import port

from ks_util import KS_ALPHA, N_SEEDS, SUMMARY_NAMES, ks_pvalues, run_summaries

pytest.importorskip("scipy")
HERE = os.path.dirname(os.path.abspath(__file__))


class _PortRunner:
    def __init__(self, grid, agents, acts, seed):
        self.r = port.OracleRun(grid, acts, seed, log_births=False)
        self.r.load(agents)

    def step(self, k):
        return self.r.step(k)

    def counts(self):
        return self.r.counts()

    def close(self):
        self.r.close()


@pytest.mark.parametrize("case", ["small", "plain_configured"])
def test_port_matches_unmodified_reference_in_distribution(case):
    ref = np.load(os.path.join(HERE, "golden", f"ks_{case}.npz"))["summaries"]
    ours = run_summaries(_PortRunner, case, range(5000, 5000 + N_SEEDS))
    p = ks_pvalues(ref, ours)
    report = ", ".join(f"{n} p={v:.3f}" for n, v in zip(SUMMARY_NAMES, p))
    print(report)
    assert (p >= KS_ALPHA).all(), report
