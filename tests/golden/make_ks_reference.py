#!/usr/bin/env python3
"""Generates tests/golden/ks_<case>.npz: per-seed summaries of the unmodified
reference, the first sample of the two-sample KS tests (tests/ks_util.py).

Each case is run with oracle/_ref/qhg_ref_well -- the reference's own
SPopulation, action and pairing code with its WELL512 generators, compiled
from the reference sources by oracle/ref/Makefile -- for seeds 1000..1063
(the seed picks both the initial population and the 16-word WELL state), with
per-cell counts dumped every 50 steps.

Run from the repository root after `make -C oracle/ref`:
    python tests/golden/make_ks_reference.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle.refsim_io import run_reference  # noqa: E402
from ks_util import CASES, N_SEEDS, OCC_AT, case_inputs, summaries  # noqa: E402

REF_SEED0 = 1000


def main():
    names = sys.argv[1:] or list(CASES)
    with tempfile.TemporaryDirectory() as work:
        for name in names:
            rows = []
            for s in range(REF_SEED0, REF_SEED0 + N_SEEDS):
                grid, agents, acts, steps = case_inputs(name, s)
                out = run_reference("well", work, grid, agents, acts, steps, s, dump_every=50, threads=8)
                counts_at = {t: out.counts[list(out.dump_steps).index(t - 1)] for t in OCC_AT}
                rows.append(summaries(out.stats[:, 0], counts_at))
            rows = np.array(rows)
            np.savez_compressed(os.path.join(HERE, f"ks_{name}.npz"), summaries=rows,
                                seeds=np.arange(REF_SEED0, REF_SEED0 + N_SEEDS))
            print(name, rows.mean(axis=0).round(4).tolist())


if __name__ == "__main__":
    main()
