"""Served execution (continuous batching): jobs that arrive over time, are
admitted under an HBM budget and run together in one batch must each give
the same result as the job run alone -- final agent table, population
trajectory and the snapshots written on the way (bit for bit)."""
import os

import numpy as np
import pytest

from qhg4_gb300.gpu import GpuRun
from qhg4_gb300.serve import Job, Server, footprint, read_snapshot
from qhg4_gb300.spec import config1_actions
from qhg4_gb300.workload import make_agents, uniform_grid

from helpers import table_diff

pytestmark = pytest.mark.gpu


def small_jobs(n=8, seed=5):
    rng = np.random.default_rng(seed)
    grids = {k: uniform_grid(k, 30.0) for k in (6, 8, 10)}
    jobs, t = [], 0.0
    for j in range(n):
        t += float(rng.exponential(0.01))
        g = grids[int(rng.choice([6, 8, 10]))]
        a = make_agents(g, int(rng.integers(2000, 9000)), seed=900 + j, age_max=50.0)
        acts = config1_actions(b0=float(rng.uniform(0.3, 0.6)), d0=float(rng.uniform(0.02, 0.05)),
                               move_p=float(rng.uniform(0.05, 0.3)))
        jobs.append(Job(j, t, g, a, acts, 70 + j, int(rng.integers(20, 80))))
    return jobs


def test_served_jobs_equal_alone(gpu_lib, tmp_path):
    jobs = small_jobs()
    # a budget for about three jobs at a time, so that later jobs queue
    budget = 3.2 * max(j.bytes for j in jobs)
    srv = Server(hbm_budget=budget, agent_capacity=400_000, cell_capacity=4_000, max_runs=4, snapshot_every=25,
                 snapshot_dir=str(tmp_path), chunk=8, clock="virtual", virtual_step_s=0.002)
    done = srv.serve(jobs)
    srv.close()
    assert len(done) == len(jobs)
    assert max(j.admitted - j.arrival for j in done) > 0.0   # some job waited for room
    for j in done:
        r = GpuRun(j.grid, j.actions, j.seed)
        r.load(j.agents)
        snaps = {read_snapshot(p)[1]: p for p in j.snapshots}
        assert sorted(snaps) == [s for s in range(25, j.steps, 25)]
        live = []
        for s in range(1, j.steps + 1):
            r.step(1)
            live.append(int(r.stats(1)[0, 0]))
            if s in snaps:
                _, step, cols = read_snapshot(snaps[s])
                ref = r.agents()
                o = np.argsort(cols["m_ulID"], kind="stable")
                assert np.array_equal(cols["m_ulID"][o], ref.id)
                assert np.array_equal(cols["m_ulCellID"][o], ref.cell)
                assert np.array_equal(cols["m_fBirthTime"][o].view(np.uint32), ref.birth.view(np.uint32))
                assert np.array_equal(cols["m_fAge"][o].view(np.uint32), ref.age.view(np.uint32))
                assert np.array_equal(cols["m_fLastBirth"][o].view(np.uint32), ref.lastb.view(np.uint32))
                assert np.array_equal(cols["m_iGender"][o], ref.gender)
                assert np.array_equal(cols["m_iLifeState"][o], ref.state)
        d = table_diff(j.result.sorted_by_id(), r.agents())
        assert d is None, f"job {j.jid}: {d}"
        assert j.live == live
        r.close()
