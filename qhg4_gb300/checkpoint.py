"""Checkpoint and resume of a run (the reference's dumpSpeciesDataQDF and
--resume, core/SPopulation.cpp:2138, app/SimParams.cpp:357).

With draws keyed by (seed, step, agent ID, action) the whole state of a run
is its agent table (+ genomes), its step and its next agent ID: a run resumed
from a checkpoint continues exactly as the uninterrupted one. Checkpoints are
.npz files (HDF5, which QDF files need, is not available here).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

from .gpu import GpuRun
from .spec import Action, Genetics
from .workload import Agents, Grid


def save(run: GpuRun, path: str) -> None:
    a = run.agents(sort_by_id=True)
    cols = dict(id=a.id, cell=a.cell, birth=a.birth, age=a.age, lastb=a.lastb, gender=a.gender, state=a.state,
                step=np.array([run.current_step()], np.int64), next_id=np.array([run.next_id()], np.int64))
    if a.genome is not None:
        cols["genome"] = a.genome
    np.savez(path, **cols)


def resume(grid: Grid, actions: Sequence[Action], seed: int, path: str, genetics: Genetics = Genetics(),
           **kw) -> GpuRun:
    d = np.load(path)
    a = Agents(d["id"], d["cell"], d["birth"], d["age"], d["lastb"], d["gender"], d["state"],
               d["genome"] if "genome" in d else None)
    run = GpuRun(grid, actions, seed, genetics, **kw)
    run.load(a, first_step=int(d["step"][0]))
    run.set_next_id(int(d["next_id"][0]))
    return run
