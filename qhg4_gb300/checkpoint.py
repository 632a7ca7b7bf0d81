"""Checkpoint and resume of a run (the reference's dumpSpeciesDataQDF and
--resume, core/SPopulation.cpp:2138, app/SimParams.cpp:357).

With draws keyed by (seed, step, agent ID, action) the state of a run is its
agent table (+ genomes), its step and its next agent ID, plus what it was
given or accumulated beside the table: K, move weights and ice set between
steps (qhg_gpu_set_capacity / qhg_gpu_set_move_weights / qhg_gpu_set_ice), the occupation history
(OccTracker) and MoveStats' per-cell arrays (what the reference's
writeAdditionalDataQDF / readAdditionalDataQDF carry, actions/MoveStats.cpp).
A run resumed from a checkpoint continues exactly as the uninterrupted one.
The checkpoint also records the seed and a digest of the action list and
genetics (spec_digest): the draws are keyed by the seed and the actions'
windows, so a resume with a different seed or action set would continue
differently, and resume() refuses it.
Checkpoints are .npz files (HDF5, which QDF files need, is not available
here).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

from .gpu import GpuRun
from .spec import Action, Genetics, spec_digest
from .workload import Agents, Grid


def save(run: GpuRun, path: str) -> None:
    a = run.agents(sort_by_id=True)
    cols = dict(id=a.id, cell=a.cell, birth=a.birth, age=a.age, lastb=a.lastb, gender=a.gender, state=a.state,
                step=np.array([run.current_step()], np.int64), next_id=np.array([run.next_id()], np.int64),
                seed=np.array([run.seed], np.uint64), spec=np.array(run.spec_digest))
    if a.genome is not None:
        cols["genome"] = a.genome
    if run.capacity_K is not None:
        cols["env_K"] = run.capacity_K
    if run.move_weights is not None:
        cols["env_W"] = run.move_weights
    if run.ice is not None:
        cols["env_ice"] = run.ice
    if run.track_occupancy:
        cols["occupancy"] = run.occupancy()
    if run.move_stats_config is not None:
        mode, lon, lat, radius, cart = run.move_stats_config
        h, d, t = run.move_stats()
        cols.update(ms_mode=np.array([mode], np.int64), ms_lon=lon, ms_lat=lat,
                    ms_radius=np.array([radius]), ms_cartesian=np.array([int(cart)], np.int64),
                    ms_hops=h, ms_dist=d, ms_time=t)
    np.savez(path, **cols)


def resume(grid: Grid, actions: Sequence[Action], seed: int, path: str, genetics: Genetics = Genetics(),
           **kw) -> GpuRun:
    d = np.load(path)
    if "seed" in d and int(d["seed"][0]) != int(seed):
        raise ValueError(f"checkpoint {path} was written by a run with seed {int(d['seed'][0])}, not {int(seed)}")
    if "spec" in d and str(d["spec"]) != spec_digest(actions, genetics):
        raise ValueError(f"checkpoint {path} was written by a run with other actions, parameters or genetics")
    a = Agents(d["id"], d["cell"], d["birth"], d["age"], d["lastb"], d["gender"], d["state"],
               d["genome"] if "genome" in d else None)
    if "occupancy" in d:
        kw = dict(kw, track_occupancy=True)
    run = GpuRun(grid, actions, seed, genetics, **kw)
    if "env_ice" in d:
        run.set_ice(d["env_ice"])
    if "env_K" in d:
        run.set_capacity(d["env_K"])
    if "env_W" in d:
        run.set_move_weights(d["env_W"])
    run.load(a, first_step=int(d["step"][0]))
    run.set_next_id(int(d["next_id"][0]))
    if "occupancy" in d:
        run.set_occupancy(d["occupancy"])
    if "ms_mode" in d:
        run.move_stats_enable(int(d["ms_mode"][0]), d["ms_lon"], d["ms_lat"], float(d["ms_radius"][0]),
                              cartesian=bool(d["ms_cartesian"][0]))
        run.set_move_stats(d["ms_hops"], d["ms_dist"], d["ms_time"])
    return run
