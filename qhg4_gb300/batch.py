"""Batched execution: many independent runs in one device table.

``GpuBatch`` binds the qhg_batch_* entry points of libqhg_gpu.so: runs of
one action list (types and order shared, parameters, seeds, grids and
populations per run) are admitted into one batch, stepped together by one
launch of each step kernel over all runs, and removed when done. Every run's
results equal those of the same run alone through ``GpuRun``.

``Autotuner`` picks the launch shape of the persistent kernels (CTAs per SM
of the action and scatter kernels) per size bucket of the batch, by timing
real steps of the batch with each candidate; because results do not depend
on the shape, tuning costs no simulation work.
"""
from __future__ import annotations

import ctypes as ct
import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np

from .gpu import AgentsSoA, QhgError, StepStats, _p, load_library
from .spec import Action, MAX_ACTIONS, execution_order
from .workload import Agents, Grid


class BatchDesc(ct.Structure):
    _fields_ = [
        ("n_actions", ct.c_int32),
        ("action_type", ct.c_int32 * MAX_ACTIONS),
        ("agent_capacity", ct.c_int64),
        ("cell_capacity", ct.c_int64),
        ("stage_capacity", ct.c_int64),
        ("max_runs", ct.c_int32),
        ("device", ct.c_int32),
    ]


class BatchRunDesc(ct.Structure):
    _fields_ = [("seed", ct.c_uint64), ("action_param", (ct.c_double * 4) * MAX_ACTIONS)]


class BatchRunStatus(ct.Structure):
    _fields_ = [("active", ct.c_int32), ("cell0", ct.c_int32), ("num_cells", ct.c_int32),
                ("steps_done", ct.c_int32)]


def _bcheck(rc: int) -> None:
    if rc != 0:
        raise QhgError(rc, load_library().qhg_batch_last_error().decode())


def action_types(actions: Sequence[Action]) -> List[int]:
    return [int(a.type) for a in execution_order(actions)]


class GpuBatch:
    """A batch of runs on one CUDA device."""

    def __init__(self, actions: Sequence[Action], agent_capacity: int, cell_capacity: int, max_runs: int,
                 stage_capacity: Optional[int] = None, device: int = 0):
        lib = load_library()
        self.types = action_types(actions)
        d = BatchDesc()
        d.n_actions = len(self.types)
        for i, t in enumerate(self.types):
            d.action_type[i] = t
        d.agent_capacity = int(agent_capacity)
        d.cell_capacity = int(cell_capacity)
        d.stage_capacity = int(stage_capacity if stage_capacity is not None else agent_capacity)
        d.max_runs = int(max_runs)
        d.device = int(device)
        self._desc = d
        h = ct.c_void_p()
        _bcheck(lib.qhg_batch_create(ct.byref(d), ct.byref(h)))
        self.h = h
        self.grids: Dict[int, Grid] = {}

    def add_run(self, grid: Grid, actions: Sequence[Action], seed: int, agents: Agents) -> int:
        """Admits a run; its agents enter at the next step. Returns its index."""
        ordered = execution_order(actions)
        if [int(a.type) for a in ordered] != self.types:
            raise ValueError("a run of a batch must have the batch's action types in the same order")
        rd = BatchRunDesc()
        rd.seed = int(seed)
        for i, a in enumerate(ordered):
            for k, v in enumerate(a.params4()):
                rd.action_param[i][k] = float(v)
        nbr = np.ascontiguousarray(grid.nbr, dtype=np.int32)
        nnbr = np.ascontiguousarray(grid.nnbr, dtype=np.uint8)
        K = np.ascontiguousarray(grid.K, dtype=np.float64)
        cols = dict(id=np.ascontiguousarray(agents.id, dtype=np.int64),
                    cell=np.ascontiguousarray(agents.cell, dtype=np.int32),
                    birth=np.ascontiguousarray(agents.birth, dtype=np.float32),
                    age=np.ascontiguousarray(agents.age, dtype=np.float32),
                    last_birth=np.ascontiguousarray(agents.lastb, dtype=np.float32),
                    gender=np.ascontiguousarray(agents.gender, dtype=np.uint8),
                    state=np.ascontiguousarray(agents.state, dtype=np.uint8))
        soa = AgentsSoA(**{k: v.ctypes.data for k, v in cols.items()})
        r = ct.c_int32()
        _bcheck(load_library().qhg_batch_add_run(self.h, ct.byref(rd), _p(nbr), _p(nnbr), _p(K), grid.num_cells,
                                                  ct.byref(soa), len(agents), ct.byref(r)))
        self.grids[int(r.value)] = grid
        return int(r.value)

    def remove_run(self, run: int) -> None:
        _bcheck(load_library().qhg_batch_remove_run(self.h, int(run)))

    def step(self, n: int = 1) -> None:
        _bcheck(load_library().qhg_batch_step(self.h, int(n)))

    def step_timed(self, n: int) -> float:
        ms = ct.c_float()
        _bcheck(load_library().qhg_batch_step_timed(self.h, int(n), ct.byref(ms)))
        return float(ms.value)

    def sync(self) -> None:
        _bcheck(load_library().qhg_batch_sync(self.h))

    def num_agents(self) -> int:
        n = ct.c_int64()
        _bcheck(load_library().qhg_batch_num_agents(self.h, ct.byref(n)))
        return int(n.value)

    def live_history(self, nsteps: int) -> np.ndarray:
        """Agents of all runs after each of the batch's last nsteps (<= 1024) steps."""
        out = np.zeros(max(1, nsteps), dtype=np.uint64)
        _bcheck(load_library().qhg_batch_live_history(self.h, int(nsteps), _p(out)))
        return out[:nsteps]

    def run_info(self, run: int) -> BatchRunStatus:
        st = BatchRunStatus()
        _bcheck(load_library().qhg_batch_run_info(self.h, int(run), ct.byref(st)))
        return st

    def steps_done(self, run: int) -> int:
        return int(self.run_info(run).steps_done)

    def stats(self, run: int, nsteps: int) -> np.ndarray:
        """Statistics of the run's last nsteps (<= 64) steps: live, births, deaths, moves."""
        buf = (StepStats * max(1, nsteps))()
        _bcheck(load_library().qhg_batch_stats(self.h, int(run), int(nsteps), ct.byref(buf)))
        return np.array([[s.live, s.births, s.deaths, s.moves] for s in buf[:nsteps]], dtype=np.uint64)

    def agents(self, run: int, sort_by_id: bool = True) -> Agents:
        cap = 1 << 16
        while True:
            out = Agents(np.zeros(cap, np.int64), np.zeros(cap, np.int32), np.zeros(cap, np.float32),
                         np.zeros(cap, np.float32), np.zeros(cap, np.float32), np.zeros(cap, np.uint8),
                         np.zeros(cap, np.uint8))
            soa = AgentsSoA(out.id.ctypes.data, out.cell.ctypes.data, out.birth.ctypes.data, out.age.ctypes.data,
                            out.lastb.ctypes.data, out.gender.ctypes.data, out.state.ctypes.data, None)
            got = ct.c_int64()
            rc = load_library().qhg_batch_download(self.h, int(run), ct.byref(soa), cap, ct.byref(got))
            n = int(got.value)
            if rc != 0 and n > cap:
                cap = n
                continue
            _bcheck(rc)
            break
        out = Agents(out.id[:n].copy(), out.cell[:n].copy(), out.birth[:n].copy(), out.age[:n].copy(),
                     out.lastb[:n].copy(), out.gender[:n].copy(), out.state[:n].copy())
        return out.sorted_by_id() if sort_by_id else out

    def counts(self, run: int) -> np.ndarray:
        c = np.zeros(self.grids[run].num_cells, dtype=np.uint32)
        _bcheck(load_library().qhg_batch_counts(self.h, int(run), _p(c)))
        return c

    def set_shape(self, actions_ctas: int, scatter_ctas: int) -> None:
        _bcheck(load_library().qhg_batch_set_shape(self.h, int(actions_ctas), int(scatter_ctas)))

    def shape(self) -> Tuple[int, int, int, int]:
        a, s, ma, ms = ct.c_int32(), ct.c_int32(), ct.c_int32(), ct.c_int32()
        _bcheck(load_library().qhg_batch_get_shape(self.h, ct.byref(a), ct.byref(s), ct.byref(ma), ct.byref(ms)))
        return int(a.value), int(s.value), int(ma.value), int(ms.value)

    def close(self) -> None:
        if getattr(self, "h", None):
            load_library().qhg_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass
class Autotuner:
    """Launch shape per size bucket (log2 of the batch's agents), chosen by
    timing ``trial_steps`` real steps of the batch with every candidate."""

    trial_steps: int = 2
    span: int = 3          # candidates: the top `span` CTAs-per-SM values of each kernel
    table: Dict[int, Tuple[int, int]] = field(default_factory=dict)
    trials: Dict[int, List[Tuple[Tuple[int, int], float]]] = field(default_factory=dict)

    @staticmethod
    def bucket(n_agents: int) -> int:
        return int(math.log2(max(1, n_agents)))

    def candidates(self, batch: GpuBatch) -> List[Tuple[int, int]]:
        _, _, ma, ms = batch.shape()
        return [(a, s) for a in range(max(1, ma - self.span + 1), ma + 1)
                for s in range(max(1, ms - self.span + 1), ms + 1)]

    def tune(self, batch: GpuBatch) -> Tuple[int, int]:
        """Sets the batch's shape for its current size, measuring once per
        bucket; steps the batch len(candidates) * trial_steps times on a
        bucket's first visit."""
        b = self.bucket(batch.num_agents())
        if b not in self.table:
            results = []
            for cand in self.candidates(batch):
                batch.set_shape(*cand)
                batch.step(1)   # graph capture outside the timed steps
                results.append((cand, batch.step_timed(self.trial_steps) / self.trial_steps))
            self.trials[b] = results
            self.table[b] = min(results, key=lambda x: x[1])[0]
        batch.set_shape(*self.table[b])
        return self.table[b]
