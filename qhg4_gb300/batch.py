"""Batched execution: many independent runs in one device table.

``GpuBatch`` binds the qhg_batch_* entry points of libqhg_gpu.so: runs of
one action list (types and order shared, parameters, seeds, grids and
populations per run) are admitted into one batch, stepped together by one
launch of each step kernel over all runs, and removed when done. Every run's
results equal those of the same run alone through ``GpuRun``.

``Autotuner`` picks the batch's launch tuning (CTAs per SM of the action and
scatter kernels, cells per scan thread, the occupancy from which steps run
the warp-per-cell form) per size bucket of the batch, by timing real steps
of the batch with each candidate; because results do not depend on the
launch, tuning costs no simulation work.
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


class BatchLaunch(ct.Structure):
    _fields_ = [("actions_ctas_per_sm", ct.c_int32), ("scatter_ctas_per_sm", ct.c_int32),
                ("scan_cells_per_thread", ct.c_int32), ("dense_cell", ct.c_int32)]


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

    def set_launch(self, actions_ctas: int, scatter_ctas: int, scan_cells_per_thread: int = 0,
                   dense_cell: int = 0) -> None:
        """The launch tuning: CTAs per SM of the action kernel and scatter,
        cells per scan thread (0: by grid size), the mean occupancy from
        which steps run the warp-per-cell form (0: default)."""
        lb = BatchLaunch(int(actions_ctas), int(scatter_ctas), int(scan_cells_per_thread), int(dense_cell))
        _bcheck(load_library().qhg_batch_set_launch(self.h, ct.byref(lb)))

    def launch(self) -> Tuple[int, int, int, int]:
        lb = BatchLaunch()
        _bcheck(load_library().qhg_batch_get_launch(self.h, ct.byref(lb)))
        return (int(lb.actions_ctas_per_sm), int(lb.scatter_ctas_per_sm), int(lb.scan_cells_per_thread),
                int(lb.dense_cell))

    def table_info(self) -> Tuple[int, int]:
        """Agents and non-empty cells of the batch's table."""
        n, ne = ct.c_int64(), ct.c_int64()
        _bcheck(load_library().qhg_batch_table_info(self.h, ct.byref(n), ct.byref(ne)))
        return int(n.value), int(ne.value)

    def set_capacity(self, run: int, K: np.ndarray) -> None:
        """A new K per cell of the run's grid from its next step on (as
        GpuRun.set_capacity for the run alone)."""
        k = np.ascontiguousarray(K, dtype=np.float64)
        if k.shape != (self.grids[run].num_cells,):
            raise ValueError("K needs one entry per cell of the run's grid")
        _bcheck(load_library().qhg_batch_set_capacity(self.h, int(run), _p(k)))

    def set_move_weights(self, run: int, W: np.ndarray) -> None:
        """WeightedMove's cumulative weights (cells x 7) of the run from its
        next step on (as GpuRun.set_move_weights)."""
        w = np.ascontiguousarray(W, dtype=np.float64)
        if w.shape != (self.grids[run].num_cells, 7):
            raise ValueError("weights need shape (cells of the run's grid, 7)")
        _bcheck(load_library().qhg_batch_set_move_weights(self.h, int(run), _p(w)))

    def set_ice(self, run: int, ice) -> None:
        """The run's ice flags per cell (None: no ice) from its next step on
        (as GpuRun.set_ice)."""
        if ice is None:
            _bcheck(load_library().qhg_batch_set_ice(self.h, int(run), None))
            return
        f = np.ascontiguousarray(np.asarray(ice) != 0, dtype=np.uint8)
        if f.shape != (self.grids[run].num_cells,):
            raise ValueError("one flag per cell of the run's grid")
        _bcheck(load_library().qhg_batch_set_ice(self.h, int(run), _p(f)))

    def enable_occupancy(self) -> None:
        """Tracks every run's occupation history (before the first run)."""
        _bcheck(load_library().qhg_batch_enable_occupancy(self.h))

    def occupancy(self, run: int) -> np.ndarray:
        """Per cell of the run's grid, the first of its steps whose table
        holds an agent there (-1 none), as GpuRun.occupancy for the run alone."""
        o = np.zeros(self.grids[run].num_cells, dtype=np.int32)
        _bcheck(load_library().qhg_batch_occupancy(self.h, int(run), _p(o)))
        return o

    def move_stats_enable(self, mode: int, radius: float = 1.0, cartesian: bool = False) -> None:
        """MoveStats for every run (before the first run), in mode
        QHG_MOVESTATS_FIRST / MIN / LAST (qhg4_gb300.gpu's constants)."""
        _bcheck(load_library().qhg_batch_move_stats_enable(self.h, int(mode), float(radius), 1 if cartesian else 0))

    def move_stats_coords(self, run: int, lon: np.ndarray, lat: np.ndarray) -> None:
        """The run's cell coordinates (degrees, or x/y with cartesian)."""
        C = self.grids[run].num_cells
        lo = np.ascontiguousarray(lon, dtype=np.float64)
        la = np.ascontiguousarray(lat, dtype=np.float64)
        if lo.shape != (C,) or la.shape != (C,):
            raise ValueError("one coordinate pair per cell of the run's grid")
        _bcheck(load_library().qhg_batch_move_stats_coords(self.h, int(run), _p(lo), _p(la)))

    def move_stats(self, run: int):
        """Per cell of the run's grid: hops, distance and time of the arrivals
        (as GpuRun.move_stats for the run alone)."""
        C = self.grids[run].num_cells
        h = np.zeros(C, dtype=np.int32)
        d = np.zeros(C, dtype=np.float64)
        t = np.zeros(C, dtype=np.float64)
        _bcheck(load_library().qhg_batch_move_stats(self.h, int(run), _p(h), _p(d), _p(t)))
        return h, d, t

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
    """Launch tuning of a batch per size bucket, chosen by timing real steps.

    The bucket is (log2 of the batch's agents, log2 of its mean agents per
    non-empty cell).  On a bucket's first visit the tuner searches one knob
    at a time, keeping the best value of each before it moves to the next:
    CTAs per SM of the action kernel and the scatter (the top ``span``
    values of each that fit), then cells per thread of the cell scan (1, 2),
    then the mean occupancy from which steps run the warp-per-cell form
    (``dense_choices``; below it, cell-aligned tiles of 512 agents in
    256-thread blocks).  Each candidate is set, stepped twice untimed (the
    step graphs of both table parities captured, the form changed) and
    timed over ``trial_steps`` steps; candidates compare by time per
    agent-step.  Every stage times the incumbent first and again last and
    removes the linear drift between the two (``drift_corrected``).  The
    steps are the batch's own (results do not depend on the launch), so
    tuning costs no simulation work.  A later visit of a known bucket just
    sets its entry."""

    trial_steps: int = 2
    span: int = 3
    dense_choices: Tuple[int, ...] = (12, 24, 48)
    table: Dict[Tuple[int, int], Tuple[int, int, int, int]] = field(default_factory=dict)
    trials: Dict[Tuple[int, int], List[Tuple[Tuple[int, int, int, int], float]]] = field(default_factory=dict)
    current: Optional[Tuple[int, int, int, int]] = None
    # the timed trial steps so far: device ms and agent-steps (they are steps
    # of the batch's runs like any other)
    trial_ms: float = 0.0
    trial_agent_steps: int = 0
    trial_steps_done: int = 0

    @staticmethod
    def bucket(n_agents: int, n_nonempty: int = 1) -> Tuple[int, int]:
        occ = max(1.0, n_agents / max(1, n_nonempty))
        return int(math.log2(max(1, n_agents))), int(math.log2(occ))

    @staticmethod
    def drift_corrected(times: List[float]) -> List[float]:
        """Times of a stage's trials, timed in order between two trials of
        the incumbent (first and last), with the linear drift between those
        two removed: the batch's runs change while it is tuned (populations
        grow or shrink, so the cost per agent-step moves), and without the
        correction a stage would favour whichever candidates came first."""
        n = len(times) - 1
        if n <= 0:
            return list(times)
        drift = times[-1] - times[0]
        return [t - drift * i / n for i, t in enumerate(times)]

    def _time(self, batch: GpuBatch, cand: Tuple[int, int, int, int]) -> float:
        batch.set_launch(*cand)
        self.current = cand
        batch.step(2)   # step graphs of both table parities captured (and the form applied) untimed
        n0, _ = batch.table_info()
        ms = batch.step_timed(self.trial_steps)
        self.trial_ms += ms
        self.trial_agent_steps += n0 * self.trial_steps
        self.trial_steps_done += self.trial_steps
        return ms / (self.trial_steps * max(1, n0))

    def tune(self, batch: GpuBatch) -> Tuple[int, int, int, int]:
        """Sets the batch's launch for its current bucket (searching on the
        bucket's first visit) and returns it."""
        n, ne = batch.table_info()
        b = self.bucket(n, ne)
        if b not in self.table:
            _, _, ma, ms = batch.shape()
            best = (ma, ms, 0, 0)
            results = []

            def consider(cands):
                nonlocal best
                cands = [c for c in cands if c != best]
                seq = [best] + cands + [best]
                times = [self._time(batch, c) for c in seq]
                corrected = self.drift_corrected(times)
                scored = list(zip(seq[:-1], corrected[:-1]))
                results.extend(scored)
                best = min(scored, key=lambda x: x[1])[0]

            consider([(a, s_, 0, 0) for a in range(max(1, ma - self.span + 1), ma + 1)
                      for s_ in range(max(1, ms - self.span + 1), ms + 1)])
            consider([(best[0], best[1], items, best[3]) for items in (1, 2)])
            consider([(best[0], best[1], best[2], d) for d in self.dense_choices])
            self.trials[b] = results
            self.table[b] = best
        if self.current != self.table[b]:   # setting it drops the batch's captured step graphs
            batch.set_launch(*self.table[b])
            self.current = self.table[b]
        return self.table[b]
