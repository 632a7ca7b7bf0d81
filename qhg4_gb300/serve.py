"""Served execution: simulation jobs arriving over time, run by continuous
batching on one GPU.

A job is one simulation (grid, initial agents, the plain method's action set
with its own parameters and seed, a step count). ``Server`` keeps one
``GpuBatch`` on the device and loops:

* arrived jobs wait in a FIFO queue;
* the head of the queue is admitted when its HBM footprint (reserved agent
  rows x bytes per row + cells x bytes per cell) fits under the budget next
  to the jobs already running, and the batch has a free run slot, cell range
  and table rows; admitted jobs join the running ones at the next step;
* the batch steps all running jobs together, in chunks that end where a job
  finishes or is due a snapshot;
* a finished job's final agent table is downloaded and the job leaves the
  batch, freeing its footprint for the queue;
* every ``snapshot_every`` steps of a job, its table is copied to page-locked
  host memory while the batch keeps stepping, and a writer thread stores it
  (``write_snapshot``).

The reference writes QDF (HDF5) files; the HDF5 library is absent on both
machines this runs on, so snapshots are raw files with the reference's agent
fields (``SNAPSHOT_FIELDS``). Job latency = completion time - arrival time.
Every job's result is the same as the job run alone (tests/test_gpu_serve.py).
"""
from __future__ import annotations

import collections
import ctypes as ct
import math
import os
import queue
import struct
import threading
import time
from dataclasses import dataclass, field
from typing import Callable, Deque, Dict, List, Optional, Sequence

import numpy as np

from .batch import GpuBatch, _bcheck
from .ensemble import grid_n
from .gpu import AgentsSoA, QhgError, load_library
from .spec import Action, config1_actions
from .workload import Agents, Grid, make_agents

QHG_ERR_CAPACITY = -7

#: device bytes per reserved agent row of a batch: two tables of id 8,
#: birth/age/last birth 12, meta 1; outcome 1, father 4, birth rank 2; staging 22
BYTES_PER_AGENT = 2 * 21 + 1 + 4 + 2 + 22
#: device bytes per cell of a batch: neighbours 24 + count 1 + reverse slots 4
#: + K 8 + Verhulst thresholds 16 + move thresholds 48 + flag 1 + run 4 +
#: class counts 32 + bases 12 + mover bases 24 + non-empty lists 2 x 8 +
#: admission 12 + scan status
BYTES_PER_CELL = 24 + 1 + 4 + 8 + 16 + 48 + 1 + 4 + 32 + 12 + 24 + 16 + 12 + 2

#: fields of a snapshot file, as the reference's agent data set names them
#: (core/SPopulation.h:43-50 and the populations' agent structs)
SNAPSHOT_FIELDS = [("m_ulID", "<i8"), ("m_ulCellID", "<i4"), ("m_fBirthTime", "<f4"), ("m_fAge", "<f4"),
                   ("m_fLastBirth", "<f4"), ("m_iGender", "u1"), ("m_iLifeState", "u1")]


def reserved_rows(cells: int, agents: int) -> int:
    """Table rows a job reserves: twice its start or 40 agents per cell
    (Verhulst keeps the plain method's populations below K = 30 per cell)."""
    return max(2 * agents, 40 * cells)


def footprint(cells: int, agents: int) -> int:
    return reserved_rows(cells, agents) * BYTES_PER_AGENT + cells * BYTES_PER_CELL


@dataclass
class Job:
    jid: int
    arrival: float
    grid: Grid
    agents: Agents
    actions: List[Action]
    seed: int
    steps: int
    # set by the server
    run: int = -1
    admit_step: int = -1          # batch steps launched when it was admitted
    admitted: Optional[float] = None
    finished: Optional[float] = None
    result: Optional[Agents] = None
    live: List[int] = field(default_factory=list)   # agents after each of its steps
    agent_steps: int = 0
    snapshots: List[str] = field(default_factory=list)

    @property
    def latency(self) -> Optional[float]:
        return None if self.finished is None else self.finished - self.arrival

    @property
    def rows(self) -> int:
        return reserved_rows(self.grid.num_cells, len(self.agents))

    @property
    def bytes(self) -> int:
        return footprint(self.grid.num_cells, len(self.agents))


def job_stream(n_jobs: int, rate: float = 20.0, seed: int = 7, grid_ns: Sequence[int] = (32, 64, 128, 256),
               n_min: float = 1e4, n_max: float = 1e7, steps_min: int = 50, steps_max: int = 1000) -> List[Job]:
    """Poisson arrivals at `rate` jobs/s; grid n uniform in grid_ns, initial
    agents log-uniform in [n_min, n_max], steps uniform in [steps_min,
    steps_max]; the plain method's action set with b0 ~ U[0.1, 0.3],
    d0 ~ U[0.02, 0.08], RandomMove p ~ U[0.05, 0.3]; job j has seed j."""
    rng = np.random.default_rng(seed)
    t = 0.0
    jobs = []
    for j in range(n_jobs):
        t += float(rng.exponential(1.0 / rate))
        n = int(rng.choice(grid_ns))
        N = int(math.exp(rng.uniform(math.log(n_min), math.log(n_max))))
        steps = int(rng.integers(steps_min, steps_max + 1))
        acts = config1_actions(b0=float(rng.uniform(0.1, 0.3)), d0=float(rng.uniform(0.02, 0.08)),
                               move_p=float(rng.uniform(0.05, 0.3)))
        g = grid_n(n)
        a = make_agents(g, N, seed=seed * 100000 + j, age_max=50.0)
        jobs.append(Job(j, t, g, a, acts, j, steps))
    return jobs


def write_snapshot(path: str, job: int, step: int, cols: Dict[str, np.ndarray]) -> None:
    """Raw snapshot: b"QHGSNAP1", u32 job, i32 step, u64 n, then the columns
    of SNAPSHOT_FIELDS in that order."""
    n = len(cols["m_ulID"])
    with open(path, "wb") as f:
        f.write(b"QHGSNAP1")
        f.write(struct.pack("<IiQ", job, step, n))
        for name, dt in SNAPSHOT_FIELDS:
            f.write(np.ascontiguousarray(cols[name], dtype=dt).tobytes())


def read_snapshot(path: str):
    with open(path, "rb") as f:
        b = f.read()
    if b[:8] != b"QHGSNAP1":
        raise ValueError("not a snapshot file")
    job, step, n = struct.unpack_from("<IiQ", b, 8)
    pos = 8 + 16
    cols = {}
    for name, dt in SNAPSHOT_FIELDS:
        d = np.dtype(dt)
        cols[name] = np.frombuffer(b, dtype=d, count=n, offset=pos).copy()
        pos += d.itemsize * n
    return job, step, cols


class _PinnedBuffer:
    """Page-locked host columns for one snapshot copy."""

    def __init__(self, n: int):
        lib = load_library()
        self.n = n
        self.ptrs = {}
        self.arrays = {}
        for name, dt in (("id", np.int64), ("cell", np.uint32), ("birth", np.float32), ("age", np.float32),
                         ("last_birth", np.float32), ("state", np.uint8)):
            p = ct.c_void_p()
            nbytes = max(1, n) * np.dtype(dt).itemsize
            _bcheck(lib.qhg_host_buffer_alloc(nbytes, ct.byref(p)))
            self.ptrs[name] = p
            buf = (ct.c_char * nbytes).from_address(p.value)
            self.arrays[name] = np.frombuffer(buf, dtype=dt, count=max(1, n))

    def soa(self) -> AgentsSoA:
        P = self.ptrs
        return AgentsSoA(P["id"].value, P["cell"].value, P["birth"].value, P["age"].value, P["last_birth"].value,
                         None, P["state"].value, None)

    def free(self) -> None:
        lib = load_library()
        for p in self.ptrs.values():
            lib.qhg_host_buffer_free(p)
        self.ptrs = {}
        self.arrays = {}


class Server:
    """Continuous batching of simulation jobs on one GPU."""

    def __init__(self, hbm_budget: float = 150e9, agent_capacity: Optional[int] = None,
                 cell_capacity: Optional[int] = None, max_runs: int = 256, snapshot_every: int = 100,
                 snapshot_dir: Optional[str] = None, chunk: int = 16, device: int = 0,
                 clock: str = "real", virtual_step_s: float = 1e-3):
        self.budget = float(hbm_budget)
        rows = agent_capacity if agent_capacity is not None else min(2**31 - 1, int(self.budget * 0.9 / BYTES_PER_AGENT))
        cells = cell_capacity if cell_capacity is not None else int(self.budget * 0.1 / BYTES_PER_CELL)
        self.batch = GpuBatch(config1_actions(), agent_capacity=rows, cell_capacity=cells, max_runs=max_runs,
                              stage_capacity=min(rows, 1 << 28), device=device)
        self.rows_cap, self.cells_cap, self.max_runs = rows, cells, max_runs
        self.snapshot_every = int(snapshot_every)
        self.snapshot_dir = snapshot_dir
        self.chunk = int(chunk)
        self.clock = clock
        self.virtual_step_s = float(virtual_step_s)
        self.gstep = 0                 # batch steps launched
        self.vtime = 0.0
        self.used_bytes = 0
        self.used_rows = 0
        self.used_cells = 0
        self.running: Dict[int, Job] = {}
        self.done: List[Job] = []
        self._t0 = None
        self._writes: "queue.Queue" = queue.Queue()
        self._writer = threading.Thread(target=self._write_loop, daemon=True)
        self._writer.start()
        self._pending_snap = []       # (job, step, buffer, n, cell0) copies in flight
        self.busy_s = 0.0

    # ------------------------------------------------------------ time
    def now(self) -> float:
        if self.clock == "virtual":
            return self.vtime
        return time.perf_counter() - self._t0

    def _wait_until(self, t: float) -> None:
        if self.clock == "virtual":
            self.vtime = max(self.vtime, t)
        else:
            dt = t - self.now()
            if dt > 0:
                time.sleep(dt)

    # ------------------------------------------------------- snapshots
    def _write_loop(self) -> None:
        while True:
            item = self._writes.get()
            if item is None:
                return
            path, jid, step, cols = item
            write_snapshot(path, jid, step, cols)

    def _flush_snapshots(self) -> None:
        """Hands finished snapshot copies to the writer thread."""
        if not self._pending_snap:
            return
        self.batch_snapshot_wait()
        for job, step, buf, n, cell0 in self._pending_snap:
            A = buf.arrays
            meta = A["state"][:n]
            cols = {"m_ulID": A["id"][:n].copy(), "m_ulCellID": (A["cell"][:n].astype(np.int64) - cell0).astype(np.int32),
                    "m_fBirthTime": A["birth"][:n].copy(), "m_fAge": A["age"][:n].copy(),
                    "m_fLastBirth": A["last_birth"][:n].copy(), "m_iGender": (meta & 1).astype(np.uint8),
                    "m_iLifeState": np.where(meta & 2, 5, 1).astype(np.uint8)}
            buf.free()
            if self.snapshot_dir:
                path = os.path.join(self.snapshot_dir, f"job{job.jid:05d}_step{step:05d}.qhgsnap")
                job.snapshots.append(path)
                self._writes.put((path, job.jid, step, cols))
        self._pending_snap = []

    def batch_snapshot_wait(self) -> None:
        _bcheck(load_library().qhg_batch_snapshot_wait(self.batch.h))

    def _snapshot(self, job: Job) -> None:
        info = self.batch.run_info(job.run)
        n = job.live[-1] if job.live else len(job.agents)
        buf = _PinnedBuffer(n)
        soa = buf.soa()
        got, step = ct.c_int64(), ct.c_int32()
        _bcheck(load_library().qhg_batch_snapshot_async(self.batch.h, job.run, ct.byref(soa), n, ct.byref(got),
                                                         ct.byref(step)))
        self._pending_snap.append((job, int(step.value), buf, int(got.value), int(info.cell0)))

    # ------------------------------------------------------------ jobs
    def _fits(self, job: Job) -> bool:
        return (len(self.running) < self.max_runs and self.used_bytes + job.bytes <= self.budget and
                self.used_rows + job.rows <= self.rows_cap and
                self.used_cells + job.grid.num_cells <= self.cells_cap)

    def _admit(self, job: Job) -> None:
        job.run = self.batch.add_run(job.grid, job.actions, job.seed, job.agents)
        job.admit_step = self.gstep
        job.admitted = self.now()
        self.used_bytes += job.bytes
        self.used_rows += job.rows
        self.used_cells += job.grid.num_cells
        self.running[job.run] = job

    def _steps_done(self, job: Job) -> int:
        return max(0, self.gstep - (job.admit_step + 1))

    def _to_next_event(self, job: Job) -> int:
        """Batch steps until the job finishes or is due a snapshot."""
        done = self._steps_done(job)
        entering = 1 if self.gstep <= job.admit_step else 0
        left = job.steps - done
        if self.snapshot_every > 0:
            nxt = (done // self.snapshot_every + 1) * self.snapshot_every
            left = min(left, nxt - done)
        return left + entering

    def _after_chunk(self, k: int) -> None:
        finished = []
        for run, job in self.running.items():
            done = self._steps_done(job)
            new = min(k, done - len(job.live))
            if new > 0:
                st = self.batch.stats(run, new)
                prev = job.live[-1] if job.live else len(job.agents)
                lives = [int(x) for x in st[:, 0]]
                job.agent_steps += prev + sum(lives[:-1])
                job.live.extend(lives)
            if done >= job.steps:
                finished.append(job)
            elif self.snapshot_every > 0 and new > 0 and done % self.snapshot_every == 0:
                self._snapshot(job)
        for job in finished:
            job.result = self.batch.agents(job.run, sort_by_id=False)
            self.batch.remove_run(job.run)
            job.finished = self.now()
            del self.running[job.run]
            self.used_bytes -= job.bytes
            self.used_rows -= job.rows
            self.used_cells -= job.grid.num_cells
            self.done.append(job)

    def serve(self, jobs: Sequence[Job], on_done: Optional[Callable[[Job], None]] = None) -> List[Job]:
        """Runs the job stream to completion; returns the jobs in completion order."""
        pending: Deque[Job] = collections.deque(sorted(jobs, key=lambda j: j.arrival))
        waiting: Deque[Job] = collections.deque()
        self._t0 = time.perf_counter()
        for j in pending:
            if j.bytes > self.budget or j.rows > self.rows_cap or j.grid.num_cells > self.cells_cap:
                raise ValueError(f"job {j.jid} can never fit the budget or the batch")
        while pending or waiting or self.running:
            t = self.now()
            while pending and pending[0].arrival <= t:
                waiting.append(pending.popleft())
            while waiting and self._fits(waiting[0]):
                try:
                    self._admit(waiting[0])
                except QhgError as e:
                    # no run slot or no contiguous cell range free yet: a leaving
                    # job frees them at the next step
                    if e.code != QHG_ERR_CAPACITY or not self.running:
                        raise
                    break
                waiting.popleft()
            if not self.running:
                if pending:
                    self._wait_until(pending[0].arrival)
                continue
            k = min([self.chunk] + [self._to_next_event(j) for j in self.running.values()])
            k = max(1, k)
            t1 = time.perf_counter()
            self.batch.step(k)
            self.batch.sync()
            self._flush_snapshots()
            self.busy_s += time.perf_counter() - t1
            self.gstep += k
            if self.clock == "virtual":
                self.vtime += k * self.virtual_step_s
            n_done = len(self.done)
            self._after_chunk(k)
            if on_done:
                for j in self.done[n_done:]:
                    on_done(j)
        self._flush_snapshots()
        self._writes.put(None)
        self._writer.join()
        return self.done

    def close(self) -> None:
        self.batch.close()


def summarize(jobs: Sequence[Job], wall_s: float) -> dict:
    lat = np.array([j.latency for j in jobs if j.latency is not None])
    total = sum(j.agent_steps for j in jobs)
    return {"jobs": len(jobs), "agent_steps": int(total), "wall_s": wall_s,
            "value": total / wall_s if wall_s > 0 else 0.0, "unit": "agent-steps/s",
            "latency_p50_s": float(np.percentile(lat, 50)) if lat.size else None,
            "latency_p99_s": float(np.percentile(lat, 99)) if lat.size else None,
            "latency_max_s": float(lat.max()) if lat.size else None}
