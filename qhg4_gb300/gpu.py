"""ctypes binding of libqhg_gpu.so (include/qhg_gpu.h).

``GpuRun`` holds one simulation on the GPU.  There is no CPU fallback: if
the library cannot be loaded or no CUDA device is present, every call
raises.
"""
from __future__ import annotations

import ctypes as ct
import os
from typing import Sequence

import numpy as np

from .spec import Action, Genetics, MAX_ACTIONS, execution_order, spec_digest
from .workload import Agents, Grid

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqhg_gpu.so")

QHG_FLAG_LOG_BIRTHS = 1
QHG_FLAG_TRACK_OCCUPANCY = 2
QHG_MOVESTATS_FIRST, QHG_MOVESTATS_MIN, QHG_MOVESTATS_LAST = 0, 1, 2   # MoveStats modes

ERRORS = {
    -1: "QHG_ERR_ARG", -2: "QHG_ERR_CUDA", -3: "QHG_ERR_NOMEM", -4: "QHG_ERR_STATE",
    -5: "QHG_ERR_CELL_TOO_LARGE", -6: "QHG_ERR_TIMEOUT", -7: "QHG_ERR_CAPACITY", -8: "QHG_ERR_DEVICE",
}

#: every symbol include/qhg_gpu.h declares
EXPORTS = [
    "qhg_gpu_last_error", "qhg_gpu_version", "qhg_gpu_create", "qhg_gpu_upload_grid",
    "qhg_gpu_upload_agents", "qhg_gpu_step", "qhg_gpu_sync", "qhg_gpu_num_agents",
    "qhg_gpu_current_step", "qhg_gpu_download", "qhg_gpu_counts", "qhg_gpu_stats",
    "qhg_gpu_birth_log", "qhg_gpu_stream", "qhg_gpu_destroy", "qhg_gpu_step_profiled",
    "qhg_gpu_step_timed", "qhg_gpu_cell_census_noalloc", "qhg_gpu_census_last_error",
    "qhg_batch_last_error", "qhg_batch_create", "qhg_batch_add_run", "qhg_batch_remove_run",
    "qhg_batch_step", "qhg_batch_step_timed", "qhg_batch_sync", "qhg_batch_num_agents",
    "qhg_batch_run_info", "qhg_batch_stats", "qhg_batch_download", "qhg_batch_counts",
    "qhg_batch_set_shape", "qhg_batch_get_shape", "qhg_batch_stream", "qhg_batch_destroy",
    "qhg_batch_live_history", "qhg_batch_snapshot_async", "qhg_batch_snapshot_wait",
    "qhg_host_buffer_alloc", "qhg_host_buffer_free", "qhg_gpu_next_id", "qhg_gpu_set_next_id",
    "qhg_gpu_test_stall_scan", "qhg_gpu_occupancy", "qhg_gpu_set_capacity", "qhg_gpu_set_move_weights", "qhg_gpu_set_ice", "qhg_gpu_stats_async", "qhg_batch_set_launch", "qhg_batch_get_launch",
    "qhg_batch_table_info", "qhg_batch_set_capacity", "qhg_batch_set_move_weights", "qhg_batch_set_ice",
    "qhg_batch_enable_occupancy", "qhg_batch_occupancy", "qhg_batch_move_stats_enable",
    "qhg_batch_move_stats_coords", "qhg_batch_move_stats",
    "qhg_gpu_move_stats_enable", "qhg_gpu_move_stats", "qhg_gpu_set_move_stats", "qhg_gpu_set_occupancy",
]


class QhgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class RunDesc(ct.Structure):
    _fields_ = [
        ("seed", ct.c_uint64),
        ("n_actions", ct.c_int32),
        ("action_type", ct.c_int32 * MAX_ACTIONS),
        ("action_param", (ct.c_double * 4) * MAX_ACTIONS),
        ("genome_size", ct.c_int32),
        ("num_crossover", ct.c_int32),
        ("mutation_rate", ct.c_double),
        ("agent_capacity", ct.c_int64),
        ("flags", ct.c_uint32),
        ("device", ct.c_int32),
    ]


class AgentsSoA(ct.Structure):
    _fields_ = [("id", ct.c_void_p), ("cell", ct.c_void_p), ("birth", ct.c_void_p), ("age", ct.c_void_p),
                ("last_birth", ct.c_void_p), ("gender", ct.c_void_p), ("state", ct.c_void_p),
                ("genome", ct.c_void_p)]


class StepStats(ct.Structure):
    _fields_ = [("live", ct.c_uint64), ("births", ct.c_uint64), ("deaths", ct.c_uint64), ("moves", ct.c_uint64)]


_lib = None


def load_library(path: str = LIB_PATH):
    """Loads libqhg_gpu.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from .build import build
        build()
    lib = ct.CDLL(path)
    P = ct.c_void_p
    I = ct.c_int
    sig = {
        "qhg_gpu_last_error": (ct.c_char_p, []),
        "qhg_gpu_version": (ct.c_char_p, []),
        "qhg_gpu_create": (I, [P, P]),
        "qhg_gpu_upload_grid": (I, [P, P, P, P, ct.c_int32]),
        "qhg_gpu_upload_agents": (I, [P, P, ct.c_int64, ct.c_int32]),
        "qhg_gpu_step": (I, [P, ct.c_int32]),
        "qhg_gpu_sync": (I, [P]),
        "qhg_gpu_num_agents": (I, [P, P]),
        "qhg_gpu_current_step": (I, [P, P]),
        "qhg_gpu_download": (I, [P, P, ct.c_int64, P]),
        "qhg_gpu_counts": (I, [P, P]),
        "qhg_gpu_stats": (I, [P, ct.c_int32, P]),
        "qhg_gpu_birth_log": (I, [P, P, P, P, ct.c_int64, P]),
        "qhg_gpu_stream": (I, [P, P]),
        "qhg_gpu_destroy": (I, [P]),
        "qhg_gpu_step_profiled": (I, [P, ct.c_int32, P]),
        "qhg_gpu_step_timed": (I, [P, ct.c_int32, P]),
        "qhg_gpu_cell_census_noalloc": (I, [P, ct.c_int64, ct.c_int32, P, P, P]),
        "qhg_gpu_census_last_error": (ct.c_char_p, []),
        "qhg_batch_last_error": (ct.c_char_p, []),
        "qhg_batch_create": (I, [P, P]),
        "qhg_batch_add_run": (I, [P, P, P, P, P, ct.c_int32, P, ct.c_int64, P]),
        "qhg_batch_remove_run": (I, [P, ct.c_int32]),
        "qhg_batch_step": (I, [P, ct.c_int32]),
        "qhg_batch_step_timed": (I, [P, ct.c_int32, P]),
        "qhg_batch_sync": (I, [P]),
        "qhg_batch_num_agents": (I, [P, P]),
        "qhg_batch_run_info": (I, [P, ct.c_int32, P]),
        "qhg_batch_stats": (I, [P, ct.c_int32, ct.c_int32, P]),
        "qhg_batch_download": (I, [P, ct.c_int32, P, ct.c_int64, P]),
        "qhg_batch_counts": (I, [P, ct.c_int32, P]),
        "qhg_batch_set_shape": (I, [P, ct.c_int32, ct.c_int32]),
        "qhg_batch_get_shape": (I, [P, P, P, P, P]),
        "qhg_batch_stream": (I, [P, P]),
        "qhg_batch_destroy": (I, [P]),
        "qhg_batch_live_history": (I, [P, ct.c_int32, P]),
        "qhg_batch_snapshot_async": (I, [P, ct.c_int32, P, ct.c_int64, P, P]),
        "qhg_batch_snapshot_wait": (I, [P]),
        "qhg_host_buffer_alloc": (I, [ct.c_int64, P]),
        "qhg_host_buffer_free": (I, [P]),
        "qhg_gpu_next_id": (I, [P, P]),
        "qhg_gpu_set_next_id": (I, [P, ct.c_int64]),
        "qhg_gpu_test_stall_scan": (I, [P, ct.c_int32]),
        "qhg_gpu_occupancy": (I, [P, P]),
        "qhg_gpu_set_capacity": (I, [P, P]),
        "qhg_gpu_set_move_weights": (I, [P, P]),
        "qhg_gpu_set_ice": (I, [P, P]),
        "qhg_gpu_stats_async": (I, [P, P]),
        "qhg_batch_set_launch": (I, [P, P]),
        "qhg_batch_get_launch": (I, [P, P]),
        "qhg_batch_table_info": (I, [P, P, P]),
        "qhg_batch_set_capacity": (I, [P, ct.c_int32, P]),
        "qhg_batch_set_move_weights": (I, [P, ct.c_int32, P]),
        "qhg_batch_set_ice": (I, [P, ct.c_int32, P]),
        "qhg_batch_enable_occupancy": (I, [P]),
        "qhg_batch_occupancy": (I, [P, ct.c_int32, P]),
        "qhg_batch_move_stats_enable": (I, [P, ct.c_int32, ct.c_double, ct.c_int32]),
        "qhg_batch_move_stats_coords": (I, [P, ct.c_int32, P, P]),
        "qhg_batch_move_stats": (I, [P, ct.c_int32, P, P, P]),
        "qhg_gpu_move_stats_enable": (I, [P, ct.c_int32, P, P, ct.c_double, ct.c_int32]),
        "qhg_gpu_move_stats": (I, [P, P, P, P]),
        "qhg_gpu_set_move_stats": (I, [P, P, P, P]),
        "qhg_gpu_set_occupancy": (I, [P, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _check(rc: int) -> None:
    if rc != 0:
        raise QhgError(rc, _lib.qhg_gpu_last_error().decode())


def _p(a: np.ndarray):
    return a.ctypes.data_as(ct.c_void_p)


def make_desc(actions: Sequence[Action], seed: int, genetics: Genetics = Genetics(), capacity: int = 0,
              flags: int = 0, device: int = 0) -> RunDesc:
    ordered = execution_order(actions)
    if len(ordered) > MAX_ACTIONS:
        raise ValueError("too many actions")
    d = RunDesc()
    d.seed = int(seed)
    d.n_actions = len(ordered)
    for i, a in enumerate(ordered):
        d.action_type[i] = int(a.type)
        for k, v in enumerate(a.params4()):
            d.action_param[i][k] = float(v)
    d.genome_size = int(genetics.genome_size)
    d.num_crossover = int(genetics.num_crossover)
    d.mutation_rate = float(genetics.mutation_rate)
    d.agent_capacity = int(capacity)
    d.flags = int(flags)
    d.device = int(device)
    return d


class HostBuffer:
    """Page-locked host memory (qhg_host_buffer_alloc) seen as a numpy array:
    copies between it and the device run at the interconnect's speed, and
    qhg_gpu_stats_async can write into it without a wait."""

    def __init__(self, shape, dtype):
        lib = load_library()
        dt = np.dtype(dtype)
        count = int(np.prod(shape))
        nbytes = max(1, count * dt.itemsize)
        p = ct.c_void_p()
        if lib.qhg_host_buffer_alloc(nbytes, ct.byref(p)) != 0:
            raise QhgError(-3, lib.qhg_batch_last_error().decode())
        self.ptr = p.value
        raw = (ct.c_uint8 * nbytes).from_address(self.ptr)
        self.array = np.frombuffer(raw, dtype=np.uint8, count=count * dt.itemsize).view(dt).reshape(shape)

    def free(self) -> None:
        if self.ptr:
            self.array = None
            _lib.qhg_host_buffer_free(ct.c_void_p(self.ptr))
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def pinned_agents(n: int, genome_words: int = 0):
    """An agent table of n rows in page-locked host memory, and the buffers
    that hold it (keep them alive while the table is used)."""
    bufs = [HostBuffer((n,), np.int64), HostBuffer((n,), np.int32), HostBuffer((n,), np.float32),
            HostBuffer((n,), np.float32), HostBuffer((n,), np.float32), HostBuffer((n,), np.uint8),
            HostBuffer((n,), np.uint8)]
    a = Agents(*(b.array for b in bufs))
    if genome_words > 0:
        g = HostBuffer((n, genome_words), np.uint64)
        bufs.append(g)
        a.genome = g.array
    return a, bufs


class GpuRun:
    """One simulation held by libqhg_gpu.so on a CUDA device."""

    def __init__(self, grid: Grid, actions: Sequence[Action], seed: int, genetics: Genetics = Genetics(),
                 log_births: bool = False, capacity: int = 0, device: int = 0, track_occupancy: bool = False):
        lib = load_library()
        flags = (QHG_FLAG_LOG_BIRTHS if log_births else 0) | (QHG_FLAG_TRACK_OCCUPANCY if track_occupancy else 0)
        self._desc = make_desc(actions, seed, genetics, capacity, flags, device)
        h = ct.c_void_p()
        _check(lib.qhg_gpu_create(ct.byref(self._desc), ct.byref(h)))
        self.h = h
        self.C = grid.num_cells
        self.genetics = genetics
        self.seed = int(seed)
        self.spec_digest = spec_digest(actions, genetics)
        self.grid = grid
        self.track_occupancy = track_occupancy
        # what the run was given beyond its grid (for checkpoints): K and
        # move weights set between steps, the MoveStats configuration
        self.capacity_K = None
        self.move_weights = None
        self.ice = None
        self.move_stats_config = None
        nbr = np.ascontiguousarray(grid.nbr, dtype=np.int32)
        nnbr = np.ascontiguousarray(grid.nnbr, dtype=np.uint8)
        K = np.ascontiguousarray(grid.K, dtype=np.float64)
        _check(lib.qhg_gpu_upload_grid(self.h, _p(nbr), _p(nnbr), _p(K), self.C))

    def load(self, a: Agents, first_step: int = 0) -> None:
        cols = dict(id=np.ascontiguousarray(a.id, dtype=np.int64), cell=np.ascontiguousarray(a.cell, dtype=np.int32),
                    birth=np.ascontiguousarray(a.birth, dtype=np.float32),
                    age=np.ascontiguousarray(a.age, dtype=np.float32),
                    last_birth=np.ascontiguousarray(a.lastb, dtype=np.float32),
                    gender=np.ascontiguousarray(a.gender, dtype=np.uint8),
                    state=np.ascontiguousarray(a.state, dtype=np.uint8))
        soa = AgentsSoA(**{k: v.ctypes.data for k, v in cols.items()})
        if self.genetics.genome_size > 0:
            g = np.ascontiguousarray(a.genome, dtype=np.uint64)
            cols["genome"] = g
            soa.genome = g.ctypes.data
        _check(_lib.qhg_gpu_upload_agents(self.h, ct.byref(soa), len(a), int(first_step)))

    def step(self, n: int = 1) -> None:
        _check(_lib.qhg_gpu_step(self.h, int(n)))

    def sync(self) -> None:
        _check(_lib.qhg_gpu_sync(self.h))

    def num_agents(self) -> int:
        n = ct.c_int64()
        _check(_lib.qhg_gpu_num_agents(self.h, ct.byref(n)))
        return int(n.value)

    def current_step(self) -> int:
        s = ct.c_int32()
        _check(_lib.qhg_gpu_current_step(self.h, ct.byref(s)))
        return int(s.value)

    def agents(self, sort_by_id: bool = True, out: Agents = None) -> Agents:
        """The current table (rows by cell, or by ID).  `out`: arrays to fill
        (e.g. pinned_agents), at least as long as the table; the result is
        then their first rows."""
        n = self.num_agents()
        if out is not None:
            if len(out) < n:
                raise ValueError("output table too small")
            out = Agents(out.id[:n], out.cell[:n], out.birth[:n], out.age[:n], out.lastb[:n], out.gender[:n],
                         out.state[:n], None if out.genome is None else out.genome[:n])
        else:
            out = Agents(np.zeros(n, np.int64), np.zeros(n, np.int32), np.zeros(n, np.float32),
                         np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.uint8),
                         np.zeros(n, np.uint8))
        soa = AgentsSoA(out.id.ctypes.data, out.cell.ctypes.data, out.birth.ctypes.data, out.age.ctypes.data,
                        out.lastb.ctypes.data, out.gender.ctypes.data, out.state.ctypes.data, None)
        if self.genetics.genome_size > 0:
            if out.genome is None:
                out.genome = np.zeros((n, 2 * self.genetics.num_blocks), dtype=np.uint64)
            soa.genome = out.genome.ctypes.data
        got = ct.c_int64()
        _check(_lib.qhg_gpu_download(self.h, ct.byref(soa), n, ct.byref(got)))
        return out.sorted_by_id() if sort_by_id else out

    def counts(self) -> np.ndarray:
        c = np.zeros(self.C, dtype=np.uint32)
        _check(_lib.qhg_gpu_counts(self.h, _p(c)))
        return c

    def set_capacity(self, K: np.ndarray) -> None:
        """A new K per cell from the next step on (VerhulstVarK; the move
        weights follow unless weights were given)."""
        k = np.ascontiguousarray(K, dtype=np.float64)
        if k.shape != (self.C,):
            raise ValueError("K needs one entry per cell")
        _check(_lib.qhg_gpu_set_capacity(self.h, _p(k)))
        self.capacity_K = k.copy()

    def set_move_weights(self, W: np.ndarray) -> None:
        """WeightedMove's cumulative weights (C x 7) from the next step on."""
        w = np.ascontiguousarray(W, dtype=np.float64)
        if w.shape != (self.C, 7):
            raise ValueError("weights need shape (cells, 7)")
        _check(_lib.qhg_gpu_set_move_weights(self.h, _p(w)))
        self.move_weights = w.copy()

    def set_ice(self, ice) -> None:
        """The Geography's ice flags per cell (None: no ice) from the next step
        on: WeightedMove registers no move into an ice cell, and weights that
        follow K give ice cells weight 0."""
        if ice is None:
            _check(_lib.qhg_gpu_set_ice(self.h, None))
            self.ice = None
            return
        f = np.ascontiguousarray(np.asarray(ice) != 0, dtype=np.uint8)
        if f.shape != (self.C,):
            raise ValueError("one flag per cell")
        _check(_lib.qhg_gpu_set_ice(self.h, _p(f)))
        self.ice = f.copy()

    def move_stats_enable(self, mode: int, lon: np.ndarray, lat: np.ndarray, radius: float = 1.0,
                          cartesian: bool = False) -> None:
        """MoveStats (QHG_MOVESTATS_FIRST / MIN / LAST = 0 / 1 / 2) over the
        cells' coordinates (lon/lat in degrees, or x/y when cartesian)."""
        lo = np.ascontiguousarray(lon, dtype=np.float64)
        la = np.ascontiguousarray(lat, dtype=np.float64)
        if lo.shape != (self.C,) or la.shape != (self.C,):
            raise ValueError("coordinates need one entry per cell")
        _check(_lib.qhg_gpu_move_stats_enable(self.h, int(mode), _p(lo), _p(la), float(radius),
                                              1 if cartesian else 0))
        self.move_stats_config = (int(mode), lo.copy(), la.copy(), float(radius), bool(cartesian))

    def set_move_stats(self, hops: np.ndarray, dist: np.ndarray, time: np.ndarray) -> None:
        """Restores MoveStats' per-cell arrays (after enabling it)."""
        h = np.ascontiguousarray(hops, dtype=np.int32)
        d = np.ascontiguousarray(dist, dtype=np.float64)
        t = np.ascontiguousarray(time, dtype=np.float64)
        if h.shape != (self.C,) or d.shape != (self.C,) or t.shape != (self.C,):
            raise ValueError("one entry per cell")
        _check(_lib.qhg_gpu_set_move_stats(self.h, _p(h), _p(d), _p(t)))

    def move_stats(self):
        """Per cell: hops (int32), distance and time (float64) of MoveStats."""
        h = np.zeros(self.C, np.int32)
        d = np.zeros(self.C, np.float64)
        t = np.zeros(self.C, np.float64)
        _check(_lib.qhg_gpu_move_stats(self.h, _p(h), _p(d), _p(t)))
        return h, d, t

    def set_occupancy(self, first_step: np.ndarray) -> None:
        """Restores the occupation history (needs track_occupancy=True)."""
        o = np.ascontiguousarray(first_step, dtype=np.int32)
        if o.shape != (self.C,):
            raise ValueError("one entry per cell")
        _check(_lib.qhg_gpu_set_occupancy(self.h, _p(o)))

    def occupancy(self) -> np.ndarray:
        """Per cell, the first step whose table holds an agent there (-1 none);
        needs track_occupancy=True."""
        o = np.zeros(self.C, dtype=np.int32)
        _check(_lib.qhg_gpu_occupancy(self.h, _p(o)))
        return o

    def stats(self, nsteps: int) -> np.ndarray:
        buf = (StepStats * max(1, nsteps))()
        _check(_lib.qhg_gpu_stats(self.h, int(nsteps), ct.byref(buf)))
        return np.array([[s.live, s.births, s.deaths, s.moves] for s in buf[:nsteps]], dtype=np.uint64)

    def stats_async(self, out: np.ndarray) -> None:
        """Queues a copy of the last launched step's statistics (live,
        births, deaths, moves) into `out` (4 uint64, page-locked memory such
        as a HostBuffer row) without waiting; valid after sync()."""
        assert out.dtype == np.uint64 and out.size == 4 and out.flags["C_CONTIGUOUS"]
        _check(_lib.qhg_gpu_stats_async(self.h, ct.c_void_p(out.ctypes.data)))

    def birth_log(self) -> np.ndarray:
        n = ct.c_int64()
        rc = _lib.qhg_gpu_birth_log(self.h, None, None, None, 0, ct.byref(n))
        total = int(n.value)
        b, m, f = np.zeros(total, np.int64), np.zeros(total, np.int64), np.zeros(total, np.int64)
        if total > 0 or rc != 0:
            _check(_lib.qhg_gpu_birth_log(self.h, _p(b), _p(m), _p(f), total, ct.byref(n)))
        o = np.argsort(b, kind="stable")
        return np.stack([b[o], m[o], f[o]], axis=1)

    def step_profiled(self, n: int) -> np.ndarray:
        """Runs n steps with per-kernel CUDA events; returns ms[n, 4]
        (actions, cell scan, scatter, genomes)."""
        t = np.zeros((max(1, n), 4), dtype=np.float32)
        _check(_lib.qhg_gpu_step_profiled(self.h, int(n), _p(t)))
        return t[:n]

    def step_timed(self, n: int) -> float:
        """Runs n steps between CUDA events on the run's stream; returns ms."""
        ms = ct.c_float()
        _check(_lib.qhg_gpu_step_timed(self.h, int(n), ct.byref(ms)))
        return float(ms.value)

    def next_id(self) -> int:
        v = ct.c_int64()
        _check(_lib.qhg_gpu_next_id(self.h, ct.byref(v)))
        return int(v.value)

    def set_next_id(self, next_id: int) -> None:
        _check(_lib.qhg_gpu_set_next_id(self.h, int(next_id)))

    def test_stall_scan(self, tile: int = 0) -> None:
        """Makes the next step fail through a bounded wait (tests of failure detection)."""
        _check(_lib.qhg_gpu_test_stall_scan(self.h, int(tile)))

    def stream_handle(self) -> int:
        s = ct.c_void_p()
        _check(_lib.qhg_gpu_stream(self.h, ct.byref(s)))
        return int(s.value or 0)

    def close(self) -> None:
        if getattr(self, "h", None):
            _lib.qhg_gpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
