"""ctypes front end of the C port oracle (oracle/qhg_oracle.c).

ORACLE / TEST INFRASTRUCTURE ONLY: imported by tests/, by
``__graft_entry__.smoke()`` as the checker and by bench.py's CPU legs.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

from qhg4_gb300.spec import Action, Genetics, execution_order
from qhg4_gb300.workload import Agents, Grid

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libqhg_oracle.so")
_lib = None


def build() -> str:
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        build()
    lib = ct.CDLL(LIB_PATH)
    P = ct.c_void_p
    lib.qo_create.restype = P
    lib.qo_create.argtypes = [ct.c_uint64, ct.c_int, P, P, ct.c_int, ct.c_int, ct.c_double,
                              ct.c_int, P, P, P]
    lib.qo_load.restype = ct.c_int
    lib.qo_load.argtypes = [P, ct.c_int64, P, P, P, P, P, P, P, P, ct.c_int32]
    lib.qo_step.restype = ct.c_int
    lib.qo_step.argtypes = [P, ct.c_int, P]
    lib.qo_num_agents.restype = ct.c_int64
    lib.qo_num_agents.argtypes = [P]
    lib.qo_next_id.restype = ct.c_int64
    lib.qo_next_id.argtypes = [P]
    lib.qo_set_next_id.argtypes = [P, ct.c_int64]
    lib.qo_current_step.restype = ct.c_int32
    lib.qo_current_step.argtypes = [P]
    lib.qo_get_agents.restype = ct.c_int
    lib.qo_get_agents.argtypes = [P] * 9
    lib.qo_get_counts.restype = ct.c_int
    lib.qo_get_counts.argtypes = [P, P]
    lib.qo_num_logged_births.restype = ct.c_int64
    lib.qo_num_logged_births.argtypes = [P]
    lib.qo_get_birth_log.restype = ct.c_int
    lib.qo_get_birth_log.argtypes = [P, P, P, P]
    lib.qo_binomial_table.restype = ct.c_int
    lib.qo_binomial_table.argtypes = [P, P, ct.c_int]
    lib.qo_set_log_births.argtypes = [P, ct.c_int]
    lib.qo_set_capacity.restype = ct.c_int
    lib.qo_set_capacity.argtypes = [P, P]
    lib.qo_set_move_weights.restype = ct.c_int
    lib.qo_set_move_weights.argtypes = [P, P]
    lib.qo_move_stats_enable.restype = ct.c_int
    lib.qo_move_stats_enable.argtypes = [P, ct.c_int, P, P, ct.c_double, ct.c_int]
    lib.qo_move_stats.restype = ct.c_int
    lib.qo_move_stats.argtypes = [P, P, P, P]
    lib.qo_set_ice.restype = ct.c_int
    lib.qo_set_ice.argtypes = [P, P]
    lib.qo_set_threads.argtypes = [ct.c_int]
    lib.qo_max_threads.restype = ct.c_int
    lib.qo_destroy.argtypes = [P]
    _lib = lib
    return lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(ct.c_void_p)


def set_threads(n: int) -> None:
    _load().qo_set_threads(int(n))


def max_threads() -> int:
    return int(_load().qo_max_threads())


class OracleRun:
    """One simulation held by the port oracle."""

    def __init__(self, grid: Grid, actions: Sequence[Action], seed: int,
                 genetics: Genetics = Genetics(), log_births: bool = True):
        lib = _load()
        ordered = execution_order(actions)
        types = np.array([a.type for a in ordered], dtype=np.int32)
        params = np.array([a.params4() for a in ordered], dtype=np.float64).reshape(-1)
        if params.size == 0:
            params = np.zeros(4, dtype=np.float64)
        self._keep = (np.ascontiguousarray(grid.nbr, dtype=np.int32),
                      np.ascontiguousarray(grid.nnbr, dtype=np.uint8),
                      np.ascontiguousarray(grid.K, dtype=np.float64), types, params)
        self.h = lib.qo_create(ct.c_uint64(seed), len(ordered), _p(types), _p(params),
                               genetics.genome_size, genetics.num_crossover,
                               ct.c_double(genetics.mutation_rate), grid.num_cells,
                               _p(self._keep[0]), _p(self._keep[1]), _p(self._keep[2]))
        if not self.h:
            raise ValueError("oracle rejected the configuration")
        self.C = grid.num_cells
        self.genetics = genetics
        lib.qo_set_log_births(self.h, 1 if log_births else 0)
        self.stats = []

    def load(self, a: Agents, first_step: int = 0) -> None:
        cols = [np.ascontiguousarray(a.id, dtype=np.int64), np.ascontiguousarray(a.cell, dtype=np.int32),
                np.ascontiguousarray(a.birth, dtype=np.float32), np.ascontiguousarray(a.age, dtype=np.float32),
                np.ascontiguousarray(a.lastb, dtype=np.float32), np.ascontiguousarray(a.gender, dtype=np.uint8),
                np.ascontiguousarray(a.state, dtype=np.uint8)]
        g = None
        if self.genetics.genome_size > 0:
            g = np.ascontiguousarray(a.genome, dtype=np.uint64)
        rc = _load().qo_load(self.h, len(a), *[_p(c) for c in cols], _p(g) if g is not None else None,
                             int(first_step))
        if rc != 0:
            raise ValueError(f"oracle load failed ({rc})")

    def step(self, n: int = 1) -> np.ndarray:
        st = np.zeros(max(n, 1) * 4, dtype=np.uint64)
        _load().qo_step(self.h, int(n), _p(st))
        st = st[:n * 4].reshape(n, 4)
        self.stats.append(st)
        return st

    def set_capacity(self, K: np.ndarray) -> None:
        """VerhulstVarK's K per cell from the next step on (and the move
        weights, unless weights were given)."""
        k = np.ascontiguousarray(K, dtype=np.float64)
        assert k.shape == (self.C,)
        _load().qo_set_capacity(self.h, _p(k))

    def set_move_weights(self, W: np.ndarray) -> None:
        """WeightedMove's cumulative weights (C x 7) from the next step on."""
        w = np.ascontiguousarray(W, dtype=np.float64)
        assert w.shape == (self.C, 7)
        _load().qo_set_move_weights(self.h, _p(w))

    def set_ice(self, ice) -> None:
        """Geography::m_abIce per cell from the next step on (None: no ice);
        WeightedMove refuses moves into ice cells."""
        if ice is None:
            _load().qo_set_ice(self.h, None)
            return
        f = np.ascontiguousarray(np.asarray(ice) != 0, dtype=np.uint8)
        assert f.shape == (self.C,)
        self._ice = f
        _load().qo_set_ice(self.h, _p(f))

    def move_stats_enable(self, mode: int, lon: np.ndarray, lat: np.ndarray, radius: float = 1.0,
                          cartesian: bool = False) -> None:
        """MoveStats (0 first, 1 min, 2 last) over the given cell coordinates."""
        self._ms = (np.ascontiguousarray(lon, dtype=np.float64), np.ascontiguousarray(lat, dtype=np.float64))
        rc = _load().qo_move_stats_enable(self.h, int(mode), _p(self._ms[0]), _p(self._ms[1]),
                                          ct.c_double(radius), 1 if cartesian else 0)
        if rc != 0:
            raise ValueError("bad MoveStats mode")

    def move_stats(self):
        """Per cell: hops, distance and time of MoveStats."""
        h = np.zeros(self.C, np.int32)
        d = np.zeros(self.C, np.float64)
        t = np.zeros(self.C, np.float64)
        if _load().qo_move_stats(self.h, _p(h), _p(d), _p(t)) != 0:
            raise ValueError("MoveStats not enabled")
        return h, d, t

    def num_agents(self) -> int:
        return int(_load().qo_num_agents(self.h))

    def agents(self) -> Agents:
        n = self.num_agents()
        out = Agents(np.zeros(n, np.int64), np.zeros(n, np.int32), np.zeros(n, np.float32),
                     np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.uint8),
                     np.zeros(n, np.uint8))
        g = None
        if self.genetics.genome_size > 0:
            g = np.zeros((n, 2 * self.genetics.num_blocks), dtype=np.uint64)
            out.genome = g
        _load().qo_get_agents(self.h, _p(out.id), _p(out.cell), _p(out.birth), _p(out.age),
                              _p(out.lastb), _p(out.gender), _p(out.state),
                              _p(g) if g is not None else None)
        return out

    def counts(self) -> np.ndarray:
        c = np.zeros(self.C, dtype=np.uint32)
        _load().qo_get_counts(self.h, _p(c))
        return c

    def birth_log(self) -> np.ndarray:
        n = int(_load().qo_num_logged_births(self.h))
        b, m, f = np.zeros(n, np.int64), np.zeros(n, np.int64), np.zeros(n, np.int64)
        _load().qo_get_birth_log(self.h, _p(b), _p(m), _p(f))
        return np.stack([b, m, f], axis=1)

    def binomial_table(self) -> np.ndarray:
        buf = np.zeros(256, dtype=np.float64)
        n = _load().qo_binomial_table(self.h, _p(buf), 256)
        return buf[:min(n, 256)].copy()

    def next_id(self) -> int:
        return int(_load().qo_next_id(self.h))

    def set_next_id(self, next_id: int) -> None:
        _load().qo_set_next_id(self.h, int(next_id))

    def current_step(self) -> int:
        return int(_load().qo_current_step(self.h))

    def close(self) -> None:
        if getattr(self, "h", None):
            _load().qo_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def run(grid: Grid, agents: Agents, actions: Sequence[Action], steps: int, seed: int,
        genetics: Genetics = Genetics(), first_step: int = 0):
    r = OracleRun(grid, actions, seed, genetics)
    r.load(agents, first_step)
    st = r.step(steps) if steps > 0 else np.zeros((0, 4), np.uint64)
    return r, st
