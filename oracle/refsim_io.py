"""Input/output files of the reference oracle programs (oracle/_ref/qhg_ref_*).

ORACLE / TEST INFRASTRUCTURE ONLY: imported by tests/ and by the golden
fixture script, never by the product.

Input (little endian):
  "QHGREF01", u32 C, u32 N, u32 steps, u32 layer_size, u64 seed, u32 n_actions,
  n_actions x (u32 type, u32 prio, f64 p[4]),
  u32 genome_size, i32 num_crossover, f64 mutation_rate, u32 dump_counts_every,
  i32 nbr[C*6], u8 nnbr[C], f64 K[C],
  i64 id[N], i32 cell[N], f32 birth[N], f32 age[N], f32 lastb[N], u8 gender[N],
  u8 state[N], u64 genome[N*2*blocks]
  optional: u32 has_weights, f64 W[C*7] if has_weights == 1 (WeightedMove's
  cumulative weights as given, in place of the SingleEvaluator over K),
  u32 n_k_changes, n_k_changes x (u32 step, f64 K[C]) (K from that step on),
  u32 movestats_mode + 1 (0 none), f64 radius, f64 lon[C], f64 lat[C]
  (a MoveStats action over a Geography with these cell coordinates, degrees),
  u32 n_kill_events, n_kill_events x (u32 step, u8 flags[C]) (before that
  step every agent in a flagged cell dies, as after a geography event),
  u32 n_mods, n_mods x (u32 step, u32 name_len, char name[name_len], f64 value)
  (runtime edits through Prioritizer::modifyAttributes before that step),
  u32 has_ice, u8 ice[C] if has_ice == 1 (the Geography's m_abIce, which
  WeightedMove reads)
Output:
  "QHGOUT01", u32 steps, u32 C, u64 stats[steps*4] (live, births, deaths, moves),
  u32 n_dumps, u32 dump_step[n_dumps], u32 counts[n_dumps*C],
  u64 n, i64 id[n], i32 cell[n], f32 birth[n], f32 age[n], f32 lastb[n],
  u8 gender[n], u8 state[n], u64 genome[n*2*blocks],
  u64 nb, i64 baby[nb], i64 mother[nb], i64 father[nb],
  u64 draw_errors, f64 seconds, u64 agent_steps, u32 threads,
  u32 has_movestats, i32 hops[C], f64 dist[C], f64 time[C] if has_movestats
"""
from __future__ import annotations

import os
import struct
import subprocess
from typing import Sequence

import numpy as np

from qhg4_gb300.spec import Action, Genetics
from qhg4_gb300.workload import Agents, Grid

REF_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_ref")


def ref_program(kind: str) -> str:
    return os.path.join(REF_DIR, "qhg_ref_" + kind)


def write_input(path: str, grid: Grid, agents: Agents, actions: Sequence[Action], steps: int,
                seed: int, genetics: Genetics = Genetics(), dump_every: int = 0,
                layer_size: int = 65536, weights=None, k_changes=(), move_stats=None, kills=(), ice=None,
                mods=()) -> None:
    C = grid.num_cells
    N = len(agents)
    with open(path, "wb") as f:
        f.write(b"QHGREF01")
        f.write(struct.pack("<IIII", C, N, steps, layer_size))
        f.write(struct.pack("<QI", seed, len(actions)))
        for a in actions:
            f.write(struct.pack("<II4d", a.type, a.prio, *a.params4()))
        f.write(struct.pack("<IidI", genetics.genome_size, genetics.num_crossover,
                            genetics.mutation_rate, dump_every))
        f.write(np.ascontiguousarray(grid.nbr, dtype="<i4").tobytes())
        f.write(np.ascontiguousarray(grid.nnbr, dtype="u1").tobytes())
        f.write(np.ascontiguousarray(grid.K, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(agents.id, dtype="<i8").tobytes())
        f.write(np.ascontiguousarray(agents.cell, dtype="<i4").tobytes())
        f.write(np.ascontiguousarray(agents.birth, dtype="<f4").tobytes())
        f.write(np.ascontiguousarray(agents.age, dtype="<f4").tobytes())
        f.write(np.ascontiguousarray(agents.lastb, dtype="<f4").tobytes())
        f.write(np.ascontiguousarray(agents.gender, dtype="u1").tobytes())
        f.write(np.ascontiguousarray(agents.state, dtype="u1").tobytes())
        if genetics.genome_size > 0:
            f.write(np.ascontiguousarray(agents.genome, dtype="<u8").tobytes())
        if (weights is not None or len(k_changes) > 0 or move_stats is not None or len(kills) > 0 or len(mods) > 0
                or ice is not None):
            f.write(struct.pack("<I", 1 if weights is not None else 0))
            if weights is not None:
                w = np.ascontiguousarray(weights, dtype="<f8")
                assert w.shape == (C, 7)
                f.write(w.tobytes())
            f.write(struct.pack("<I", len(k_changes)))
            for step, K in k_changes:
                k = np.ascontiguousarray(K, dtype="<f8")
                assert k.shape == (C,)
                f.write(struct.pack("<I", int(step)))
                f.write(k.tobytes())
            if move_stats is not None:
                mode, lon, lat, radius = move_stats
                f.write(struct.pack("<Id", int(mode) + 1, float(radius)))
                f.write(np.ascontiguousarray(lon, dtype="<f8").tobytes())
                f.write(np.ascontiguousarray(lat, dtype="<f8").tobytes())
            else:
                f.write(struct.pack("<I", 0))
            f.write(struct.pack("<I", len(kills)))
            for step, flags in kills:
                fl = np.ascontiguousarray(flags, dtype="u1")
                assert fl.shape == (C,)
                f.write(struct.pack("<I", int(step)))
                f.write(fl.tobytes())
            f.write(struct.pack("<I", len(mods)))
            for step, name, value in mods:
                nb = name.encode()
                f.write(struct.pack("<II", int(step), len(nb)))
                f.write(nb)
                f.write(struct.pack("<d", float(value)))
            if ice is not None:
                fi = np.ascontiguousarray(np.asarray(ice) != 0, dtype="u1")
                assert fi.shape == (C,)
                f.write(struct.pack("<I", 1))
                f.write(fi.tobytes())
            else:
                f.write(struct.pack("<I", 0))


class RefOutput:
    pass


def read_output(path: str, genome_blocks: int = 0) -> RefOutput:
    with open(path, "rb") as f:
        b = f.read()
    o = RefOutput()
    pos = 0

    def take(dtype, count):
        nonlocal pos
        dt = np.dtype(dtype)
        a = np.frombuffer(b, dtype=dt, count=count, offset=pos).copy()
        pos += dt.itemsize * count
        return a

    if b[:8] != b"QHGOUT01":
        raise ValueError("not a reference oracle output file")
    pos = 8
    steps, C = take("<u4", 2)
    o.stats = take("<u8", int(steps) * 4).reshape(int(steps), 4)
    nd = int(take("<u4", 1)[0])
    o.dump_steps = take("<u4", nd)
    o.counts = take("<u4", nd * int(C)).reshape(nd, int(C))
    n = int(take("<u8", 1)[0])
    o.agents = Agents(take("<i8", n), take("<i4", n), take("<f4", n), take("<f4", n),
                      take("<f4", n), take("u1", n), take("u1", n))
    if genome_blocks > 0:
        o.agents.genome = take("<u8", n * 2 * genome_blocks).reshape(n, 2 * genome_blocks)
    nb = int(take("<u8", 1)[0])
    o.births = np.stack([take("<i8", nb), take("<i8", nb), take("<i8", nb)], axis=1)
    o.draw_errors = int(take("<u8", 1)[0])
    o.seconds = float(take("<f8", 1)[0])
    o.agent_steps = int(take("<u8", 1)[0])
    o.threads = int(take("<u4", 1)[0])
    o.move_stats = None
    if pos < len(b) and int(take("<u4", 1)[0]) == 1:
        o.move_stats = (take("<i4", int(C)), take("<f8", int(C)), take("<f8", int(C)))
    return o


def run_reference(kind: str, workdir: str, grid: Grid, agents: Agents, actions: Sequence[Action],
                  steps: int, seed: int, genetics: Genetics = Genetics(), dump_every: int = 0,
                  threads: int = 0, timeout: float = 3600.0, weights=None, k_changes=(),
                  move_stats=None, kills=(), mods=(), ice=None) -> RefOutput:
    """Run qhg_ref_well or qhg_ref_philox on the given input; `weights`
    (C x 7 cumulative) replace the weights from K, `k_changes` holds
    (step, K) pairs: K from that step on; `move_stats` = (mode, lon, lat,
    radius) adds a MoveStats action; `kills` holds (step, cell flags) pairs:
    before that step every agent in a flagged cell dies; `mods` holds
    (step, attribute name, value) runtime edits."""
    exe = ref_program(kind)
    if not os.path.exists(exe):
        raise FileNotFoundError(exe)
    os.makedirs(workdir, exist_ok=True)
    pin = os.path.join(workdir, f"in_{kind}_{seed}.bin")
    pout = os.path.join(workdir, f"out_{kind}_{seed}.bin")
    write_input(pin, grid, agents, actions, steps, seed, genetics, dump_every, weights=weights,
                k_changes=k_changes, move_stats=move_stats, kills=kills, mods=mods, ice=ice)
    env = dict(os.environ)
    if threads > 0:
        env["OMP_NUM_THREADS"] = str(threads)
    r = subprocess.run([exe, pin, pout], env=env, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE,
                       timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"{exe} failed ({r.returncode}): {r.stderr.decode()[-2000:]}")
    return read_output(pout, genetics.num_blocks)
