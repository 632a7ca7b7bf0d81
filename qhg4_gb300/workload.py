"""Synthetic inputs: the icosahedral cell grid and the initial populations.

The reference builds its grids offline (icosa/EQsahedron, tools_io/GridFactory)
and reads them from QDF files into ``SCellGrid`` (core/SCellGrid.cpp:20-60):
every cell has up to 6 neighbours, -1 padded, and the 12 pentagon cells have
5.  This module writes the same kind of table directly: subdivision ``n`` of
the icosahedron gives 10*n^2 + 2 cells (icosa/EQsahedron.h:44 with s = n-1).

Cells are numbered in the order they first appear when the 20 faces are
walked row by row, which keeps neighbours close in index; neighbours are
listed counter-clockwise around the outward normal, starting from the one
closest to the local east direction.

All generators are seeded and deterministic (numpy PCG64).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Dict, Optional

import numpy as np

_PHI = (1.0 + math.sqrt(5.0)) / 2.0

_ICO_VERTS = np.array([
    [-1, _PHI, 0], [1, _PHI, 0], [-1, -_PHI, 0], [1, -_PHI, 0],
    [0, -1, _PHI], [0, 1, _PHI], [0, -1, -_PHI], [0, 1, -_PHI],
    [_PHI, 0, -1], [_PHI, 0, 1], [-_PHI, 0, -1], [-_PHI, 0, 1],
], dtype=np.float64)

_ICO_FACES = np.array([
    [0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
    [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
    [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
    [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1],
], dtype=np.int64)


@dataclass
class Grid:
    """Cell grid: neighbour table (int32[C,6], -1 padded), neighbour counts
    (uint8[C]), unit-sphere cell centres (float64[C,3]) and carrying
    capacity K (float64[C])."""

    n: int
    nbr: np.ndarray
    nnbr: np.ndarray
    xyz: np.ndarray
    K: np.ndarray

    @property
    def num_cells(self) -> int:
        return int(self.nbr.shape[0])


_GRID_CACHE: Dict[int, tuple] = {}


def ico_grid_tables(n: int):
    """Neighbour table, neighbour counts and centres of the subdivision-n
    icosahedral grid (cached per n)."""
    if n in _GRID_CACHE:
        return _GRID_CACHE[n]
    if n < 1:
        raise ValueError("subdivision must be >= 1")
    # lattice points (i, j) of a face, i + j <= n, weights (n-i-j, i, j)
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    m = (ii + jj) <= n
    fi = ii[m].astype(np.int64)
    fj = jj[m].astype(np.int64)
    npf = fi.size
    loc = -np.ones((n + 1, n + 1), dtype=np.int64)
    loc[fi, fj] = np.arange(npf)

    F = _ICO_FACES.shape[0]
    w = np.stack([n - fi - fj, fi, fj], axis=1)  # [npf, 3]
    keys = np.zeros((F * npf, 6), dtype=np.int64)
    for f in range(F):
        vids = np.broadcast_to(_ICO_FACES[f], (npf, 3)).copy()
        ww = w.copy()
        vids[ww == 0] = 99  # zero weights do not identify the point
        order = np.argsort(vids, axis=1, kind="stable")
        vs = np.take_along_axis(vids, order, axis=1)
        ws = np.take_along_axis(ww, order, axis=1)
        keys[f * npf:(f + 1) * npf, 0::2] = vs
        keys[f * npf:(f + 1) * npf, 1::2] = ws
    _, first, inv = np.unique(keys, axis=0, return_index=True, return_inverse=True)
    inv = inv.reshape(-1)
    # renumber by first appearance (face-major, row by row)
    rank = np.empty(first.size, dtype=np.int64)
    rank[np.argsort(first, kind="stable")] = np.arange(first.size)
    gid = rank[inv]
    C = first.size
    if C != 10 * n * n + 2:
        raise RuntimeError(f"icosahedral grid n={n}: {C} cells, expected {10 * n * n + 2}")

    # centres
    xyz = np.zeros((C, 3), dtype=np.float64)
    for f in range(F):
        A, B, Cc = _ICO_VERTS[_ICO_FACES[f]]
        p = (A[None, :] * (n - fi - fj)[:, None] + B[None, :] * fi[:, None] + Cc[None, :] * fj[:, None]) / n
        xyz[gid[f * npf:(f + 1) * npf]] = p
    xyz /= np.linalg.norm(xyz, axis=1, keepdims=True)

    # lattice edges of every face
    es = []
    for di, dj in ((1, 0), (0, 1), (-1, 1)):
        a_i, a_j = fi, fj
        b_i, b_j = fi + di, fj + dj
        ok = (b_i >= 0) & (b_j >= 0) & (b_i + b_j <= n)
        la = loc[a_i[ok], a_j[ok]]
        lb = loc[b_i[ok], b_j[ok]]
        for f in range(F):
            es.append(np.stack([gid[f * npf + la], gid[f * npf + lb]], axis=1))
    E = np.concatenate(es, axis=0)
    E = np.concatenate([E, E[:, ::-1]], axis=0)
    E = np.unique(E, axis=0)
    src, dst = E[:, 0], E[:, 1]
    deg = np.bincount(src, minlength=C)
    if deg.max() > 6 or deg.min() < 5:
        raise RuntimeError("unexpected vertex degree in icosahedral grid")

    # order neighbours counter-clockwise around the outward normal
    p = xyz[src]
    q = xyz[dst] - p
    zaxis = np.array([0.0, 0.0, 1.0])
    xaxis = np.array([1.0, 0.0, 0.0])
    ref = np.where(np.abs(p[:, 2:3]) > 0.999, xaxis[None, :], zaxis[None, :])
    e1 = np.cross(ref, p)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(p, e1)
    ang = np.arctan2(np.einsum("ij,ij->i", q, e2), np.einsum("ij,ij->i", q, e1))
    ang = np.mod(ang, 2.0 * math.pi)
    order = np.lexsort((ang, src))
    src, dst = src[order], dst[order]
    start = np.zeros(C + 1, dtype=np.int64)
    np.cumsum(deg, out=start[1:])
    slot = np.arange(src.size) - start[src]
    nbr = -np.ones((C, 6), dtype=np.int32)
    nbr[src, slot] = dst.astype(np.int32)
    nnbr = deg.astype(np.uint8)
    _GRID_CACHE[n] = (nbr, nnbr, xyz)
    return nbr, nnbr, xyz


def uniform_grid(n: int, K: float) -> Grid:
    nbr, nnbr, xyz = ico_grid_tables(n)
    return Grid(n, nbr, nnbr, xyz, np.full(nbr.shape[0], float(K), dtype=np.float64))


def altitude(xyz: np.ndarray, seed: int) -> np.ndarray:
    """Altitude field in metres: sum over k=1..16 of a_k sin(f_k (d_k . x) + phi_k)
    with d_k uniform on the sphere, f_k ~ U[2,20], phi_k ~ U[0, 2 pi) and
    a_k ~ N(0, (1000/k)^2), evaluated in float64 and rounded to float32."""
    rng = np.random.default_rng(seed)
    alt = np.zeros(xyz.shape[0], dtype=np.float64)
    for k in range(1, 17):
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        f = rng.uniform(2.0, 20.0)
        phi = rng.uniform(0.0, 2.0 * math.pi)
        a = rng.normal(0.0, 1000.0 / k)
        alt += a * np.sin(f * (xyz @ d) + phi)
    return alt.astype(np.float32)


def terrain_grid(n: int, seed: int) -> Grid:
    """Grid whose K follows the altitude: 0 below sea level, else
    100 * max(0, 1 - alt/3000) (float32 K widened to float64)."""
    nbr, nnbr, xyz = ico_grid_tables(n)
    alt = altitude(xyz, seed)
    K = np.where(alt < 0, np.float32(0.0),
                 np.float32(100.0) * np.maximum(np.float32(0.0), np.float32(1.0) - alt / np.float32(3000.0)))
    return Grid(n, nbr, nnbr, xyz, K.astype(np.float32).astype(np.float64))


@dataclass
class Agents:
    """Agent table, one row per agent (SoA)."""

    id: np.ndarray       # int64
    cell: np.ndarray     # int32
    birth: np.ndarray    # float32
    age: np.ndarray      # float32
    lastb: np.ndarray    # float32
    gender: np.ndarray   # uint8
    state: np.ndarray    # uint8 (1 alive, 5 fertile)
    genome: Optional[np.ndarray] = None  # uint64[N, 2*blocks]

    def __len__(self) -> int:
        return int(self.id.size)

    def sorted_by_id(self) -> "Agents":
        o = np.argsort(self.id, kind="stable")
        return Agents(self.id[o], self.cell[o], self.birth[o], self.age[o], self.lastb[o],
                      self.gender[o], self.state[o], None if self.genome is None else self.genome[o])


def make_agents(grid: Grid, N: int, seed: int, age_max: float, proportional_to_K: bool = False,
                fert_min: float = 15.0, fert_max: float = 45.0, genome_blocks: int = 0) -> Agents:
    """N agents with IDs 0..N-1 placed uniformly over the cells (or with
    probability proportional to K), age ~ U[0, age_max) in float32, birth time
    -age (the first step is at time 0), last birth 0, gender Bernoulli(0.5)
    and the state the Fertility rule gives at their age (ignoring the
    interbirth gap).  With genome_blocks > 0, every genome bit is
    Bernoulli(0.5)."""
    rng = np.random.default_rng(seed)
    C = grid.num_cells
    if proportional_to_K:
        w = np.maximum(grid.K, 0.0)
        if w.sum() <= 0:
            raise ValueError("K is zero everywhere")
        cell = rng.choice(C, size=N, p=w / w.sum()).astype(np.int32)
    else:
        cell = rng.integers(0, C, size=N).astype(np.int32)
    age = rng.uniform(0.0, age_max, size=N).astype(np.float32)
    gender = rng.integers(0, 2, size=N).astype(np.uint8)
    fert = np.where(gender == 0, (age > fert_min) & (age < fert_max), age > fert_min)
    state = np.where(fert, 5, 1).astype(np.uint8)
    genome = None
    if genome_blocks > 0:
        genome = rng.integers(0, np.iinfo(np.uint64).max, size=(N, 2 * genome_blocks),
                              dtype=np.uint64, endpoint=True)
    return Agents(np.arange(N, dtype=np.int64), cell, (-age).astype(np.float32), age,
                  np.zeros(N, dtype=np.float32), gender, state, genome)
