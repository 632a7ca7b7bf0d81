"""The synthetic grid and populations."""
import numpy as np
import pytest

from qhg4_gb300.workload import altitude, ico_grid_tables, make_agents, terrain_grid, uniform_grid


@pytest.mark.parametrize("n", [1, 2, 5, 32])
def test_icosahedral_grid(n):
    nbr, nnbr, xyz = ico_grid_tables(n)
    C = 10 * n * n + 2
    assert nbr.shape == (C, 6) and nnbr.shape == (C,)
    assert np.bincount(nnbr, minlength=7)[5] == 12          # the 12 pentagons
    assert (nnbr[nnbr != 5] == 6).all()
    assert (nbr[nnbr == 5, 5] == -1).all()                   # -1 padded
    for c in range(C):                                       # links are symmetric
        for j in range(nnbr[c]):
            assert c in nbr[nbr[c, j], :nnbr[nbr[c, j]]]
    assert np.allclose(np.linalg.norm(xyz, axis=1), 1.0)


def test_terrain_capacity():
    g = terrain_grid(16, seed=3)
    alt = altitude(g.xyz, 3)
    assert (g.K[alt < 0] == 0).all()
    assert (g.K >= 0).all() and (g.K <= 100).all()
    land = alt >= 0
    assert np.allclose(g.K[land], np.float32(100) * np.maximum(np.float32(0), np.float32(1) - alt[land] / np.float32(3000)))


def test_agents():
    g = uniform_grid(4, 30.0)
    a = make_agents(g, 1000, seed=1, age_max=50.0)
    assert (a.id == np.arange(1000)).all()
    assert (a.birth == -a.age).all() and (a.age >= 0).all() and (a.age < 50).all()
    assert set(np.unique(a.state)) <= {1, 5}
    t = terrain_grid(8, seed=2)
    b = make_agents(t, 5000, seed=2, age_max=60.0, proportional_to_K=True)
    assert (t.K[b.cell] > 0).all()
