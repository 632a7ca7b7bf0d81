"""The population plugin's host code under QHG4's step loop, without a GPU.

tests/plugin_host/plugin_drive.cpp runs GpuSexualPop (qhg4_gb300/plugin) as
QHG4 runs a population -- agents in its LayerBuf, preLoop, initializeStep /
doActions / finalizeStep per step, preWrite -- linked against
tests/plugin_host/qhg_gpu_fake.c, a stand-in for libqhg_gpu.so that runs
the C ABI on the oracle.  What it copies back into its LayerBuf must equal
the reference's own tutorial actions run by the Philox test build: this
checks the plugin's glue (seed, parameters and priorities, the upload from
the LayerBuf, the copy back), the part no machine here can run against the
real library.  Needs the reference tree (headers, template code and the
support objects built by oracle/ref/Makefile).
"""
import os
import subprocess

import numpy as np
import pytest

from oracle.refpath import REFERENCE_DIR

from oracle.refsim_io import ref_program, run_reference, write_input
from qhg4_gb300.spec import CROSSOVER_POISSON1, Genetics, config1_actions, config3_actions
from qhg4_gb300.workload import Agents, make_agents, uniform_grid

from helpers import table_diff

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = REFERENCE_DIR
HERE = os.path.join(ROOT, "tests", "plugin_host")


def build_driver(out: str) -> str:
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref")], check=True, capture_output=True,
                   timeout=1200)
    fake = os.path.join(out, "libqhg_gpu.so")
    subprocess.run(["gcc", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-std=c11", "-shared",
                    "-I" + os.path.join(ROOT, "include"), os.path.join(HERE, "qhg_gpu_fake.c"),
                    os.path.join(ROOT, "oracle", "qhg_oracle.c"), "-lm", "-o", fake], check=True, timeout=300)
    refobj = os.path.join(ROOT, "oracle", "_ref", "well")
    objs = [os.path.join(refobj, f) for f in sorted(os.listdir(refobj)) if f.endswith(".o") and f != "harness.o"]
    inc = ["-I" + os.path.join(REF, d) for d in ("core", "actions", "utils", "io", "genes", "utils_qhg", "icosa",
                                                   "populations", "geoinfo")]
    exe = os.path.join(out, "plugin_drive")
    r = subprocess.run(["g++", "-std=c++20", "-O1", "-fopenmp", "-w", "-I" + os.path.join(ROOT, "oracle", "ref", "shim")]
                       + inc + ["-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "qhg4_gb300", "plugin"),
                                os.path.join(HERE, "plugin_drive.cpp")] + objs
                       + ["-L" + out, "-Wl,-rpath," + out, "-lqhg_gpu", "-lz", "-o", exe],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    if not os.path.isdir(REF):
        pytest.skip("the reference tree is not present")
    return build_driver(str(tmp_path_factory.mktemp("plugin_drive")))


def read_drive_output(path: str):
    b = open(path, "rb").read()
    pos = 0

    def take(dt, n):
        nonlocal pos
        a = np.frombuffer(b, dtype=dt, count=n, offset=pos).copy()
        pos += np.dtype(dt).itemsize * n
        return a

    n = int(take("<u8", 1)[0])
    a = Agents(take("<i8", n), take("<i4", n), take("<f4", n), take("<f4", n), take("<f4", n), take("u1", n),
               take("u1", n))
    C = int(take("<u4", 1)[0])
    counts = take("<u4", C)
    words = int(take("<u4", 1)[0])
    if words > 0:
        a.genome = take("<u8", n * words).reshape(n, words)
    read_drive_output.generators_next = int(take("<i8", 1)[0])
    return a, counts


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference tree is not present")
@pytest.mark.parametrize("write_every", [0, 4], ids=["no_snapshots", "snapshot_every_4"])
def test_plugin_population_equals_reference_actions(tmp_path, driver, write_every):
    out = str(tmp_path)
    exe = driver
    grid = uniform_grid(8, 30.0)
    agents = make_agents(grid, 15000, seed=71, age_max=50.0)
    acts = config1_actions(b0=0.3, d0=0.03, move_p=0.2)
    pin, pout = os.path.join(out, "in.bin"), os.path.join(out, "drive.bin")
    write_input(pin, grid, agents, acts, 25, 4711)
    r = subprocess.run([exe, pin, pout, str(write_every)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got, counts = read_drive_output(pout)
    ref = run_reference("philox", out, grid, agents, acts, 25, 4711, threads=2)
    assert ref.draw_errors == 0
    got = got.sorted_by_id()
    d = table_diff(got, ref.agents)
    assert d is None, d
    assert np.array_equal(counts, np.bincount(ref.agents.cell, minlength=grid.num_cells).astype(np.uint32))
    assert len(got) > 5000
    # the application's ID generators were moved past the run's newborn IDs
    assert read_drive_output.generators_next > int(ref.births[:, 0].max())


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference tree is not present")
@pytest.mark.parametrize("genetics", [Genetics(512, CROSSOVER_POISSON1, 1e-3), Genetics(200, 2, 5e-3)],
                         ids=["poisson_512", "fixed2_200"])
def test_plugin_population_with_genomes(tmp_path, driver, genetics):
    """With genomes kept beside the agents (setGpuGenetics): uploaded with the
    LayerBuf, crossed and mutated by the run, written back by preWrite --
    against the reference's Genetics / BitGeneUtils in the Philox test build."""
    out = str(tmp_path)
    exe = driver
    grid = uniform_grid(5, 40.0)
    agents = make_agents(grid, 3000, seed=72, age_max=50.0, genome_blocks=genetics.num_blocks)
    acts = config3_actions()
    pin, pout = os.path.join(out, "in.bin"), os.path.join(out, "drive.bin")
    write_input(pin, grid, agents, acts, 15, 4712, genetics)
    r = subprocess.run([exe, pin, pout, "5"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got, counts = read_drive_output(pout)
    ref = run_reference("philox", out, grid, agents, acts, 15, 4712, genetics, threads=2)
    assert ref.draw_errors == 0
    d = table_diff(got.sorted_by_id(), ref.agents)
    assert d is None, d
    assert len(ref.births) > 0


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference tree is not present")
@pytest.mark.parametrize("case", range(4))
def test_plugin_population_configured_like_the_reference(tmp_path, driver, case):
    """A plugin population whose actions are GpuParamActions, configured from
    one module per action and the priorities (random action lists, ties
    included), equals the reference's population configured the same way."""
    from qhg4_gb300.spec import (ACT_ATANDEATH, ACT_FERTILITY, ACT_GETOLD, ACT_OLDAGEDEATH, ACT_RANDOMMOVE,
                                 ACT_RANDOMPAIR, ACT_VERHULST, ACT_VERHULSTVARK, ACT_WEIGHTEDMOVE, Action)
    from qhg4_gb300.workload import terrain_grid
    rng = np.random.default_rng(900 + case)

    def prio():
        return int(rng.integers(1, 6))

    acts = [Action(ACT_FERTILITY, prio(), (15.0, 45.0, float(rng.uniform(0, 3)))), Action(ACT_RANDOMPAIR, prio())]
    if case % 2 == 0:
        acts.append(Action(ACT_VERHULST, prio(), (float(rng.uniform(0.2, 0.5)), 0.03, 0.01, 50.0)))
    else:
        acts.append(Action(ACT_VERHULSTVARK, prio(), (float(rng.uniform(0.2, 0.5)), 0.03, 0.01)))
    acts.append(Action(ACT_WEIGHTEDMOVE if case < 2 else ACT_RANDOMMOVE, prio(), (float(rng.uniform(0.1, 0.4)),)))
    acts.append(Action(ACT_OLDAGEDEATH, prio(), (62.0, 0.08)))
    if case >= 2:
        acts.append(Action(ACT_ATANDEATH, prio(), (55.0, 12.0, 0.3)))
    acts.append(Action(ACT_GETOLD, prio()))
    grid = terrain_grid(8, seed=910 + case)
    agents = make_agents(grid, 6000, seed=920 + case, age_max=75.0, proportional_to_K=True)
    out = str(tmp_path)
    pin, pout = os.path.join(out, "in.bin"), os.path.join(out, "drive.bin")
    write_input(pin, grid, agents, acts, 15, 930 + case)
    r = subprocess.run([driver, pin, pout, "6", "param"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got, counts = read_drive_output(pout)
    ref = run_reference("philox", out, grid, agents, acts, 15, 930 + case, threads=2)
    assert ref.draw_errors == 0
    d = table_diff(got.sorted_by_id(), ref.agents)
    assert d is None, (d, [(a.type, a.prio) for a in acts])


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference tree is not present")
@pytest.mark.parametrize("given_weights", [False, True], ids=["weights_from_K", "given_weights"])
def test_plugin_population_environment_events(tmp_path, driver, given_weights):
    """GpuPop's environment arrays: given move weights, and K rewritten with
    an environment event before steps 4 and 9, handed to the run by the next
    initializeStep -- against the reference's classes with the same weights
    and K changes."""
    from qhg4_gb300.spec import config2_actions
    from qhg4_gb300.workload import terrain_grid
    from helpers import move_weights
    grid = terrain_grid(9, seed=940)
    agents = make_agents(grid, 8000, seed=941, age_max=70.0, proportional_to_K=True)
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.3)
    rng = np.random.default_rng(942)
    changes = [(4, grid.K * rng.uniform(0.3, 1.5, grid.num_cells)),
               (9, np.where(rng.random(grid.num_cells) < 0.2, 0.0, grid.K * 1.2))]
    W = move_weights(grid, 943) if given_weights else None
    out = str(tmp_path)
    pin, pout = os.path.join(out, "in.bin"), os.path.join(out, "drive.bin")
    write_input(pin, grid, agents, acts, 14, 944, weights=W, k_changes=changes)
    r = subprocess.run([driver, pin, pout, "0", "param"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got, counts = read_drive_output(pout)
    ref = run_reference("philox", out, grid, agents, acts, 14, 944, threads=2, weights=W, k_changes=changes)
    assert ref.draw_errors == 0
    d = table_diff(got.sorted_by_id(), ref.agents)
    assert d is None, d


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference tree is not present")
def test_plugin_population_removes_agents_in_cells(tmp_path, driver):
    """GpuPop::removeAgentsInCells (a geography event's drowning, as
    FlatExpPop::updateEvent does it) before steps 5 and 11, with genomes,
    against the reference's registerDeath / recycleDeadSpaceNew path."""
    from qhg4_gb300.workload import uniform_grid as ug
    gen = Genetics(256, CROSSOVER_POISSON1, 2e-3)
    grid = ug(6, 40.0)
    agents = make_agents(grid, 9000, seed=961, age_max=50.0, genome_blocks=gen.num_blocks)
    acts = config3_actions()
    rng = np.random.default_rng(962)
    kills = [(5, (rng.random(grid.num_cells) < 0.2).astype(np.uint8)),
             (11, (rng.random(grid.num_cells) < 0.3).astype(np.uint8))]
    out = str(tmp_path)
    pin, pout = os.path.join(out, "in.bin"), os.path.join(out, "drive.bin")
    write_input(pin, grid, agents, acts, 16, 963, gen, kills=kills)
    r = subprocess.run([driver, pin, pout, "7"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got, counts = read_drive_output(pout)
    ref = run_reference("philox", out, grid, agents, acts, 16, 963, gen, threads=2, kills=kills)
    assert ref.draw_errors == 0
    d = table_diff(got.sorted_by_id(), ref.agents)
    assert d is None, d


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference tree is not present")
def test_plugin_population_runtime_edits(tmp_path, driver):
    """Runtime edits through Prioritizer::modifyAttributes: WeightedMove's
    probability changes from step 4 (the plugin rebuilds its run with the
    table, step and next ID kept), and a Verhulst edit changes nothing, as in
    the reference (its LinearBirth / LinearDeath know other names)."""
    from qhg4_gb300.spec import config2_actions
    from qhg4_gb300.workload import terrain_grid
    grid = terrain_grid(9, seed=970)
    agents = make_agents(grid, 8000, seed=971, age_max=70.0, proportional_to_K=True)
    acts = config2_actions(b0=0.3, d0=0.03, move_p=0.1)
    mods = [(4, "WeightedMove_prob", 0.6), (7, "Verhulst_b0", 0.9), (9, "WeightedMove_prob", 0.02)]
    out = str(tmp_path)
    pin, pout = os.path.join(out, "in.bin"), os.path.join(out, "drive.bin")
    write_input(pin, grid, agents, acts, 14, 972, mods=mods)
    r = subprocess.run([driver, pin, pout, "5", "param"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    got, counts = read_drive_output(pout)
    ref = run_reference("philox", out, grid, agents, acts, 14, 972, threads=2, mods=mods)
    assert ref.draw_errors == 0
    d = table_diff(got.sorted_by_id(), ref.agents)
    assert d is None, d
    plain = run_reference("philox", out, grid, agents, acts, 14, 972, threads=2)
    assert table_diff(plain.agents, ref.agents) is not None   # the edits matter
