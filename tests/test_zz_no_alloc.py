"""The census entry point that allocates nothing, checked against the run's
own per-cell counts.

qhg_gpu_cell_census_noalloc exists for callers that cannot allocate device
memory when they need a census of an agent table: a host runtime that owns
a fixed device pool, a real-time loop that must not call cudaMalloc/cudaFree,
or a device whose heap is full.  It keeps its scratch in a file-scope device
array and takes the caller's device buffers for input and output.  The test
allocates those buffers itself (with torch), runs a small simulation through
the regular C ABI, and compares the census of its agent table -- twice in a
row, so that the second call proves the shared scratch is reset -- with
qhg_gpu_counts, exactly (counts are integers).

The file is named to be collected last: a failure here leaves every other
test already run.
"""
import ctypes as ct

import numpy as np
import pytest

from qhg4_gb300.gpu import GpuRun

from helpers import case_config1

pytestmark = pytest.mark.gpu


def _census(lib, torch, cells: np.ndarray, C: int):
    d_cell = torch.from_numpy(np.ascontiguousarray(cells, dtype=np.int32)).cuda()
    d_counts = torch.zeros(C, dtype=torch.int32, device="cuda")
    d_first = torch.zeros(C + 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = lib.qhg_gpu_cell_census_noalloc(ct.c_void_p(d_cell.data_ptr()), len(cells), C,
                                         ct.c_void_p(d_counts.data_ptr()), ct.c_void_p(d_first.data_ptr()), None)
    assert rc == 0, lib.qhg_gpu_census_last_error().decode()
    return d_counts.cpu().numpy().view(np.uint32), d_first.cpu().numpy().view(np.uint32)


def test_census_noalloc_matches_run_counts(gpu_lib):
    torch = pytest.importorskip("torch")
    grid, agents, acts = case_config1(n=16, N=60000, seed=3)
    C = grid.num_cells
    run = GpuRun(grid, acts, 7)
    run.load(agents)
    run.step(5)
    expect = run.counts()
    table = run.agents(sort_by_id=False)
    n = len(table)
    for trial in range(2):
        cells = np.random.default_rng(trial).permutation(table.cell)
        counts, first = _census(gpu_lib, torch, cells, C)
        assert np.array_equal(counts, expect), f"call {trial}: counts differ"
        assert first[0] == 0 and first[-1] == n
        assert np.array_equal(first[1:], np.cumsum(expect, dtype=np.uint64).astype(np.uint32))
    run.close()


def test_census_noalloc_rejects_oversized_grid(gpu_lib):
    rc = gpu_lib.qhg_gpu_cell_census_noalloc(None, 0, 4194305, ct.c_void_p(8), ct.c_void_p(8), None)
    assert rc == -1
    assert b"QHG_CENSUS_MAX_CELLS" in gpu_lib.qhg_gpu_census_last_error()


def test_census_noalloc_many_tiles_then_fewer_then_maximum(gpu_lib):
    """Synthetic cell arrays without a run, checked against np.bincount:
    about 1M cells (hundreds of scan tiles, so that tiles combine the
    aggregates of tiles still waiting for their prefix), then a grid of a
    few tiles on the next call (the status words the first call left behind
    must count as stale), then exactly QHG_CENSUS_MAX_CELLS cells (every
    status word of the static array in use), and the small grid again."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    for C, n in ((1_000_003, 3_000_000), (5_000, 40_000), (4_194_304, 6_000_000), (5_000, 1)):
        cells = rng.integers(0, C, size=n, dtype=np.int64).astype(np.int32)
        # a dense stretch of cells holding many agents each, and empty ones
        cells[: n // 4] = (cells[: n // 4] % max(1, C // 64)).astype(np.int32)
        counts, first = _census(gpu_lib, torch, cells, C)
        expect = np.bincount(cells, minlength=C).astype(np.uint64)
        assert np.array_equal(counts.astype(np.uint64), expect), f"C={C}: counts differ"
        assert first[0] == 0 and int(first[-1]) == n
        assert np.array_equal(first[1:].astype(np.uint64), np.cumsum(expect)), f"C={C}: first rows differ"


def test_census_noalloc_reports_a_bad_cell(gpu_lib):
    """A cell index outside the grid is reported (never counted) and the
    next call is unaffected."""
    torch = pytest.importorskip("torch")
    C = 3000
    cells = np.arange(10_000, dtype=np.int32) % C
    cells[1234] = C + 5
    d_cell = torch.from_numpy(cells).cuda()
    d_counts = torch.zeros(C, dtype=torch.int32, device="cuda")
    d_first = torch.zeros(C + 1, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    rc = gpu_lib.qhg_gpu_cell_census_noalloc(ct.c_void_p(d_cell.data_ptr()), len(cells), C,
                                             ct.c_void_p(d_counts.data_ptr()), ct.c_void_p(d_first.data_ptr()), None)
    assert rc == -1
    assert b"1234" in gpu_lib.qhg_gpu_census_last_error()
    cells[1234] = 0
    counts, first = _census(gpu_lib, torch, cells, C)
    assert np.array_equal(counts.astype(np.int64), np.bincount(cells, minlength=C))
