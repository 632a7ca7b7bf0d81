"""The dynpops population plugins (qhg4_gb300/plugin: GpuPop<T>, GpuSexualPop,
GpuFlatExpPop)
compiles against the reference's own population headers and template code
and exports the loader's entry points, createPop and getInfo
(dynpops/WrapperTemplate.cpp.tmp).  Needs the reference tree; QHG4's HDF5 and
OpenSSL headers are stood in for by the oracle build's shim headers."""
import os
import subprocess

import pytest

from oracle.refpath import REFERENCE_DIR

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = REFERENCE_DIR


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference tree is not present")
def test_plugin_builds_and_exports_loader_symbols(tmp_path):
    from qhg4_gb300.build import build
    lib = build()
    out = str(tmp_path)
    os.symlink(lib, os.path.join(out, "libqhg_gpu.so"))
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "qhg4_gb300", "plugin"), "REF=" + REF, "OUT=" + out,
                        "EXTRA_INC=-I" + os.path.join(ROOT, "oracle", "ref", "shim")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    for pop in ("GpuSexualPop", "GpuFlatExpPop"):
        so = os.path.join(out, f"lib{pop}Wrapper.so")
        syms = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
        for name in ("createPop", "getInfo"):
            assert f" T {name}" in syms, (pop, name)
        needed = subprocess.run(["nm", "-D", "--undefined-only", so], capture_output=True, text=True).stdout
        for name in ("qhg_gpu_create", "qhg_gpu_upload_grid", "qhg_gpu_upload_agents", "qhg_gpu_step",
                     "qhg_gpu_download", "qhg_gpu_counts", "qhg_gpu_set_move_weights"):
            assert name in needed, (pop, name)


@pytest.mark.skipif(not os.path.isdir(REF), reason="the reference tree is not present")
def test_plugin_reads_actions_from_configuration(tmp_path):
    """GpuParamActions take their priorities (SPopulation::setPrioList) and
    attributes (Prioritizer::getActionAttributes) from the configuration
    modules the reference's actions read; the run's action list follows.
    A module without one of its attributes is refused.  No GPU is used."""
    from qhg4_gb300.build import build
    lib = build()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle", "ref")], check=True, capture_output=True,
                   timeout=1200)
    out = str(tmp_path)
    os.symlink(lib, os.path.join(out, "libqhg_gpu.so"))
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "qhg4_gb300", "plugin"), "REF=" + REF, "OUT=" + out,
                        "EXTRA_INC=-I" + os.path.join(ROOT, "oracle", "ref", "shim"), "param_check"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    run = subprocess.run([os.path.join(out, "param_check")], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0, run.stdout[-2000:] + run.stderr[-2000:]
    rows = [ln.split() for ln in run.stdout.splitlines() if ln[:1].isdigit()]
    got = [(int(t), int(p), n, [float(x) for x in v]) for t, p, n, *v in rows]
    want = [(1, 2, "Fertility", [15, 45.5, 2, 0]), (2, 3, "RandomPair", [0, 0, 0, 0]),
            (5, 4, "OldAgeDeath", [64, 0.078125, 0, 0]), (8, 5, "ATanDeath", [55, 12, 0.35, 0]),
            (3, 6, "Verhulst", [0.2, 0.05, 0.01, 30]), (4, 6, "VerhulstVarK", [0.25, 0.04, 0.02, 0]),
            (6, 7, "RandomMove", [0.1, 0, 0, 0]), (7, 7, "WeightedMove", [0.2, 0, 0, 0]),
            (0, 8, "GetOld", [0, 0, 0, 0])]
    assert got == want
    missing = [ln for ln in run.stdout.splitlines() if ln.startswith("missing ")]
    assert missing and int(missing[0].split()[1]) != 0
    assert "equal 1" in run.stdout.splitlines()
    assert "edited 0 0" in run.stdout.splitlines()
