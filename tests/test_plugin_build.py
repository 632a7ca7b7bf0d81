"""The dynpops population plugins (qhg4_gb300/plugin: GpuPop<T>, GpuSexualPop,
GpuFlatExpPop)
compiles against the reference's own population headers and template code
and exports the loader's entry points, createPop and getInfo
(dynpops/WrapperTemplate.cpp.tmp).  Needs the reference tree; QHG4's HDF5 and
OpenSSL headers are stood in for by the oracle build's shim headers."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = "/root/reference/QHG4"


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
