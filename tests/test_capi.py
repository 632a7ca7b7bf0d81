"""The C ABI library builds for sm_103a, loads, and exports every function
include/qhg_gpu.h declares (no device calls: this runs without a GPU)."""
import ctypes
import os
import re

from qhg4_gb300.build import build
from qhg4_gb300.gpu import EXPORTS

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "qhg_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(qhg_(?:gpu|batch|host)_\w+)\s*\(", src)))


def test_library_exports_header():
    lib = ctypes.CDLL(build())
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(EXPORTS) == names


def test_version_string():
    lib = ctypes.CDLL(build())
    lib.qhg_gpu_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.qhg_gpu_version()
