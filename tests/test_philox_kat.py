"""Philox4x32-10 known-answer vectors (Random123 kat_vectors: counter, key,
expected output) for the generator the oracles use (oracle/philox4x32.h)."""
import ctypes
import os
import subprocess

import pytest

KAT = [
    ((0x00000000, 0x00000000, 0x00000000, 0x00000000), (0x00000000, 0x00000000),
     (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff, 0xffffffff, 0xffffffff, 0xffffffff), (0xffffffff, 0xffffffff),
     (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]

SRC = r"""
#include "philox4x32.h"
void kat(const unsigned *ctr, const unsigned *key, unsigned *out) { qhg_oracle_philox4x32_10(ctr, key, out); }
"""


@pytest.fixture(scope="module")
def katlib(tmp_path_factory):
    d = tmp_path_factory.mktemp("kat")
    src = d / "kat.c"
    src.write_text(SRC)
    so = d / "libkat.so"
    inc = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle")
    subprocess.run(["gcc", "-O2", "-shared", "-fPIC", "-I", inc, str(src), "-o", str(so)], check=True)
    return ctypes.CDLL(str(so))


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_philox_kat(katlib, ctr, key, expect):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    katlib.kat(c, k, o)
    assert tuple(o) == expect
