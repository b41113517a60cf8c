"""Host-side logic without a GPU: the C-ABI library loads and exports every
symbol its header declares; the x87 extended-precision model; the restated
libstdc++ float orders."""

import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            with open(os.path.join(ROOT, "include", name)) as f:
                syms |= set(re.findall(r"\b(kgb_[a-z0-9_]+)\s*\(", f.read()))
    return syms


def test_library_exports_every_declared_symbol(kg):
    path = kg.library_path()
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (kgb_[a-z0-9_]+)$", out, re.M))
    declared = _declared_symbols()
    assert declared, "no declarations found"
    assert declared <= exported, f"missing: {sorted(declared - exported)}"
    lib = ctypes.CDLL(path)
    for s in declared:
        assert hasattr(lib, s)
    lib.kgb_version.restype = ctypes.c_char_p
    assert lib.kgb_version().startswith(b"kodama_gb300")


def test_python_mirror_lists_exports(kg):
    from kodama_gb300 import _native
    assert _declared_symbols() == set(_native.EXPORTED)


def test_ext80_against_native_long_double(orc):
    lib = orc._LIB
    lib.ext80_selftest.restype = ctypes.c_int
    bad = lib.ext80_selftest(200000, ctypes.c_ulonglong(7))
    if bad < 0:
        pytest.skip("long double is not the x87 format on this host")
    assert bad == 0


def test_dot_order_matches_reference_shape(orc):
    # 16 lane partial sums, then the lane combine, then the tail: a sum whose
    # result depends on that order
    a = np.array([1e8, 1.0, -1e8, 1.0] * 5 + [3.0, 5.0], np.float32)
    b = np.ones_like(a)
    p = np.zeros(16, np.float32)
    for i in range(0, 16):
        p[i] = np.float32(p[i] + a[i] * b[i])
    lanes = [np.float32(np.float32(p[l] + p[4 + l]) + np.float32(p[8 + l] + p[12 + l])) for l in range(4)]
    s = np.float32(np.float32(np.float32(lanes[0] + lanes[1]) + lanes[2]) + lanes[3])
    for i in range(16, len(a)):
        s = np.float32(s + np.float32(a[i] * b[i]))
    assert orc.dot_x86(a, b) == s
