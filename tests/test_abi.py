"""The C-ABI library builds for sm_103a and exports every entry point that
include/*.h declares (no compute calls: this runs without a GPU)."""
import ctypes
import glob
import os
import re

import pytest

import pi_gb300
from pi_gb300 import build as B

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b(pimul_\w+)\s*\(", text, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("pimul_mul", "pimul_mul_device", "pimul_init", "pimul_last_error"):
        assert must in names


def test_library_builds_and_exports_all_symbols():
    path = B.build()
    assert os.path.exists(path)
    lib = ctypes.CDLL(path)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_version_and_plan_without_gpu():
    # pimul_plan is pure host arithmetic: N = next_pow2(4la + 4lb - 1) (ntt.rs:810-813)
    assert "sm_103a" in pi_gb300.version()
    assert pi_gb300.plan(1, 1) == (8, 0)
    n, p = pi_gb300.plan(1 << 24, 1 << 24)
    assert n == 1 << 27 and p == 3
    n, p = pi_gb300.plan(1 << 24, 1 << 14)
    assert n == 1 << 27
    with pytest.raises(pi_gb300.PimulError):
        pi_gb300.plan(1 << 30, 1 << 30)


def test_decimal_to_hex_host_checks_without_gpu():
    # verify_hex.rs:563-569 prefix check and the E = 0 case return before any
    # device work; the output length h + 2 (h = floor(E log2(10) / 4)) is
    # reported before the buffer is checked
    with pytest.raises(pi_gb300.PimulError, match="doesn't start"):
        pi_gb300.decimal_to_hex("2.718")
    with pytest.raises(pi_gb300.PimulError, match="doesn't start"):
        pi_gb300.decimal_to_hex("  ")
    assert pi_gb300.decimal_to_hex(" 3.\n") == "3."
    n = ctypes.c_size_t(0)
    rc = pi_gb300.lib().pimul_decimal_to_hex(b"3." + b"1" * 1000, 1002, None, 0, ctypes.byref(n), None)
    assert rc != 0 and n.value == 2 + int(1000 * (__import__("math").log2(10.0) / 4.0))
