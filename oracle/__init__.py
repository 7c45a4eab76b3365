"""CPU oracle for the big-integer multiply path (test infrastructure only).

This package wraps ``oracle/_build/libpimul_oracle.so``, a plain-C
restatement of the reference's CPU multiply (joelodom/pi,
``crates/bignum/src/ntt.rs`` and ``crates/bignum/src/integer.rs``) and of
its BBP digit extractor (``crates/pi-core/src/bbp.rs``).  Only the tests,
``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` use it, and only
as the checker or as the timed CPU baseline; the product path in
``pi_gb300`` never imports it.

Parity pinning: the restatement is checked against the reference's own
known-answer tests (see ``tests/golden/``) and against Python's exact
integer multiply.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libpimul_oracle.so")
_lib = None

_u64p = ctypes.POINTER(ctypes.c_uint64)
_sz = ctypes.c_size_t
_u64 = ctypes.c_uint64


def build(force: bool = False) -> str:
    """Compile the oracle with the committed Makefile (gcc + OpenMP)."""
    src = os.path.join(_HERE, "pimul_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        for name in ("orc_gl_add", "orc_gl_sub", "orc_gl_mul", "orc_gl_reduce128", "orc_gl_pow"):
            getattr(L, name).restype = _u64
            getattr(L, name).argtypes = [_u64, _u64]
        for name in ("orc_gl_inv", "orc_gl_root"):
            getattr(L, name).restype = _u64
            getattr(L, name).argtypes = [_u64]
        for name in ("orc_ntt_forward", "orc_ntt_inverse", "orc_four_step_forward",
                     "orc_four_step_inverse", "orc_bit_reverse"):
            getattr(L, name).restype = None
            getattr(L, name).argtypes = [_u64p, _sz]
        L.orc_pack.restype = None
        L.orc_pack.argtypes = [_u64p, _sz, _u64p, _sz]
        L.orc_unpack.restype = _sz
        L.orc_unpack.argtypes = [_u64p, _sz, _u64p, _sz]
        for name in ("orc_mul_mag_ntt", "orc_mul_mag", "orc_schoolbook"):
            getattr(L, name).restype = _sz
            getattr(L, name).argtypes = [_u64p, _sz, _u64p, _sz, _u64p, _sz]
        L.orc_mul_mag_dispatch.restype = _sz
        L.orc_mul_mag_dispatch.argtypes = [_u64p, _sz, _u64p, _sz, _u64p, _sz, _sz]
        L.orc_set_thresholds.restype = None
        L.orc_set_thresholds.argtypes = [_sz, _sz, _sz, _sz]
        L.orc_set_threads.restype = None
        L.orc_set_threads.argtypes = [ctypes.c_int]
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_max_threads.argtypes = []
        L.orc_bbp_hex_digits_at.restype = ctypes.c_int
        L.orc_bbp_hex_digits_at.argtypes = [_u64, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint32)]
        L.orc_mul_abi.restype = ctypes.c_int
        L.orc_mul_abi.argtypes = [_u64p, _sz, _u64p, _sz, _u64p, _sz, ctypes.POINTER(_sz)]
        L.orc_bbp_batch.restype = None
        L.orc_bbp_batch.argtypes = [_u64p, _sz, ctypes.POINTER(ctypes.c_uint32)]
        L.orc_bbp_hex_digits_deep.restype = ctypes.c_uint32
        L.orc_bbp_hex_digits_deep.argtypes = [_u64]
        _lib = L
    return _lib


P = 0xFFFFFFFF00000001


def _p(a: np.ndarray):
    return a.ctypes.data_as(_u64p)


def _as_u64(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint64))


# ---------------------------------------------------------------- field
def gl_add(a, b): return lib().orc_gl_add(a, b)
def gl_sub(a, b): return lib().orc_gl_sub(a, b)
def gl_mul(a, b): return lib().orc_gl_mul(a, b)
def gl_pow(a, e): return lib().orc_gl_pow(a, e)
def gl_inv(a): return lib().orc_gl_inv(a)
def gl_root(n): return lib().orc_gl_root(n)


def gl_reduce128(x: int) -> int:
    return lib().orc_gl_reduce128(x & (2**64 - 1), x >> 64)


# ---------------------------------------------------------------- transforms
def _inplace(fn, a):
    a = _as_u64(a).copy()
    getattr(lib(), fn)(_p(a), a.size)
    return a


def ntt_forward(a): return _inplace("orc_ntt_forward", a)
def ntt_inverse(a): return _inplace("orc_ntt_inverse", a)
def four_step_forward(a): return _inplace("orc_four_step_forward", a)
def four_step_inverse(a): return _inplace("orc_four_step_inverse", a)
def bit_reverse(a): return _inplace("orc_bit_reverse", a)


def pack(limbs, n_coeffs: int) -> np.ndarray:
    limbs = _as_u64(limbs)
    out = np.empty(n_coeffs, dtype=np.uint64)
    lib().orc_pack(_p(limbs), limbs.size, _p(out), n_coeffs)
    return out


def unpack(coeffs) -> np.ndarray:
    coeffs = _as_u64(coeffs)
    cap = (coeffs.size + 3) // 4 + 4
    out = np.empty(cap, dtype=np.uint64)
    n = lib().orc_unpack(_p(coeffs), coeffs.size, _p(out), cap)
    return out[:n].copy()


def _mul(fn, a, b, *extra):
    a = _as_u64(a)
    b = _as_u64(b)
    cap = a.size + b.size + 1
    out = np.empty(max(cap, 1), dtype=np.uint64)
    n = getattr(lib(), fn)(_p(a), a.size, _p(b), b.size, _p(out), cap, *extra)
    if n == ctypes.c_size_t(-1).value:
        raise RuntimeError(f"{fn}: output capacity too small")
    return out[:n].copy()


def mul_mag_ntt(a, b): return _mul("orc_mul_mag_ntt", a, b)
def mul_mag(a, b): return _mul("orc_mul_mag", a, b)
def schoolbook(a, b): return _mul("orc_schoolbook", a, b)
def mul_mag_dispatch(a, b, ntt_max_coeffs): return _mul("orc_mul_mag_dispatch", a, b, ntt_max_coeffs)


def set_thresholds(karatsuba=32, parallel_karatsuba=512, ntt=8192, four_step=1 << 25):
    """Reference defaults: crates/bignum/src/config.rs:94-127."""
    lib().orc_set_thresholds(karatsuba, parallel_karatsuba, ntt, four_step)


def set_threads(n: int):
    lib().orc_set_threads(n)


def max_threads() -> int:
    return lib().orc_max_threads()


def mul_abi_pointer():
    """Address of orc_mul_abi (a pimul_mul_fn-compatible multiply)."""
    return ctypes.cast(lib().orc_mul_abi, ctypes.c_void_p).value


# ---------------------------------------------------------------- BBP
def bbp_hex_digits_at(n: int, stop: bool = False):
    flag = ctypes.c_int(1 if stop else 0)
    out = ctypes.c_uint32(0)
    rc = lib().orc_bbp_hex_digits_at(n, ctypes.byref(flag), ctypes.byref(out))
    return None if rc else out.value


def bbp_batch(positions) -> np.ndarray:
    pos = _as_u64(positions)
    out = np.empty(pos.size, dtype=np.uint32)
    lib().orc_bbp_batch(_p(pos), pos.size, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)))
    return out


def bbp_deep(n: int) -> int:
    """Digits at one deep position, each series' terms split over all
    OpenMP threads (same bits as bbp_hex_digits_at; the series sum is
    wrapping addition, so the split does not matter)."""
    return int(lib().orc_bbp_hex_digits_deep(int(n)))


# ---------------------------------------------------------------- verify-hex
_WS = " \t\n\r\x0b\x0c"


def decimal_to_hex(text) -> str:
    """Restatement of crates/pi-cli/src/verify_hex.rs:553-629
    (convert_decimal_to_hex up to the file write) with Python's exact
    integers: trim, require "3." and digits (:563-574), N = the digits
    with the point removed (:575-581; parse_radix, integer.rs:102-153),
    h = floor((D-1) * log2(10) / 4) in f64 (:584-585), m = N 16^h div
    10^(D-1) (:592-593), and "3." + hex(m)[1:] after the leading-'3' check
    (:597-613, to_string_radix(16) at integer.rs:169-177: lower case, no
    leading zeros).  Raises ValueError with the reference's messages."""
    import math
    import sys

    if hasattr(sys, "set_int_max_str_digits"):
        sys.set_int_max_str_digits(0)
    if isinstance(text, (bytes, bytearray)):
        text = bytes(text).decode("ascii", errors="replace")
    t = text.strip(_WS)
    if not t.startswith("3."):
        raise ValueError("doesn't start with \"3.\"")
    frac = t[2:]
    if not all("0" <= c <= "9" for c in frac):
        raise ValueError("has non-digit characters after \"3.\"")
    e = len(frac)
    if e > 0xFFFFFFFF:
        raise ValueError("fractional decimal digit count exceeds u32::MAX")
    n = int("3" + frac)
    h = int(float(e) * (math.log2(10.0) / 4.0))
    m = (n << (4 * h)) // (10 ** e)
    x = format(m, "x")
    if not x.startswith("3"):
        raise ValueError("internal: hex conversion didn't produce a leading '3'")
    return "3." + x[1:]


# ---------------------------------------------------------------- helpers
def limbs_to_int(x) -> int:
    x = _as_u64(x)
    return int.from_bytes(x.astype("<u8").tobytes(), "little") if x.size else 0


def int_to_limbs(v: int) -> np.ndarray:
    if v == 0:
        return np.zeros(0, dtype=np.uint64)
    nbytes = (v.bit_length() + 63) // 64 * 8
    return np.frombuffer(v.to_bytes(nbytes, "little"), dtype="<u8").astype(np.uint64)
