"""pi_gb300 — GB300-native big-integer multiply engine (Python host side).

The engine is ``pi_gb300/_build/libpimul.so`` (hand-written sm_103a CUDA
behind the C ABI in ``include/pimul.h``).  This module loads it with ctypes
and exposes the reference's multiply interface:

* :func:`mul_mag_ntt` — drop-in for ``mul_mag_ntt(a: &[u64], b: &[u64]) ->
  Vec<u64>`` (joelodom/pi ``crates/bignum/src/ntt.rs:806``): little-endian
  u64 limb arrays in, trimmed product out, empty means zero.
* :func:`mul_device` — the same product on device buffers (torch CUDA
  tensors), asynchronous on the current torch stream.

There is no CPU fallback: if the library is missing or CUDA fails, every call
raises :class:`PimulError`.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

__all__ = [
    "PimulError", "lib", "load", "version", "init", "mul_mag_ntt", "mul_device",
    "plan", "sync", "bbp_hex_digits", "LIB_PATH",
]

LIB_PATH = _build.LIB

PIMUL_OK = 0
ERRORS = {1: "EINVAL", 2: "ENOMEM", 3: "ECUDA", 4: "ETIMEDOUT", 5: "ENOTFOUND", 6: "ECANCELED"}


class PimulError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"pimul {ERRORS.get(code, code)}: {msg}")
        self.code = code


_lib = None
_u64p = ctypes.POINTER(ctypes.c_uint64)
_sz = ctypes.c_size_t


def load(build_if_stale: bool = True):
    """Load libpimul.so (compiling it first when sources are newer)."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_stale:
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise PimulError(3, f"{LIB_PATH} is missing; run `python -m pi_gb300.build`")
    L = ctypes.CDLL(LIB_PATH)
    L.pimul_version.restype = ctypes.c_char_p
    L.pimul_last_error.restype = ctypes.c_char_p
    L.pimul_init.argtypes = [ctypes.c_int]
    L.pimul_shutdown.argtypes = []
    L.pimul_mul.argtypes = [_u64p, _sz, _u64p, _sz, _u64p, _sz, ctypes.POINTER(_sz)]
    L.pimul_mul_device.argtypes = [ctypes.c_void_p, _sz, ctypes.c_void_p, _sz, ctypes.c_void_p, ctypes.c_void_p]
    L.pimul_plan.argtypes = [_sz, _sz, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_int)]
    L.pimul_sync.argtypes = []
    L.pimul_bbp_hex_digits.argtypes = [_u64p, _sz, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)]
    L.pimul_bbp_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


lib = load


def _check(rc: int):
    if rc != PIMUL_OK:
        raise PimulError(rc, lib().pimul_last_error().decode())


def version() -> str:
    return lib().pimul_version().decode()


def init(device: int = 0):
    _check(lib().pimul_init(device))


def shutdown():
    _check(lib().pimul_shutdown())


def sync():
    _check(lib().pimul_sync())


def _limbs(x) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint64))


def mul_mag_ntt(a, b) -> np.ndarray:
    """Exact product of two little-endian u64 limb arrays (trimmed)."""
    a = _limbs(a)
    b_is_a = b is a
    b = a if b_is_a else _limbs(b)
    if a.size == 0 or b.size == 0:
        return np.zeros(0, dtype=np.uint64)
    out = np.empty(a.size + b.size, dtype=np.uint64)
    n = _sz(0)
    _check(lib().pimul_mul(a.ctypes.data_as(_u64p), a.size, b.ctypes.data_as(_u64p), b.size,
                           out.ctypes.data_as(_u64p), out.size, ctypes.byref(n)))
    return out[: n.value]


def mul_device(d_a, d_b, d_out, stream=None):
    """d_out[:la+lb] = d_a * d_b on torch CUDA uint64/int64 tensors (async)."""
    la, lb = d_a.numel(), d_b.numel()
    if d_out.numel() < la + lb:
        raise PimulError(1, "output tensor too small")
    if stream is None:
        import torch
        stream = torch.cuda.current_stream(d_out.device).cuda_stream
    _check(lib().pimul_mul_device(d_a.data_ptr(), la, d_b.data_ptr(), lb, d_out.data_ptr(),
                                  ctypes.c_void_p(stream)))


def bbp_hex_digits(positions, stop=None) -> np.ndarray:
    """8 hex digits of pi at each position (crates/pi-core/src/bbp.rs:52).

    `stop` may be a ctypes.c_int; setting it non-zero from another thread
    cancels the call (PimulError with code ECANCELED), like the reference's
    hex_digits_at_interruptible (bbp.rs:63)."""
    pos = np.ascontiguousarray(np.asarray(positions, dtype=np.uint64))
    out = np.zeros(pos.size, dtype=np.uint32)
    if pos.size == 0:
        return out
    rc = lib().pimul_bbp_hex_digits(pos.ctypes.data_as(_u64p), pos.size,
                                    out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                                    ctypes.byref(stop) if stop is not None else None)
    if rc:
        raise PimulError(rc, lib().pimul_bbp_last_error().decode())
    return out


def plan(la: int, lb: int):
    """(N, passes) the engine uses for an la x lb limb product."""
    n = ctypes.c_uint64(0)
    p = ctypes.c_int(0)
    _check(lib().pimul_plan(la, lb, ctypes.byref(n), ctypes.byref(p)))
    return n.value, p.value
