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
    "PimulError", "lib", "load", "version", "init", "mul_mag_ntt", "mul_device", "sum_batch", "SumJob",
    "plan", "sync", "bbp_hex_digits", "mul_batch", "BatchPlan", "autotune",
    "tuning_apply", "PimulJob", "set_budget", "upload", "submit", "wait", "download", "free",
    "handle_size", "pi_chudnovsky", "pi_gauss_legendre", "service_stats", "service_reset_stats", "OP_MUL", "OP_SQR", "OP_ADD", "OP_SUB", "release", "adopt", "handle_device", "pi_chudnovsky_served", "LIB_PATH",
    "decimal_to_hex", "convert_decimal_to_hex",
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
    L.pimul_mul_batch.argtypes = [ctypes.c_void_p, _sz, ctypes.c_void_p]
    L.pimul_addsub_batch.argtypes = [ctypes.c_void_p, _sz, ctypes.c_void_p]
    L.pimul_sum_batch.argtypes = [ctypes.c_void_p, _sz, ctypes.c_void_p]
    L.pimul_sum_batch_ex.argtypes = [ctypes.c_void_p, _sz, ctypes.c_void_p, ctypes.c_uint]
    L.pimul_top_limbs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _sz, ctypes.c_void_p, ctypes.c_void_p]
    L.pimul_batch_plan_create.argtypes = [ctypes.POINTER(_sz), ctypes.POINTER(_sz), _sz, ctypes.POINTER(ctypes.c_void_p)]
    L.pimul_batch_plan_run.argtypes = [ctypes.c_void_p, ctypes.c_void_p, _sz, ctypes.c_void_p]
    L.pimul_batch_plan_destroy.argtypes = [ctypes.c_void_p]
    L.pimul_autotune.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_char_p, _sz]
    L.pimul_tuning_set.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.pimul_set_budget.argtypes = [ctypes.c_uint64]
    L.pimul_twiddle_cache.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_service_config.argtypes = [ctypes.c_int, ctypes.c_int]
    L.pimul_upload.argtypes = [_u64p, _sz, ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_submit.argtypes = [ctypes.c_int, ctypes.c_uint64, ctypes.c_uint64, ctypes.POINTER(ctypes.c_uint64),
                               ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_wait.argtypes = [ctypes.c_uint64, ctypes.c_int64]
    L.pimul_handle_size.argtypes = [ctypes.c_uint64, ctypes.POINTER(_sz)]
    L.pimul_download.argtypes = [ctypes.c_uint64, _u64p, _sz, ctypes.POINTER(_sz)]
    L.pimul_free.argtypes = [ctypes.c_uint64]
    L.pimul_release.argtypes = [ctypes.c_uint64]
    L.pimul_adopt.argtypes = [ctypes.c_void_p, _sz, ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_handle_device.argtypes = [ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(_sz)]
    L.pimul_pi_chudnovsky_served.argtypes = [ctypes.c_uint64, ctypes.c_char_p, _sz, ctypes.c_uint64,
                                             ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64),
                                             ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_service_stats.argtypes = [ctypes.POINTER(ctypes.c_double)] * 2 + [ctypes.POINTER(ctypes.c_uint64)] * 3
    L.pimul_service_reset_stats.argtypes = []
    L.pimul_pi_chudnovsky.argtypes = [ctypes.c_uint64, ctypes.c_char_p, _sz, ctypes.c_void_p, ctypes.c_uint64,
                                      ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64),
                                      ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_pi_chudnovsky_batched.argtypes = [ctypes.c_uint64, ctypes.c_char_p, _sz, ctypes.c_uint64,
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64),
                                              ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_to_decimal.argtypes = [_u64p, _sz, ctypes.c_char_p, _sz, ctypes.POINTER(_sz), ctypes.c_int]
    L.pimul_decimal_to_hex.argtypes = [ctypes.c_char_p, _sz, ctypes.c_char_p, _sz, ctypes.POINTER(_sz),
                                       ctypes.POINTER(ctypes.c_double)]
    L.pimul_pi_gauss_legendre_ex.argtypes = [ctypes.c_uint64, ctypes.c_char_p, _sz, ctypes.c_void_p, ctypes.c_uint64,
                                             ctypes.c_uint32, ctypes.POINTER(ctypes.c_double),
                                             ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_pi_gauss_legendre.argtypes = [ctypes.c_uint64, ctypes.c_char_p, _sz, ctypes.c_void_p, ctypes.c_uint64,
                                          ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_uint64)]
    L.pimul_bbp_hex_digits.argtypes = [_u64p, _sz, ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int)]
    L.pimul_bbp_last_error.restype = ctypes.c_char_p
    L.pimul_bbp_modops.argtypes = [_u64p, _u64p, _u64p, _sz, _u64p, _u64p]
    L.pimul_bbp_terms.argtypes = [_u64p, _u64p, _sz, _u64p]
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


class AddSubJob(ctypes.Structure):
    _fields_ = [("x", ctypes.c_void_p), ("nx", _sz), ("y", ctypes.c_void_p), ("ny", _sz),
                ("out", ctypes.c_void_p), ("nout", _sz), ("sub", ctypes.c_int)]


def addsub_batch(jobs, stream=None):
    """Batched add/subtract of torch CUDA uint64/int64 tensors:
    jobs = [(x, y, out, sub)], out = x + y or x - y (x >= y) over out.numel()
    limbs (pimul_addsub_batch; synchronous)."""
    arr = (AddSubJob * len(jobs))()
    for i, (x, y, out, sub) in enumerate(jobs):
        arr[i] = AddSubJob(x.data_ptr() if x.numel() else None, x.numel(), y.data_ptr() if y.numel() else None,
                           y.numel(), out.data_ptr(), out.numel(), int(bool(sub)))
    if stream is None and jobs:
        import torch
        stream = torch.cuda.current_stream(jobs[0][2].device).cuda_stream
    _check(lib().pimul_addsub_batch(arr, len(jobs), ctypes.c_void_p(stream) if stream else None))


class SumJob(ctypes.Structure):
    """struct pimul_sum_job of include/pimul.h (device pointers)."""
    _fields_ = [("a1", ctypes.c_void_p), ("la1", _sz), ("b1", ctypes.c_void_p), ("lb1", _sz),
                ("a2", ctypes.c_void_p), ("la2", _sz), ("b2", ctypes.c_void_p), ("lb2", _sz),
                ("out", ctypes.c_void_p), ("nout", _sz)]


def sum_batch(jobs, stream=None, wrap=False):
    """out = a1 * b1 + a2 * b2 for torch CUDA uint64/int64 tensors:
    jobs = [(a1, b1, a2, b2, out)] (a2, b2 may be None), over out.numel()
    limbs (pimul_sum_batch; asynchronous on the current torch stream).
    wrap=True: pimul_sum_batch_ex with PIMUL_BATCH_WRAP (half-full long
    transforms run as cyclic products of half the length)."""
    arr = (SumJob * max(len(jobs), 1))()

    def ptr(t):
        return (t.data_ptr() if t.numel() else None, t.numel()) if t is not None else (None, 0)

    for i, (a1, b1, a2, b2, out) in enumerate(jobs):
        arr[i] = SumJob(*ptr(a1), *ptr(b1), *ptr(a2), *ptr(b2), out.data_ptr(), out.numel())
    if stream is None and jobs:
        import torch
        stream = torch.cuda.current_stream(jobs[0][4].device).cuda_stream
    if wrap:
        _check(lib().pimul_sum_batch_ex(arr, len(jobs), ctypes.c_void_p(stream) if stream else None, 1))
    else:
        _check(lib().pimul_sum_batch(arr, len(jobs), ctypes.c_void_p(stream) if stream else None))


def top_limbs(arrays, stream=None):
    """Trimmed lengths of torch CUDA limb tensors (pimul_top_limbs)."""
    n = len(arrays)
    ptrs = (ctypes.c_uint64 * n)(*[a.data_ptr() for a in arrays])
    lens = (_sz * n)(*[a.numel() for a in arrays])
    out = (_sz * n)()
    if stream is None and arrays:
        import torch
        stream = torch.cuda.current_stream(arrays[0].device).cuda_stream
    _check(lib().pimul_top_limbs(ptrs, lens, n, out, ctypes.c_void_p(stream) if stream else None))
    return list(out)


class PimulJob(ctypes.Structure):
    """struct pimul_job of include/pimul.h (device pointers)."""
    _fields_ = [("a", ctypes.c_void_p), ("la", ctypes.c_size_t), ("b", ctypes.c_void_p),
                ("lb", ctypes.c_size_t), ("out", ctypes.c_void_p)]


def _job_array(jobs):
    """jobs: iterable of (d_a, d_b, d_out) torch CUDA tensors, or of
    (a_ptr, la, b_ptr, lb, out_ptr) integer tuples."""
    items = list(jobs)
    arr = (PimulJob * max(len(items), 1))()
    for i, j in enumerate(items):
        if len(j) == 3:
            a, b, o = j
            arr[i] = PimulJob(a.data_ptr(), a.numel(), b.data_ptr(), b.numel(), o.data_ptr())
        else:
            arr[i] = PimulJob(*j)
    return arr, len(items)


def _stream_ptr(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream


def mul_batch(jobs, stream=None):
    """Batched device products (one call for many independent products)."""
    arr, n = _job_array(jobs)
    _check(lib().pimul_mul_batch(ctypes.cast(arr, ctypes.c_void_p), n, ctypes.c_void_p(_stream_ptr(stream))))


class BatchPlan:
    """A fixed batch shape with its launch schedule captured in a CUDA graph."""

    def __init__(self, la, lb):
        la = list(la)
        lb = list(lb)
        if len(la) != len(lb):
            raise PimulError(1, "la and lb differ in length")
        self.n = len(la)
        A = (ctypes.c_size_t * max(self.n, 1))(*la)
        B = (ctypes.c_size_t * max(self.n, 1))(*lb)
        h = ctypes.c_void_p()
        _check(lib().pimul_batch_plan_create(A, B, self.n, ctypes.byref(h)))
        self._h = h

    def run(self, jobs, stream=None):
        arr, n = _job_array(jobs)
        _check(lib().pimul_batch_plan_run(self._h, ctypes.cast(arr, ctypes.c_void_p), n,
                                          ctypes.c_void_p(_stream_ptr(stream))))

    def close(self):
        if self._h:
            lib().pimul_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


def autotune(log_n_min=7, log_n_max=19, reps=8) -> dict:
    """Run the autotuner; returns its choices (also applied in-process)."""
    import json
    buf = ctypes.create_string_buffer(4096)
    _check(lib().pimul_autotune(log_n_min, log_n_max, reps, buf, 4096))
    return json.loads(buf.value.decode() or "{}")


def tuning_apply(choices: dict):
    """Re-apply choices returned by autotune() (e.g. loaded from a file)."""
    for k, v in choices.items():
        if k.startswith("np_"):
            _check(lib().pimul_tuning_set(int(k[3:]), int(v), 0))
        elif k == "small_ctas_per_sm":
            _check(lib().pimul_tuning_set(-1, 0, int(v)))


# ----------------------------------------------------------------- served form
OP_MUL, OP_SQR, OP_ADD, OP_SUB = 0, 1, 2, 3


def set_budget(nbytes: int):
    """HBM admission budget of the multiply service (default 120 GiB)."""
    _check(lib().pimul_set_budget(int(nbytes)))


def service_config(big_log_n: int = 0, max_batch: int = 0):
    """Service admission policy: transforms of 2^big_log_n and longer run
    alone; groups hold at most max_batch requests (0 leaves a value)."""
    _check(lib().pimul_service_config(int(big_log_n), int(max_batch)))


def twiddle_cache(max_bytes: int) -> int:
    """Cap of the pass-twiddle table cache in bytes (0: build no more
    tables; tables already built stay until shutdown).  Returns the bytes
    held."""
    held = ctypes.c_uint64(0)
    _check(lib().pimul_twiddle_cache(int(max_bytes), ctypes.byref(held)))
    return held.value


def upload(limbs) -> int:
    """Copy an integer (u64 limbs) to the device; returns its handle."""
    x = _limbs(limbs)
    h = ctypes.c_uint64(0)
    _check(lib().pimul_upload(x.ctypes.data_as(_u64p), x.size, ctypes.byref(h)))
    return h.value


def submit(a: int, b: int = None, op: int = None):
    """Queue a * b (or a * a); returns (result_handle, ticket) immediately."""
    if op is None:
        op = OP_SQR if b is None else OP_MUL
    h, t = ctypes.c_uint64(0), ctypes.c_uint64(0)
    _check(lib().pimul_submit(op, a, a if b is None else b, ctypes.byref(h), ctypes.byref(t)))
    return h.value, t.value


def wait(ticket: int, timeout_us: int = -1):
    _check(lib().pimul_wait(ticket, timeout_us))


def handle_size(h: int) -> int:
    n = _sz(0)
    _check(lib().pimul_handle_size(h, ctypes.byref(n)))
    return n.value


def download(h: int) -> np.ndarray:
    """The handle's value (trimmed limbs); waits for its producer."""
    cap = handle_size(h)
    out = np.zeros(max(cap, 1), dtype=np.uint64)
    n = _sz(0)
    _check(lib().pimul_download(h, out.ctypes.data_as(_u64p), out.size, ctypes.byref(n)))
    return out[: n.value].copy()


def free(h: int):
    _check(lib().pimul_free(h))


def release(h: int):
    """Free the handle once its producer and the requests reading it are done
    (returns at once)."""
    _check(lib().pimul_release(h))


def adopt(device_ptr: int, n: int) -> int:
    """A handle for n limbs of device memory the caller owns and keeps."""
    h = ctypes.c_uint64(0)
    _check(lib().pimul_adopt(ctypes.c_void_p(device_ptr), n, ctypes.byref(h)))
    return h.value


def handle_device(h: int):
    """(device address, stored limbs) of a handle; waits for its producer."""
    d = ctypes.c_void_p(0)
    n = _sz(0)
    _check(lib().pimul_handle_device(h, ctypes.byref(d), ctypes.byref(n)))
    return d.value, n.value


def _digit_buffer(n: int):
    """An uninitialised n + 1-byte output buffer for a driver that writes n
    digits (no zero fill of up to a gigabyte)."""
    buf = np.empty(n + 1, dtype=np.uint8)
    return buf, ctypes.cast(buf.ctypes.data, ctypes.c_char_p)


def _digits_str(buf, n: int) -> str:
    # one copy: ASCII bytes of the buffer straight into the str
    return str(memoryview(buf)[:n], "ascii")


def pi_chudnovsky_served(digits: int, serve_nodes: int = 0):
    """Digits of pi by Chudnovsky with the splitting tree's upper levels
    (above about serve_nodes nodes, 0: 512) submitted to the multiply service
    as chained handles (pimul_pi_chudnovsky_served).  Returns (digits_str, info)."""
    buf, pbuf = _digit_buffer(digits)
    ph = (ctypes.c_double * 3)()
    n = ctypes.c_uint64(0)
    req = ctypes.c_uint64(0)
    _check(lib().pimul_pi_chudnovsky_served(digits, pbuf, digits + 1, serve_nodes, ph, ctypes.byref(n),
                                            ctypes.byref(req)))
    info = {"binary_splitting_ms": ph[0], "final_assembly_ms": ph[1], "decimal_conversion_ms": ph[2],
            "ntt_products": n.value, "service_requests": req.value}
    return _digits_str(buf, digits), info


def service_stats() -> dict:
    p50, p99 = ctypes.c_double(0), ctypes.c_double(0)
    c, b, u = ctypes.c_uint64(0), ctypes.c_uint64(0), ctypes.c_uint64(0)
    _check(lib().pimul_service_stats(ctypes.byref(p50), ctypes.byref(p99), ctypes.byref(c), ctypes.byref(b),
                                     ctypes.byref(u)))
    return {"p50_ms": p50.value, "p99_ms": p99.value, "completed": c.value, "batches": b.value,
            "bytes_in_use": u.value}


def service_reset_stats():
    _check(lib().pimul_service_reset_stats())


def pi_chudnovsky(digits: int, backend=None, ntt_threshold: int = 0):
    """Digits of pi ("31415...") by Chudnovsky with large products on the GPU
    (crates/pi-core/src/algorithm/chudnovsky.rs:75).  `backend`: address of
    a pimul_mul_fn-compatible multiply (None = the GPU engine).  Returns
    (digits_str, info) with phase times and the backend-call histogram."""
    buf, pbuf = _digit_buffer(digits)
    ph = (ctypes.c_double * 3)()
    n = ctypes.c_uint64(0)
    hist = (ctypes.c_uint64 * 33)()
    _check(lib().pimul_pi_chudnovsky(digits, pbuf, digits + 1, ctypes.c_void_p(backend) if backend else None,
                                     ntt_threshold, ph, ctypes.byref(n), hist))
    info = {"binary_splitting_ms": ph[0], "final_assembly_ms": ph[1], "decimal_conversion_ms": ph[2],
            "ntt_products": n.value, "ntt_hist": {f"2^{L}": hist[L] for L in range(33) if hist[L]}}
    return _digits_str(buf, digits), info


def served_backend():
    """Address of pimul_mul_served (pimul_mul's contract through the served
    form), usable as the `backend` of pi_chudnovsky / pi_gauss_legendre."""
    return ctypes.cast(lib().pimul_mul_served, ctypes.c_void_p).value


def pi_chudnovsky_batched(digits: int, leaf_terms: int = 0):
    """Digits of pi by Chudnovsky with the binary splitting run level by level
    through the batched GPU multiply (pimul_pi_chudnovsky_batched); same
    digits as pi_chudnovsky.  Returns (digits_str, info)."""
    buf, pbuf = _digit_buffer(digits)
    ph = (ctypes.c_double * 3)()
    n = ctypes.c_uint64(0)
    lv = ctypes.c_uint64(0)
    hist = (ctypes.c_uint64 * 33)()
    _check(lib().pimul_pi_chudnovsky_batched(digits, pbuf, digits + 1, leaf_terms, ph, ctypes.byref(n),
                                             ctypes.byref(lv), hist))
    info = {"binary_splitting_ms": ph[0], "final_assembly_ms": ph[1], "decimal_conversion_ms": ph[2],
            "ntt_products": n.value, "batched_levels": lv.value,
            "ntt_hist": {f"2^{L}": hist[L] for L in range(33) if hist[L]}}
    return _digits_str(buf, digits), info


def to_decimal(limbs, batched: bool = True) -> str:
    """Decimal string of a non-negative integer given as u64 limbs
    (pimul_to_decimal; crates/bignum/src/integer.rs:892)."""
    a = _limbs(limbs)
    n = _sz(0)
    rc = lib().pimul_to_decimal(a.ctypes.data_as(_u64p), a.size, None, 0, ctypes.byref(n), int(batched))
    if n.value == 0:  # the length query itself failed
        _check(rc)
    buf = ctypes.create_string_buffer(n.value + 1)
    _check(lib().pimul_to_decimal(a.ctypes.data_as(_u64p), a.size, buf, n.value + 1, ctypes.byref(n),
                                  int(batched)))
    return buf.raw[: n.value].decode()


def decimal_to_hex(text, phases: bool = False):
    """verify-hex's conversion of pi's decimal text "3.ddd..." to "3.hhh..."
    (pimul_decimal_to_hex; crates/pi-cli/src/verify_hex.rs:553-629): the
    floor(N 16^h / 10^E) hex digits, computed on the GPU.  With phases, also
    returns the phase times in ms (parse, power of ten, quotient, hex)."""
    raw = text.encode() if isinstance(text, str) else bytes(text)
    n = _sz(0)
    rc = lib().pimul_decimal_to_hex(raw, len(raw), None, 0, ctypes.byref(n), None)
    if n.value == 0:  # the text was rejected before its length was known
        _check(rc)
    out = bytearray(n.value)  # written in place (no zero-filled ctypes buffer and copy)
    ph = (ctypes.c_double * 4)()
    dst = ctypes.cast((ctypes.c_char * len(out)).from_buffer(out), ctypes.c_char_p)
    _check(lib().pimul_decimal_to_hex(raw, len(raw), dst, n.value, ctypes.byref(n), ph))
    del dst
    res = out.decode("ascii")
    return (res, list(ph)) if phases else res


def convert_decimal_to_hex(decimal_path, hex_path):
    """The file form of verify_hex.rs:553-629: reads the decimal file, writes
    "3." + hex digits + a newline to hex_path through a .tmp file and a
    rename."""
    with open(decimal_path, "rb") as f:
        raw = f.read()
    out = decimal_to_hex(raw)
    hex_path = os.fspath(hex_path)
    tmp = os.path.splitext(hex_path)[0] + ".tmp"
    with open(tmp, "wb") as f:
        f.write(out.encode() + b"\n")
        f.flush()
        os.fsync(f.fileno())
    os.replace(tmp, hex_path)


def pi_gauss_legendre(digits: int, backend=None, ntt_threshold: int = 0, fast_sqrt: bool = False,
                      device_decimal: bool = False, device_agm: bool = False):
    """Digits of pi by the Gauss-Legendre AGM
    (crates/pi-core/src/algorithm/gauss_legendre.rs:61); fast_sqrt takes the
    square roots by a multiplication-only Newton iteration, device_decimal
    converts with the nodes on the GPU, device_agm runs the whole iteration
    on the GPU in fixed point (same digits)."""
    buf, pbuf = _digit_buffer(digits)
    ph = (ctypes.c_double * 3)()
    n = ctypes.c_uint64(0)
    flags = (1 if fast_sqrt else 0) | (2 if device_decimal else 0) | (4 if device_agm else 0)
    _check(lib().pimul_pi_gauss_legendre_ex(digits, pbuf, digits + 1, ctypes.c_void_p(backend) if backend else None,
                                            ntt_threshold, flags, ph, ctypes.byref(n)))
    return _digits_str(buf, digits), {"iterations_ms": ph[0], "decimal_conversion_ms": ph[2],
                                       "ntt_products": n.value}


def bbp_modops(e, d, p):
    """16^e mod d and floor(p 2^64 / d) on the device (pimul_bbp_modops)."""
    e, d, p = (np.ascontiguousarray(np.asarray(x, dtype=np.uint64)) for x in (e, d, p))
    pw = np.zeros(e.size, dtype=np.uint64)
    fr = np.zeros(e.size, dtype=np.uint64)
    rc = lib().pimul_bbp_modops(e.ctypes.data_as(_u64p), d.ctypes.data_as(_u64p), p.ctypes.data_as(_u64p), e.size,
                                pw.ctypes.data_as(_u64p), fr.ctypes.data_as(_u64p))
    if rc:
        raise PimulError(rc, lib().pimul_bbp_last_error().decode())
    return pw, fr


def bbp_terms(e, d):
    """floor((16^e mod d) 2^64 / d) on the device, the term the extractor
    sums (pimul_bbp_terms)."""
    e, d = (np.ascontiguousarray(np.asarray(x, dtype=np.uint64)) for x in (e, d))
    out = np.zeros(e.size, dtype=np.uint64)
    rc = lib().pimul_bbp_terms(e.ctypes.data_as(_u64p), d.ctypes.data_as(_u64p), e.size, out.ctypes.data_as(_u64p))
    if rc:
        raise PimulError(rc, lib().pimul_bbp_last_error().decode())
    return out


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
