"""Host-side pi pipeline (the caller of the multiply), run on the CPU with
the oracle's multiply as its backend: digits must equal an independent
mpmath computation (tests/golden/pi_digits_100k.txt) and the reference's
FIRST_100 constant (crates/pi-core/src/algorithm/util.rs:126-127)."""
import os

import pytest

import oracle as O
import pi_gb300 as pm

HERE = os.path.dirname(os.path.abspath(__file__))


def ref_digits():
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        return f.read().strip()


def test_first_100(golden):
    s, _ = pm.pi_chudnovsky(100, backend=O.mul_abi_pointer())
    assert s == golden["first_100_digits"].replace(".", "")


@pytest.mark.parametrize("digits,thr", [(1, 0), (2, 0), (50, 0), (1000, 0), (4321, 64), (30000, 64)])
def test_digits_vs_mpmath(digits, thr):
    s, info = pm.pi_chudnovsky(digits, backend=O.mul_abi_pointer(), ntt_threshold=thr)
    assert s == ref_digits()[:digits]
    if thr:
        assert info["ntt_products"] > 0  # the backend saw the large products


@pytest.mark.parametrize("digits,thr", [(1, 0), (100, 0), (3000, 64), (20000, 256)])
def test_gauss_legendre_vs_mpmath(digits, thr):
    s, info = pm.pi_gauss_legendre(digits, backend=O.mul_abi_pointer(), ntt_threshold=thr)
    assert s == ref_digits()[:digits]


@pytest.mark.parametrize("digits,thr", [(1, 0), (100, 0), (5000, 64), (30000, 256)])
def test_gauss_legendre_fast_sqrt_vs_mpmath(digits, thr):
    s, _ = pm.pi_gauss_legendre(digits, backend=O.mul_abi_pointer(), ntt_threshold=thr, fast_sqrt=True)
    assert s == ref_digits()[:digits]


def test_concurrent_calls_are_independent():
    # The drivers keep their backend, threshold, error and statistics per
    # call: two Chudnovsky runs and a Gauss-Legendre run with different
    # thresholds, started from three host threads at once, each give the
    # golden digits and count only their own backend calls.
    import threading

    ref = ref_digits()
    res = {}

    def run(key, fn):
        try:
            res[key] = fn()
        except Exception as e:  # noqa: BLE001
            res[key] = e

    jobs = {
        "ch64": lambda: pm.pi_chudnovsky(100_000, backend=O.mul_abi_pointer(), ntt_threshold=64),
        "ch8192": lambda: pm.pi_chudnovsky(100_000, backend=O.mul_abi_pointer()),
        "gl256": lambda: pm.pi_gauss_legendre(30_000, backend=O.mul_abi_pointer(), ntt_threshold=256),
    }
    th = [threading.Thread(target=run, args=(k, f)) for k, f in jobs.items()]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for k, v in res.items():
        assert not isinstance(v, Exception), (k, v)
    assert res["ch64"][0] == ref and res["ch8192"][0] == ref
    assert res["gl256"][0] == ref[:30_000]
    # the 8192-limb threshold sends nothing to the backend at 10^5 digits
    assert res["ch8192"][1]["ntt_products"] == 0
    assert res["ch64"][1]["ntt_products"] > 0


def test_backend_error_stops_the_run():
    # A backend that fails (PIMUL_ENOMEM) stops the pipeline at once: the
    # call returns that code and issues no further products (at most the
    # few already in flight on other helper threads reach the backend).
    import ctypes
    import time

    calls = []
    FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t,
                          ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t))

    def failing(a, la, b, lb, out, cap, n):
        calls.append(la + lb)
        return 2  # PIMUL_ENOMEM

    cb = FN(failing)
    addr = ctypes.cast(cb, ctypes.c_void_p).value
    for run in (lambda: pm.pi_chudnovsky(100_000, backend=addr, ntt_threshold=64),
                lambda: pm.pi_gauss_legendre(20_000, backend=addr, ntt_threshold=64)):
        calls.clear()
        t0 = time.perf_counter()
        with pytest.raises(pm.PimulError) as e:
            run()
        assert e.value.code == 2
        assert 1 <= len(calls) <= 16, len(calls)
        assert time.perf_counter() - t0 < 5.0
    # a good run afterwards is unaffected
    s, _ = pm.pi_chudnovsky(2000, backend=O.mul_abi_pointer(), ntt_threshold=64)
    assert s == ref_digits()[:2000]
