"""Parity of the CUDA multiply (through the C ABI) with the CPU oracle.

Bit-exact integer equality is the bar: every product must equal the
reference's CPU multiply on the same operands.
"""
import os
import threading

import numpy as np
import pytest

import oracle as O
import pi_gb300 as pm
from conftest import hexlimbs, rand_limbs, splitmix64_limbs

pytestmark = pytest.mark.gpu
M64 = (1 << 64) - 1
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def check(a, b, square=False):
    got = pm.mul_mag_ntt(a, a if square else b)
    want = O.mul_mag_ntt(a, a if square else b)
    assert got.dtype == np.uint64
    assert got.size == want.size, (got.size, want.size)
    assert np.array_equal(got, want)
    return got


def test_golden_products(golden):
    for c in golden["mul_cases"]:
        if "a" not in c:
            continue
        got = pm.mul_mag_ntt(hexlimbs(c["a"]), hexlimbs(c["b"]))
        assert np.array_equal(got, hexlimbs(c["out"])), c["name"]


def test_golden_digest_32768(golden):
    import hashlib
    c = next(c for c in golden["mul_cases"] if c["name"] == "bit_reverse_parallel_via_ntt_32768")
    P = O.P
    def rv(n, seed):
        s = (seed * 0x9E3779B97F4A7C15 + 1) & M64
        out = []
        for _ in range(n):
            s = (s * 6364136223846793005 + 1442695040888963407) & M64
            out.append(s % P)
        return np.array(out, dtype=np.uint64)
    got = pm.mul_mag_ntt(rv(32768, 0xAA), rv(32768, 0xBB))
    h = hashlib.sha256(got.astype("<u8").tobytes()).hexdigest()
    assert got.size == c["out_len"] and h == c["sha256"]


SIZES = [(1, 1), (1, 4), (4, 4), (8, 5), (32, 16), (60, 60), (200, 200), (255, 256), (256, 256),
         (511, 512), (512, 512), (513, 512), (1000, 3000), (3000, 1000), (1, 5000), (8192, 8192),
         (4096, 1), (10000, 12345), (1 << 15, 1 << 15), (1 << 16, 1 << 16), (1 << 17, 1 << 16),
         (1 << 18, 1 << 18),
         (1 << 18, 5), (3, 1 << 18), (1 << 19, 1 << 19)]


@pytest.mark.parametrize("la,lb", SIZES)
def test_sizes_vs_oracle(la, lb):
    check(rand_limbs(la, 7 * la + 1), rand_limbs(lb, 11 * lb + 2))


@pytest.mark.parametrize("n", [1, 2, 17, 256, 512, 1024, 4096, 1 << 14, 1 << 17, 1 << 20])
def test_squares(n):
    check(rand_limbs(n, n), None, square=True)


def test_splitmix_operands():
    check(splitmix64_limbs(3000, 1), splitmix64_limbs(2000, 2))


@pytest.mark.parametrize("n", [1, 3, 64, 1000, 1 << 12, 1 << 16, 1 << 18])
def test_all_ones_carry_chains(n):
    ones = np.full(n, M64, dtype=np.uint64)
    check(ones, ones)  # (2^k - 1)^2
    # (2^k - 1) * (2^k + 1) = 2^2k - 1: every output limb is all-ones,
    # so every window propagates and the carry scan crosses every chunk.
    plus = np.zeros(n + 1, dtype=np.uint64)
    plus[0] = 1
    plus[n] = 1
    got = pm.mul_mag_ntt(ones, plus)
    assert got.size == 2 * n and np.all(got == np.uint64(M64))


def test_sparse_and_unnormalised():
    a = np.zeros(5000, dtype=np.uint64)
    a[0], a[4999] = 1, 1 << 63
    b = np.zeros(7000, dtype=np.uint64)
    b[3500] = 12345
    check(a, b)
    # top zero limbs: the product is trimmed like the reference's unpack
    z = rand_limbs(300, 5)
    z[-10:] = 0
    check(z, rand_limbs(400, 6))
    e = np.zeros(0, dtype=np.uint64)
    assert pm.mul_mag_ntt(e, rand_limbs(10, 1)).size == 0
    assert pm.mul_mag_ntt(np.zeros(9, dtype=np.uint64), rand_limbs(10, 1)).size == 0


def test_errors_do_not_touch_gpu():
    lib = pm.lib()
    import ctypes
    a = rand_limbs(4, 1)
    out = np.empty(3, dtype=np.uint64)
    n = ctypes.c_size_t(0)
    p = a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64))
    rc = lib.pimul_mul(p, 4, p, 4, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), 3, ctypes.byref(n))
    assert rc == 1 and b"out_cap" in lib.pimul_last_error()


def test_device_api_matches_host_api():
    import torch
    a, b = rand_limbs(70000, 1), rand_limbs(50000, 2)
    want = O.mul_mag_ntt(a, b)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        da = torch.from_numpy(a.view(np.int64)).cuda()
        db = torch.from_numpy(b.view(np.int64)).cuda()
        out = torch.empty(a.size + b.size, dtype=torch.int64, device="cuda")
        pm.mul_device(da, db, out)
        # square through the device API (same pointer twice)
        sq = torch.empty(2 * a.size, dtype=torch.int64, device="cuda")
        pm.mul_device(da, da, sq)
    s.synchronize()
    got = out.cpu().numpy().view(np.uint64)
    got = got[: want.size] if got[-1] == 0 else got
    assert np.array_equal(np.trim_zeros(got, "b"), want)
    sq_got = np.trim_zeros(sq.cpu().numpy().view(np.uint64), "b")
    assert np.array_equal(sq_got, O.mul_mag_ntt(a, a))


def test_concurrent_callers():
    # mul_mag_ntt is called from many rayon workers at once in the reference
    # (crates/pi-core/src/algorithm/chudnovsky.rs:349-359); the C ABI is
    # re-entrant: each calling thread gets its own stream.
    jobs = [(rand_limbs(3000 + 17 * i, i), rand_limbs(2000 + 31 * i, 100 + i)) for i in range(8)]
    wants = [O.mul_mag_ntt(a, b) for a, b in jobs]
    errs = []

    def work(k):
        try:
            for _ in range(3):
                a, b = jobs[k]
                if not np.array_equal(pm.mul_mag_ntt(a, b), wants[k]):
                    errs.append(k)
        except Exception as e:  # noqa: BLE001
            errs.append(repr(e))

    th = [threading.Thread(target=work, args=(k,)) for k in range(8)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errs, errs


# --------------------------------------------------------------- full sizes
# The isolated-multiply sweep's sizes, compared with the oracle bit for bit
# (the oracle runs a 2^30 x 2^30-bit product in a few seconds on all host
# cores): balanced 2^24, 2^28 and 2^30 bits, the unbalanced 2^30 x 2^20,
# and squares at 2^24, 2^28 and 2^30 bits.
@pytest.mark.parametrize("bits_a,bits_b", [(1 << 24, 1 << 24), (1 << 28, 1 << 28), (1 << 30, 1 << 30),
                                           (1 << 30, 1 << 20), (1 << 20, 1 << 30)])
def test_full_size_exact_vs_oracle(bits_a, bits_b):
    la, lb = bits_a // 64, bits_b // 64
    got = check(rand_limbs(la, 101 + la), rand_limbs(lb, 202 + lb))
    assert got.size == la + lb or got.size == la + lb - 1


@pytest.mark.parametrize("bits", [1 << 24, 1 << 28, 1 << 30])
def test_full_size_square_exact_vs_oracle(bits):
    n = bits // 64
    got = check(rand_limbs(n, 303 + n), None, square=True)
    assert got.size in (2 * n, 2 * n - 1)


def test_computed_twiddles_match_oracle_in_fresh_process():
    # With the twiddle-table cache capped at 0 before the first product, every
    # pass computes its twiddles from the root tables (the path transforms
    # longer than 2^28 take, and the no-alloc entry point's): products at
    # N = 2^21, 2^24 and 2^27 must still equal the oracle's.
    import subprocess
    import sys
    code = r"""
import sys, numpy as np
sys.path.insert(0, %r)
import pi_gb300 as pm, oracle as O
from conftest import rand_limbs
pm.init(0)
assert pm.twiddle_cache(0) == 0
for la, lb in ((1 << 18, 1 << 18), (1 << 21, 1 << 21), (1 << 24, 1 << 24), (1 << 21, 3)):
    a, b = rand_limbs(la, la + 5), rand_limbs(lb, lb + 6)
    assert np.array_equal(pm.mul_mag_ntt(a, b), O.mul_mag_ntt(a, b)), (la, lb)
assert pm.twiddle_cache(0) == 0
print("ok")
""" % (os.path.dirname(os.path.abspath(__file__)),)
    env = dict(os.environ)
    env["PYTHONPATH"] = os.pathsep.join([ROOT, env.get("PYTHONPATH", "")])
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr


def test_twiddle_tables_are_cached():
    # the first product at a length builds its tables; later ones reuse them
    before = pm.twiddle_cache(8 << 30)
    a, b = rand_limbs(5000, 1), rand_limbs(7000, 2)
    check(a, b)
    mid = pm.twiddle_cache(8 << 30)
    check(a, b)
    assert pm.twiddle_cache(8 << 30) == mid >= before
