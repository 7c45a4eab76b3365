"""The multiply entry point that allocates nothing (pimul_mul_device_noalloc).

It serves callers that cannot allocate device memory while they multiply:
a GPU whose memory is owned by another allocator, a loop where cudaMalloc's
implicit synchronisation is not allowed, a runtime that allocates only at
start-up.  Its scratch is a fixed array inside the library, so products are
limited to la + lb <= 262144 limbs.

The test calls it through the C ABI, twice in a row (the second call finds
the first call's data still in the shared scratch), and requires each result
to equal the pool-backed entry point's result bit for bit.  All device
buffers are allocated by the test before the calls.
"""
import ctypes

import numpy as np
import pytest

import pi_gb300 as pm
from conftest import rand_limbs

pytestmark = pytest.mark.gpu


def _fn(lib):
    f = lib.pimul_mul_device_noalloc
    f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                  ctypes.c_void_p]
    f.restype = ctypes.c_int
    return f


def _dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x).view(np.int64)).cuda()


# (la, lb) pairs, each run as two calls in a row: a one-CTA product (N <= 2^12)
# followed by a 2-pass one (3000 x 1500 limbs, N = 2^15); two multi-pass
# products; a product at the size limit (N = 2^20) followed by a small one
CASES = [
    ((3, 5), (3000, 1500)),
    ((20000, 9000), (1 << 17, 1 << 17)),
    ((100000, 162144), (4096, 4096)),
]


@pytest.mark.parametrize("first,second", CASES)
def test_noalloc_matches_pool_entry_point_twice(first, second):
    import torch
    lib = pm.lib()
    noalloc = _fn(lib)
    s = torch.cuda.Stream()
    jobs = []
    for k, (la, lb) in enumerate((first, second)):
        a = rand_limbs(la, 1000 + 7 * k + la)
        b = rand_limbs(lb, 2000 + 11 * k + lb)
        with torch.cuda.stream(s):
            da, db = _dev(a), _dev(b)
            ref = torch.zeros(la + lb, dtype=torch.int64, device="cuda")
            got = torch.full((la + lb,), -1, dtype=torch.int64, device="cuda")
        s.synchronize()
        jobs.append((da, la, db, lb, ref, got))
    sp = ctypes.c_void_p(s.cuda_stream)
    for da, la, db, lb, ref, _ in jobs:
        assert lib.pimul_mul_device(da.data_ptr(), la, db.data_ptr(), lb, ref.data_ptr(), sp) == 0
    s.synchronize()
    # two calls in a row on the shared scratch
    for da, la, db, lb, _, got in jobs:
        rc = noalloc(da.data_ptr(), la, db.data_ptr(), lb, got.data_ptr(), sp)
        assert rc == 0, lib.pimul_last_error()
    s.synchronize()
    for da, la, db, lb, ref, got in jobs:
        assert torch.equal(got, ref), (la, lb)


@pytest.mark.parametrize("n", [50000, 1 << 17])
def test_noalloc_square_and_repeat(n):
    # 2^17 limbs squared is the largest square the fixed scratch holds (N = 2^20)
    import torch
    lib = pm.lib()
    noalloc = _fn(lib)
    a = rand_limbs(n, 77 + n)
    da = _dev(a)
    ref = torch.zeros(2 * a.size, dtype=torch.int64, device="cuda")
    out1 = torch.zeros_like(ref)
    out2 = torch.zeros_like(ref)
    torch.cuda.synchronize()
    assert lib.pimul_mul_device(da.data_ptr(), a.size, da.data_ptr(), a.size, ref.data_ptr(), None) == 0
    lib.pimul_sync()
    for out in (out1, out2):
        assert noalloc(da.data_ptr(), a.size, da.data_ptr(), a.size, out.data_ptr(), None) == 0
        torch.cuda.synchronize()
    assert torch.equal(out1, ref) and torch.equal(out2, ref)


def test_noalloc_rejects_products_above_the_limit():
    import torch
    lib = pm.lib()
    noalloc = _fn(lib)
    t = torch.zeros(4, dtype=torch.int64, device="cuda")
    p = t.data_ptr()
    # the size check runs on the host before any device work
    assert noalloc(p, 1 << 17, p, (1 << 17) + 1, p, None) == 1
    assert b"262144" in lib.pimul_last_error()
    # sizes whose sum wraps around in size_t are rejected too
    assert noalloc(p, (1 << 64) - 1, p, 2, p, None) == 1
    assert noalloc(p, 1 << 63, p, 1 << 63, p, None) == 1
    assert noalloc(p, 2, p, (1 << 64) - 1, p, None) == 1
