"""Batched add/subtract and trimmed lengths on the device (the T sums of a
binary-splitting level, crates/bignum/src/integer.rs:351-421), against
Python's exact integers."""
import numpy as np
import pytest

import oracle as O
import pi_gb300 as pm

pytestmark = pytest.mark.gpu


def _t(v, n=None):
    import torch
    a = O.int_to_limbs(v)
    if n is not None:
        a = np.concatenate([a, np.zeros(n - a.size, dtype=np.uint64)])
    return torch.from_numpy(a.view(np.int64).copy()).cuda()


def _val(t):
    return O.limbs_to_int(t.cpu().numpy().view(np.uint64))


def test_random_adds_and_subtracts():
    import torch
    rng = np.random.default_rng(3)
    jobs, want = [], []
    for nx, ny in [(1, 1), (5, 3), (3, 5), (1000, 999), (4096, 1), (70000, 69000), (300000, 7)]:
        x = O.limbs_to_int(rng.integers(0, 2**64, nx, dtype=np.uint64))
        y = O.limbs_to_int(rng.integers(0, 2**64, ny, dtype=np.uint64))
        for sub in (0, 1):
            a, b = (max(x, y), min(x, y)) if sub else (x, y)
            n = max(nx, ny) + (0 if sub else 1)
            out = torch.empty(n, dtype=torch.int64, device="cuda")
            jobs.append((_t(a), _t(b), out, sub))
            want.append(a - b if sub else a + b)
    pm.addsub_batch(jobs)
    torch.cuda.synchronize()
    for (_, _, out, _), w in zip(jobs, want):
        assert _val(out) == w


def test_carries_and_borrows_across_chunks():
    import torch
    n = 50000  # many 1024-limb chunks
    cases = [((1 << (64 * n)) - 1, 1, 0), (1 << (64 * n), 1, 1), ((1 << (64 * n)) - 1, (1 << (64 * n)) - 1, 1)]
    jobs = []
    for x, y, sub in cases:
        out = torch.empty(n + 1, dtype=torch.int64, device="cuda")
        jobs.append((_t(x, n + 1), _t(y), out, sub))
    pm.addsub_batch(jobs)
    for (x, y, sub), (_, _, out, _) in zip(cases, jobs):
        assert _val(out) == (x - y if sub else x + y)
    lens = pm.top_limbs([j[2] for j in jobs])
    assert lens == [n + 1, n, 0]


def test_borrow_out_of_the_top_is_reported():
    import torch
    out = torch.empty(3, dtype=torch.int64, device="cuda")
    with pytest.raises(pm.PimulError):
        pm.addsub_batch([(_t(5, 3), _t(7), out, 1)])
