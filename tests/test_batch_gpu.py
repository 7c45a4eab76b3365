"""Batched and graph-planned products: every product equals the plain
per-call product (and the CPU oracle) bit for bit."""
import numpy as np
import pytest

import oracle as O
import pi_gb300 as pm

pytestmark = pytest.mark.gpu


def _rand_sizes(n, lo_bits, hi_bits, seed):
    rng = np.random.default_rng(seed)
    bits = np.exp(rng.uniform(np.log(lo_bits), np.log(hi_bits), size=(n, 2)))
    return np.maximum(1, (bits // 64).astype(np.int64))


def _make(sizes, seed, squares=()):
    import torch
    rng = np.random.default_rng(seed)
    jobs, host = [], []
    for k, (la, lb) in enumerate(sizes):
        a = rng.integers(0, 1 << 64, size=int(la), dtype=np.uint64)
        a[-1] |= np.uint64(1 << 63)
        da = torch.from_numpy(a.view(np.int64)).cuda()
        if k in squares:
            b, db = a, da
        else:
            b = rng.integers(0, 1 << 64, size=int(lb), dtype=np.uint64)
            b[-1] |= np.uint64(1 << 63)
            db = torch.from_numpy(b.view(np.int64)).cuda()
        out = torch.full((a.size + b.size,), -1, dtype=torch.int64, device="cuda")
        jobs.append((da, db, out))
        host.append((a, b))
    return jobs, host


def _plain(jobs):
    import torch
    outs = []
    for da, db, o in jobs:
        r = torch.zeros_like(o)
        pm.mul_device(da, db, r)
        outs.append(r)
    torch.cuda.synchronize()
    return outs


def test_batch_matches_plain_and_oracle():
    import torch
    sizes = _rand_sizes(300, 2 ** 10, 2 ** 20, 1)
    sizes = np.concatenate([sizes, [[1, 1], [3, 700], [40000, 30000], [65536, 65536], [1, 60000]]])
    jobs, host = _make(sizes, 2, squares={5, 17, 301})
    pm.mul_batch(jobs)
    torch.cuda.synchronize()
    ref = _plain(jobs)
    for (da, db, o), r in zip(jobs, ref):
        assert torch.equal(o, r)
    for k in (0, 5, 17, 123, 301, 303):
        a, b = host[k]
        got = np.trim_zeros(jobs[k][2].cpu().numpy().view(np.uint64), "b")
        assert np.array_equal(got, O.mul_mag_ntt(a, b))


def test_plan_replays_with_new_operands():
    import torch
    sizes = _rand_sizes(200, 2 ** 10, 2 ** 22, 3)
    sizes[7, 1] = sizes[7, 0]  # job 7 becomes a square in the second run
    plan = pm.BatchPlan(sizes[:, 0], sizes[:, 1])
    try:
        for seed in (4, 5):
            jobs, _ = _make(sizes, seed, squares={7} if seed == 5 else ())
            plan.run(jobs)
            torch.cuda.synchronize()
            for (da, db, o), r in zip(jobs, _plain(jobs)):
                assert torch.equal(o, r)
    finally:
        plan.close()


def test_plan_rejects_other_shapes():
    sizes = _rand_sizes(10, 2 ** 10, 2 ** 14, 6)
    plan = pm.BatchPlan(sizes[:, 0], sizes[:, 1])
    try:
        jobs, _ = _make(sizes[:9], 7)
        with pytest.raises(pm.PimulError):
            plan.run(jobs)
    finally:
        plan.close()


def test_autotune_keeps_products_exact():
    import torch
    choices = pm.autotune(12, 15, 2)
    assert "np_13" in choices and "small_ctas_per_sm" in choices
    pm.tuning_apply(choices)
    sizes = _rand_sizes(64, 2 ** 10, 2 ** 17, 9)
    jobs, _ = _make(sizes, 10)
    pm.mul_batch(jobs)
    torch.cuda.synchronize()
    for (da, db, o), r in zip(jobs, _plain(jobs)):
        assert torch.equal(o, r)
    # a split with no compiled first-pass kernel (2^6 x 2^6 x 2^6) is refused
    with pytest.raises(pm.PimulError):
        pm.tuning_apply({"np_18": 3})


def test_forced_four_pass_split_matches_oracle():
    # 2^25 transform: default 2^9 x 2^8 x 2^8, forced 2^7 x 2^6 x 2^6 x 2^6
    # (two middle column passes); both must give the oracle's product
    rng = np.random.default_rng(12)
    a = rng.integers(0, 2**63, 3_000_000, dtype=np.uint64) | np.uint64(1)
    b = rng.integers(0, 2**63, 2_900_000, dtype=np.uint64) | np.uint64(1)
    assert pm.plan(a.size, b.size) == (1 << 25, 3)
    want = O.mul_mag(a, b)
    pm.tuning_apply({"np_25": 4})
    try:
        assert pm.plan(a.size, b.size) == (1 << 25, 4)
        got4 = pm.mul_mag_ntt(a, b)
    finally:
        pm.tuning_apply({"np_25": 0})
    got3 = pm.mul_mag_ntt(a, b)
    assert np.array_equal(got3, want)
    assert np.array_equal(got4, want)


def test_empty_batch_and_zero_lengths():
    import torch
    pm.mul_batch([])
    z = torch.zeros(0, dtype=torch.int64, device="cuda")
    x = torch.ones(5, dtype=torch.int64, device="cuda")
    out = torch.full((5,), 7, dtype=torch.int64, device="cuda")
    pm.mul_batch([(z, x, out)])
    torch.cuda.synchronize()
    assert torch.equal(out, torch.full((5,), 7, dtype=torch.int64, device="cuda"))
