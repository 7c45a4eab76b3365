"""Sums of two products in the transform domain (pimul_sum_batch) and
spectra shared by products with the same operand b (pimul_mul_batch and
pimul_sum_batch), against Python's exact integers.  These are the engine's
forms of a binary-splitting level's T = T_L Q_R + P_L T_R and of a decimal
conversion level's products by one divisor
(crates/pi-core/src/algorithm/chudnovsky.rs:399-413,
crates/bignum/src/integer.rs:892-983)."""
import numpy as np
import pytest

import oracle as O
import pi_gb300 as pm

pytestmark = pytest.mark.gpu


def _t(v):
    import torch
    return torch.from_numpy(O.int_to_limbs(v).view(np.int64).copy()).cuda()


def _rand(rng, n):
    v = rng.integers(0, 2**64, n, dtype=np.uint64)
    v[-1] |= np.uint64(1 << 63)
    return O.limbs_to_int(v)


def _val(t):
    return O.limbs_to_int(t.cpu().numpy().view(np.uint64))


def test_sums_of_products_match_python():
    import torch
    rng = np.random.default_rng(11)
    shapes = [  # (la1, lb1, la2, lb2): short, long, unbalanced, one pair empty
        (3, 5, 2, 2), (700, 600, 500, 650), (2000, 2100, 1500, 2500), (9000, 8000, 7000, 9500),
        (40000, 39000, 25000, 41000), (100000, 3, 99000, 5), (5000, 6000, 0, 0), (0, 0, 7000, 300),
        (131072, 131072, 131071, 131072)]
    jobs, want = [], []
    for la1, lb1, la2, lb2 in shapes:
        a1, b1 = (_rand(rng, la1), _rand(rng, lb1)) if la1 else (0, 0)
        a2, b2 = (_rand(rng, la2), _rand(rng, lb2)) if la2 else (0, 0)
        n = max(la1 + lb1, la2 + lb2) + 3  # extra limbs must come back zero
        out = torch.full((n,), -1, dtype=torch.int64, device="cuda")
        jobs.append((_t(a1) if la1 else None, _t(b1) if la1 else None,
                     _t(a2) if la2 else None, _t(b2) if la2 else None, out))
        want.append(a1 * b1 + a2 * b2)
    pm.sum_batch(jobs)
    torch.cuda.synchronize()
    for j, w in zip(jobs, want):
        assert _val(j[4]) == w


def test_sums_with_squares_and_all_ones():
    import torch
    rng = np.random.default_rng(12)
    x = (1 << (64 * 30000)) - 1  # all-ones limbs: the largest coefficients and carries
    y = _rand(rng, 30000)
    tx, ty = _t(x), _t(y)
    outs = [torch.empty(60001, dtype=torch.int64, device="cuda") for _ in range(3)]
    pm.sum_batch([(tx, tx, ty, ty, outs[0]), (tx, ty, tx, ty, outs[1]), (tx, tx, tx, tx, outs[2])])
    torch.cuda.synchronize()
    assert _val(outs[0]) == x * x + y * y
    assert _val(outs[1]) == 2 * x * y
    assert _val(outs[2]) == 2 * x * x


def test_shared_operand_spectra_in_a_batch():
    import torch
    rng = np.random.default_rng(13)
    v = _rand(rng, 20000)
    tv = _t(v)
    xs = [_rand(rng, 20000 + 37 * k) for k in range(6)]
    outs = [torch.empty(20000 + 37 * k + 20000, dtype=torch.int64, device="cuda") for k in range(6)]
    # six products with the same b; plus a second length sharing nothing
    w = _rand(rng, 3000)
    tw = _t(w)
    o2 = torch.empty(3000 + 20000, dtype=torch.int64, device="cuda")
    pm.mul_batch([(_t(x), tv, o) for x, o in zip(xs, outs)] + [(tw, tv, o2)])
    torch.cuda.synchronize()
    for x, o in zip(xs, outs):
        assert _val(o) == x * v
    assert _val(o2) == w * v


def test_sum_sharing_b_with_a_product():
    # the splitting level's shape: Q = Q_L Q_R and T = T_L Q_R + P_L T_R in
    # one batch share Q_R's spectrum
    import torch
    rng = np.random.default_rng(14)
    for n in (5000, 60000):
        ql, qr, tl, tr, pl = (_rand(rng, n + d) for d in (0, 3, 5, 7, -n // 3))
        tqr = _t(qr)
        oq = torch.empty(2 * n + 3, dtype=torch.int64, device="cuda")
        ot = torch.empty(2 * n + 13, dtype=torch.int64, device="cuda")
        pm.sum_batch([(_t(ql), tqr, None, None, oq), (_t(tl), tqr, _t(pl), _t(tr), ot)])
        torch.cuda.synchronize()
        assert _val(oq) == ql * qr
        assert _val(ot) == tl * qr + pl * tr


def test_wrapped_products_and_sums_match_unwrapped():
    # PIMUL_BATCH_WRAP: jobs whose coefficients fill at most 5/8 of their
    # transform run as cyclic products of half the length plus a short
    # product of the low limbs; results must equal the plain batch's (and
    # Python's for the smaller shapes).  Shapes: just past 2^20 and 2^22
    # coefficients, a fused sum, two products sharing b, a square, all-ones
    # operands (largest coefficients and carries), and one job too full to wrap.
    import torch
    rng = np.random.default_rng(21)
    ones = (1 << (64 * 140000)) - 1
    b_shared = _rand(rng, 135000)
    sq = _rand(rng, 140000)
    specs = [  # (a1, b1, a2, b2, check with Python)
        (_rand(rng, 140000), _rand(rng, 140000), 0, 0, True),
        (_rand(rng, 140000), _rand(rng, 135000), _rand(rng, 100000), _rand(rng, 170000), True),
        (_rand(rng, 150000), b_shared, 0, 0, True),
        (_rand(rng, 145000), b_shared, 0, 0, False),
        (sq, sq, 0, 0, True),
        (ones, ones, 0, 0, True),
        (_rand(rng, 550000), _rand(rng, 560000), 0, 0, False),
        (_rand(rng, 200000), _rand(rng, 200000), 0, 0, False),
        # 3 wrapped coefficients; the largest wrap allowed (2^18 - 1 of 2^20)
        (_rand(rng, 131073), _rand(rng, 131072), 0, 0, True),
        (_rand(rng, 163840), _rand(rng, 163840), 0, 0, True),
    ]
    tens = {}

    def t(v):
        if id(v) not in tens:
            tens[id(v)] = _t(v)
        return tens[id(v)]

    def lim(v):
        return (v.bit_length() + 63) // 64

    plain, wrapped = [], []
    for a1, b1, a2, b2, _ in specs:
        n = max(lim(a1) + lim(b1), lim(a2) + lim(b2)) + (1 if a2 else 0)
        for dst in (plain, wrapped):
            out = torch.full((n,), -1, dtype=torch.int64, device="cuda")
            dst.append((t(a1), t(b1), t(a2) if a2 else None, t(b2) if a2 else None, out))
    pm.sum_batch(plain)
    pm.sum_batch(wrapped, wrap=True)
    torch.cuda.synchronize()
    for (a1, b1, a2, b2, check), p, w in zip(specs, plain, wrapped):
        assert torch.equal(p[4], w[4]), (lim(a1), lim(b1), lim(a2), lim(b2))
        if check:
            assert _val(w[4]) == a1 * b1 + a2 * b2
