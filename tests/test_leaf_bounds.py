"""The device leaf kernel (pi_gb300/csrc/leaves.cu) keeps every level of a
leaf in fixed shared-memory slots: for a node of m terms (k < 2^31) |P| in
2m limbs, Q in 3m and |T| in 3m + 2, and every merge's untrimmed |T| in
3m + 3.  Checked here with exact integers on term ranges up to 2^31, with
the splitting's static signs (P of m terms has sign (-1)^m, T < 0)."""
import random

A, B, C3_24 = 13591409, 545140134, 10939058860032000  # crates/pi-core/src/algorithm/chudnovsky.rs:57-61


def limbs(x):
    return (abs(x).bit_length() + 63) // 64


def pqt(a, b):
    if b - a == 1:
        k = a
        p = -(6 * k - 5) * (2 * k - 1) * (6 * k - 1)
        return p, C3_24 * k ** 3, p * (A + B * k)
    m = (a + b) // 2
    p1, q1, t1 = pqt(a, m)
    p2, q2, t2 = pqt(m, b)
    return p1 * p2, q1 * q2, t1 * q2 + p1 * t2


def test_leaf_slot_bounds_and_static_signs():
    rng = random.Random(7)
    starts = [1, 2, 1000, 70_000_000, 2 ** 31 - 64] + [rng.randint(1, 2 ** 31 - 64) for _ in range(6)]
    for k0 in starts:
        for m in (1, 2, 3, 4, 8, 16, 31, 32, 64):
            p, q, t = pqt(k0, k0 + m)
            assert limbs(p) <= 2 * m and limbs(q) <= 3 * m and limbs(t) <= 3 * m + 2, (k0, m)
            assert (p < 0) == (m % 2 == 1) and t < 0 and q > 0, (k0, m)
            if m >= 2:  # the merge that makes this node: untrimmed |T| length
                h = m // 2
                pl, ql, tl = pqt(k0, k0 + h)
                pr, qr, tr = pqt(k0 + h, k0 + m)
                assert max(limbs(tl) + limbs(qr), limbs(pl) + limbs(tr)) + 1 <= 3 * m + 3, (k0, m)
