"""The arithmetic the BBP series kernel relies on, restated step for step
with Python integers and checked against exact division (no GPU).

The kernel sums floor((16^e mod d) 2^64 / d) over terms (bbp.rs:117-140)
and computes each term without a division:
  * d = 2^t m with m odd, p = 16^e mod d, r' = 2^(4e + 64 - t) mod m;
  * then q = ((p mod 2^t) 2^(64-t) - r') m^-1 mod 2^64 is exactly the
    floor, since p 2^(64-t) = q m + r' with q < 2^64;
  * r' comes from Montgomery squarings (R = 2^32 below 2^32) with one
    doubling per set exponent bit;
  * the Montgomery product's carry and borrow test is done in 32-bit words.
"""
import random

M32 = (1 << 32) - 1
M64 = (1 << 64) - 1


def mont_mul32(a, b, m, minv):
    # 32-bit words: t = a b = (th:tl), u = tl minv; t + u m has low word 0
    # and carries into the high word exactly when tl != 0
    t = a * b
    tl, th = t & M32, t >> 32
    u = (tl * minv) & M32
    s = th + ((u * m) >> 32) + (1 if tl else 0)
    h, c = s & M32, s >> 32
    borrow = 1 if h < m else 0
    return (h - m) & M32 if c - borrow >= 0 else h


def dbl_mod32(x, m):
    s = 2 * x
    lo, c = s & M32, s >> 32
    return (lo - m) & M32 if c - (1 if lo < m else 0) >= 0 else lo


def pow2_mod_odd32(E, m):
    minv = (-pow(m, -1, 1 << 32)) % (1 << 32)
    x = ((1 << 32) - m) % m  # R mod m, the Montgomery one
    eh = E >> 32
    if eh:
        top = eh.bit_length() - 1
        x = dbl_mod32(x, m)
        for b in range(top - 1, -1, -1):
            x = mont_mul32(x, x, m, minv)
            if (eh >> b) & 1:
                x = dbl_mod32(x, m)
    el = E & M32
    for _ in range(32):
        x = mont_mul32(x, x, m, minv)
        if el & 0x80000000:
            x = dbl_mod32(x, m)
        el = (el << 1) & M32
    return mont_mul32(x, 1, m, minv)


def term(e, d):
    if d == 1:
        return 0
    t = (d & -d).bit_length() - 1
    m = d >> t
    lo = 0 if (t == 0 or 4 * e >= t) else 1 << (4 * e + 64 - t)
    if m == 1:
        return lo
    E = 4 * e + 64 - t
    r = pow2_mod_odd32(E, m) if m < (1 << 32) else pow(2, E, m)
    return ((lo - r) * pow(m, -1, 1 << 64)) & M64


def test_montgomery_carry_and_doubling():
    rng = random.Random(1)
    for _ in range(20000):
        m = rng.randrange(3, 1 << 32) | 1
        if rng.random() < 0.3:
            m = (1 << 32) - 1 - 2 * rng.randrange(1000)
        minv = (-pow(m, -1, 1 << 32)) % (1 << 32)
        a, b = rng.randrange(m), rng.randrange(m)
        assert mont_mul32(a, b, m, minv) == a * b * pow(1 << 32, -1, m) % m
        assert dbl_mod32(a, m) == 2 * a % m


def test_power_of_two_by_montgomery():
    rng = random.Random(2)
    for _ in range(3000):
        m = rng.randrange(3, 1 << 32) | 1
        E = rng.choice([rng.randrange(62, 300), rng.randrange(1 << 30, 1 << 32), rng.randrange(1 << 32, 1 << 35)])
        assert pow2_mod_odd32(E, m) == pow(2, E, m)


def test_exact_two_adic_term():
    rng = random.Random(3)
    cases = [(e, d) for e in range(12) for d in range(1, 80)]
    cases += [(rng.randrange(1 << 31), 8 * rng.randrange(1 << 31) + rng.choice([1, 4, 5, 6])) for _ in range(1500)]
    cases += [(rng.randrange(1 << 31), rng.randrange(1, 1 << 34)) for _ in range(1500)]
    for e, d in cases:
        assert term(e, d) == (pow(16, e, d) << 64) // d, (e, d)
