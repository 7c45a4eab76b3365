"""Decimal conversion of big integers (crates/bignum/src/integer.rs:892-983):
the reference's recursive divide and conquer on the host (CPU-only sizes
here) and the level-batched form with its nodes on the GPU, both against
Python's str()."""
import sys

import numpy as np
import pytest

import oracle as O
import pi_gb300 as pm


@pytest.fixture(autouse=True)
def _long_int_strings():
    old = sys.get_int_max_str_digits()
    sys.set_int_max_str_digits(0)
    yield
    sys.set_int_max_str_digits(old)


def _cases(rng):
    out = [0, 1, 9, 10, 10**19 - 1, 10**19, 10**38, 2**64 - 1, 2**64]
    for k in (300, 607, 608, 1000, 4000):
        out += [10**k, 10**k - 1, 10**k + 1]
    for nlimbs in (1, 3, 31, 32, 33, 257, 500, 1500):
        v = O.limbs_to_int(rng.integers(0, 2**63, nlimbs, dtype=np.uint64) | np.uint64(1 << 62))
        out.append(v)
    return out


def test_host_conversion_matches_python():
    rng = np.random.default_rng(5)
    for v in _cases(rng):
        assert pm.to_decimal(O.int_to_limbs(v), batched=False) == str(v)


@pytest.mark.gpu
def test_batched_conversion_matches_python():
    rng = np.random.default_rng(6)
    cases = _cases(rng)
    for nlimbs in (257, 2049, 20000):
        cases.append(O.limbs_to_int(rng.integers(0, 2**64, nlimbs, dtype=np.uint64)))
    # long runs of zero and nine chunks stress the quotient corrections
    cases += [10**6000 * 7 + 3, (10**5000 - 1) * 10**3000, 2**40000 - 1]
    # the level divisors 10^(19 2^k) themselves and their neighbours
    for k in (6, 8, 10):
        p = 10 ** (19 * 2**k)
        cases += [p - 1, p, p + 1, p * p - 1, 3 * p + p // 7]
    for v in cases:
        assert pm.to_decimal(O.int_to_limbs(v), batched=True) == str(v)


@pytest.mark.gpu
def test_batched_conversion_corrects_low_quotients(monkeypatch):
    # test hook: every quotient estimate lowered by one on the device, so
    # that every remainder goes through the r >= P correction
    monkeypatch.setenv("PIMUL_DEC_TEST_LOWER_Q", "1")
    rng = np.random.default_rng(7)
    p = 10 ** (19 * 2**8)
    cases = [10**6000 * 7 + 3, (10**5000 - 1) * 10**3000, 2**40000 - 1, p - 1, p, p * p - 1]
    for nlimbs in (257, 2049, 20000):
        cases.append(O.limbs_to_int(rng.integers(0, 2**64, nlimbs, dtype=np.uint64)))
    for v in cases:
        assert pm.to_decimal(O.int_to_limbs(v), batched=True) == str(v)


@pytest.mark.gpu
def test_conversion_of_large_values_with_long_carries():
    # above the host's parallel-loop size (2^18 limbs): all-ones limbs make
    # every chunked add/subtract ripple its carries across chunk boundaries
    for v in (2 ** (64 * 300_000) - 1, 10 ** 6_000_000 + 1):
        want = str(v)
        assert pm.to_decimal(O.int_to_limbs(v), batched=True) == want
        assert pm.to_decimal(O.int_to_limbs(v), batched=False) == want
