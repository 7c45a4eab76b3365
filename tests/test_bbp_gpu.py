"""Batched BBP hex digits on the GPU vs the reference's known values and the
CPU oracle (crates/pi-core/src/bbp.rs:52-140)."""
import ctypes
import threading

import numpy as np
import pytest

import oracle as O
import pi_gb300 as pm

pytestmark = pytest.mark.gpu


def test_known_values(golden):
    # bbp.rs:153-175
    for n, v in golden["bbp_known"].items():
        assert int(pm.bbp_hex_digits([int(n)])[0]) == v
    d = pm.bbp_hex_digits(np.arange(16))
    assert [int(x) >> 28 for x in d] == golden["pi_hex_prefix"]


def test_overlap_property():
    # bbp.rs:177-187: low 7 nibbles at n equal the top 7 at n + 1
    d = pm.bbp_hex_digits(np.arange(64))
    for n in range(63):
        assert int(d[n]) & 0x0FFFFFFF == int(d[n + 1]) >> 4


def test_matches_oracle_on_seeded_positions():
    rng = np.random.default_rng(8)
    pos = np.concatenate([np.arange(0, 40), rng.integers(0, 200_000, 200), [99_999, 100_000, 131_071]])
    got = pm.bbp_hex_digits(pos)
    want = O.bbp_batch(pos)
    assert np.array_equal(got, want)


def test_deeper_positions_match_oracle():
    pos = np.array([300_000, 999_983, 1_000_000], dtype=np.uint64)
    assert np.array_equal(pm.bbp_hex_digits(pos), O.bbp_batch(pos))


@pytest.mark.parametrize("n", [12_345_678, 87_654_321, 550_000_007])
def test_deep_positions_match_oracle(n):
    # Positions of config 5's range [0, 8e8).  At 550,000,007 the odd moduli
    # d = 8k + 1 and 8k + 5 pass 2^32 for k >= 2^29, so the kernel's 64-bit
    # Montgomery branch computes about 2.6e7 of the terms; below 5.4e8 every
    # odd part stays under 2^32.  The oracle splits each series over all
    # host threads (tens of seconds at the deepest position).
    got = int(pm.bbp_hex_digits(np.array([n], dtype=np.uint64))[0])
    assert got == O.bbp_deep(n), n


def test_stop_flag_cancels():
    # bbp.rs:199-204: a stop flag set before the call returns without digits
    flag = ctypes.c_int(1)
    with pytest.raises(pm.PimulError) as e:
        pm.bbp_hex_digits(np.full(64, 3_000_000, dtype=np.uint64), stop=flag)
    assert e.value.code == 6


def test_stop_flag_from_another_thread():
    import time
    flag = ctypes.c_int(0)
    t = threading.Timer(0.3, lambda: setattr(flag, "value", 1))
    t.start()
    t0 = time.perf_counter()
    with pytest.raises(pm.PimulError):
        # a few seconds of work if not cancelled (bounded either way)
        pm.bbp_hex_digits(np.full(256, 100_000_000, dtype=np.uint64), stop=flag)
    t.join()
    assert time.perf_counter() - t0 < 2.0


def test_rejects_positions_above_limit():
    with pytest.raises(pm.PimulError):
        pm.bbp_hex_digits([1 << 32])


def test_modular_building_blocks_at_large_moduli():
    # 16^e mod d and floor(p 2^64 / d) against Python's integers, over the
    # whole modulus range the extractor uses (d = 8k + j < 2^34, even and odd)
    rng = np.random.default_rng(21)
    d = np.concatenate([rng.integers(1, 1 << 34, 4000, dtype=np.uint64),
                        np.array([1, 2, 3, 4, 6, 7, 9, 12, (1 << 34) - 1, (1 << 34) - 2, (1 << 33) + 1, 2**32 - 5],
                                 dtype=np.uint64),
                        8 * rng.integers(0, 1 << 31, 2000, dtype=np.uint64) + np.uint64(4)])
    e = rng.integers(0, 1 << 31, d.size, dtype=np.uint64)
    e[:20] = np.arange(20)
    p = np.array([int(rng.integers(0, int(x))) if x > 1 else 0 for x in d], dtype=np.uint64)
    p[-5:] = d[-5:] - np.uint64(1)
    pw, fr = pm.bbp_modops(e, d, p)
    for i in range(d.size):
        dd, ee, pp = int(d[i]), int(e[i]), int(p[i])
        assert int(pw[i]) == pow(16, ee, dd), (ee, dd)
        assert int(fr[i]) == (pp << 64) // dd, (pp, dd)


def test_terms_exact_division_at_large_moduli():
    # the summed term floor((16^e mod d) 2^64 / d) (bbp.rs:117-140) as the
    # series kernel computes it, against Python's integers: both Montgomery
    # widths (odd part below and above 2^32), t = 0, 1, 2 and larger powers
    # of two, e = 0 and exponents near 2^31
    rng = np.random.default_rng(33)
    k = rng.integers(0, 1 << 31, 3000, dtype=np.uint64)
    d = np.concatenate([8 * k[:750] + np.uint64(1), 8 * k[750:1500] + np.uint64(4),
                        8 * k[1500:2250] + np.uint64(5), 8 * k[2250:] + np.uint64(6),
                        rng.integers(1, 1 << 34, 2000, dtype=np.uint64),
                        np.array([1, 2, 3, 4, 5, 6, 8, 12, 13, 14, 16, 1 << 20, 3 << 30, (1 << 32) - 1, (1 << 32) + 1,
                                  (1 << 33) + 12, (1 << 34) - 1, (1 << 34) - 2, 2**32 - 5], dtype=np.uint64)])
    e = rng.integers(0, 1 << 31, d.size, dtype=np.uint64)
    e[:40] = np.arange(40)
    e[-19:] = np.array([0, 1, 0, 1, 2, 0, 1, 0, 3, 7, 1, 5, 9, (1 << 31) - 1, 1 << 30, 12345, 0, 1, 77],
                       dtype=np.uint64)
    got = pm.bbp_terms(e, d)
    for i in range(d.size):
        dd, ee = int(d[i]), int(e[i])
        assert int(got[i]) == (pow(16, ee, dd) << 64) // dd, (ee, dd)
