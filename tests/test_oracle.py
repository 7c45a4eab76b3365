"""Pin the CPU oracle to the reference's own known-answer tests.

Every case here comes from the reference's unit tests (file:line in
tests/golden/reference_vectors.json) or restates one of them; the expected
products were computed with Python's exact integer multiply.
"""
import hashlib

import numpy as np
import pytest

import oracle as O
from conftest import hexlimbs, rand_limbs

P = O.P
M64 = (1 << 64) - 1


def digest(limbs):
    h = hashlib.sha256()
    for x in np.asarray(limbs, dtype=np.uint64):
        h.update(int(x).to_bytes(8, "little"))
    return h.hexdigest()


# ---------------------------------------------------------------- field
def test_reduce128_battery(golden):
    # crates/bignum/src/ntt.rs:1155-1179
    for x_hex, want_hex in golden["reduce128"]:
        assert O.gl_reduce128(int(x_hex, 16)) == int(want_hex, 16)


def test_field_basics():
    # ntt.rs:1116-1152
    assert O.gl_add(P - 1, 1) == 0
    assert O.gl_add(P - 1, P - 1) == P - 2
    assert O.gl_sub(0, 1) == P - 1
    assert O.gl_sub(0, P - 1) == 1
    assert O.gl_mul(P - 1, P - 1) == 1
    assert O.gl_mul((P + 1) // 2, 2) == 1


def test_mul_grid_vs_naive():
    # ntt.rs:1182-1196
    eps = 0xFFFFFFFF
    xs = [0, 1, 2, 100, eps, eps + 1, P - 1, P // 2, P // 3,
          0xDEADBEEFCAFEBABE & (P - 1), 0x123456789ABCDEF0 & (P - 1)]
    for a in xs:
        for b in xs:
            assert O.gl_mul(a, b) == (a * b) % P


def test_pow_inv_roots():
    # ntt.rs:1199-1212, 1424-1436
    for a in (2, 3, 7, 12345, P - 1, P // 2):
        assert O.gl_pow(a, P - 1) == 1
        assert O.gl_mul(a, O.gl_inv(a)) == 1
    for lg in (1, 2, 4, 8, 16, 20, 32):
        w = O.gl_root(1 << lg)
        assert O.gl_pow(w, 1 << lg) == 1
        assert O.gl_pow(w, 1 << (lg - 1)) == P - 1


# ---------------------------------------------------------------- transforms
def test_bit_reverse_known(golden):
    # ntt.rs:1240-1246
    assert list(O.bit_reverse(np.arange(8, dtype=np.uint64))) == golden["bit_reverse8"]


def random_vec(n, seed):
    s = (seed * 0x9E3779B97F4A7C15 + 1) & M64
    out = []
    for _ in range(n):
        s = (s * 6364136223846793005 + 1442695040888963407) & M64
        out.append(s % P)
    return np.array(out, dtype=np.uint64)


@pytest.mark.parametrize("lg", [1, 2, 3, 4, 8, 12])
def test_ntt_round_trip(lg):
    # ntt.rs:1249-1258
    x = random_vec(1 << lg, lg)
    assert np.array_equal(O.ntt_inverse(O.ntt_forward(x)), x)


@pytest.mark.parametrize("lg", [2, 3, 4, 5, 7, 8, 9, 10, 11])
def test_four_step_round_trip(lg):
    # ntt.rs:1796-1836 (square) and 1925-1970 (non-square)
    x = random_vec(1 << lg, 0xABCD + lg)
    assert np.array_equal(O.four_step_inverse(O.four_step_forward(x)), x)


def naive_conv(a, b, n):
    out = [0] * n
    for i, x in enumerate(a):
        for j, y in enumerate(b):
            out[i + j] = (out[i + j] + int(x) * int(y)) % P
    return out


def test_known_convolutions(golden):
    # ntt.rs:1840-1865 and 1975-1993, via both transforms
    for c in golden["convolutions"]:
        n = c["n"]
        a = np.zeros(n, dtype=np.uint64)
        b = np.zeros(n, dtype=np.uint64)
        for k, v in c["a"].items():
            a[int(k)] = v
        for k, v in c["b"].items():
            b[int(k)] = v
        want = np.zeros(n, dtype=np.uint64)
        for k, v in c["want"].items():
            want[int(k)] = v
        for fwd, inv in ((O.four_step_forward, O.four_step_inverse), (O.ntt_forward, O.ntt_inverse)):
            fa, fb = fwd(a), fwd(b)
            prod = np.array([O.gl_mul(int(x), int(y)) for x, y in zip(fa, fb)], dtype=np.uint64)
            assert np.array_equal(inv(prod), want), c["name"]


@pytest.mark.parametrize("in_len,seed", [(7, 1), (15, 2), (31, 3), (63, 4), (127, 5)])
def test_convolution_random(in_len, seed):
    # ntt.rs:1261-1316
    a = random_vec(in_len, seed) & np.uint64(0xFFFF)
    b = random_vec(in_len, seed ^ 0xFF) & np.uint64(0xFFFF)
    n_out = 2 * in_len - 1
    n = 1 << (n_out - 1).bit_length()
    pa = np.zeros(n, dtype=np.uint64)
    pb = np.zeros(n, dtype=np.uint64)
    pa[:in_len], pb[:in_len] = a, b
    fa, fb = O.ntt_forward(pa), O.ntt_forward(pb)
    prod = np.array([O.gl_mul(int(x), int(y)) for x, y in zip(fa, fb)], dtype=np.uint64)
    got = O.ntt_inverse(prod)[:n_out]
    assert list(got) == naive_conv(a, b, n_out)


# ---------------------------------------------------------------- pack / unpack
def test_pack_unpack_round_trips():
    # ntt.rs:1320-1356
    for limbs in ([0xDEADBEEFCAFEBABE],
                  [0xDEADBEEFCAFEBABE, 0x123456789ABCDEF0, 0x5555AAAA5555AAAA, M64, 1]):
        x = np.array(limbs, dtype=np.uint64)
        assert np.array_equal(O.unpack(O.pack(x, 4 * len(limbs) + 5)), x)
    x = random_vec(40, 12345)
    assert np.array_equal(O.unpack(O.pack(x, 170)), np.trim_zeros(x, "b"))


def test_unpack_parallel_matches_serial():
    # ntt.rs:1729-1768: coefficient streams above the 2^20 parallel threshold,
    # with high values to stress the cross-chunk carry merge.
    n = (1 << 20) + 4321
    i = np.arange(n, dtype=np.uint64)
    c = ((i * np.uint64(0x123456789ABCDEF0)) >> np.uint64(8)) & np.uint64(0xFFFFFFFF)
    got = O.unpack(c)
    want = sum(int(v) << (16 * k) for k, v in enumerate(c[:5000]))  # prefix check below
    val = O.limbs_to_int(got)
    assert val & ((1 << (16 * 4000)) - 1) == want & ((1 << (16 * 4000)) - 1)
    # full check against Python on a cheaper exact formula: sum c_k 2^(16k)
    total = 0
    for k in range(0, n, 4096):
        chunk = c[k:k + 4096]
        part = sum(int(v) << (16 * j) for j, v in enumerate(chunk))
        total += part << (16 * k)
    assert val == total


# ---------------------------------------------------------------- products
def test_golden_products(golden):
    for c in golden["mul_cases"]:
        if "a" in c:
            a, b = hexlimbs(c["a"]), hexlimbs(c["b"])
        else:
            continue
        want = hexlimbs(c["out"])
        assert np.array_equal(O.mul_mag(a, b), want), c["name"]
        assert np.array_equal(O.mul_mag_ntt(a, b), want), c["name"]
        assert np.array_equal(O.schoolbook(a, b), want), c["name"]


def test_golden_large_digest(golden):
    c = next(c for c in golden["mul_cases"] if c["name"] == "bit_reverse_parallel_via_ntt_32768")
    a, b = random_vec(32768, 0xAA), random_vec(32768, 0xBB)
    got = O.mul_mag_ntt(a, b)
    assert len(got) == c["out_len"] and digest(got) == c["sha256"]


def test_four_step_forced(golden):
    # ntt.rs:2056-2101 with the four-step threshold lowered to 1
    O.set_thresholds(four_step=1)
    try:
        for name in ("four_step_dispatch_300", "four_step_nonsquare_600"):
            c = next(c for c in golden["mul_cases"] if c["name"] == name)
            assert np.array_equal(O.mul_mag_ntt(hexlimbs(c["a"]), hexlimbs(c["b"])), hexlimbs(c["out"]))
    finally:
        O.set_thresholds()


def test_karatsuba_above_ntt(golden):
    # integer.rs:1727-1754: ntt_max_coeffs=100 forces Karatsuba, ntt_threshold=50
    c = next(c for c in golden["mul_cases"] if c["name"] == "karatsuba_above_ntt_200")
    a, b, want = hexlimbs(c["a"]), hexlimbs(c["b"]), hexlimbs(c["out"])
    O.set_thresholds(ntt=50)
    try:
        assert np.array_equal(O.mul_mag_dispatch(a, b, 100), want)
        assert np.array_equal(O.mul_mag_dispatch(a, b, 1 << 32), want)
    finally:
        O.set_thresholds()


@pytest.mark.parametrize("la,lb", [(8192, 8192), (9000, 20000), (20000, 9000), (1, 70000)])
def test_dispatch_vs_python(la, lb):
    a, b = rand_limbs(la, la), rand_limbs(lb, lb + 1)
    want = O.limbs_to_int(a) * O.limbs_to_int(b)
    assert O.limbs_to_int(O.mul_mag(a, b)) == want
    assert O.limbs_to_int(O.mul_mag_ntt(a, b)) == want


def test_empty_and_zero_limbs():
    e = np.zeros(0, dtype=np.uint64)
    assert O.mul_mag_ntt(e, np.array([5], dtype=np.uint64)).size == 0
    z = np.zeros(3, dtype=np.uint64)
    assert O.mul_mag_ntt(z, np.array([5, 6], dtype=np.uint64)).size == 0
    ones = np.full(50, M64, dtype=np.uint64)
    want = ((1 << 3200) - 1) ** 2
    assert O.limbs_to_int(O.mul_mag_ntt(ones, ones)) == want


# ---------------------------------------------------------------- BBP
def test_bbp_known(golden):
    # crates/pi-core/src/bbp.rs:153-175
    for n, v in golden["bbp_known"].items():
        assert O.bbp_hex_digits_at(int(n)) == v
    for n, nib in enumerate(golden["pi_hex_prefix"]):
        assert (O.bbp_hex_digits_at(n) >> 28) & 0xF == nib


def test_bbp_overlap_and_interrupt():
    # bbp.rs:177-216
    for n in range(16):
        assert O.bbp_hex_digits_at(n) & 0x0FFFFFFF == O.bbp_hex_digits_at(n + 1) >> 4
    assert O.bbp_hex_digits_at(10_000_000, stop=True) is None
    got = O.bbp_batch([0, 1, 7, 8, 100, 999])
    assert list(got) == [O.bbp_hex_digits_at(n) for n in (0, 1, 7, 8, 100, 999)]


# ---------------------------------------------------------------- verify-hex conversion
def test_decimal_to_hex_pinned_to_bbp(golden):
    # crates/pi-cli/src/verify_hex.rs:553-629 on the first 100 decimal digits
    # (util.rs:126-127) against the reference's hex prefix and BBP known
    # values (bbp.rs:153-175); the last TAIL_SKIP = 32 digits are exempt
    # (verify_hex.rs:540-547)
    x = O.decimal_to_hex(golden["first_100_digits"])
    assert x.startswith("3.")
    frac = x[2:]
    assert len(frac) == int(99 * (np.log2(10.0) / 4.0))
    assert [int(c, 16) for c in frac[: len(golden["pi_hex_prefix"])]] == golden["pi_hex_prefix"]
    for n, v in golden["bbp_known"].items():
        assert frac[int(n): int(n) + 8] == format(v, "08x")
    for n in range(0, len(frac) - 32 - 8):
        assert frac[n: n + 8] == format(O.bbp_hex_digits_at(n), "08x")


def test_decimal_to_hex_edges_and_errors():
    # h = floor(E log2(10) / 4): "3." -> no digits, "3.1" -> none, "3.14" -> one
    assert O.decimal_to_hex("3.") == "3."
    assert O.decimal_to_hex(" 3.1\n") == "3."
    assert O.decimal_to_hex("3.14") == "3.2"
    assert O.decimal_to_hex("3.5000") == "3.800"
    for bad, msg in (("2.14", "3."), ("314", "3."), ("3.1a4", "non-digit"), ("", "3.")):
        with pytest.raises(ValueError, match=msg.replace(".", r"\.")):
            O.decimal_to_hex(bad)
