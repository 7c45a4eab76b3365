"""verify-hex's decimal -> hex conversion on the GPU (pimul_decimal_to_hex)
against the oracle's exact-integer restatement of
crates/pi-cli/src/verify_hex.rs:553-629, and against BBP hex digits."""
import os
import random

import numpy as np
import pytest

import oracle as O
import pi_gb300 as pm

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def pi_text(n_digits: int) -> str:
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        d = f.read().strip()[:n_digits]
    return "3." + d[1:]


def rand_text(e: int, rng: random.Random) -> str:
    return "3." + "".join(rng.choice("0123456789") for _ in range(e))


def test_small_and_boundary_lengths():
    rng = random.Random(7)
    lengths = list(range(0, 80)) + [1215, 1216, 1217, 2431, 2432, 2433]
    # D = E + 1 digits around chunk (19), leaf (1216) and level (19 2^k) edges
    for k in range(1, 12):
        for dd in (-1, 0, 1):
            lengths.append(19 * (1 << k) + dd - 1)
    for e in sorted(set(lengths)):
        t = rand_text(e, rng)
        assert pm.decimal_to_hex(t) == O.decimal_to_hex(t), e


def test_exact_quotients_and_extremes():
    # remainders of zero (3.000..., 3.5000...) and values next to 4
    for e in (1, 5, 19, 40, 1300, 5000, 40000):
        for t in ("3." + "0" * e, "3.5" + "0" * (e - 1), "3." + "9" * e, "3." + "0" * (e - 1) + "1"):
            assert pm.decimal_to_hex(t) == O.decimal_to_hex(t), (e, t[:8])


def test_pi_100k_matches_oracle_and_bbp():
    t = pi_text(100_000)
    x, ph = pm.decimal_to_hex(t, phases=True)
    assert x == O.decimal_to_hex(t)
    frac = x[2:]
    assert frac.startswith("243f6a8885a308d3")
    h = len(frac)
    pos = np.array([0, 8, 1000, 12345, 50000, h - 32 - 8], dtype=np.uint64)
    d = pm.bbp_hex_digits(pos)
    for p, v in zip(pos, d):
        assert frac[int(p): int(p) + 8] == format(int(v), "08x"), p
    assert len(ph) == 4 and all(v >= 0 for v in ph)


def test_pi_1e6_matches_oracle():
    s, _ = pm.pi_chudnovsky_batched(1_000_000)
    t = "3." + s[1:]
    assert pm.decimal_to_hex(t) == O.decimal_to_hex(t)


def test_random_large():
    rng = random.Random(11)
    for e in (100_003, 262_143):
        t = rand_text(e, rng)
        assert pm.decimal_to_hex(t) == O.decimal_to_hex(t), e


def test_whitespace_and_errors(tmp_path):
    assert pm.decimal_to_hex(" \t3.14159265358979\r\n") == O.decimal_to_hex("3.14159265358979")
    assert pm.decimal_to_hex("3.") == "3."
    for bad, msg in (("2.14", "doesn't start"), ("314", "doesn't start"), ("", "doesn't start"),
                     ("3.14a59", "non-digit"), ("3.1 4", "non-digit"), ("3." + "1" * 3000 + "x", "non-digit")):
        with pytest.raises(pm.PimulError, match=msg):
            pm.decimal_to_hex(bad)
    # the file form: "3." + hex digits + newline, through a .tmp and a rename
    src, dst = tmp_path / "pi.txt", tmp_path / "pi.hex"
    src.write_text(pi_text(5000) + "\n")
    pm.convert_decimal_to_hex(src, dst)
    assert dst.read_text() == O.decimal_to_hex(pi_text(5000)) + "\n"
    assert not (tmp_path / "pi.tmp").exists()
