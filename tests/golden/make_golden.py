"""Generate tests/golden/*.json from the reference's own unit tests.

Reads the reference's Rust test sources as text (a checkout of joelodom/pi,
given as the first argument or in PI_REFERENCE) and records, for every known-answer
test on the multiply path, the inputs and the exact expected output.
Expected products come from Python's exact integer multiply, which is
independent of both the CPU oracle and the CUDA engine.  Known constants
(digits of pi, BBP hex values) are parsed out of the reference source text.

Run:  python tests/golden/make_golden.py /path/to/joelodom-pi
  or: PI_REFERENCE=/path/to/joelodom-pi python tests/golden/make_golden.py
"""
from __future__ import annotations

import hashlib
import json
import os
import re
import sys

REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PI_REFERENCE", "")
if __name__ == "__main__" and not os.path.isdir(REF):
    sys.exit("usage: make_golden.py <path to a joelodom/pi checkout> (or set PI_REFERENCE)")
HERE = os.path.dirname(os.path.abspath(__file__))
P = 0xFFFFFFFF00000001
M64 = (1 << 64) - 1


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def random_vec(n, seed):
    """LCG of crates/bignum/src/ntt.rs:1216-1226 (values reduced mod P)."""
    s = (seed * 0x9E3779B97F4A7C15 + 1) & M64
    out = []
    for _ in range(n):
        s = (s * 6364136223846793005 + 1442695040888963407) & M64
        out.append(s % P)
    return out


def to_int(limbs):
    return sum(int(x) << (64 * i) for i, x in enumerate(limbs))


def to_limbs(v):
    out = []
    while v:
        out.append(v & M64)
        v >>= 64
    return out


def digest(limbs):
    h = hashlib.sha256()
    for x in limbs:
        h.update(int(x).to_bytes(8, "little"))
    return h.hexdigest()


def case(name, cite, a, b, store_full=True):
    prod = to_limbs(to_int(a) * to_int(b))
    c = {"name": name, "cite": cite, "la": len(a), "lb": len(b), "out_len": len(prod),
         "sha256": digest(prod)}
    if store_full:
        c["a"] = [f"{x:016x}" for x in a]
        c["b"] = [f"{x:016x}" for x in b]
        c["out"] = [f"{x:016x}" for x in prod]
    return c


def main():
    ntt = read("crates/bignum/src/ntt.rs")
    integer = read("crates/bignum/src/integer.rs")
    util = read("crates/pi-core/src/algorithm/util.rs")
    bbp = read("crates/pi-core/src/bbp.rs")

    cases = []
    # ntt.rs:1384-1392 tiny 3*7
    cases.append(case("ntt_mul_matches_schoolbook_tiny", "ntt.rs:1384-1392", [3], [7]))
    # ntt.rs:1394-1411: (len_a, len_b, seed) table parsed from the source
    m = re.search(r"fn ntt_mul_matches_schoolbook_small_random\(\)\s*\{(.*?)\n    \}", ntt, re.S)
    table = re.findall(r"\((\d+)(?:_usize)?,\s*(\d+)(?:_usize)?,\s*(\d+)(?:_u64)?\)", m.group(1))
    assert len(table) >= 7, table
    for la, lb, seed in table:
        la, lb, seed = int(la), int(lb), int(seed)
        cases.append(case(f"small_random_{la}x{lb}_s{seed}", "ntt.rs:1394-1411",
                          random_vec(la, seed), random_vec(lb, seed ^ 0xFF)))
    # ntt.rs:1414-1421 u64::MAX squared
    cases.append(case("ntt_mul_one_limb_max_values", "ntt.rs:1414-1421", [M64], [M64]))
    # ntt.rs:1480-1487 500x500
    s = 0xDEADBEEFCAFEBABE
    cases.append(case("medium_random_500", "ntt.rs:1480-1487", random_vec(500, s), random_vec(500, s ^ 0xFF)))
    # ntt.rs:1548-1567 pool reuse cases
    cases.append(case("pool_reuse_300_ab", "ntt.rs:1548-1567", random_vec(300, 0xCAFE0001), random_vec(300, 0xBEEF0002)))
    cases.append(case("pool_reuse_300_cd", "ntt.rs:1548-1567", random_vec(300, 0xDEAD0003), random_vec(300, 0xFACE0004)))
    # ntt.rs:1523-1541 repeated 200x200
    cases.append(case("pool_caps_200", "ntt.rs:1523-1541", random_vec(200, 0x123456789ABCDEF0), random_vec(200, 0x0FEDCBA987654321)))
    # ntt.rs:1657-1667 twiddle cache 400x400
    cases.append(case("twiddle_cache_400", "ntt.rs:1657-1667", random_vec(400, 0x1111222233334444), random_vec(400, 0x5555666677778888)))
    # ntt.rs:1712-1722 32768x32768 (digest only)
    cases.append(case("bit_reverse_parallel_via_ntt_32768", "ntt.rs:1712-1722",
                      random_vec(32768, 0xAA), random_vec(32768, 0xBB), store_full=False))
    # ntt.rs:2056-2101 forced four-step (300 and 600 limbs)
    cases.append(case("four_step_dispatch_300", "ntt.rs:2056-2071", random_vec(300, 0x1357), random_vec(300, 0x2468)))
    cases.append(case("four_step_nonsquare_600", "ntt.rs:2087-2101", random_vec(600, 0xAB), random_vec(600, 0xCD)))
    # integer.rs:1727-1754 Karatsuba-above-NTT operands
    a = [(0xDEADBEEFCAFE0001 * (i + 1)) & M64 for i in range(200)]
    b = [(0xFACEF00D12345678 * (i + 7)) & M64 for i in range(200)]
    cases.append(case("karatsuba_above_ntt_200", "integer.rs:1727-1754", a, b))
    # integer.rs:1413-1434 seven squarings of two seeds, then their product
    x, y = 0xDEADBEEFCAFEF00D, 0x0123456789ABCDEF
    for _ in range(7):
        x, y = x * x, y * y
    cases.append(case("karatsuba_squarings", "integer.rs:1413-1434", to_limbs(x), to_limbs(y)))
    # integer.rs:1502-1514 (3 << 10000) * 0xFEDCBA9876543210
    cases.append(case("karatsuba_asymmetric", "integer.rs:1502-1514", to_limbs(3 << 10000), [0xFEDCBA9876543210]))
    # integer.rs:1398-1410 2^64 * 2^64 = 2^128 (decimal string from the source)
    dec = re.search(r'"(340282366920938463463374607431768211456)"', integer).group(1)
    assert int(dec) == 1 << 128
    cases.append(case("mul_large_carry", "integer.rs:1398-1410", [0, 1], [0, 1]))

    # known convolutions in the four-step tests (ntt.rs:1868-1891, 1989-2006)
    conv = []
    for fn in ("four_step_square_convolution_n16", "four_step_nonsquare_convolution_n8"):
        body = re.search(r"fn " + fn + r"\(\)\s*\{(.*?)\n    \}", ntt, re.S).group(1)
        av = {int(i): int(v) for i, v in re.findall(r"a\[(\d+)\] = (\d+);", body)}
        bv = {int(i): int(v) for i, v in re.findall(r"b\[(\d+)\] = (\d+);", body)}
        wv = {int(i): int(v) for i, v in re.findall(r"want\[(\d+)\] = (\d+);", body)}
        n = int(re.search(r"let n = (\d+)", body).group(1))
        conv.append({"name": fn, "n": n, "a": av, "b": bv, "want": wv})
    # ntt.rs:1240-1246 bit reverse of length 8
    br = re.search(r"fn bit_reverse_known\(\).*?assert_eq!\(a, vec!\[([\d, ]+)\]\)", ntt, re.S).group(1)
    bit_reverse8 = [int(v) for v in br.split(",")]
    # ntt.rs:1155-1179 reduce128 battery (expected = x % P)
    body = re.search(r"fn reduce128_matches_naive_mod\(\).*?let cases: &\[u128\] = &\[(.*?)\];", ntt, re.S).group(1)
    red = []
    for tok in re.findall(r"^\s*([^/\n][^\n]*?),\s*$", body, re.M):
        expr = tok.replace("_", "").replace(" as u128", "").replace("u128::MAX", str((1 << 128) - 1)).replace("P", str(P))
        v = eval(expr, {"__builtins__": {}})
        red.append([f"{v:032x}", f"{v % P:016x}"])
    # first digits of pi (util.rs:126-127)
    first100 = re.search(r'pub const FIRST_100: &str =\s*"([0-9.]+)"', util).group(1)
    # BBP known values (bbp.rs:148-174)
    bbp_known = {int(n): int(v.replace("_", ""), 16)
                 for n, v in re.findall(r"assert_eq!\(hex_digits_at\((\d+)\), 0x([0-9A-Fa-f_]+)\)", bbp)}
    prefix = re.search(r"PI_HEX_PREFIX: \[u8; 16\] = \[(.*?)\];", bbp, re.S).group(1)
    pi_hex_prefix = [int(v, 16) for v in re.findall(r"0x([0-9A-Fa-f])", prefix)]

    out = {
        "source": "joelodom/pi unit tests (crates/bignum/src/ntt.rs, integer.rs; crates/pi-core/src/bbp.rs, algorithm/util.rs)",
        "mul_cases": cases,
        "convolutions": conv,
        "bit_reverse8": bit_reverse8,
        "reduce128": red,
        "first_100_digits": first100,
        "bbp_known": {str(k): v for k, v in bbp_known.items()},
        "pi_hex_prefix": pi_hex_prefix,
    }
    path = os.path.join(HERE, "reference_vectors.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0)
    print(f"wrote {path}: {len(cases)} multiply cases, {len(red)} reduce128 cases")


if __name__ == "__main__":
    main()
