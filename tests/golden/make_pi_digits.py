"""Pi digit fixtures computed with mpmath (an independent arbitrary-precision
implementation):
  tests/golden/pi_digits_100k.txt   first 100,000 digits ("31415...", no point)
  tests/golden/pi_digits_hashes.json SHA-256 and last 20 of the first 10^6 and
                                     10^7 digits (10^7 takes about 10 minutes)
Run: python tests/golden/make_pi_digits.py"""
import hashlib
import json
import os

import mpmath

HERE = os.path.dirname(os.path.abspath(__file__))


def digits(n):
    mpmath.mp.dps = n + 50
    return mpmath.nstr(mpmath.pi, n + 20, strip_zeros=False).replace(".", "")[:n]


def main():
    s = digits(100_000)
    with open(os.path.join(HERE, "pi_digits_100k.txt"), "w") as f:
        f.write(s + "\n")
    out = {}
    for n in (1_000_000, 10_000_000):
        d = digits(n)
        out[str(n)] = {"sha256": hashlib.sha256(d.encode()).hexdigest(), "last20": d[-20:]}
    with open(os.path.join(HERE, "pi_digits_hashes.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(out)


if __name__ == "__main__":
    main()
