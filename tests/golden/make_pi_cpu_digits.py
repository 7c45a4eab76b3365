"""SHA-256 and last 20 digits of pi from the CPU pipeline: the host
restatement of pi-core's Chudnovsky (binary splitting, final assembly,
recursive decimal conversion) with every product through the oracle, the C
restatement of the reference's CPU multiply (crates/bignum/src/ntt.rs:806-865
behind integer.rs:445-486).  No GPU is used, so this runs on any host.

The record goes into tests/golden/pi_digits_hashes.json under the digit
count, with "source": "cpu-restatement" (the 10^6 and 10^7 entries come from
mpmath, make_pi_digits.py).  10^8 digits take about 20 minutes on 8 cores.

Run: python tests/golden/make_pi_cpu_digits.py [digits]   (default 10^8)
"""
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def main():
    import oracle
    import pi_gb300 as pm

    d = int(float(sys.argv[1])) if len(sys.argv) > 1 else 100_000_000
    oracle.build()
    t0 = time.perf_counter()
    s, info = pm.pi_chudnovsky(d, backend=oracle.mul_abi_pointer())
    wall = time.perf_counter() - t0
    rec = {"sha256": hashlib.sha256(s.encode()).hexdigest(), "last20": s[-20:], "source": "cpu-restatement",
           "wall_s": round(wall, 1), "cores": oracle.max_threads()}
    path = os.path.join(HERE, "pi_digits_hashes.json")
    with open(path) as f:
        table = json.load(f)
    table[str(d)] = rec
    with open(path, "w") as f:
        json.dump(table, f, indent=1)
    print(json.dumps({str(d): rec, "phases_ms": {k: round(v) for k, v in info.items() if k.endswith("_ms")}}))


if __name__ == "__main__":
    main()
