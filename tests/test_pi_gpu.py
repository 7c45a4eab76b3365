"""Configuration 1: Chudnovsky pi with every product above the reference's
NTT threshold going through the GPU multiply (one call per product); digits
must equal the independent mpmath digits and the same pipeline with the CPU
multiply (the reference's CPU path)."""
import hashlib
import json
import os

import pytest

import oracle as O
import pi_gb300 as pm

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_1e5_digits_lowered_threshold():
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        ref = f.read().strip()
    s, info = pm.pi_chudnovsky(100_000, ntt_threshold=512)
    assert s == ref
    assert info["ntt_products"] > 50


def test_1e6_digits_reference_threshold():
    with open(os.path.join(HERE, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["1000000"]
    s, info = pm.pi_chudnovsky(1_000_000)
    assert info["ntt_products"] > 0
    assert s[-20:] == want["last20"]
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]
    cpu, _ = pm.pi_chudnovsky(1_000_000, backend=O.mul_abi_pointer())
    assert cpu == s


def test_gauss_legendre_1e5_equals_chudnovsky():
    # the reference's own acceptance check: both algorithms byte-identical
    g, info = pm.pi_gauss_legendre(100_000, ntt_threshold=512)
    c, _ = pm.pi_chudnovsky(100_000, ntt_threshold=512)
    assert g == c
    assert info["ntt_products"] > 0


def test_1e7_digits_against_mpmath():
    with open(os.path.join(HERE, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["10000000"]
    s, info = pm.pi_chudnovsky(10_000_000)
    assert info["ntt_products"] > 100
    assert s[-20:] == want["last20"]
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]


@pytest.mark.parametrize("leaf", [7, 64])
def test_batched_binary_splitting_1e5(leaf):
    # level-batched splitting (odd node counts at some levels for leaf 7)
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        ref = f.read().strip()
    s, info = pm.pi_chudnovsky_batched(100_000, leaf)
    assert s == ref
    assert info["batched_levels"] > 5 and info["ntt_products"] > 100


def test_batched_binary_splitting_1e6_matches_mpmath_and_plain():
    with open(os.path.join(HERE, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["1000000"]
    s, info = pm.pi_chudnovsky_batched(1_000_000)
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]
    plain, _ = pm.pi_chudnovsky(1_000_000)
    assert plain == s


def test_gauss_legendre_through_served_form():
    # every product at or above 512 limbs goes upload -> submit -> wait -> download
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        ref = f.read().strip()
    g, info = pm.pi_gauss_legendre(100_000, backend=pm.served_backend(), ntt_threshold=512)
    assert g == ref
    assert info["ntt_products"] > 0


def test_gauss_legendre_fast_sqrt_1e6_matches_mpmath():
    with open(os.path.join(HERE, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["1000000"]
    s, _ = pm.pi_gauss_legendre(1_000_000, backend=pm.served_backend(), fast_sqrt=True)
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]


def test_gauss_legendre_device_agm_matches_golden():
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        ref = f.read().strip()
    for d in (100, 5000, 100_000):
        s, _ = pm.pi_gauss_legendre(d, device_agm=True)
        assert s == ref[:d], d
    with open(os.path.join(HERE, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["1000000"]
    s, _ = pm.pi_gauss_legendre(1_000_000, device_agm=True)
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]


def test_gauss_legendre_device_decimal_1e6_matches_mpmath():
    with open(os.path.join(HERE, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["1000000"]
    s, _ = pm.pi_gauss_legendre(1_000_000, backend=pm.served_backend(), fast_sqrt=True, device_decimal=True)
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]


@pytest.mark.parametrize("digits,leaf", [(1, 0), (17, 0), (500, 3), (1000, 0), (5000, 1), (20000, 5)])
def test_batched_small_and_odd_shapes(digits, leaf):
    # one leaf, a single-term leaf size, odd leaf counts at every level
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        ref = f.read().strip()
    s, _ = pm.pi_chudnovsky_batched(digits, leaf)
    assert s == ref[:digits]


def test_1e8_digits_batched_and_device_agm_match_cpu_restatement():
    # 10^8 digits against the CPU pipeline's digits (the host restatement of
    # pi-core's Chudnovsky with every product through the oracle, recorded by
    # tests/golden/make_pi_cpu_digits.py): the level-batched device-resident
    # Chudnovsky run and the device Gauss-Legendre AGM both match it.
    with open(os.path.join(HERE, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["100000000"]
    assert want["source"] == "cpu-restatement"
    s, info = pm.pi_chudnovsky_batched(100_000_000)
    assert s[-20:] == want["last20"]
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]
    del s
    g, _ = pm.pi_gauss_legendre(100_000_000, device_agm=True)
    assert hashlib.sha256(g.encode()).hexdigest() == want["sha256"]


@pytest.mark.parametrize("digits,leaf", [(3000, 2), (20000, 4), (100_000, 6), (100_000, 64), (1_000_000, 0),
                                         (3_000_000, 0)])
def test_merged_splitting_levels_match_batched_levels(digits, leaf, monkeypatch):
    # the lowest splitting levels merged pair by pair in one CTA (fused
    # P, Q, T products, graph-captured schedule) against the same levels
    # through pimul_sum_batch; even leaf sizes, odd node counts on the way up
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        ref = f.read().strip()
    monkeypatch.setenv("PIMUL_PI_MERGED_LEVELS", "0")
    plain, _ = pm.pi_chudnovsky_batched(digits, leaf)
    monkeypatch.setenv("PIMUL_PI_MERGED_LEVELS", "1")
    merged, info = pm.pi_chudnovsky_batched(digits, leaf)
    assert merged == plain
    assert merged[:100_000] == ref[:min(digits, 100_000)]


def test_1e9_digits_batched_match_recorded_hash():
    # the top levels of a 10^9-digit tree run wrapped products (cyclic
    # transforms of half the length, PIMUL_BATCH_WRAP); the digits must be
    # the recorded ones, on which Chudnovsky and the Gauss-Legendre AGM agree
    with open(os.path.join(HERE, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["1000000000"]
    s, info = pm.pi_chudnovsky_batched(1_000_000_000)
    assert s[-20:] == want["last20"]
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]
