"""Host-side pi pipeline (the caller of the multiply), run on the CPU with
the oracle's multiply as its backend: digits must equal an independent
mpmath computation (tests/golden/pi_digits_100k.txt) and the reference's
FIRST_100 constant (crates/pi-core/src/algorithm/util.rs:126-127)."""
import os

import pytest

import oracle as O
import pi_gb300 as pm

HERE = os.path.dirname(os.path.abspath(__file__))


def ref_digits():
    with open(os.path.join(HERE, "golden", "pi_digits_100k.txt")) as f:
        return f.read().strip()


def test_first_100(golden):
    s, _ = pm.pi_chudnovsky(100, backend=O.mul_abi_pointer())
    assert s == golden["first_100_digits"].replace(".", "")


@pytest.mark.parametrize("digits,thr", [(1, 0), (2, 0), (50, 0), (1000, 0), (4321, 64), (30000, 64)])
def test_digits_vs_mpmath(digits, thr):
    s, info = pm.pi_chudnovsky(digits, backend=O.mul_abi_pointer(), ntt_threshold=thr)
    assert s == ref_digits()[:digits]
    if thr:
        assert info["ntt_products"] > 0  # the backend saw the large products


@pytest.mark.parametrize("digits,thr", [(1, 0), (100, 0), (3000, 64), (20000, 256)])
def test_gauss_legendre_vs_mpmath(digits, thr):
    s, info = pm.pi_gauss_legendre(digits, backend=O.mul_abi_pointer(), ntt_threshold=thr)
    assert s == ref_digits()[:digits]


@pytest.mark.parametrize("digits,thr", [(1, 0), (100, 0), (5000, 64), (30000, 256)])
def test_gauss_legendre_fast_sqrt_vs_mpmath(digits, thr):
    s, _ = pm.pi_gauss_legendre(digits, backend=O.mul_abi_pointer(), ntt_threshold=thr, fast_sqrt=True)
    assert s == ref_digits()[:digits]
