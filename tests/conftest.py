import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_vectors.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running case")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this container")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as f:
        return json.load(f)


def hexlimbs(xs):
    return np.array([int(x, 16) for x in xs], dtype=np.uint64)


M64 = (1 << 64) - 1


def splitmix64_limbs(n, seed):
    """Seeded SplitMix64 limbs with the top limb's bit 63 set (exact bit length)."""
    out = np.empty(n, dtype=np.uint64)
    s = seed & M64
    for i in range(n):
        s = (s + 0x9E3779B97F4A7C15) & M64
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        out[i] = z ^ (z >> 31)
    if n:
        out[-1] |= np.uint64(1 << 63)
    return out


def rand_limbs(n, seed, top=True):
    """Fast seeded uniform limbs (numpy PCG64); top limb bit 63 set when top."""
    rng = np.random.default_rng(seed)
    x = rng.integers(0, 1 << 64, size=n, dtype=np.uint64, endpoint=False)
    if n and top:
        x[-1] |= np.uint64(1 << 63)
    return x
