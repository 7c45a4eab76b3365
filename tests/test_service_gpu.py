"""Served form: device-resident handles, chained requests, HBM admission
budget and continuous batching.  Every result must be the same whether the
request runs alone or in a mix, and equal the CPU oracle."""
import numpy as np
import pytest

import oracle as O
import pi_gb300 as pm
from conftest import rand_limbs

pytestmark = pytest.mark.gpu


def _stream(n, seed, lo_bits=2 ** 12, hi_bits=2 ** 20, chain=0.3, sq=0.25):
    """Request list: (op, x, y) where x / y are base-operand indices (>= 0) or
    results of earlier requests (encoded as -(k+1))."""
    rng = np.random.default_rng(seed)
    nbase = n
    bits = np.exp(rng.uniform(np.log(lo_bits), np.log(hi_bits), size=nbase)).astype(np.int64)
    base = [rand_limbs(max(1, int(b) // 64), 1000 + i) for i, b in enumerate(bits)]
    reqs = []
    for k in range(n):
        x = int(rng.integers(0, nbase))
        if k > 0 and rng.random() < chain:
            x = -(int(rng.integers(0, k)) + 1)
        if rng.random() < sq:
            reqs.append(("sqr", x, x))
        else:
            reqs.append(("mul", x, int(rng.integers(0, nbase))))
    return base, reqs


def _host_results(base, reqs):
    res = []
    for op, x, y in reqs:
        a = base[x] if x >= 0 else res[-x - 1]
        b = a if op == "sqr" else (base[y] if y >= 0 else res[-y - 1])
        res.append(pm.mul_mag_ntt(a, b))
    return res


def _served(base, reqs, budget=None):
    if budget is not None:
        pm.set_budget(budget)
    hb = [pm.upload(x) for x in base]
    outs, tickets = [], []
    for op, x, y in reqs:
        ha = hb[x] if x >= 0 else outs[-x - 1]
        if op == "sqr":
            h, t = pm.submit(ha)
        else:
            hy = hb[y] if y >= 0 else outs[-y - 1]
            h, t = pm.submit(ha, hy)
        outs.append(h)
        tickets.append(t)
    for t in tickets:
        pm.wait(t)
    res = [pm.download(h) for h in outs]
    for h in outs + hb:
        pm.free(h)
    pm.set_budget(120 << 30)
    return res


def test_served_results_match_plain_and_oracle():
    base, reqs = _stream(120, 1)
    want = _host_results(base, reqs)
    got = _served(base, reqs)
    for k, (g, w) in enumerate(zip(got, want)):
        assert np.array_equal(g, w), k
    # spot-check against the CPU oracle (chained ones included)
    for k in (0, 1, 7, 50, 119):
        op, x, y = reqs[k]
        a = base[x] if x >= 0 else want[-x - 1]
        b = a if op == "sqr" else (base[y] if y >= 0 else want[-y - 1])
        assert np.array_equal(want[k], O.mul_mag_ntt(a, b))


def test_same_result_alone_and_in_the_mix():
    base, reqs = _stream(200, 2)
    mixed = _served(base, reqs)
    for k in (3, 77, 150, 199):
        op, x, y = reqs[k]
        # resolve chains on the host, then run the request alone
        a = base[x] if x >= 0 else mixed[-x - 1]
        b = a if op == "sqr" else (base[y] if y >= 0 else mixed[-y - 1])
        ha = pm.upload(a)
        hb = ha if op == "sqr" else pm.upload(b)
        h, t = pm.submit(ha) if op == "sqr" else pm.submit(ha, hb)
        pm.wait(t)
        alone = pm.download(h)
        for z in {h, ha, hb}:
            pm.free(z)
        assert np.array_equal(alone, mixed[k]), k


def test_budget_admission_still_completes():
    # budget below the sum of the requests' scratch: they are admitted a few
    # at a time as earlier ones release memory
    base, reqs = _stream(40, 3, lo_bits=2 ** 18, hi_bits=2 ** 22, chain=0.2)
    want = _host_results(base, reqs)
    got = _served(base, reqs, budget=64 << 20)
    for g, w in zip(got, want):
        assert np.array_equal(g, w)


def test_request_larger_than_budget_is_rejected():
    pm.set_budget(1 << 20)
    try:
        small = pm.upload(rand_limbs(10, 1))
        big = pm.upload(rand_limbs(60000, 3))  # 480 KB fits the 1 MiB budget
        with pytest.raises(pm.PimulError) as e:
            pm.submit(big, big, pm.OP_MUL)  # result + 8 MiB of scratch do not
        assert e.value.code == 2
        pm.free(small)
        pm.free(big)
    finally:
        pm.set_budget(120 << 30)


def test_wait_timeout_and_errors():
    a = pm.upload(rand_limbs(1 << 21, 5))
    h, t = pm.submit(a)
    with pytest.raises(pm.PimulError) as e:
        pm.wait(t, 0)
    assert e.value.code in (4,)  # ETIMEDOUT (the product needs far longer than 0 us)
    pm.wait(t)
    assert pm.download(h).size > 0
    pm.free(h)
    pm.free(a)
    with pytest.raises(pm.PimulError) as e:
        pm.free(a)
    assert e.value.code == 5
    with pytest.raises(pm.PimulError):
        pm.wait(1 << 60)


def test_free_waits_for_readers():
    a = pm.upload(rand_limbs(1 << 18, 6))
    b = pm.upload(rand_limbs(1 << 18, 7))
    h, t = pm.submit(a, b)
    pm.free(a)  # returns only after the product has read it
    pm.wait(t)
    got = pm.download(h)
    assert np.array_equal(got, O.mul_mag_ntt(rand_limbs(1 << 18, 6), rand_limbs(1 << 18, 7)))
    pm.free(b)
    pm.free(h)


def _int(x):
    return O.limbs_to_int(x)


def test_add_and_subtract_requests_chained():
    # sums and differences as service requests, chained on products without
    # a host round trip: s = a b + c, d = s - c (= a b), e = d - a b = 0,
    # with operands of different stored lengths in both orders
    cases = [(300, 200, 5), (5, 300, 200), (4000, 4000, 4001), (1, 1, 1), (70000, 3000, 65000)]
    for la, lb, lc in cases:
        a, b, c = rand_limbs(la, la + 1), rand_limbs(lb, lb + 2), rand_limbs(lc, lc + 3)
        ha, hb, hc = pm.upload(a), pm.upload(b), pm.upload(c)
        p, _ = pm.submit(ha, hb)
        s, _ = pm.submit(p, hc, op=pm.OP_ADD)
        d, _ = pm.submit(s, hc, op=pm.OP_SUB)
        e, t = pm.submit(d, p, op=pm.OP_SUB)
        pm.wait(t)
        want = _int(a) * _int(b)
        assert _int(pm.download(s)) == want + _int(c)
        assert _int(pm.download(d)) == want
        assert pm.download(e).size == 0
        for h in (ha, hb, hc, p, s, d, e):
            pm.free(h)


def test_release_frees_after_readers_and_adopt_keeps_caller_memory():
    import torch
    a, b = rand_limbs(5000, 11), rand_limbs(7000, 12)
    ta = torch.from_numpy(a.view(np.int64)).cuda()
    torch.cuda.synchronize()
    ha = pm.adopt(ta.data_ptr(), a.size)
    hb = pm.upload(b)
    p, _ = pm.submit(ha, hb)
    q, t = pm.submit(p, ha)  # reads p and the adopted a
    pm.release(p)            # freed once q has read it
    pm.release(ha)           # the adopted memory stays the caller's
    pm.wait(t)
    assert _int(pm.download(q)) == _int(a) * _int(b) * _int(a)
    dq, nq = pm.handle_device(q)
    assert dq != 0 and nq == 2 * a.size + b.size
    assert np.array_equal(ta.cpu().numpy().view(np.uint64), a)
    with pytest.raises(pm.PimulError):
        pm.download(p)       # released and freed
    pm.free(q)
    pm.free(hb)


def test_served_chudnovsky_matches_golden():
    import hashlib
    import json
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "golden", "pi_digits_100k.txt")) as f:
        ref = f.read().strip()
    for d, nodes in ((1000, 0), (100_000, 0), (100_000, 7), (100_000, 4096)):
        s, info = pm.pi_chudnovsky_served(d, nodes)
        assert s == ref[:d], (d, nodes)
    assert info["service_requests"] > 0
    with open(os.path.join(here, "golden", "pi_digits_hashes.json")) as f:
        want = json.load(f)["1000000"]
    s, info = pm.pi_chudnovsky_served(1_000_000)
    assert hashlib.sha256(s.encode()).hexdigest() == want["sha256"]
    assert info["service_requests"] >= 5 * 100
