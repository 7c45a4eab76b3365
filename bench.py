#!/usr/bin/env python3
"""Benchmark: the isolated big-integer multiply on one GB300.

Headline workload: one balanced 2^30-bit x 2^30-bit product per step
(2^24 x 2^24 limbs, Goldilocks NTT length N = 2^27), seeded synthetic limbs
(uniform, top limb's bit 63 set).  The metric is NTT-multiply GB/s on the
algorithmic-bytes model of a two-pass transform:

    B_mul(N) = 96 N + 16 (la + lb) bytes per product.

`value` times products whose operands are already resident in HBM (device
API, CUDA events on the launching stream); `e2e` times the drop-in host API
(pimul_mul) with pinned host buffers, so every step includes the
host->device copy of both operands and the device->host copy of the product.

`--impl reference` times the CPU restatement of the reference's multiply
(the oracle, all host threads) on the same workload.  With --gpus N > 1
under torchrun, every rank runs an independent replica (the multiply does
not shard): value = all ranks' bytes / max rank time.
"""
from __future__ import annotations

import argparse
import hashlib
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

PROJECT_METRIC = "1e9-digit pi wall-s; NTT-mul GB/s, batched ops/s & p99 vs plain GPU, bit-exact"


def mul_metric():
    """metric of the isolated multiply (both arms), at the operand size in use."""
    return f"NTT-mul GB/s (2^{BITS_A.bit_length() - 1} x 2^{BITS_B.bit_length() - 1}-bit product)"


BITS_A = 1 << 30
BITS_B = 1 << 30

# DRAM traffic of the dominant kernel class (forward passes) per transform
# word: dram__bytes_read.sum + dram__bytes_write.sum from one ncu capture of
# each of k_col_mid<9,fwd> (15.60 bytes per word) and k_fwd_last<9> (15.53)
# of a 2^30 x 2^30-bit product (N = 2^27); the class runs the first twice
# and the second once per transform: 15.58 N bytes per launch.
NCU_TRAFFIC_BYTES_PER_WORD = 15.58


def b_mul(n, la, lb, square=False):
    return (64 * n + 24 * la) if square else (96 * n + 16 * (la + lb))


def next_pow2_log(x):
    return (x - 1).bit_length()


def mul_workload(la, lb, L):
    """config.workload of the isolated multiply (the same string in both arms)."""
    return (f"isolated multiply, balanced 2^{(64 * la).bit_length() - 1} x 2^{(64 * lb).bit_length() - 1} bits "
            f"({la} x {lb} limbs), N = 2^{L}")


def make_operands(la, lb, seed=20241203):
    rng = np.random.default_rng(seed)
    a = rng.integers(0, 1 << 64, size=la, dtype=np.uint64)
    b = rng.integers(0, 1 << 64, size=lb, dtype=np.uint64)
    a[-1] |= np.uint64(1 << 63)
    b[-1] |= np.uint64(1 << 63)
    return a, b


# ----------------------------------------------------------------- distributed
def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def dist_init(ws, backend):
    if ws <= 1:
        return None
    import torch.distributed as dist
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    dist.init_process_group(backend=backend)
    return dist


def reduce_max(dist, x, device="cpu"):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_value(world_size, bytes_per_step, steps, ms_total_max):
    """GB/s over all ranks: every rank runs an independent replica, timed
    by the slowest rank (max over ranks)."""
    return world_size * bytes_per_step * steps / (ms_total_max * 1e-3) / 1e9


def barrier(dist, device=None):
    if dist is None:
        return
    if device is not None:
        dist.barrier(device_ids=[device])
    else:
        dist.barrier()


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0, period_ms=50):
        self.gpu = gpu_index
        self.period = period_ms
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", f"-lms={self.period}"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ----------------------------------------------------------------- peaks
def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ----------------------------------------------------------------- kernel stats
def stats(lib):
    out = {}
    name = ctypes.c_char_p()
    launches = ctypes.c_uint64()
    timed = ctypes.c_uint64()
    ms = ctypes.c_double()
    k = 0
    while lib.pimul_stats_get(k, ctypes.byref(name), ctypes.byref(launches), ctypes.byref(timed),
                              ctypes.byref(ms)) == 0:
        out[name.value.decode()] = {"launches": launches.value, "timed": timed.value, "ms": ms.value}
        k += 1
    return out


# ALU-pipe warp instructions per transform word, per launch of each pass
# kernel (smsp__inst_executed_pipe_alu.sum / N from one ncu capture per
# kernel of a 2^30 x 2^30-bit product, N = 2^27, plan 2^9 x 2^9 x 2^9;
# k_fwd_first<9> with the half-zero first round from a 2^28 x 2^28-bit
# product, N = 2^25, the same kernel); "carry" is the three carry kernels
# together.  Instruction counts do not depend on the clock or on timing.
NCU_ALU_PER_WORD = {
    "k_fwd_first": 2.68, "k_col_mid_fwd": 2.82, "k_fwd_last": 2.22, "k_mid": 4.36,
    "k_col_mid_inv": 2.66, "k_inv_first_carry": 3.04, "carry": 0.46,
}
# The integer ALU pipe retires 16 lanes per clock per SM sub-partition:
# half a warp instruction per clock, four sub-partitions per SM.
ALU_WARP_INSTR_PER_CLK_PER_SM = 4 * 0.5


def alu_per_word(kind):
    """Mean ALU warp instructions per word of one launch of a kernel class."""
    a = NCU_ALU_PER_WORD
    return {"pack": a["k_fwd_first"], "pass_fwd": (2 * a["k_col_mid_fwd"] + a["k_fwd_last"]) / 3,
            "pass_inv": (a["k_col_mid_inv"] + a["k_inv_first_carry"]) / 2, "pointwise": a["k_mid"],
            "carry": a["carry"] / 3}.get(kind, 0.0)


def kernel_bytes_per_launch(kind, n, la, lb):
    """Algorithmic bytes of one launch of each kernel class."""
    if kind in ("pass_fwd", "pass_inv"):
        return 16 * n              # read and write the N-word array once
    if kind == "pack":
        return 8 * n + 8 * la      # read limbs, write N coefficients
    if kind == "pointwise":
        return 24 * n              # read two arrays, write one
    if kind == "carry":
        return 8 * n + 8 * (la + lb)
    return 0


# ----------------------------------------------------------------- GPU arm
def run_gpu(args):
    import torch
    ws, rank, local = dist_info()
    torch.cuda.set_device(local)
    dist = dist_init(ws, "nccl")
    import pi_gb300 as pm
    lib = pm.lib()
    pm.init(local)
    la, lb = BITS_A // 64, BITS_B // 64
    L = next_pow2_log(4 * la + 4 * lb - 1)
    N = 1 << L
    bytes_step = b_mul(N, la, lb)
    a, b = make_operands(la, lb, seed=20241203 + rank)
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        da = torch.from_numpy(a.view(np.int64)).cuda()
        db = torch.from_numpy(b.view(np.int64)).cuda()
        dout = torch.empty(la + lb, dtype=torch.int64, device="cuda")
    stream.synchronize()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def step():
        rc = lib.pimul_mul_device(ctypes.c_void_p(da.data_ptr()), la, ctypes.c_void_p(db.data_ptr()), lb,
                                  ctypes.c_void_p(dout.data_ptr()), sp)
        if rc:
            raise RuntimeError(lib.pimul_last_error().decode())

    for _ in range(args.warmup):
        step()
    stream.synchronize()
    # correctness spot check of the warm-up result (low limbs exact)
    low = dout[:8].cpu().numpy().view(np.uint64)
    ia = sum(int(x) << (64 * i) for i, x in enumerate(a[:8]))
    ib = sum(int(x) << (64 * i) for i, x in enumerate(b[:8]))
    want = (ia * ib) % (1 << 512)
    got = sum(int(x) << (64 * i) for i, x in enumerate(low))
    if got != want:
        raise RuntimeError("bench: product low limbs mismatch")

    lib.pimul_stats_reset()
    lib.pimul_stats_enable(1)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier(dist, local)
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
        barrier(dist, local)
    lib.pimul_stats_enable(0)
    ks = stats(lib)
    ms_total = ev0.elapsed_time(ev1)
    ms_total = reduce_max(dist, ms_total, device=f"cuda:{local}")
    ms_step = ms_total / args.steps
    value = whole_job_value(ws, bytes_step, args.steps, ms_total)

    # ---- e2e through the drop-in host API, pinned host buffers
    pa = torch.from_numpy(a.view(np.int64)).pin_memory()
    pb = torch.from_numpy(b.view(np.int64)).pin_memory()
    pout = torch.empty(la + lb, dtype=torch.int64).pin_memory()
    u64p = ctypes.POINTER(ctypes.c_uint64)
    ap = ctypes.cast(ctypes.c_void_p(pa.data_ptr()), u64p)
    bp = ctypes.cast(ctypes.c_void_p(pb.data_ptr()), u64p)
    op = ctypes.cast(ctypes.c_void_p(pout.data_ptr()), u64p)
    olen = ctypes.c_size_t(0)

    def e2e_step():
        rc = lib.pimul_mul(ap, la, bp, lb, op, la + lb, ctypes.byref(olen))
        if rc:
            raise RuntimeError(lib.pimul_last_error().decode())

    e2e_steps = max(3, min(args.steps, 10))
    if args.no_e2e:
        e2e_steps = 0
    else:
        e2e_step()
    barrier(dist, local)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    t1 = time.perf_counter()
    e2e_s = reduce_max(dist, t1 - t0, device=f"cuda:{local}")
    e2e_value = ws * bytes_step * e2e_steps / e2e_s / 1e9 if e2e_steps else None

    # ---- roofline of the dominant kernel class
    peak, peak_kind = measured_peaks()
    dom = max((k for k in ks if ks[k]["timed"]), key=lambda k: ks[k]["ms"])
    avg_ms = ks[dom]["ms"] / ks[dom]["timed"]
    per_launch = kernel_bytes_per_launch(dom, N, la, lb)
    achieved = per_launch / (avg_ms * 1e-3) / 1e9
    step_achieved = bytes_step / (ms_step * 1e-3) / 1e9
    launches = sum(v["launches"] for v in ks.values())
    # integer-pipe roofline: ALU warp instructions (ncu counts per word) over
    # the pipe's capacity at the SM clock sampled during the timed region
    clocks = clk.summary()
    n_sm = torch.cuda.get_device_properties(local).multi_processor_count
    f_sm = (clocks["sm_mhz"] or clocks["sm_max_mhz"] or 2070.0) * 1e6
    alu_cap = n_sm * ALU_WARP_INSTR_PER_CLK_PER_SM * f_sm  # warp instructions / s
    int_frac = alu_per_word(dom) * N / (avg_ms * 1e-3) / alu_cap
    step_alu = sum(alu_per_word(k) * N * ks[k]["launches"] / args.steps for k in ks)
    int_frac_step = step_alu / (ms_step * 1e-3) / alu_cap

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline_sample(la, lb, N)

    if rank == 0:
        line = {
            "metric": mul_metric(),
            "project_metric": PROJECT_METRIC,
            "value": round(value, 2),
            "unit": "GB/s",
            "n_gpus": ws,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": round(ms_step, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "u64",
            "data": "synthetic: seeded uniform u64 limbs, top limb bit 63 set (numpy PCG64)",
            "config": {
                "workload": mul_workload(la, lb, L),
                "bits_a": BITS_A, "bits_b": BITS_B, "la": la, "lb": lb, "transform_len": N,
                "bytes_per_step_model": "B_mul(N) = 96N + 16(la+lb)",
                "bytes_per_step": bytes_step,
                "l2": "inputs + scratch (2.3 GiB) exceed the 129 MB L2; no flush needed",
                "parallelism": f"replicas x{ws}",
            },
            "e2e": None if not e2e_steps else {
                    "value": round(e2e_value, 2), "unit": "GB/s", "ms_per_step": round(1e3 * e2e_s / e2e_steps, 3),
                    "h2d_bytes_per_step": 8 * (la + lb), "d2h_bytes_per_step": 8 * (la + lb),
                    "api": "pimul_mul (host buffers, pinned)",
                    "host_link": "pinned copies measured on this box at 209 GB/s H2D and 192 GB/s D2H (copy engines "
                                 "and SM copy kernels alike): a's upload and the product's download cannot overlap "
                                 "the multiply; b's upload is hidden behind a's forward transform"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak,
                         "peak_source": peak_kind, "unit": "GB/s", "frac": round(achieved / peak, 4),
                         "traffic": round(NCU_TRAFFIC_BYTES_PER_WORD * N) if dom == "pass_fwd" else None,
                         "bytes_per_launch": per_launch, "avg_launch_ms": round(avg_ms, 4),
                         "step_achieved": round(step_achieved, 1),
                         "step_frac": round(step_achieved / peak, 4),
                         "int_frac": round(int_frac, 4), "int_frac_step": round(int_frac_step, 4),
                         "int_model": {"alu_warp_instr_per_word": round(alu_per_word(dom), 3),
                                       "alu_warp_instr_per_step": round(step_alu),
                                       "peak_warp_instr_per_s": round(alu_cap),
                                       "sms": n_sm, "sm_mhz": f_sm / 1e6,
                                       "model": "ALU-pipe warp instructions per word from ncu x N, over "
                                                "SMs x 4 sub-partitions x 0.5 warp instr/clk x sampled SM clock"},
                         "binding_unit": "integer ALU pipe (int_frac), not HBM (frac)",
                         "io_effective_gbs": round(16 * (la + lb) / (ms_step * 1e-3) / 1e9, 1),
                         "integer_model": {
                             "butterflies": 3 * (N // 2) * L, "pointwise_mulmods": 2 * N,
                             "butterflies_per_s": round(3 * (N // 2) * L / (ms_step * 1e-3), 1),
                             "model": "3 (N/2) log2 N radix-2-equivalent butterflies + 2N pointwise/scale "
                                      "products per multiply"}},
            "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3)} for k, v in ks.items()},
            "gpu_launches": launches,
            "clocks": clocks,
            "cpu_baseline": cpu,
        }
        if ws == 1:
            run_extras(line, args, peak)
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


# ----------------------------------------------------------------- extras
# The other configurations, measured in the same default run and reported
# as keys of the headline line: the isolated-multiply sweep, the batched
# uneven products, the served stream at several offered loads, pi runs and
# a BBP sample.
SWEEP = [("mul", 16, 16), ("mul", 20, 20), ("mul", 24, 24), ("mul", 28, 28), ("mul", 30, 30), ("mul", 30, 20),
         ("sqr", 16, 16), ("sqr", 20, 20), ("sqr", 24, 24), ("sqr", 28, 28), ("sqr", 30, 30)]
L2_FLUSH_BYTES = 512 << 20  # written between timed calls: larger than the 129 MB L2


def sweep_measure(peak):
    """Config 2's sweep: balanced 2^16..2^30-bit products, 2^30 x 2^20 and
    squares, operands resident in HBM.  Every call is timed alone with CUDA
    events on its stream after a 512 MiB write that flushes L2; the median
    over the repetitions is reported, with GB/s on the two-pass bytes model
    and a SHA-256 prefix of the product."""
    import hashlib
    import torch
    import pi_gb300 as pm
    lib = pm.lib()
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda")
    rows = []
    for kind, ba, bb in SWEEP:
        sq = kind == "sqr"
        la, lb = (1 << ba) // 64, (1 << bb) // 64
        a, b = make_operands(la, lb, seed=1000 + ba + 64 * bb)
        with torch.cuda.stream(stream):
            da = torch.from_numpy(a.view(np.int64)).cuda()
            db = da if sq else torch.from_numpy(b.view(np.int64)).cuda()
            dout = torch.empty(la + (la if sq else lb), dtype=torch.int64, device="cuda")
        stream.synchronize()
        lb_eff = la if sq else lb

        def one():
            rc = lib.pimul_mul_device(ctypes.c_void_p(da.data_ptr()), la, ctypes.c_void_p(db.data_ptr()), lb_eff,
                                      ctypes.c_void_p(dout.data_ptr()), sp)
            if rc:
                raise RuntimeError(lib.pimul_last_error().decode())

        for _ in range(3):
            one()
        stream.synchronize()
        L = next_pow2_log(4 * la + 4 * lb_eff - 1)
        n = 1 << L
        reps = 20 if L >= 25 else 50
        times = []
        with torch.cuda.stream(stream):
            for _ in range(reps):
                flush.fill_(1)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                one()
                e1.record(stream)
                times.append((e0, e1))
        stream.synchronize()
        ms = statistics.median(e0.elapsed_time(e1) for e0, e1 in times)
        by = b_mul(n, la, lb_eff, square=sq)
        gbs = by / (ms * 1e-3) / 1e9
        digest = hashlib.sha256(dout.cpu().numpy().tobytes()).hexdigest()[:16]
        rows.append({"case": f"square 2^{ba} bits" if sq else f"2^{ba} x 2^{bb} bits", "la": la, "lb": lb_eff,
                     "transform_len": f"2^{L}", "ms": round(ms, 4), "gbs": round(gbs, 1),
                     "hbm_frac": round(gbs / peak, 4), "io_gbs": round(16 * (la + lb_eff) / (ms * 1e-3) / 1e9, 1),
                     "reps": reps, "product_sha256_16": digest})
        del da, db, dout
    del flush
    torch.cuda.empty_cache()
    return {"model": "B_mul(N) = 96N + 16(la+lb), B_sqr(N) = 64N + 24la bytes; hbm_frac of measured HBM GB/s",
            "timing": "each call alone: CUDA events around one pimul_mul_device after a 512 MiB L2 flush; median",
            "parity": "bit-exact vs the oracle in tests/test_mul_gpu.py (full sizes included)",
            "rows": rows}


def pi_measure():
    """Chudnovsky pi to 10^9 digits through the level-batched, device-resident
    splitting, and 10^8 digits both batched and plain (one GPU call per
    product); wall times, phase splits and SHA-256 of the digits, compared
    with the recorded hashes (10^8: the CPU restatement's digits)."""
    import hashlib
    import pi_gb300 as pm
    pm.init(0)
    golden = {}
    path = os.path.join(ROOT, "tests", "golden", "pi_digits_hashes.json")
    if os.path.exists(path):
        with open(path) as f:
            golden = json.load(f)
    out = {}
    pm.pi_chudnovsky_batched(100_000)  # warm-up (tables, pools, kernels)
    pm.pi_chudnovsky(100_000)
    for D in (10 ** 9, 10 ** 8):
        t0 = time.perf_counter()
        s, info = pm.pi_chudnovsky_batched(D)
        wall = time.perf_counter() - t0
        h = hashlib.sha256(s.encode()).hexdigest()
        rec = golden.get(str(D))
        key = "pi_1e9" if D == 10 ** 9 else "pi_1e8_plain_vs_batched"
        out[key] = {"digits": D, "batched_wall_s": round(wall, 3),
                    "phases_ms": {k: round(v, 1) for k, v in info.items() if k.endswith("_ms")},
                    "gpu_products": info["ntt_products"], "sha256": h, "last20": s[-20:],
                    "matches_recorded": None if rec is None else (h == rec["sha256"]),
                    "recorded_source": None if rec is None else rec.get("source", "mpmath")}
        if D == 10 ** 8:
            t1 = time.perf_counter()
            sp_, _ = pm.pi_chudnovsky(D)
            pwall = time.perf_counter() - t1
            out[key].update({"plain_wall_s": round(pwall, 3), "speedup_batched_vs_plain": round(pwall / wall, 2),
                             "plain_identical": sp_ == s})
            del sp_
            # the splitting tree's upper levels through the multiply service
            # (chained handles submitted as the recursion unfolds)
            pm.pi_chudnovsky_served(100_000)
            t2 = time.perf_counter()
            ss_, sinfo = pm.pi_chudnovsky_served(D)
            swall = time.perf_counter() - t2
            out[key].update({"served_wall_s": round(swall, 3), "served_identical": ss_ == s,
                             "served_service_requests": sinfo["service_requests"],
                             "served_phases_ms": {k: round(v, 1) for k, v in sinfo.items() if k.endswith("_ms")}})
            del ss_
        del s
    return out


def bbp_measure(positions=64, max_pos=8e8):
    """A seeded sample of config 5's BBP spot checks, one batched launch."""
    import pi_gb300 as pm
    rng = np.random.default_rng(2025)
    pos = rng.integers(0, int(max_pos), size=positions, dtype=np.uint64)
    pm.bbp_hex_digits(np.arange(64, dtype=np.uint64))
    t0 = time.perf_counter()
    d = pm.bbp_hex_digits(pos)
    dt = time.perf_counter() - t0
    terms = 4.0 * float((pos.astype(np.float64) + 1).sum())
    return {"positions": positions, "range": f"[0, {int(max_pos)})", "wall_s": round(dt, 3),
            "positions_per_s": round(positions / dt, 3), "terms_per_s": round(terms / dt, 1),
            "extrapolated_65536_positions_s": round(dt * 65536 / positions, 1),
            "first_digits": [f"{int(x):08x}" for x in d[:4]]}


def run_extras(line, args, peak):
    """Adds the other configurations to the headline line (rank 0, one GPU)."""
    import torch
    steps = [("sweep", lambda: sweep_measure(peak)),
             ("batch4096", lambda: batch_measure(10, 3, tune=True, cpu=not args.no_cpu_baseline)),
             ("served", lambda: served_measure(args.requests, [0.8, 1.0, 1.5, 2.0])),
             ("pi", pi_measure),
             ("bbp", bbp_measure)]
    only = set(args.extras.split(",")) if args.extras not in ("all", "none") else None
    for name, fn in steps:
        if args.extras == "none" or (only is not None and name not in only):
            continue
        t0 = time.perf_counter()
        try:
            r = fn()
        except Exception as e:  # noqa: BLE001 - one failing extra must not lose the headline
            r = {"error": f"{type(e).__name__}: {e}"}
        torch.cuda.empty_cache()
        if name == "pi" and "error" not in r:
            line.update(r)
        else:
            for k in ("project_metric", "n_gpus", "vs_baseline", "dtype", "scaling"):
                r.pop(k, None)
            line[name] = r
        line.setdefault("extras_wall_s", {})[name] = round(time.perf_counter() - t0, 1)


# ----------------------------------------------------------------- batched form
def batch_sizes(n=4096, lo=10, hi=22, seed=20241203):
    """Operand bit lengths log-uniform in [2^lo, 2^hi], independent per operand."""
    rng = np.random.default_rng(seed)
    bits = np.exp(rng.uniform(lo * np.log(2), hi * np.log(2), size=(n, 2))).astype(np.int64)
    return np.maximum(bits, 1)


def make_exact_bits(rng, bits):
    limbs = (bits + 63) // 64
    x = rng.integers(0, 1 << 64, size=limbs, dtype=np.uint64)
    top = (bits - 1) % 64
    x[-1] &= np.uint64((1 << (top + 1)) - 1) if top < 63 else np.uint64(0xFFFFFFFFFFFFFFFF)
    x[-1] |= np.uint64(1 << top)
    return x


def run_batch(args):
    print(json.dumps(batch_measure(args.steps, args.warmup, tune=not args.no_tune, cpu=not args.no_cpu_baseline)),
          flush=True)


def batch_measure(steps, warmup, tune=True, cpu=True):
    """Config 3: 4,096 independent products of uneven sizes; the graph-planned
    batch vs the direct batch vs one pimul_mul_device call per product."""
    import torch
    import pi_gb300 as pm
    pm.init(0)
    lib = pm.lib()
    bits = batch_sizes()
    rng = np.random.default_rng(7)
    ops_a = [make_exact_bits(rng, int(b)) for b in bits[:, 0]]
    ops_b = [make_exact_bits(rng, int(b)) for b in bits[:, 1]]
    la = np.array([x.size for x in ops_a])
    lb = np.array([x.size for x in ops_b])
    flat = np.concatenate(ops_a + ops_b)
    d_in = torch.from_numpy(flat.view(np.int64)).cuda()
    offs_a = np.concatenate([[0], np.cumsum(la)[:-1]])
    offs_b = la.sum() + np.concatenate([[0], np.cumsum(lb)[:-1]])
    out_off = np.concatenate([[0], np.cumsum(la + lb)[:-1]])
    d_out = torch.zeros(int((la + lb).sum()), dtype=torch.int64, device="cuda")
    d_ref = torch.zeros_like(d_out)
    base, obase, rbase = d_in.data_ptr(), d_out.data_ptr(), d_ref.data_ptr()
    jobs = [(base + 8 * int(offs_a[i]), int(la[i]), base + 8 * int(offs_b[i]), int(lb[i]),
             obase + 8 * int(out_off[i])) for i in range(len(la))]
    rjobs = [(a, x, b, y, rbase + 8 * int(out_off[i])) for i, (a, x, b, y, _) in enumerate(jobs)]
    tune = pm.autotune(7, 19, 4) if tune else {}
    stream = torch.cuda.Stream()
    sp = stream.cuda_stream
    plan = pm.BatchPlan(la, lb)
    arr, n = pm._job_array(jobs)

    def step_plan():
        lib.pimul_batch_plan_run(plan._h, ctypes.cast(arr, ctypes.c_void_p), n, ctypes.c_void_p(sp))

    def step_direct():
        lib.pimul_mul_batch(ctypes.cast(arr, ctypes.c_void_p), n, ctypes.c_void_p(sp))

    def step_plain():
        for (a, x, b, y, o) in rjobs:
            lib.pimul_mul_device(ctypes.c_void_p(a), x, ctypes.c_void_p(b), y, ctypes.c_void_p(o),
                                 ctypes.c_void_p(sp))

    def timeit(fn, steps, warm):
        for _ in range(warm):
            fn()
        stream.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        lat = []
        e0.record(stream)
        for _ in range(steps):
            t = time.perf_counter()
            fn()
            lat.append(time.perf_counter() - t)
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1) / steps

    ms_plan = timeit(step_plan, steps, warmup)
    ms_direct = timeit(step_direct, steps, warmup)
    ms_plain = timeit(step_plain, max(2, steps // 4), 1)
    step_plan()
    step_plain()
    stream.synchronize()
    exact = bool(torch.equal(d_out, d_ref))
    nprod = len(la)
    total_bits = float((la.astype(np.float64) * 64).sum() + (lb.astype(np.float64) * 64).sum())
    bytes_model = 0
    for x, y in zip(la, lb):
        N = 1 << next_pow2_log(4 * int(x) + 4 * int(y) - 1)
        bytes_model += b_mul(N, int(x), int(y))
    line = {
        "metric": "batched products/s (4096 uneven products)",
        "project_metric": PROJECT_METRIC,
        "value": round(nprod / (ms_plan * 1e-3), 1),
        "unit": "products/s",
        "n_gpus": 1, "steps": steps, "warmup": warmup,
        "ms_per_step": round(ms_plan, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic: operand bit lengths log-uniform in [2^10, 2^22], uniform limbs (seeded)",
        "config": {"workload": "4096 independent products, each operand's bit length log-uniform in [2^10, 2^22]",
                   "limbs_total": int(la.sum() + lb.sum())},
        "plain_per_call_ms": round(ms_plain, 3),
        "direct_batch_ms": round(ms_direct, 3),
        "speedup_plan_vs_plain": round(ms_plain / ms_plan, 2),
        "speedup_direct_vs_plain": round(ms_plain / ms_direct, 2),
        "bits_per_s": round(total_bits / (ms_plan * 1e-3), 1),
        "model_gbs": round(bytes_model / (ms_plan * 1e-3) / 1e9, 1),
        "bit_exact_vs_plain": exact,
        "autotune": tune,
        "cpu_baseline": batch_cpu_baseline(ops_a, ops_b, d_out, out_off) if cpu else None,
    }
    plan.close()
    return line


def batch_cpu_baseline(ops_a, ops_b, d_out, out_off):
    """The oracle's mul_mag (the reference's dispatch: schoolbook, Karatsuba,
    NTT at >= 8192 limbs) on the same products: all 4096 across a pool of
    single-threaded workers (one product per task), and a seeded 1/8
    subsample one after another on one thread (scaled to 4096)."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor
    oracle.build()
    threads = oracle.max_threads()
    n = len(ops_a)

    def one(i):
        oracle.set_threads(1)  # this worker's OpenMP setting
        return oracle.mul_mag(ops_a[i], ops_b[i])

    try:
        t0 = time.perf_counter()
        with ThreadPoolExecutor(max_workers=threads) as ex:
            res = list(ex.map(one, range(n)))
        t_pool = time.perf_counter() - t0
        sub = np.random.default_rng(9).choice(n, size=n // 8, replace=False)
        oracle.set_threads(1)
        t1 = time.perf_counter()
        for i in sub:
            oracle.mul_mag(ops_a[i], ops_b[i])
        t_serial = (time.perf_counter() - t1) * n / len(sub)
    finally:
        oracle.set_threads(threads)
    # the pool's products against the GPU's (device output, trimmed)
    out = d_out.cpu().numpy().view(np.uint64)
    same = all(np.array_equal(res[i], np.trim_zeros(out[int(out_off[i]): int(out_off[i]) + ops_a[i].size +
                                                         ops_b[i].size], "b")) for i in range(n))
    return {"value": round(n / t_pool, 1), "unit": "products/s", "cores": threads, "kind": "port",
            "seconds": round(t_pool, 3),
            "sample": f"the same {n} products through the C restatement of mul_mag (integer.rs:445-486 dispatch), "
                      f"a pool of {threads} single-threaded workers",
            "serial_one_core": {"value": round(n / t_serial, 1), "unit": "products/s",
                                "seconds_scaled": round(t_serial, 3),
                                "sample": f"{n // 8} seeded products of the batch on one thread, scaled to {n}"},
            "gpu_matches_cpu": bool(same)}


# ----------------------------------------------------------------- served form
def served_stream(n, seed=20241204, lo=12, hi=28, chain=0.3, sq=0.25):
    """Config 4 request stream: operand bit lengths log-uniform in
    [2^lo, 2^hi]; about 30 % of requests consume an earlier result (only
    results below 2^27 bits are chained, so chains stay bounded); a quarter
    of the requests are squares."""
    rng = np.random.default_rng(seed)
    bits = np.exp(rng.uniform(lo * np.log(2), hi * np.log(2), size=n)).astype(np.int64)
    base = [make_exact_bits(rng, int(b)) for b in bits]
    reqs, out_limbs = [], []
    for k in range(n):
        x = k
        if k > 0 and rng.random() < chain:
            cands = [j for j in range(max(0, k - 64), k) if out_limbs[j] * 64 < (1 << 27)]
            if cands:
                x = -(int(rng.choice(cands)) + 1)
        la = base[x].size if x >= 0 else out_limbs[-x - 1]
        if rng.random() < sq:
            reqs.append(("sqr", x, x))
            out_limbs.append(2 * la)
        else:
            y = int(rng.integers(0, n))
            reqs.append(("mul", x, y))
            out_limbs.append(la + base[y].size)
    return base, reqs


def run_served(args):
    loads = [float(x) for x in str(args.load).split(",")]
    print(json.dumps(served_measure(args.requests, loads)), flush=True)


def served_measure(n, loads):
    """Config 4: Poisson request stream through the device-resident service
    (continuous batching, chained handles, HBM budget) vs the plain per-call
    path fed by one worker in arrival order, at each offered load (a multiple
    of the plain path's measured capacity; above 1 the plain path saturates).
    Latency = completion - arrival.  Results are compared bit for bit with
    the plain path's at the first load."""
    import torch
    import pi_gb300 as pm
    pm.init(0)
    lib = pm.lib()
    base, reqs = served_stream(n)
    pm.set_budget(120 << 30)
    # ---- plain path: device operands as torch tensors, results kept
    dbase = [torch.from_numpy(x.view(np.int64)).cuda() for x in base]
    stream = torch.cuda.Stream()
    sp = ctypes.c_void_p(stream.cuda_stream)

    def plain_one(k, res):
        op, x, y = reqs[k]
        a = dbase[x] if x >= 0 else res[-x - 1]
        b = a if op == "sqr" else (dbase[y] if y >= 0 else res[-y - 1])
        out = torch.empty(a.numel() + b.numel(), dtype=torch.int64, device="cuda")
        lib.pimul_mul_device(ctypes.c_void_p(a.data_ptr()), a.numel(), ctypes.c_void_p(b.data_ptr()), b.numel(),
                             ctypes.c_void_p(out.data_ptr()), sp)
        stream.synchronize()
        return out

    # capacity of the plain path (back to back, no arrivals)
    res = []
    for k in range(min(n, 32)):  # warm-up
        res.append(plain_one(k, res))
    res = []
    t0 = time.perf_counter()
    for k in range(n):
        res.append(plain_one(k, res))
    t_serial = time.perf_counter() - t0
    capacity = n / t_serial
    del res
    torch.cuda.empty_cache()
    hb = [pm.upload(x) for x in base]
    runs = []
    exact = None
    # every load with the default admission policy (transforms of 2^24 and
    # longer run alone, smaller ones are batched), then the highest load
    # again with 2^20 and longer alone (mid-size products one at a time)
    plan = [(load, 24) for load in loads] + [(max(loads), 20)]
    for li, (load, big) in enumerate(plan):
        pm.service_config(big_log_n=big)
        lam = load * capacity
        rng = np.random.default_rng(99)
        arrivals = np.cumsum(rng.exponential(1.0 / lam, size=n))
        # ---- plain path under the arrival process (one worker, FIFO)
        res = []
        lat_plain = []
        t0 = time.perf_counter()
        for k in range(n):
            while time.perf_counter() - t0 < arrivals[k]:
                pass
            res.append(plain_one(k, res))
            lat_plain.append(time.perf_counter() - t0 - arrivals[k])
        span_plain = time.perf_counter() - t0
        plain_host = [np.trim_zeros(r.cpu().numpy().view(np.uint64), "b") for r in res] if li == 0 else None
        del res
        torch.cuda.empty_cache()
        # ---- served path
        pm.service_reset_stats()
        outs, tickets = [], []
        t0 = time.perf_counter()
        for k, (op, x, y) in enumerate(reqs):
            while time.perf_counter() - t0 < arrivals[k]:
                pass
            ha = hb[x] if x >= 0 else outs[-x - 1]
            if op == "sqr":
                h, t = pm.submit(ha)
            else:
                h, t = pm.submit(ha, hb[y] if y >= 0 else outs[-y - 1])
            outs.append(h)
            tickets.append(t)
        for t in tickets:
            pm.wait(t)
        span_served = time.perf_counter() - t0
        st = pm.service_stats()
        if plain_host is not None:
            served_host = [pm.download(h) for h in outs]
            exact = all(np.array_equal(a, b) for a, b in zip(served_host, plain_host))
            del served_host, plain_host
        for h in outs:
            pm.free(h)
        lp = np.array(lat_plain) * 1e3
        runs.append({
            "offered_load": load, "lambda_rps": round(lam, 1), "alone_from_log_n": big,
            "served": {"p50_ms": round(st["p50_ms"], 3), "p99_ms": round(st["p99_ms"], 3),
                       "ops_per_s": round(n / span_served, 1), "batches": st["batches"]},
            "plain": {"p50_ms": round(float(np.percentile(lp, 50)), 3),
                      "p99_ms": round(float(np.percentile(lp, 99)), 3), "ops_per_s": round(n / span_plain, 1)},
            "throughput_served_over_plain": round(span_plain / span_served, 3)})
    pm.service_config(big_log_n=24)
    for h in hb:
        pm.free(h)
    first = runs[0]
    return {
        "metric": "served request stream: p50/p99 latency and ops/s vs plain per-call",
        "project_metric": PROJECT_METRIC,
        "value": first["served"]["ops_per_s"], "unit": "requests/s",
        "n_gpus": 1, "steps": 1, "warmup": 1, "ms_per_step": round(1e3 * n / first["served"]["ops_per_s"], 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic: Poisson arrivals (seeded), operand bits log-uniform in [2^12, 2^28], "
                "30% chained on earlier results, 25% squares",
        "config": {"workload": f"{n} requests per offered load, loads {loads} of the plain path's capacity",
                   "plain_capacity_rps": round(capacity, 1), "hbm_budget_bytes": 120 << 30},
        "served": first["served"], "plain": first["plain"], "loads": runs,
        "bit_exact_served_vs_plain": bool(exact),
    }


# ----------------------------------------------------------------- pi runs
def run_pi(args):
    """Config 1: Chudnovsky pi to D digits; every product at or above the
    reference's NTT threshold goes through the GPU multiply, one call per
    product.  The same pipeline with the CPU restatement of the reference's
    multiply is the CPU run; digits must be byte-identical."""
    import hashlib
    import pi_gb300 as pm
    pm.init(0)
    D = args.digits
    other_same = None
    gl_backend = pm.served_backend() if args.gl_backend == "served" else None

    def gl_run(d, **kw):
        return pm.pi_gauss_legendre(d, backend=kw.get("backend", gl_backend), fast_sqrt=args.gl_sqrt == "newton",
                                    device_decimal=args.gl_decimal == "device",
                                    device_agm=args.gl_backend == "device")

    if args.algorithm == "both":
        gl_run(min(D, 100_000))
        t0 = time.perf_counter()
        g, _ = gl_run(D)
        gl_wall = time.perf_counter() - t0
        args.algorithm = "chudnovsky"
        args.gl_wall = gl_wall
        args.gl_digits = g
    run = gl_run if args.algorithm == "gl" else pm.pi_chudnovsky
    run(min(D, 100_000))  # warm-up (tables, pools, kernels)
    batched = None
    if args.algorithm == "chudnovsky" and args.pi_mode in ("batched", "both"):
        pm.pi_chudnovsky_batched(min(D, 100_000), args.leaf_terms)
        t0 = time.perf_counter()
        sb, binfo = pm.pi_chudnovsky_batched(D, args.leaf_terms)
        bwall = time.perf_counter() - t0
        batched = {"wall_s": round(bwall, 3), "leaf_terms": args.leaf_terms or "auto (at most 64, per eighth of the terms)",
                   "phases_ms": {k: round(v, 1) for k, v in binfo.items() if k.endswith("_ms")},
                   "gpu_products": binfo["ntt_products"], "batched_levels": binfo["batched_levels"],
                   "sha256": hashlib.sha256(sb.encode()).hexdigest()}
    if batched is not None and args.pi_mode == "batched":
        s, info, wall = sb, binfo, bwall
    else:
        t0 = time.perf_counter()
        s, info = run(D)
        wall = time.perf_counter() - t0
    if batched is not None and args.pi_mode == "both":
        batched["digits_identical_to_plain"] = sb == s
        batched["speedup_vs_plain"] = round(wall / bwall, 3)
    cpu = None
    same = None
    if not args.no_cpu_baseline:
        import oracle
        oracle.build()
        t1 = time.perf_counter()
        sc, cinfo = run(D, backend=oracle.mul_abi_pointer())
        cwall = time.perf_counter() - t1
        same = sc == s
        cpu = {"value": round(cwall, 3), "unit": "s", "cores": oracle.max_threads(), "kind": "port",
               "sample": f"the same {D}-digit run with the C restatement of mul_mag_ntt "
                         "(crates/bignum/src/ntt.rs:806-865) as the multiply",
               "phases_ms": {k: round(v, 1) for k, v in cinfo.items() if k.endswith("_ms")}}
    if getattr(args, "gl_digits", None) is not None:
        other_same = args.gl_digits == s
    golden = None
    path = os.path.join(ROOT, "tests", "golden", "pi_digits_hashes.json")
    if os.path.exists(path):
        with open(path) as f:
            g = json.load(f).get(str(D))
        if g:
            golden = hashlib.sha256(s.encode()).hexdigest() == g["sha256"]
    line = {
        "metric": f"pi wall-s ({'Gauss-Legendre' if args.algorithm == 'gl' else 'Chudnovsky'}, {D} digits)",
        "project_metric": PROJECT_METRIC,
        "value": round(wall, 3), "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": round(1e3 * wall, 1), "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64", "data": "deterministic (no random input)",
        "config": {"workload": f"{'Gauss-Legendre AGM' if args.algorithm == 'gl' else 'Chudnovsky binary splitting'}"
                               f" for pi to {D} decimal digits, "
                               + ("binary splitting level by level through the batched GPU multiply, "
                                  "other products >= 8192 limbs one call each"
                                  if args.pi_mode == "batched" and args.algorithm == "chudnovsky" else
                                  "products >= 8192 limbs on the GPU (one call per product)")},
        "phases_ms": {k: round(v, 1) for k, v in info.items() if k.endswith("_ms")},
        "gpu_products": info["ntt_products"], "gpu_products_by_length": info.get("ntt_hist"),
        "digits_match_cpu_run": same, "digits_match_mpmath_sha256": golden,
        "batched_binary_splitting": batched,
        "gauss_legendre": None if other_same is None else {"wall_s": round(args.gl_wall, 3),
                                                           "multiply": args.gl_backend,
                                                           "sqrt": ("multiplication-only Newton" if args.gl_sqrt == "newton"
                                                                    else "reference (division-based)"),
                                                           "decimal": ("device-resident level-batched"
                                                                       if args.gl_decimal == "device"
                                                                       else "reference recursion"),
                                                           "digits_identical_to_chudnovsky": other_same},
        "sha256": hashlib.sha256(s.encode()).hexdigest(),
        "last_digits": s[-20:], "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- verify-hex
def run_hex(args):
    """verify-hex's decimal -> hex conversion (crates/pi-cli/src/verify_hex.rs:
    553-629) of D digits of pi computed by the batched Chudnovsky run
    (untimed): wall time of pimul_decimal_to_hex from host text to host
    text, hex digits spot-checked against BBP at seeded positions.  The CPU
    baseline is the oracle's exact-integer restatement on a bounded sample."""
    import hashlib
    import pi_gb300 as pm
    pm.init(0)
    D = args.digits
    if args.hex_input == "pi":
        s, _ = pm.pi_chudnovsky_batched(D)
        text = "3." + s[1:]
        del s
    else:  # seeded uniform digits: the conversion alone (profiling)
        digs = np.random.default_rng(2027).integers(0, 10, size=D - 1, dtype=np.uint8) + ord("0")
        text = "3." + digs.tobytes().decode()
        del digs
    pm.decimal_to_hex(text[: min(len(text), 100_002)])  # warm-up
    t0 = time.perf_counter()
    x, ph = pm.decimal_to_hex(text, phases=True)
    wall = time.perf_counter() - t0
    frac = x[2:]
    h = len(frac)
    if args.hex_input != "pi":
        args.hex_checks = 0
    rng = np.random.default_rng(2026)
    # seeded positions over the whole text, the first and the last one before
    # verify-hex's 32-digit tail (verify_hex.rs:540-547); at 2^31 and above
    # the BBP kernel's moduli would pass 2^34
    hi = max(1, min(h - 40, 1 << 31))
    pos = np.unique(np.concatenate([[0, hi - 1], rng.integers(0, hi, size=args.hex_checks)]).astype(np.uint64))
    bbp_ok = None
    if args.hex_input == "pi":
        d = pm.bbp_hex_digits(pos)
        bbp_ok = all(frac[int(p): int(p) + 8] == format(int(v), "08x") for p, v in zip(pos, d))
    cpu = None
    if not args.no_cpu_baseline:
        import oracle
        n = min(D, args.hex_cpu_digits)
        t1 = time.perf_counter()
        xc = oracle.decimal_to_hex(text[: n + 1])
        ct = time.perf_counter() - t1
        xg = pm.decimal_to_hex(text[: n + 1])
        cpu = {"value": round(ct, 3), "unit": "s", "cores": 1, "kind": "port",
               "sample": f"the first {n} digits through the oracle's restatement of verify_hex.rs:553-629 with "
                         "Python's exact integers (CPython's subquadratic string parse and division; the "
                         "reference's own parse is quadratic, integer.rs:127-148)",
               "gpu_same_sample_s": None, "gpu_matches_cpu": xc == xg}
        t2 = time.perf_counter()
        pm.decimal_to_hex(text[: n + 1])
        cpu["gpu_same_sample_s"] = round(time.perf_counter() - t2, 4)
    line = {
        "metric": f"decimal->hex conversion wall-s ({D} digits of pi)", "project_metric": PROJECT_METRIC,
        "value": round(wall, 3), "unit": "s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": round(1e3 * wall, 1), "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64", "data": ("pi's digits from the batched Chudnovsky run (deterministic)" if args.hex_input == "pi"
                                 else "seeded uniform decimal digits after \"3.\""),
        "config": {"workload": f"verify-hex conversion of {D} decimal digits to {h} hex digits, host text in and out"},
        "phases_ms": {k: round(v, 1) for k, v in zip(("parse", "power_of_ten", "quotient", "hex_digits"), ph)},
        "hex_digits": h, "bbp_positions_checked": int(pos.size) if bbp_ok is not None else 0, "bbp_matches": bbp_ok,
        "sha256": hashlib.sha256(x.encode()).hexdigest(), "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- BBP
def run_bbp(args):
    """Config 5's spot checks: batched BBP hex digits at seeded positions
    uniform in [0, max_pos); positions/s and modular multiplies/s.  The CPU
    oracle times a smaller seeded subsample (scaled linearly in n)."""
    import pi_gb300 as pm
    rng = np.random.default_rng(2025)
    pos = rng.integers(0, int(args.max_pos), size=args.positions, dtype=np.uint64)
    pm.bbp_hex_digits(np.arange(64, dtype=np.uint64))  # warm-up
    # launches of at most --bbp-batch positions (a full 65,536-position run
    # takes tens of minutes; each launch is bounded)
    bs = max(1, args.bbp_batch)
    t0 = time.perf_counter()
    d = np.concatenate([pm.bbp_hex_digits(pos[i:i + bs]) for i in range(0, pos.size, bs)])
    dt = time.perf_counter() - t0
    terms = 4.0 * float((pos.astype(np.float64) + 1).sum())
    digest = hashlib.sha256("".join(f"{int(p)} {int(x):08x}\n" for p, x in zip(pos, d)).encode()).hexdigest()
    check = None
    if args.check_digits:
        # every position against the hex digits of pi computed independently:
        # batched Chudnovsky to D decimal digits, then verify-hex's conversion
        D = int(args.check_digits)
        t1 = time.perf_counter()
        sdig, _ = pm.pi_chudnovsky_batched(D)
        hx = pm.decimal_to_hex("3." + sdig[1:])
        del sdig
        frac = hx[2:]
        limit = len(frac) - 40  # verify-hex leaves its last 32 hex digits unchecked
        ok = bad = 0
        for p_, x in zip(pos, d):
            if int(p_) + 8 <= limit:
                if frac[int(p_): int(p_) + 8] == f"{int(x):08x}":
                    ok += 1
                else:
                    bad += 1
        check = {"decimal_digits": D, "hex_digits": len(frac), "checked_below": limit, "positions_checked": ok + bad,
                 "matches": ok, "mismatches": bad, "seconds": round(time.perf_counter() - t1, 1)}
        del hx, frac
    line = {
        "metric": "BBP hex-digit spot checks (positions/s)", "project_metric": PROJECT_METRIC,
        "value": round(args.positions / dt, 3), "unit": "positions/s", "n_gpus": 1, "steps": 1, "warmup": 1,
        "ms_per_step": round(1e3 * dt, 1), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u64+f64", "data": f"seeded positions uniform in [0, {int(args.max_pos)})",
        "config": {"workload": f"{args.positions} positions in one batched launch"},
        "terms_per_s": round(terms / dt, 1),
        "extrapolated_65536_positions_s": round(dt * 65536 / args.positions, 1),
        "first_digits": [f"{int(x):08x}" for x in d[:4]],
        "digits_sha256": digest, "digits_format": "one line per position in seeded order: '<position> <8 hex>'",
        "cross_check": check,
    }
    if not args.no_cpu_baseline:
        import oracle
        oracle.build()
        sub = pos[: args.cpu_positions]
        scale = float(args.cpu_depth) / float(max(1, sub.mean()))
        sub = np.maximum((sub.astype(np.float64) * scale).astype(np.uint64), 1)
        t1 = time.perf_counter()
        cd = oracle.bbp_batch(sub)
        ct = time.perf_counter() - t1
        gd = pm.bbp_hex_digits(sub)
        cterms = 4.0 * float((sub.astype(np.float64) + 1).sum())
        line["cpu_baseline"] = {"value": round(cterms / ct, 1), "unit": "terms/s", "cores": oracle.max_threads(),
                                "kind": "port",
                                "sample": f"{sub.size} positions scaled to mean depth {args.cpu_depth} "
                                          "(C restatement of crates/pi-core/src/bbp.rs:52-140, OpenMP)",
                                "gpu_matches_cpu": bool(np.array_equal(cd, gd))}
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------- CPU legs
def cpu_baseline_sample(la, lb, n):
    """The oracle (CPU restatement of the reference's mul_mag_ntt) on one
    full-size product, all host threads."""
    import oracle
    oracle.build()
    threads = oracle.max_threads()
    a, b = make_operands(la, lb, seed=7)
    t0 = time.perf_counter()
    oracle.mul_mag_ntt(a, b)
    dt = time.perf_counter() - t0
    # one core: a bounded sample (a 2^26 x 2^26-bit product), same bytes model
    sa, sb = make_operands(1 << 20, 1 << 20, seed=8)
    sn = 1 << next_pow2_log(4 * (2 << 20) - 1)
    oracle.set_threads(1)
    try:
        t1 = time.perf_counter()
        oracle.mul_mag_ntt(sa, sb)
        dt1 = time.perf_counter() - t1
    finally:
        oracle.set_threads(threads)
    return {"value": round(b_mul(n, la, lb) / dt / 1e9, 3), "unit": "GB/s", "cores": threads,
            "kind": "port", "seconds": round(dt, 2),
            "sample": f"one {la}x{lb}-limb product (the full workload) through the C restatement of "
                      f"mul_mag_ntt (crates/bignum/src/ntt.rs:806-865), OpenMP on {threads} threads",
            "one_core": {"value": round(b_mul(sn, 1 << 20, 1 << 20) / dt1 / 1e9, 3), "unit": "GB/s",
                         "seconds": round(dt1, 2),
                         "sample": "one 2^26 x 2^26-bit product (2^20 x 2^20 limbs) on 1 thread"}}


def run_reference(args):
    ws, rank, local = dist_info()
    if rank != 0:
        return
    import oracle
    oracle.build()
    threads = oracle.max_threads()
    la, lb = BITS_A // 64, BITS_B // 64
    L = next_pow2_log(4 * la + 4 * lb - 1)
    N = 1 << L
    a, b = make_operands(la, lb)
    warm = min(args.warmup, 1)
    steps = max(1, min(args.steps, 3))
    for _ in range(warm):
        oracle.mul_mag_ntt(a, b)
    t0 = time.perf_counter()
    for _ in range(steps):
        oracle.mul_mag_ntt(a, b)
    dt = time.perf_counter() - t0
    value = b_mul(N, la, lb) * steps / dt / 1e9
    sample = (f"{steps} timed + {warm} warm-up full {la}x{lb}-limb products (requested {args.steps}/"
              f"{args.warmup}; capped so the CPU run stays within minutes)")
    line = {
        "impl": "reference",
        "metric": mul_metric(),
        "project_metric": PROJECT_METRIC,
        "value": round(value, 3),
        "unit": "GB/s",
        "n_gpus": ws,
        "steps": steps,
        "warmup": warm,
        "ms_per_step": round(1e3 * dt / steps, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "u64",
        "data": "synthetic: seeded uniform u64 limbs, top limb bit 63 set (numpy PCG64)",
        "config": {"workload": mul_workload(la, lb, L),
                   "bits_a": BITS_A, "bits_b": BITS_B, "la": la, "lb": lb, "transform_len": N,
                   "bytes_per_step_model": "B_mul(N) = 96N + 16(la+lb)"},
        "cpu_baseline": {"value": round(value, 3), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": sample + "; C restatement of crates/bignum/src/ntt.rs:806-865 "
                                            "(the Rust reference cannot be built here: no cargo/rustc)"},
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["engine", "reference"], default="engine")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-API leg (profiling runs)")
    ap.add_argument("--digits", type=int, default=1_000_000)
    ap.add_argument("--algorithm", choices=["chudnovsky", "gl", "both"], default="chudnovsky")
    ap.add_argument("--pi-mode", choices=["plain", "batched", "both"], default="both",
                    help="Chudnovsky binary splitting: one GPU call per product, level-batched, or both")
    ap.add_argument("--leaf-terms", type=int, default=0,
                    help="terms per binary-splitting leaf (0 = chosen per eighth of the terms, at most 64)")
    ap.add_argument("--gl-backend", choices=["plain", "served", "device"], default="plain",
                    help="Gauss-Legendre products: one pimul_mul call each, through the served form, or the whole "
                         "iteration on the device in fixed point")
    ap.add_argument("--gl-sqrt", choices=["reference", "newton"], default="reference",
                    help="Gauss-Legendre square roots: the reference's division-based iteration or the "
                         "multiplication-only one (same digits)")
    ap.add_argument("--gl-decimal", choices=["reference", "device"], default="reference",
                    help="Gauss-Legendre decimal conversion: the reference's recursion (products one call "
                         "each) or level-batched with the nodes on the GPU (same digits)")
    ap.add_argument("--positions", type=int, default=256)
    ap.add_argument("--max-pos", type=float, default=8e8)
    ap.add_argument("--cpu-positions", type=int, default=16)
    ap.add_argument("--cpu-depth", type=float, default=2e6)
    ap.add_argument("--bbp-batch", type=int, default=8192, help="BBP positions per launch")
    ap.add_argument("--check-digits", type=float, default=0,
                    help="BBP: also compute pi to this many decimal digits, convert to hex and compare every position")
    ap.add_argument("--workload", choices=["mul", "batch", "served", "pi", "bbp", "hex"], default="mul",
                    help="mul: the 2^30-bit product (headline); batch: 4096 uneven products; "
                         "served: Poisson request stream through the multiply service")
    ap.add_argument("--requests", type=int, default=1000)
    ap.add_argument("--extras", default="all",
                    help="other configurations added to the headline line: all, none, or a comma-separated "
                         "subset of sweep,batch4096,served,pi,bbp")
    ap.add_argument("--hex-checks", type=int, default=8, help="BBP spot checks of the hex conversion")
    ap.add_argument("--hex-cpu-digits", type=int, default=1_000_000)
    ap.add_argument("--hex-input", choices=["pi", "random"], default="pi",
                    help="text to convert: pi's digits (BBP-checked) or seeded random digits")
    ap.add_argument("--load", default="0.8,1.0,1.5,2.0",
                    help="offered loads of the served workload, comma-separated multiples of plain capacity")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--bits", type=int, default=30,
                    help="log2 bits per operand (30 = the headline workload; smaller for profiling)")
    args = ap.parse_args()
    global BITS_A, BITS_B
    BITS_A = BITS_B = 1 << args.bits
    if args.warmup < 3 and args.impl == "engine":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "served":
        run_served(args)
    elif args.workload == "pi":
        run_pi(args)
    elif args.workload == "bbp":
        run_bbp(args)
    elif args.workload == "hex":
        run_hex(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
