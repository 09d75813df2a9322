#!/usr/bin/env python3
"""Benchmark of the batched fused polymul (N = 2^16, L = 32, 16 pairs).

One step = one fused polymul over the whole batch: for each of the 16 pairs
and each of the 32 RNS limbs, NTT(a), NTT(b), pointwise product, INTT = 3
limb-NTTs per limb, 1536 limb-NTTs per step.  A is uniform, B a centred
discrete Gaussian (sigma 3.2, |e| <= 19) mapped per limb, both from
splitmix64 seeds.  Each step touches 768 MiB of operands and results plus
256 MiB of scratch, well above the 129 MB L2, so no flush is needed between
steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs its own batch on its own GPU (weak scaling,
no collective on the data path); the timed region is bracketed by barriers
and the max over ranks is reported.  --impl reference times the reference's
CPU algorithm (the reference's own sources when they were built here, else
the oracle's C restatement of them) on all host cores, rank 0 only.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "limb-NTTs/s at N=2^16 batched vs per-call on 1 GB300; served p50/p99 polymul"
UNIT = "limb-NTT/s"
LOG_N, L, PAIRS = 16, 32, 16
LIMB_NTTS_PER_STEP = 3 * L * PAIRS
N = 1 << LOG_N
SEED = 3
WORKLOAD = f"fused polymul N=2^{LOG_N}, L={L} (P[0..{L - 1}]), {PAIRS} pairs"

# Algorithmic bytes of one launch of each pipeline kernel per limb (pair):
# reads + writes of the words it must move (twiddles excluded).
ALGO_BYTES_PER_LIMB = {
    "polymul_col_fwd": 32 * N,     # read a and b, write their NTT pass-1 outputs
    "polymul_rows": 24 * N,        # read both pass-1 outputs, write pass-1 of the INTT
    "polymul_col_inv": 16 * N,     # read, write the product
    "polymul_whole": 24 * N,
}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_inputs(rank: int, pairs: int = PAIRS):
    from yell_gb300.inputs import gaussian_polys, uniform_polys
    import yell_gb300 as y

    ps = y.primes(L)
    seed = SEED + 1000 * rank
    a = uniform_polys(seed, PAIRS, L, LOG_N, ps)[:pairs]
    b = gaussian_polys(seed, PAIRS, L, LOG_N, ps, offset=PAIRS * L * N)[:pairs]
    return np.ascontiguousarray(a), np.ascontiguousarray(b)


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons in the background."""

    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.uuid = (uuid or "").lower()
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self):
        rows = self.rows
        if self.uuid:
            mine = [r for r in rows if self.uuid in r[0].lower()]
            rows = mine or rows
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [num(r[1]) for r in rows if num(r[1]) is not None]
        smax = [num(r[2]) for r in rows if num(r[2]) is not None]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for name, val in zip(names, r[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(rows),
                "power_w_max": max((num(r[3]) or 0.0) for r in rows),
                "reasons": sorted(reasons)}


def device_uuid(torch, dev: int):
    try:
        u = str(torch.cuda.get_device_properties(dev).uuid)
        return u.replace("GPU-", "")
    except Exception:
        return None


REF_SAMPLE_PAIRS = 4  # pairs per reference-arm step (a bounded sample of the batch)


def cpu_reference_run(a, b, threads: int):
    """One polymul batch of a.shape[0] pairs on the CPU; returns (seconds, kind)."""
    import oracle

    if oracle.ref_available():
        try:
            orc = oracle.Oracle("ref")
            kind = "reference"
        except OSError:
            orc = oracle.Oracle("port")
            kind = "port"
    else:
        orc = oracle.Oracle("port")
        kind = "port"
    _, secs = orc.polymul_batch(a, b, a.shape[0], L, LOG_N, threads)
    return secs, kind


def rows_cpu_baseline(dc_host) -> dict:
    """CPU timings of the rows beside the polymul path, on bounded samples of
    the same workloads (single thread: the restatements are scalar C / Python):
    samplers (oracle/samplers_oracle.c), CRT lifting (the big-integer
    restatement of gmp::poly2mpz in oracle/crt.py), the 32-bit polymul
    (oracle/yell_oracle32.c, or the reference's 32-bit build where present)."""
    import oracle
    from oracle.crt import poly2bigint

    orc = oracle.Oracle("port")
    out = {}

    def timed(fn, min_s=0.5):
        reps, t0 = 0, time.perf_counter()
        while True:
            fn()
            reps += 1
            el = time.perf_counter() - t0
            if el >= min_s or reps >= 50:
                return el / reps

    words = L * N  # one poly of L = 32 limbs, N = 2^16
    for name, fn in (("uniform", lambda: orc.sample_uniform(1, L, LOG_N, seed=1)),
                     ("zo", lambda: orc.sample_zo(1, L, LOG_N, seed=2)),
                     ("gaussian", lambda: orc.sample_gaussian(1, L, LOG_N, seed=3)),
                     ("hwt_192", lambda: orc.sample_hwt(1, L, LOG_N, 192, seed=4))):
        sec = timed(fn)
        out[f"sample_{name}"] = {"gbs": 8 * words / sec / 1e9, "cores": 1, "kind": "port",
                                 "sample": f"1 poly x {L} limbs x 2^{LOG_N}"}
    ncoef = 1024
    limbs = np.ascontiguousarray(dc_host[0, :, :ncoef])
    primes = [orc.prime(j) for j in range(L)]
    sec = timed(lambda: poly2bigint(limbs, primes), min_s=1.0)
    out["crt_lift"] = {"coefficients_per_s": ncoef / sec, "cores": 1, "kind": "port",
                       "sample": f"{ncoef} coefficients at L = {L} (Python integers, gmp::poly2mpz steps)"}
    o32 = oracle.Oracle32("ref") if oracle.ref32_available() else oracle.Oracle32("port")
    n32 = 1 << 15
    rng = np.random.default_rng(0)
    a32 = (rng.integers(0, 1 << 29, (L, n32))).astype(np.uint32)
    b32 = (rng.integers(0, 1 << 29, (L, n32))).astype(np.uint32)
    sec = timed(lambda: o32.polymul(a32, b32, 15), min_s=1.0)
    out["polymul32"] = {"limb_ntts_per_s": 3 * L / sec, "cores": 1, "kind": o32.which if o32.which == "port" else "reference",
                        "sample": f"1 pair x {L} limbs at N = 2^15"}
    return out


def init_host_group(world: int):
    """gloo process group over the ranks (None for one rank)."""
    if world <= 1:
        return None
    import datetime

    import torch.distributed as dist

    dist.init_process_group("gloo", timeout=datetime.timedelta(minutes=10))
    return dist


def host_max(dist, v: float) -> float:
    if dist is None:
        return v
    import torch

    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(args, rank: int, world: int) -> int:
    dist = init_host_group(world)
    try:
        return run_reference_rank0(args, world) if rank == 0 else 0
    finally:
        if dist is not None:
            dist.barrier()  # the other ranks do no work; they wait for rank 0's line
            dist.destroy_process_group()


def run_reference_rank0(args, world: int) -> int:
    import oracle

    oracle_dir = os.path.join(ROOT, "oracle")
    if not os.path.exists(os.path.join(oracle_dir, "liboracle.so")):
        oracle.build()
    from yell_gb300.inputs import gaussian_polys, uniform_polys

    orc_port = oracle.Oracle("port")
    ps = np.array([orc_port.prime(i) for i in range(L)], dtype=np.uint64)
    a = uniform_polys(SEED, PAIRS, L, LOG_N, ps)[:REF_SAMPLE_PAIRS].copy()
    b = gaussian_polys(SEED, PAIRS, L, LOG_N, ps, offset=PAIRS * L * N)[:REF_SAMPLE_PAIRS].copy()
    per_step = 3 * L * REF_SAMPLE_PAIRS
    threads = os.cpu_count() or 1
    kind = None
    for _ in range(args.warmup):
        _, kind = cpu_reference_run(a, b, threads)
    times = []
    for _ in range(args.steps):
        secs, kind = cpu_reference_run(a, b, threads)
        times.append(secs)
    total = sum(times)
    value = per_step * args.steps / total
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic: splitmix64 seed 3, B discrete Gaussian sigma 3.2",
        "config": {"workload": WORKLOAD, "log_n": LOG_N, "L": L, "pairs": PAIRS,
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"{REF_SAMPLE_PAIRS} of the {PAIRS} pairs (x {L} limbs, "
                                   f"{per_step} limb-NTTs) per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args, rank: int, world: int, local_rank: int) -> int:
    import torch

    import yell_gb300 as y

    if local_rank >= torch.cuda.device_count():
        print(f"bench.py: rank {rank} needs GPU {local_rank}, the box has {torch.cuda.device_count()}",
              file=sys.stderr)
        return 2
    torch.cuda.set_device(local_rank)
    # Replicas: no collective on the data path.  The ranks only meet on the
    # host (barriers around the timed region, the max of their times), so a
    # gloo group on host tensors is all they need.
    dist = init_host_group(world)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(v: float) -> float:
        return host_max(dist, v)

    pairs = args.pairs
    a, b = make_inputs(rank, pairs)
    da = torch.from_numpy(a.view(np.int64)).cuda()
    db = torch.from_numpy(b.view(np.int64)).cuda()
    dc = torch.empty_like(da)
    scratch = torch.empty(y.polymul_scratch_words(pairs, L, LOG_N), dtype=torch.int64,
                          device="cuda")
    y.init_ntt_tables(LOG_N, L)
    # autotune the launch variant of this degree at this size (same words for every variant)
    if args.no_autotune:
        tuned_variant = y.get_variant(LOG_N)
    else:
        tuned_variant, _ = y.autotune(LOG_N, L, pairs)
    stream = torch.cuda.Stream()

    def step():
        y.dev_polymul(dc, da, db, pairs, L, LOG_N, 0, scratch=scratch, stream=stream)

    if args.rows_only:  # profiling entry: one product, then the rows alone
        step()
        torch.cuda.synchronize()
        rows = run_rows(torch, y, stream, dc)
        if rank == 0:
            print(json.dumps({"rows": rows}), flush=True)
        return 0
    if args.uneven_only:  # profiling entry: the uneven batch (graphs, one queue launch, per call) alone
        uneven = run_uneven(torch, y, stream, lambda: torch.cuda.synchronize(), lambda v: v, 1, args.no_autotune)
        uneven.pop("_items")
        uneven.pop("_mix")
        if rank == 0:
            print(json.dumps({"uneven_batch": uneven}), flush=True)
        return 0

    # ---- device-resident throughput (value) ---------------------------
    for _ in range(max(args.warmup, 3)):
        step()
    barrier()
    sampler = ClockSampler(device_uuid(torch, local_rank)) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.3)
    barrier()
    launches0 = y.kernel_launches()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    launches = y.kernel_launches() - launches0
    barrier()
    if sampler:
        sampler.stop()
    ms = max_over_ranks(e0.elapsed_time(e1))
    ms_per_step = ms / args.steps
    per_step = 3 * L * pairs
    value = world * per_step * args.steps / (ms * 1e-3)

    # ---- per-kernel device time (same workload, instrumented) -----------
    prof_steps = min(args.steps, 20)
    barrier()
    y.profile_start()
    for _ in range(prof_steps):
        step()
    torch.cuda.synchronize()
    kernels = y.profile_stop()
    total_ms = sum(t for _, t in kernels.values())
    dom = max(kernels, key=lambda k: kernels[k][1])
    dom_launches, dom_ms = kernels[dom]
    per_launch_ms = dom_ms / dom_launches
    algo = ALGO_BYTES_PER_LIMB[dom] * L * pairs
    hbm, peak_kind = peaks()
    achieved = algo / (per_launch_ms * 1e-3) / 1e9
    traffic = read_ncu_traffic(dom)
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                "frac": achieved / hbm, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": algo, "launch_ms": per_launch_ms,
                "traffic": traffic,
                "share": {k: round(t / total_ms, 4) for k, (_, t) in kernels.items()},
                "pipeline": {"algorithmic_bytes_per_step": 24 * N * L * pairs,
                             "achieved": 24 * N * L * pairs / (ms_per_step * 1e-3) / 1e9,
                             "frac": 24 * N * L * pairs / (ms_per_step * 1e-3) / 1e9 / hbm}}
    roofline["traffic_kind"] = traffic_kind(dom)
    roofline["integer"] = integer_roofline(y, kernels, ms_per_step, pairs, y.variants(LOG_N)[tuned_variant])
    k1 = roofline["integer"]["k1"]
    if k1 is not None:
        # distinct twiddle pairs {w, w'} (16 B) one launch reads, once per prime: the row
        # step reads the forward and inverse tables above index 2^k1, the column passes
        # the 2^k1 - 1 entries below it; not part of the algorithmic bytes
        tw = {"polymul_rows": 2 * 16 * (N - (1 << k1)) * L, "polymul_col_fwd": 16 * ((1 << k1) - 1) * L,
              "polymul_col_inv": 16 * ((1 << k1) - 1) * L}
        roofline["twiddle_bytes_per_launch"] = tw.get(dom)
    if args.device_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT,
                              "ms_per_step": ms_per_step, "pairs": pairs, "roofline": roofline,
                              "gpu_launches": launches}), flush=True)
        return 0

    # ---- plain per-call path: one launch per reference call -------------
    ta = da.clone().reshape(-1)
    tb = db.clone().reshape(-1)

    def per_call():
        for pi in range(pairs):
            for l in range(L):
                off = (pi * L + l) * N
                va = ta[off:off + N]
                vb = tb[off:off + N]
                y.dev_ntt(va, 1, 1, LOG_N, l, y.YELL_FORWARD, stream=stream)
                y.dev_ntt(vb, 1, 1, LOG_N, l, y.YELL_FORWARD, stream=stream)
                y.dev_elementwise(y.YELL_OP_MULMOD, va, va, vb, 1, 1, LOG_N, l, stream=stream)
                y.dev_ntt(va, 1, 1, LOG_N, l, y.YELL_BACKWARD, stream=stream)

    per_call()
    barrier()
    pc_steps = 2
    e0.record(stream)
    for _ in range(pc_steps):
        per_call()
    e1.record(stream)
    torch.cuda.synchronize()
    pc_ms = max_over_ranks(e0.elapsed_time(e1)) / pc_steps
    per_call_value = world * per_step / (pc_ms * 1e-3)
    del ta, tb

    # ---- uneven batch (512 polymuls, log2 N in 10..16, L in 1..16) ----------
    uneven = serving = None
    if not args.no_uneven:
        uneven = run_uneven(torch, y, stream, barrier, max_over_ranks, world, args.no_autotune)
        if not args.no_serve:
            serving = run_serving(torch, y, uneven, args.serve_seconds)
        uneven.pop("_items")
        uneven.pop("_mix")

    rows = None if args.no_rows else run_rows(torch, y, stream, dc)
    config2 = None if args.no_rows else run_config2(torch, y, stream)

    # ---- end to end through the host-memory C ABI call --------------------
    pa = y.PinnedBuffer(a.shape)
    pb = y.PinnedBuffer(b.shape)
    pc = y.PinnedBuffer(a.shape)
    pa.array[:] = a
    pb.array[:] = b
    e2e_steps = max(3, min(args.steps, 20))
    y.polymul_host(pa.array, pb.array, LOG_N, out=pc.array)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        y.polymul_host(pa.array, pb.array, LOG_N, out=pc.array)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0)
    e2e_value = world * per_step * e2e_steps / e2e_s
    e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(a.nbytes + b.nbytes),
           "d2h_bytes_per_step": int(a.nbytes), "ms_per_step": 1e3 * e2e_s / e2e_steps,
           "path": "yell_polymul_host from pinned host buffers"}
    for buf in (pa, pb, pc):
        buf.free()
    # the same call on plain (pageable) numpy arrays: moved by kernels that
    # access the host memory in place where the device supports it
    out = np.empty_like(a)
    y.polymul_host(a, b, LOG_N, out=out)
    barrier()
    t0 = time.perf_counter()
    for _ in range(3):
        y.polymul_host(a, b, LOG_N, out=out)
    torch.cuda.synchronize()
    pg_s = max_over_ranks(time.perf_counter() - t0)
    e2e["pageable"] = {"value": world * per_step * 3 / pg_s, "unit": UNIT, "ms_per_step": 1e3 * pg_s / 3,
                       "host_access": y.host_access(),
                       "path": "yell_polymul_host from pageable numpy arrays"}
    del out
    if not args.no_facade:
        e2e["facade"] = run_e2e_facade(y, a, b, dc.cpu().numpy().view(np.uint64).reshape(a.shape))
        barrier()

    # ---- CPU baseline (rank 0 at N=1 only) --------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        # Repeat the whole batch until about 2 s of wall time (10-30 core-seconds).
        total, reps, kind = 0.0, 0, None
        while (reps < 3 or total < 2.0) and reps < 200:
            secs, kind = cpu_reference_run(a, b, threads)
            total += secs
            reps += 1
        cpu = {"value": reps * 3 * L * pairs / total, "unit": UNIT, "cores": threads,
               "kind": kind,
               "sample": f"{reps} x the full batch ({pairs} pairs x {L} limbs), {total:.2f} s wall, "
                         f"~{total * threads:.0f} core-s"}
        # one host core, on one pair of the batch repeated for about a second
        total1, reps1 = 0.0, 0
        while (reps1 < 2 or total1 < 1.0) and reps1 < 50:
            secs, _ = cpu_reference_run(a[:1], b[:1], 1)
            total1 += secs
            reps1 += 1
        cpu["single_core"] = {"value": reps1 * 3 * L / total1, "unit": UNIT, "cores": 1,
                              "sample": f"{reps1} x 1 pair x {L} limbs, {total1:.2f} s"}
        if rows is not None:
            rows["cpu_baseline"] = rows_cpu_baseline(dc.cpu().numpy().view(np.uint64).reshape(pairs, L, N))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic: splitmix64 seed 3 (+1000 per rank), B discrete Gaussian sigma 3.2",
            "config": {"workload": WORKLOAD, "log_n": LOG_N, "L": L, "pairs": PAIRS,
                       "parallelism": f"replicas x{world}",
                       "launch_variant": y.variants(LOG_N)[tuned_variant],
                       "l2": "inputs larger than L2 (768 MiB operands+result per step)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches,
            "clocks": sampler.summary() if sampler else None,
            "per_call": {"value": per_call_value, "unit": UNIT, "ms_per_step": pc_ms,
                         "path": "one launch per reference call: forward(a), forward(b), "
                                 "mulmod, backward per limb"},
            "batched_vs_per_call": value / per_call_value,
            "uneven_batch": uneven,
            "serving": serving,
            "batched_ntt": config2,
            "rows": rows,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def run_e2e_facade(y, a, b, want, steps: int = 2) -> dict:
    """The drop-in path a YELL user hits: for each pair, a.forward();
    b.forward(); c = a * b; c.backward() through yell_poly_forward /
    yell_poly_mulmod / yell_poly_backward, on the reference's data layout:
    every limb its own pageable host allocation (poly<N> allocates each limb
    separately).  Each call copies its limbs to the device and back and waits,
    as the reference's calls return with the work done.  The first pass runs
    on fresh copies and is checked against the fused device result."""
    import ctypes

    lib = y.load()
    pairs = a.shape[0]
    ptrs = ctypes.c_void_p * L

    def limbs(x):
        return [[np.array(x[p, l], copy=True) for l in range(L)] for p in range(pairs)]

    A, B = limbs(a), limbs(b)
    C = [[np.empty(N, np.uint64) for _ in range(L)] for _ in range(pairs)]
    keep = [[ptrs(*[v.ctypes.data for v in X[p]]) for p in range(pairs)] for X in (A, B, C)]
    pa, pb, pc = ([ctypes.addressof(t) for t in arrs] for arrs in keep)

    def ok(st):
        if st != 0:
            raise RuntimeError(lib.yell_last_error().decode())

    def step():
        for p in range(pairs):
            ok(lib.yell_poly_forward(pa[p], L, LOG_N))
            ok(lib.yell_poly_forward(pb[p], L, LOG_N))
            ok(lib.yell_poly_mulmod(pc[p], pa[p], pb[p], L, LOG_N))
            ok(lib.yell_poly_backward(pc[p], L, LOG_N))

    step()
    got = np.stack([np.stack(C[p]) for p in range(pairs)])
    if not np.array_equal(got, want):
        raise RuntimeError("facade path differs from the fused polymul")
    t0 = time.perf_counter()
    for _ in range(steps):
        step()
    secs = (time.perf_counter() - t0) / steps
    limb = N * 8
    h2d = pairs * L * limb * 5  # forward a, forward b, mulmod reads a and b, backward
    d2h = pairs * L * limb * 4
    return {"value": 3 * L * pairs / secs, "unit": UNIT, "ms_per_step": 1e3 * secs,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": steps,
            "path": "yell_poly_forward x2, yell_poly_mulmod, yell_poly_backward per pair on per-limb "
                    "pageable host allocations (the reference's poly<N> layout and call pattern)"}


def run_config2(torch, y, stream, reps: int = 10, groups: int = 3):
    """Batched NTT without a product: forward then inverse NTT of 64 polys x
    L = 8 x N = 2^14 (P[0..7]), device-resident, one call per direction (a
    column launch and a row launch each), against the same 1024 limb-NTTs as
    one call per limb.  CUDA events on `stream`, the fastest of `groups`
    averages over `reps`; the words are checked to come back unchanged."""
    from yell_gb300.inputs import uniform_polys

    log_n, L2, polys = 14, 8, 64
    n = 1 << log_n
    hbm, _ = peaks()
    x0 = uniform_polys(2, polys, L2, log_n, y.primes(L2))
    x = torch.from_numpy(x0.view(np.int64).reshape(-1).copy()).cuda()
    y.init_ntt_tables(log_n, L2)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(groups):
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / reps)
        return best

    fwd = lambda: y.dev_ntt(x, polys, L2, log_n, 0, y.YELL_FORWARD, stream=stream)
    inv = lambda: y.dev_ntt(x, polys, L2, log_n, 0, y.YELL_BACKWARD, stream=stream)
    fwd_ms, inv_ms = timed(fwd), timed(inv)
    both_ms = timed(lambda: (fwd(), inv()))
    ok = bool(np.array_equal(x.cpu().numpy().view(np.uint64).reshape(x0.shape), x0))
    limbs = [x[i * n:(i + 1) * n] for i in range(polys * L2)]

    def per_call():
        for i, v in enumerate(limbs):
            y.dev_ntt(v, 1, 1, log_n, i % L2, y.YELL_FORWARD, stream=stream)
        for i, v in enumerate(limbs):
            y.dev_ntt(v, 1, 1, log_n, i % L2, y.YELL_BACKWARD, stream=stream)

    pc_ms = timed(per_call)
    limb_ntts = 2 * polys * L2
    half = polys * L2 * (n // 2) * log_n  # butterflies of one direction over the batch
    ct, gs = y.calibrate_butterflies()
    out = {"workload": f"forward + inverse NTT, N=2^{log_n}, L={L2} (P[0..{L2 - 1}]), {polys} polys",
           "value": limb_ntts / (both_ms * 1e-3), "unit": UNIT, "ms_per_batch": both_ms,
           "forward_ms": fwd_ms, "inverse_ms": inv_ms, "round_trip_identity": ok,
           "roofline": {"bound": "hbm", "algorithmic_bytes": 16 * n * limb_ntts,
                        "achieved_gbs": 16 * n * limb_ntts / (both_ms * 1e-3) / 1e9,
                        "frac": 16 * n * limb_ntts / (both_ms * 1e-3) / 1e9 / hbm},
           "integer": {"forward_frac": integer_ceiling_s(half, 0, ct, gs) / (fwd_ms * 1e-3),
                       "inverse_frac": integer_ceiling_s(0, half, ct, gs) / (inv_ms * 1e-3),
                       "formula": "frac = (n_ct / ct_rate + n_gs / gs_rate) / measured time"},
           "per_call": {"value": limb_ntts / (pc_ms * 1e-3), "unit": UNIT, "ms_per_batch": pc_ms,
                        "path": "one yell_dev_ntt call per limb and direction (1024 launches)"},
           "batched_vs_per_call": pc_ms / both_ms}
    return out


def run_rows(torch, y, stream, dc, reps: int = 10, groups: int = 3):
    """Device throughput of the rows beside the polymul path, at the polymul
    workload's sizes: seeded samplers filling 16 polys of N = 2^16, L = 32;
    CRT lifting of the 16 product polys; the 32-bit moduli polymul at
    N = 2^15, L = 32, 16 pairs.  Each timed with CUDA events on `stream`:
    the fastest of `groups` averages over `reps` launches, after one warm-up."""
    from yell_gb300 import moduli32 as m32

    hbm, peak_kind = peaks()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def timed(fn):
        fn()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(groups):
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) / reps)
        return best

    out = {"peak_hbm_gbs": hbm, "peak_kind": peak_kind}
    words = PAIRS * L * N
    buf = torch.empty(words, dtype=torch.int64, device="cuda")
    samplers = {
        "uniform": lambda: y.sample_uniform(buf, PAIRS, L, LOG_N, seed=1, stream=stream),
        "zo": lambda: y.sample_zo(buf, PAIRS, L, LOG_N, seed=2, stream=stream),
        "gaussian": lambda: y.sample_gaussian(buf, PAIRS, L, LOG_N, seed=3, stream=stream),
        "hwt_192": lambda: y.sample_hwt(buf, PAIRS, L, LOG_N, 192, seed=4, stream=stream),
    }
    # what a write-only kernel reaches here: a device fill of the same bytes (a library kernel,
    # timed as the reference point of the samplers, not as work of this library)
    with torch.cuda.stream(stream):
        fill_ms = timed(lambda: buf.fill_(1))
    fill_gbs = 8 * words / (fill_ms * 1e-3) / 1e9
    out["device_fill"] = {"ms": fill_ms, "achieved_gbs": fill_gbs, "frac": fill_gbs / hbm,
                          "bytes": 8 * words, "what": "torch fill_ of the sampler buffer (write-only ceiling)"}
    for name, fn in samplers.items():
        ms = timed(fn)
        gbs = 8 * words / (ms * 1e-3) / 1e9
        out[f"sample_{name}"] = {"ms": ms, "achieved_gbs": gbs, "frac": gbs / hbm,
                                 "frac_of_device_fill": fill_ms / ms,
                                 "algorithmic_bytes": 8 * words, "bound": "hbm (writes)"}
    del buf
    # CRT lifting of the polymul output (16 polys, L = 32 -> W words per coefficient)
    W = y.crt_words(L)
    lifted = torch.empty(PAIRS * N * W, dtype=torch.int64, device="cuda")
    ms = timed(lambda: y.dev_crt_lift(lifted, dc, PAIRS, L, LOG_N, stream=stream))
    coeffs = PAIRS * N
    byts = coeffs * 8 * (L + W)
    out["crt_lift"] = {"ms": ms, "coefficients_per_s": coeffs / (ms * 1e-3),
                       "achieved_gbs": byts / (ms * 1e-3) / 1e9, "frac": byts / (ms * 1e-3) / 1e9 / hbm,
                       "algorithmic_bytes": byts, "words_per_coefficient": W,
                       "mac64_per_s": coeffs * L * (W + 1) / (ms * 1e-3),
                       "bound": "integer multiply-add (L x (W+1) 64-bit MACs per coefficient)"}
    del lifted
    # 32-bit moduli polymul
    n32, log32 = 1 << 15, 15
    w32 = PAIRS * L * n32
    a32 = torch.randint(0, 1 << 29, (w32,), dtype=torch.int32, device="cuda")
    b32 = torch.randint(0, 1 << 29, (w32,), dtype=torch.int32, device="cuda")
    c32 = torch.empty_like(a32)
    m32.init_ntt_tables(log32, L)
    ms = timed(lambda: m32.dev_polymul(c32, a32, b32, PAIRS, L, log32, stream=stream))
    byts = 12 * n32 * L * PAIRS
    # integer roofline: 3 NTTs of (N/2) log N butterflies per limb pair (2 CT, 1 GS)
    n_ct32 = 2 * L * PAIRS * (1 << (log32 - 1)) * log32
    n_gs32 = n_ct32 // 2
    ct32, gs32 = m32.calibrate_butterflies()
    floor_s = integer_ceiling_s(n_ct32, n_gs32, ct32, gs32)
    out["polymul32"] = {"ms": ms, "limb_ntts_per_s": 3 * L * PAIRS / (ms * 1e-3),
                        "achieved_gbs": byts / (ms * 1e-3) / 1e9, "frac": byts / (ms * 1e-3) / 1e9 / hbm,
                        "algorithmic_bytes": byts, "workload": "N=2^15, L=32, 16 pairs, 30-bit primes",
                        "integer": {"bfly_per_s": (n_ct32 + n_gs32) / (ms * 1e-3),
                                    "ceiling_ct_bfly_per_s": ct32, "ceiling_gs_bfly_per_s": gs32,
                                    "frac": floor_s / (ms * 1e-3),
                                    "formula": "frac = (n_ct / ct_rate + n_gs / gs_rate) / measured time",
                                    "note": "ceiling = register-only 32-bit CT/GS butterflies "
                                            "(yell32_calibrate_butterflies); pointwise products not counted"}}
    return out


def run_uneven(torch, y, stream, barrier, max_over_ranks, world, no_autotune=False):
    """512 polymuls of mixed degree and limb count (seed 4): one batched call
    (bucketed, CUDA graph per batch shape), one launch of the persistent
    work-queue kernel, the queue's items as three phase launches, and 512
    plain per-call calls."""
    from yell_gb300.workloads import mix_limb_ntts, mix_operands, uneven_mix

    mix = uneven_mix(4, 512)
    ops = mix_operands(mix, y.primes(16), 4)
    items, singles = [], []
    for (log_n, L), (a, b) in zip(mix, ops):
        da = torch.from_numpy(a.view(np.int64)).cuda()
        db = torch.from_numpy(b.view(np.int64)).cuda()
        dc = torch.empty_like(da)
        items.append((dc, da, db, log_n, L, 0))
        sw = y.polymul_scratch_words(1, L, log_n)
        singles.append(torch.empty(sw, dtype=torch.int64, device="cuda") if sw else None)
    for log_n in range(10, 17):
        y.init_ntt_tables(log_n, 16)
        if not no_autotune:
            y.autotune(log_n, 8, 4)
    limb_ntts = mix_limb_ntts(mix)
    tuned = {f"2^{d}": y.variants(d)[y.get_variant(d)] for d in range(10, 17)}
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def batched():
        y.dev_polymul_batch(items, stream=stream)

    def queue():
        y.dev_polymul_batch_queue(items, stream=stream)

    def phased():
        y.dev_polymul_batch_phased(items, stream=stream)

    def per_call():
        for (dc, da, db, log_n, L, cm0), sc in zip(items, singles):
            y.dev_polymul(dc, da, db, 1, L, log_n, cm0, scratch=sc, stream=stream)

    out = {"workload": "512 polymuls, log2 N uniform in 10..16, L uniform in 1..16 (seed 4)",
           "limb_ntts": limb_ntts,
           "launch_variants": tuned}
    for name, fn, steps in (("batched", batched, 10), ("persistent_queue", queue, 10), ("phased_queue", phased, 10),
                            ("per_call", per_call, 3)):
        for _ in range(2):
            fn()
        barrier()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        ms = max_over_ranks(e0.elapsed_time(e1)) / steps
        out[name] = {"value": world * limb_ntts / (ms * 1e-3), "unit": UNIT, "ms_per_batch": ms}
    out["batched"]["path"] = "degree buckets on forked streams, one CUDA graph per batch shape"
    out["persistent_queue"]["path"] = "one launch: resident CTAs take work items from a device queue"
    out["persistent_queue"]["status"] = y.batch_queue_status()
    out["phased_queue"]["path"] = "the queue's items as three launches, one per phase, no device waits"
    out["batched_vs_per_call"] = out["batched"]["value"] / out["per_call"]["value"]
    out["queue_vs_per_call"] = out["persistent_queue"]["value"] / out["per_call"]["value"]
    out["_items"] = items
    out["_mix"] = mix
    return out


def run_serving(torch, y, uneven, duration_s: float):
    """Poisson arrivals of polymul requests drawn from the uneven mix, offered
    at 10%..120% of the measured batched peak, against the continuous-batching
    server (120 GiB HBM budget) and against a per-call server (one request per
    launch sequence); device-resident operands."""
    from yell_gb300.serve import Server

    items, mix = uneven["_items"], uneven["_mix"]
    templates = [(da, db, log_n, L, cm0) for (dc, da, db, log_n, L, cm0) in items]
    peak_rps = len(mix) / (uneven["batched"]["ms_per_batch"] * 1e-3)
    loads = (0.1, 0.4, 0.8, 1.0, 1.2)
    out = {"workload": "Poisson arrivals from the uneven mix (seed 5), device-resident operands",
           "batched_peak_rps": peak_rps, "duration_s_per_point": duration_s}
    for name, max_batch, dur in (("continuous_batching", 1024, duration_s),
                                 ("per_call", 1, min(duration_s, 0.25))):
        points = []
        with Server(hbm_budget_bytes=0, max_inflight=4, max_batch=max_batch) as srv:
            srv.load_test(templates, 0.1 * peak_rps, 0.25, seed=1)  # warm-up
            for f in loads:
                st = srv.load_test(templates, f * peak_rps, dur, seed=5)
                points.append({"load": f, "offered_rps": f * peak_rps,
                               "achieved_rps": st["requests_per_s"],
                               "limb_ntts_per_s": st["limb_ntts_per_s"], "p50_us": st["p50_us"],
                               "p99_us": st["p99_us"], "max_us": st["max_us"],
                               "requests": st["completed"], "batches": st["batches"]})
            out["hbm_budget_bytes"] = st["hbm_budget"]
        out[name] = points
    out["p99_us_at_80pct"] = [p["p99_us"] for p in out["continuous_batching"] if p["load"] == 0.8][0]
    return out


def integer_ceiling_s(n_ct: float, n_gs: float, ct_rate: float, gs_rate: float) -> float:
    """Shortest time the calibrated butterfly rates allow for n_ct CT and n_gs
    GS butterflies (each kind at its own register-only rate).  Used for every
    kernel and for both word sizes, so the fractions are comparable."""
    return n_ct / ct_rate + n_gs / gs_rate


def integer_roofline(y, kernels: dict, ms_per_step: float, pairs: int, variant_name: str) -> dict:
    """Butterflies of the fused polymul step and of each of its kernels against
    the register-only ceiling (yell_calibrate_butterflies).  Stage counts
    follow the launch variant: k1 column stages, log N - k1 row stages; the
    forward NTTs of a and b are CT butterflies, the inverse GS (its scaled last
    layer counted as one GS stage).  The pointwise products (N L pairs of them,
    Montgomery products in the fused kernels) and the final reductions are not
    counted, so each fraction understates the kernel's use of the multiplier
    slightly."""
    import re

    ct_rate, gs_rate = y.calibrate_butterflies()
    m = re.search(r"k1=(\d+)", variant_name)
    k1 = int(m.group(1)) if m else None
    half = L * pairs * (N // 2)  # butterflies per stage over the batch
    out = {"bound": "imad (64-bit modmul from 32-bit IMAD)",
           "ceiling_ct_bfly_per_s": ct_rate, "ceiling_gs_bfly_per_s": gs_rate,
           "formula": "frac = (n_ct / ct_rate + n_gs / gs_rate) / measured time",
           "variant": variant_name, "k1": k1,
           "note": "ceiling = register-only CT/GS butterflies on every SM; the pointwise products not counted"}
    n_ct, n_gs = 2 * half * LOG_N, half * LOG_N
    out["pipeline_bfly_per_s"] = (n_ct + n_gs) / (ms_per_step * 1e-3)
    out["pipeline_frac"] = integer_ceiling_s(n_ct, n_gs, ct_rate, gs_rate) / (ms_per_step * 1e-3)
    if k1 is not None:
        rows = LOG_N - k1
        work = {"polymul_col_fwd": (2 * half * k1, 0), "polymul_rows": (2 * half * rows, half * rows),
                "polymul_col_inv": (0, half * k1)}
        out["row_stages"], out["column_stages"] = rows, k1
        for name, (c, g) in work.items():
            if name not in kernels:
                continue
            launches, total_ms = kernels[name]
            t = total_ms / launches * 1e-3
            out[name] = {"ct_bfly": c, "gs_bfly": g, "launch_ms": t * 1e3,
                         "bfly_per_s": (c + g) / t, "frac": integer_ceiling_s(c, g, ct_rate, gs_rate) / t}
        if "polymul_rows" in out:
            out["rows_kernel_frac"] = out["polymul_rows"]["frac"]
    return out


NCU_TRAFFIC = os.path.join(ROOT, "profiles", "ncu_traffic.txt")


def read_ncu_traffic(kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    try:
        with open(NCU_TRAFFIC) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 2 and parts[0] == kernel:
                    return float(parts[1])
    except OSError:
        pass
    return None


def traffic_kind(kernel: str) -> str | None:
    """What roofline.traffic is: the header line of the committed ncu summary."""
    try:
        with open(NCU_TRAFFIC) as f:
            kinds = [ln[1:].strip() for ln in f if ln.startswith("#")]
        return " ".join(kinds) if read_ncu_traffic(kernel) is not None else None
    except OSError:
        return None


def main() -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-batch comparison")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving sweep")
    ap.add_argument("--uneven-only", action="store_true",
                    help="run only the uneven-batch comparison (for profiling)")
    ap.add_argument("--rows-only", action="store_true",
                    help="run only the sampler, CRT-lifting and 32-bit measurements (for profiling)")
    ap.add_argument("--no-rows", action="store_true",
                    help="skip the sampler, CRT-lifting and 32-bit-moduli measurements")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the selected launch variants (default or YELL_GB300_TUNE_FILE)")
    ap.add_argument("--serve-seconds", type=float, default=0.5, help="seconds per serving load point")
    ap.add_argument("--device-only", action="store_true",
                    help="time only the device-resident batch (for profiler captures)")
    ap.add_argument("--pairs", type=int, default=PAIRS,
                    help="pairs per batch (profiling of a smaller case; default 16)")
    ap.add_argument("--no-facade", action="store_true",
                    help="skip the end-to-end figure through the per-limb host drop-in calls")
    args = ap.parse_args()
    if args.gpus < 1:
        ap.error("--gpus must be at least 1")
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        # not under torchrun: start the N ranks here, one process per GPU
        return spawn_ranks(args.gpus, sys.argv[1:])
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world != args.gpus:
        print(f"bench.py: --gpus {args.gpus} but WORLD_SIZE {world}", file=sys.stderr)
        return 2
    if args.impl == "reference":
        return run_reference(args, rank, world)
    return run_ours(args, rank, world, local_rank)


def spawn_ranks(n: int, argv: list[str]) -> int:
    """Runs this script as n ranks (RANK / LOCAL_RANK / WORLD_SIZE /
    MASTER_ADDR / MASTER_PORT set as torchrun sets them), one per GPU, and
    returns the first non-zero exit code.  Rank 0 prints the JSON line."""
    import socket

    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n),
                   LOCAL_WORLD_SIZE=str(n), MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, os.path.abspath(__file__), *argv], env=env))
    codes = [p.wait() for p in procs]
    return next((c for c in codes if c != 0), 0)


if __name__ == "__main__":
    sys.exit(main())
