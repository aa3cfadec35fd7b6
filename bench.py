#!/usr/bin/env python3
"""Benchmark: exact cgMLST Hamming distances, pairs/s on one GB300.

Workload: the long-tail outbreak shape, 63 005 profiles x 1 142 loci
(synthetic, seeded: per-locus Zipf(1.2) alleles with lognormal distinct counts,
median 60, tail to ~2 500; 1-5% missing per locus; 5% hashed 64-bit ids).  One
step = the whole upper triangle of the u16 distance matrix,
n (n - 1) / 2 = 1 984 783 510 exact pairs.

    value  device-resident: operands and rare groups already in HBM (device
           encoder), the step is one tch_solver_stripe over the whole upper
           triangle: the dense rare-count kernel (u16 block of the stripe),
           then the tensor-core tile pass that subtracts it (u16 output in
           HBM).  Inputs (operands ~1 GB, rare counts 8 GB) exceed L2.
    e2e    the reference-facing C ABI, tch_run, with host buffers: H2D of the
           bit-packed operands and CSR, device expansion, stripes, D2H of every
           stripe into pinned memory and the stripe callback, per step.
    roofline   the tile-pass kernel (tc_stripe_kernel), tensor-pipe bound:
           algorithmic MACs (unpadded K = L + D per pair, 2 ops per MAC) per
           launch / CUDA-event duration of that launch alone (the two passes
           are timed apart through tch_solver_rare_counts and
           tch_solver_stripe_counts), against the measured fp4 (kind::mxf4)
           tcgen05 peak of the same GPU.
    cpu_baseline   the brute-force count of the reference's exactness check
           (the C restatement in oracle/), all host threads, bounded sample.

--impl reference runs that CPU brute force alone (the reference's CPU path
for the matrix, restated in C in oracle/) on every host thread and prints its
line; it loads nothing of the package: the profiles come from synth.py loaded
by file path and are ranked by the oracle.  Each of its steps counts the rows
k, k + s, k + 2 s, ... of the upper triangle (a sample spread over the whole
triangle; s consecutive steps cover every row once), and value = pairs
counted / seconds over the timed steps.

Only one-GPU runs are offered (the library drives one device per process, and
the workload is quoted on one GPU): under torchrun with WORLD_SIZE > 1 the GPU
arm refuses to run (the reference arm runs on rank 0 and the other ranks
exit).
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "cgmlst-hamming-gpu_gb300"

METRIC = "exact_pairs_per_s"
DTYPE = "fp4(e2m1 0/+-1, block scales 1.0) -> fp32 exact ints -> u16"
UNIT = "pairs/s"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def workload_config(n: int, L: int) -> dict:
    """The workload as both arms name it (the same dict in both lines)."""
    return {"workload": f"long-tail outbreak profiles {n} x {L} (synthetic, seeded)", "n": n, "loci": L,
            "pairs": n * (n - 1) // 2,
            "l2": "inputs larger than L2 (operands ~1 GB, rare groups and per-step rare counts of several GB)"}


def load_synth():
    """synth.py by file path: the generator without importing the package."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("tch_synth", os.path.join(ROOT, PKG, "synth.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def load_oracle():
    d = os.path.join(ROOT, "oracle")
    if d not in sys.path:
        sys.path.insert(0, d)
    import oracle

    return oracle


def cpu_count_steps(x: np.ndarray, stride: int, k0: int, steps: int):
    """The oracle's brute-force count (all host threads) over the rows k,
    k + stride, ... of the upper triangle for k = k0 .. k0 + steps - 1 (mod
    stride), one call per step.  Returns (pairs, seconds)."""
    import ctypes

    lib = load_oracle().lib()
    n, L = x.shape
    x = np.ascontiguousarray(x, dtype=np.uint16)
    xp = x.ctypes.data_as(ctypes.POINTER(ctypes.c_uint16))
    pairs, secs = 0, 0.0
    for k in range(k0, k0 + steps):
        acc = ctypes.c_uint64(0)
        t = time.perf_counter()
        pairs += lib.orc_upper_rows_step(xp, n, L, k % stride, stride, ctypes.byref(acc), 0)
        secs += time.perf_counter() - t
    return pairs, secs


def reference_arm(args) -> dict:
    """The reference's CPU path for the matrix (the brute-force count of
    tensorcore/rs/check.py:39-44, restated in C with OpenMP), all host
    threads, rows k, k + s, ... per step."""
    import ctypes

    oracle = load_oracle()
    synth = load_synth()
    t0 = time.perf_counter()
    A = synth.longtail(n=args.n, L=args.L)
    x, _ = oracle.dense_ranks(A)
    n, L = x.shape
    log(f"reference arm: generated + ranked {n}x{L} in {time.perf_counter() - t0:.1f}s")
    s = max(1, args.ref_stride)
    cpu_count_steps(x, s, 0, args.warmup)
    pairs, secs = cpu_count_steps(x, s, args.warmup, args.steps)
    v = pairs / secs
    threads = oracle.lib().orc_num_threads()
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": secs / max(args.steps, 1) * 1e3,
            "higher_is_better": True, "scaling": "strong", "vs_baseline": None, "dtype": "u16",
            "data": "synthetic", "config": workload_config(n, L),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"brute-force count (check.py:39-44 restated in C, OpenMP, {threads} threads) "
                                       f"over rows k, k+{s}, k+{2 * s}, ... of the upper triangle per step "
                                       f"(~1/{s} of its pairs; {s} consecutive steps cover every row); "
                                       f"{pairs} pairs in {secs:.1f} s over {args.steps} steps"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def parity_rows(x: np.ndarray, out, rows: int = 256) -> dict:
    """Spread rows i of the device output (row i at out[i], column j at
    out[i, j]) against the oracle's count for every j in (i, n)."""
    oracle = load_oracle()
    n = x.shape[0]
    idx = sorted(set(np.linspace(0, n - 2, rows).astype(int).tolist()) | {0, n - 2})
    cells = bad = 0
    for i in idx:
        got = out[i, i + 1:n].cpu().numpy().view(np.uint16)
        want = oracle.hamming_block(x, i, i + 1, i + 1, n)[0]
        cells += got.size
        bad += int((got != want).sum())
    return {"rows": len(idx), "cells": cells, "mismatches": bad,
            "oracle": "orc_hamming_block (check.py:39-44 restated in C)"}


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def tc_peaks():
    """Measured rates of this GPU's arithmetic paths (the tch-peak probe).
    The fp4 probe runs in a process of its own."""
    exe = os.path.join(ROOT, PKG, "bin", "tch-peak")
    res = {}
    for paths in (["b1", "s8", "e4m3", "popc", "tc_f8"], ["tc_f4"]):
        try:
            out = subprocess.run([exe, *paths], capture_output=True, text=True, timeout=120).stdout
            res.update(json.loads(out.strip().splitlines()[-1]))
        except Exception as e:  # noqa: BLE001
            log("peak probe failed:", paths, e)
    return res


def time_whole(tch, A, tau, device, out, ldo, stream, reps=3, sched=(0, 0)):
    """(median device ms, tau used) of one whole-triangle solve of a fresh
    solver at this tau and schedule (sub-stripe rows, raster group)."""
    import torch

    n = A.shape[0]
    with tch.Solver.from_calls(A, tau=tau, device=device) as s:
        s.set_schedule(*sched)
        used = s.info()["tau"]
        s.stripe(0, n, out.data_ptr(), ldo, stream.cuda_stream)
        ms = []
        for _ in range(reps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.stripe(0, n, out.data_ptr(), ldo, stream.cuda_stream)
            e1.record(stream)
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
        s.check()
    return statistics.median(ms), used


def host_link(device, mib=512, reps=3):
    """Page-locked copy rates (GB/s) of the host link at this moment: the e2e
    and serving figures move with it (other jobs on the host share it)."""
    import torch

    h = torch.empty(mib << 20, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(mib << 20, dtype=torch.uint8, device=f"cuda:{device}")
    st = torch.cuda.Stream(device=device)
    res = {}
    with torch.cuda.stream(st):
        for name, dst, src in (("d2h", h, d), ("h2d", d, h)):
            dst.copy_(src, non_blocking=True)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(st)
            for _ in range(reps):
                dst.copy_(src, non_blocking=True)
            e1.record(st)
            st.synchronize()
            res[name + "_gbs"] = round(reps * h.numel() / (e0.elapsed_time(e1) * 1e-3) / 1e9, 1)
    del h, d
    return res


def serving_bench(tch, synth, args, device):
    """Resident database of n_db profiles x 1 142 loci (Zipf s = 1.2, 3 %
    missing), Poisson query arrivals (mean 50/s) of batches log-uniform in
    [1, 2 000] new profiles from the same generator, through tch_server."""
    import threading

    n_db, L, pool_rows = args.serve_db, 1142, 40000
    t0 = time.perf_counter()

    def distinct(rng, L):
        return np.clip(np.rint(rng.lognormal(np.log(60.0), 1.26, L)), 2, 3000).astype(np.int64)

    A = synth.zipf_profiles(n_db + pool_rows, L, 5, 1.2, distinct, lambda rng, L: np.full(L, 0.03),
                            hashed_frac=0.05)
    db_calls = A[:n_db]
    # the query profiles in page-locked memory, as a server receiving them
    # into pinned buffers has them (a pageable source is staged by the driver
    # and held up the other requests' copies)
    pool = tch.pinned_empty(A[n_db:].shape, A.dtype)
    pool[:] = A[n_db:]
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    db = tch.Database(db_calls, device=device)
    build_s = time.perf_counter() - t0
    dbi = db.info()
    rng = np.random.default_rng(11)
    R = args.serve_requests
    sizes = np.minimum(2000, np.floor(np.exp(rng.uniform(0, np.log(2001), R)))).astype(int)
    arrivals = np.cumsum(rng.exponential(1 / 50.0, R))
    starts = rng.integers(0, pool_rows - 2000, R)
    slots = 4
    # results go to page-locked buffers, reused: a request waits for a free one
    # (that wait counts in its latency)
    import queue as _queue

    nbuf = 8
    bufs = [(tch.pinned_empty((2000, n_db)), tch.pinned_empty((2000 * 2000,))) for _ in range(nbuf)]
    free = _queue.Queue()
    for k in range(nbuf):
        free.put(k)
    sv = tch.Server(db, slots=slots)
    # warm the kernels, grow the database's stream-ordered pool to `slots`
    # concurrent batches of the largest size, and write every result buffer
    # once from the GPU: the first device write into freshly pinned pages ran
    # at 11-35 GB/s instead of the link's ~190 (a server allocates its result
    # buffers once; the steady state is what the latencies describe)
    for k0 in range(0, nbuf, slots):
        warm = [sv.submit(pool[:2000], out=bufs[k][0], out_qq=bufs[k][1].reshape(2000, 2000))
                for k in range(k0, min(nbuf, k0 + slots))]
        for w in warm:
            sv.wait(w)
    rids = [None] * R
    bslot = [None] * R
    submit_delay = np.zeros(R)

    def submitter():
        for k in range(R):
            t = tb + arrivals[k]
            d = t - time.perf_counter()
            if d > 0:
                time.sleep(d)
            m = int(sizes[k])
            j = free.get()
            bslot[k] = j
            rids[k] = sv.submit(pool[starts[k]:starts[k] + m], out=bufs[j][0][:m],
                                out_qq=bufs[j][1][:m * m].reshape(m, m))
            submit_delay[k] = time.perf_counter() - t

    link_before = host_link(device)  # first use of torch here: outside the arrival clock
    tb = time.perf_counter() + 0.05
    th = threading.Thread(target=submitter)
    th.start()
    lat = np.zeros(R)
    queued = np.zeros(R)
    for k in range(R):
        while rids[k] is None:
            time.sleep(0.0005)
        _, _, q_s, l_s = sv.wait(rids[k])
        free.put(bslot[k])
        lat[k] = submit_delay[k] + l_s  # from the request's arrival
        queued[k] = q_s
    th.join()
    makespan = time.perf_counter() - tb
    link_after = host_link(device)
    sv.close()
    db.close()
    pairs = int(sum(m * n_db + m * (m - 1) // 2 for m in sizes))
    return {"db": f"{n_db} x {L} (Zipf s=1.2, lognormal distinct median 60, 3% missing, 5% 64-bit ids)",
            "db_tau": dbi["tau"], "db_device_gb": dbi["device_bytes"] / 1e9, "db_build_s": build_s,
            "requests": R, "arrival": "Poisson, mean 50/s", "batch": "log-uniform 1-2000 profiles",
            "query_rows": int(sizes.sum()), "slots": slots,
            "p50_ms": float(np.percentile(lat, 50) * 1e3), "p99_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_ms": float(lat.mean() * 1e3), "max_ms": float(lat.max() * 1e3),
            "slowest": [{"m": int(sizes[k]), "ms": float(lat[k] * 1e3), "queued_ms": float(queued[k] * 1e3),
                         "submit_delay_ms": float(submit_delay[k] * 1e3)} for k in np.argsort(-lat)[:4]],
            "queued_p50_ms": float(np.percentile(queued, 50) * 1e3),
            "pairs": pairs, "pairs_per_s": pairs / makespan, "makespan_s": makespan,
            "host_link_gbs": {"before": link_before, "after": link_after},
            "note": "latency = arrival -> q x db and q x q distances in (page-locked, reused) host memory, "
                    f"each of the {nbuf} result buffers written once by a warm-up query before the arrivals; "
                    f"generation {gen_s:.1f} s outside the timed region"}


def batch_bench(tch, args, device):
    """512 independent matrices, n log-uniform in [50, 5 000], L from {1 142,
    1 343, 2 794, 3 016}, Zipf s in [1.0, 1.4] over lognormal distinct counts,
    0-8 % missing: encoded once, then every upper triangle in one graph replay
    with the autotuned schedule and tau chosen per matrix."""
    import torch

    b, shapes, build_s = batch_sets(tch, args.batch_count, device)
    pairs = sum(n * (n - 1) // 2 for n, _ in shapes)
    off, ld = b.layout()
    out = torch.empty(int(off[-1]) + 8, dtype=torch.int16, device=f"cuda:{device}")
    stream = torch.cuda.Stream(device=device)
    t0 = time.perf_counter()
    tuned = b.tune(out.data_ptr(), stream.cuda_stream, reps=3)
    tune_s = time.perf_counter() - t0
    for _ in range(3):
        b.run(out.data_ptr(), stream.cuda_stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    reps = 10
    e0.record(stream)
    for _ in range(reps):
        b.run(out.data_ptr(), stream.cuda_stream)
    e1.record(stream)
    torch.cuda.synchronize()
    b.check()
    ms = e0.elapsed_time(e1) / reps
    taus = b.info()["taus"]
    b.close()
    return {"matrices": args.batch_count, "pairs": pairs, "ms_per_batch": ms, "pairs_per_s": pairs / (ms / 1e3),
            "schedule": tuned, "graph": ("one CUDA graph per replay: " + ("two persistent launches over every set"
                                       if tuned["branches"] == 0 else "fork/join over the tuned branch count")),
            "tau_per_matrix": {"min": int(min(taus)), "median": int(np.median(taus)), "max": int(max(taus))},
            "encode_s": build_s, "tune_s": tune_s}


DEFAULT_GROUP = 8  # the library's raster group of the tile pass when none is set


def picks(tch, A, device):
    """The analytic model's pick (its tau, the default schedule) and the
    learned model's pick (tau, sub-stripe rows, raster group) of a profile
    set, from the library's candidate rows; None without a shipped model."""
    if not os.path.exists(tch.TAU_MLP_PATH):
        return None
    w = tch.load_tau_mlp()
    c = tch.tau_features(A, device)
    pred = tch.mlp_predict(w, c["feats"], device)
    il = int(np.argmin(pred))
    dflt = (c["subs"] == 0) & (c["groups"] == DEFAULT_GROUP)
    ia = int(np.argmin(np.where(dflt, c["est"], np.inf)))
    analytic = (int(c["taus"][ia]), 0, 0)
    # the library takes the model's pick for sets of at most 65 536 profiles
    learned = (int(c["taus"][il]), int(c["subs"][il]), int(c["groups"][il])) if len(A) <= 65536 else analytic
    return {"analytic": analytic, "learned": learned}


def big_config_bench(tch, synth, args, device):
    """The all-frequent and the large-Zipf shapes (the reference's L4 could not
    hold the first on its tensor cores: ~250 k one-hot columns).

    founders   50 000 x 5 000 loci, 50 founder alleles per locus, 1 %
               mutations to fresh ids, 2 % missing: device encoder with the
               operand split along K into allocations of at most
               --founders-chunk-mb, the whole upper triangle in one stripe.
    zipf_big   200 000 x 3 000 loci, Zipf(1.1): the upper triangle (2.0e10
               pairs, 40 GB of u16) in stripes of --big-stripe rows written
               into one reused device buffer.
    Each: pairs/s of the device-resident solve (CUDA events; the step is the
    whole triangle) at the learned model's tau and at the analytic model's
    tau, and spread rows of the last stripe against the oracle's count on the
    raw ids."""
    import torch

    oracle = load_oracle()
    out_legs = {}
    stream = torch.cuda.Stream(device=device)
    sp = stream.cuda_stream
    for name in ("founders", "zipf_big"):
        t0 = time.perf_counter()
        A = synth.make(name)
        gen_s = time.perf_counter() - t0
        n, L = A.shape
        pairs = n * (n - 1) // 2
        chunk = (args.founders_chunk_mb << 20) if name == "founders" else 0
        S = n if name == "founders" else min(n, args.big_stripe)
        ldo = (n + 7) // 8 * 8
        stripes = [(r0, min(S, n - r0)) for r0 in range(0, n, S)]
        pk = picks(tch, A, device) or {}
        variants = [("learned", 0)] if pk else []
        variants.append(("analytic", pk["analytic"][0] if pk else 0))
        leg = {"shape": f"{n} x {L}", "pairs": pairs, "stripe_rows": S, "stripes": len(stripes),
               "chunk_limit_bytes": chunk, "generate_s": gen_s, "picks": pk}
        for vname, vtau in variants:
            if vname == "analytic" and pk:
                tch.set_tau_mlp(None)  # vtau is the analytic pick: nothing learned is consulted
            tch.set_max_chunk_bytes(chunk)
            try:
                t0 = time.perf_counter()
                s = tch.Solver.from_calls(A, tau=vtau, device=device)
                enc_s = time.perf_counter() - t0
            finally:
                tch.set_max_chunk_bytes(0)
                if pk:
                    tch.load_tau_mlp()
            with s:
                info = s.info()
                buf = torch.empty((S, ldo), dtype=torch.int16, device=f"cuda:{device}")

                def solve():
                    for r0, rows in stripes:
                        s.stripe(r0, rows, buf.data_ptr(), ldo, sp)

                with torch.cuda.stream(stream):
                    solve()  # warm-up
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                reps = 2
                e0.record(stream)
                for _ in range(reps):
                    solve()
                e1.record(stream)
                torch.cuda.synchronize()
                s.check()
                ms = e0.elapsed_time(e1) / reps
                k_alg = L + int(info["d_onehot"])
                v = {"tau": info["tau"], "sub_rows": info["sub_rows"], "tile_group": info["tile_group"],
                     "ms": ms, "pairs_per_s": pairs / (ms / 1e3),
                     "onehot_columns": int(info["d_onehot"]), "k_chunks": int(info["k_chunks"]),
                     "device_gb": info["device_bytes"] / 1e9, "rare_pairs": int(info["n_rare"]),
                     "ops_per_step": 2.0 * pairs * k_alg,
                     "whole_step_tflops": 2.0 * pairs * k_alg / (ms / 1e3) / 1e12, "encode_s": enc_s}
                if vname == variants[0][0]:
                    # the last stripe's rows against the oracle (raw ids, no ranking)
                    r0, rows = stripes[-1]
                    idx = sorted(set(np.linspace(r0, r0 + rows - 2, 24).astype(int).tolist()))
                    bad = cells = 0
                    for i in idx:
                        got = buf[i - r0, i + 1 - r0:n - r0].cpu().numpy().view(np.uint16)
                        want = oracle.hamming_block_calls(A, i, i + 1, i + 1, n)[0]
                        cells += got.size
                        bad += int((got != want).sum())
                    v["parity"] = {"rows": len(idx), "cells": cells, "mismatches": bad,
                                   "oracle": "orc_hamming_block_u64 (check.py:39-44 restated in C, on the raw ids)"}
                leg[vname] = v
                del buf
            torch.cuda.empty_cache()
        first = leg[variants[0][0]]
        leg.update(ms=first["ms"], pairs_per_s=first["pairs_per_s"], parity=first.get("parity"))
        log(name, leg)
        out_legs[name] = leg
        del A
    return out_legs


def linkage_timing(tch, synth, args, device):
    """--linkage-timing: the consumers of the matrix on the long-tail set of
    --n profiles.  The full matrix is put in device memory once (the solver's
    upper triangle, mirrored); then the minimum spanning tree and the k = 10
    and k = 32 nearest neighbours of every profile are computed from it,
    --reps times each (wall time of the call: kernels, the copy of the result
    to host memory, and the sort of the tree's edges), and the tree once more
    through the solver (its full matrix included).  Checks that need no full
    oracle matrix: the tree has n - 1 edges and joins every profile (the call
    checks that itself), every edge's distance equals the count on the ranks,
    every sampled row's lightest edge is in the tree (the cut property of a
    single profile), and the sampled rows' neighbours equal the oracle's row."""
    import torch

    oracle = load_oracle()
    n = args.n
    A = synth.longtail(n=n, L=args.L)
    x, _ = tch.dense_ranks(A)
    ld = (n + 7) // 8 * 8
    dev = f"cuda:{device}"
    out = {"workload": f"longtail {n}x{args.L}", "n": n}
    with tch.Solver.from_calls(A, device=device) as s:
        H = torch.empty((n, ld), dtype=torch.int16, device=dev)
        st = torch.cuda.current_stream().cuda_stream
        s.stripe(0, n, H.data_ptr(), ld, st)
        torch.cuda.synchronize()
        U = torch.triu(H[:, :n], 1)
        H[:, :n] = U + U.T
        del U
        torch.cuda.synchronize()
        times = {"mst": [], "k10": [], "k32": []}
        for _ in range(args.reps):
            t0 = time.perf_counter()
            u, v, w = tch.mst_device(H.data_ptr(), ld, n, st)
            times["mst"].append(time.perf_counter() - t0)
            for k in (10, 32):
                t0 = time.perf_counter()
                idx, dist = tch.neighbors_device(H.data_ptr(), ld, n, k, st)
                times[f"k{k}"].append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        u2, v2, w2 = s.mst()
        solver_mst_s = time.perf_counter() - t0
    del H
    torch.cuda.empty_cache()
    for key, ts in times.items():
        out[f"{key}_ms"] = round(float(np.median(ts)) * 1e3, 2)
        out[f"{key}_samples_ms"] = [round(t * 1e3, 2) for t in ts]
    out["solver_mst_ms"] = round(solver_mst_s * 1e3, 1)
    out["mst_weight"] = int(w.astype(np.int64).sum())
    same = bool((u == u2).all() and (v == v2).all() and (w == w2).all())
    # checks
    xu, xv = x[u.astype(np.int64)], x[v.astype(np.int64)]
    w_ref = ((xu != xv) & (xu > 0) & (xv > 0)).sum(1)
    del xu, xv
    tree = set(zip(u.tolist(), v.tolist()))
    rows = np.linspace(0, n - 1, 64).astype(np.int64)
    cut_bad = nbr_bad = 0
    for r in rows.tolist():
        d = oracle.hamming_block(x, r, r + 1, 0, n)[0].astype(np.int64)
        key = (d << 42) | (np.minimum(np.arange(n), r) << 21) | np.maximum(np.arange(n), r)
        key[r] = np.iinfo(np.int64).max
        j = int(key.argmin())
        cut_bad += (min(r, j), max(r, j)) not in tree
        order = np.lexsort((np.arange(n), np.where(np.arange(n) == r, 1 << 20, d)))[:32]
        nbr_bad += int((idx[r] != order).sum() + (dist[r] != d[order]).sum())
    out["checks"] = {"edges": int(len(u)), "edge_distance_mismatches": int((w_ref != w).sum()),
                     "sampled_rows": int(len(rows)), "cut_property_violations": int(cut_bad),
                     "neighbor_mismatches": int(nbr_bad), "solver_tree_equal": same}
    print(json.dumps(out), flush=True)


def step_timing(tch, synth, args, device):
    """--step-timing: the two passes of one whole-triangle solve of the
    long-tail generator at --n profiles and --tau (rare counts, then the tile
    pass), timed apart with CUDA events, --reps times.  The small case the
    kernel profiles are captured on: one launch of each kernel per rep."""
    import torch

    n = args.n
    A = synth.longtail(n=n, L=args.L)
    with tch.Solver.from_calls(A, tau=args.tau, kernel=args.kernel, device=device) as s:
        info = s.info()
        log(info)
        ldr = (n + 255) // 256 * 256
        ldo = (n + 7) // 8 * 8
        R = torch.empty((n, ldr), dtype=torch.int16, device=f"cuda:{device}")
        out = torch.empty((n, ldo), dtype=torch.int16, device=f"cuda:{device}")
        st = torch.cuda.current_stream().cuda_stream
        for _ in range(args.reps):
            e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
            e0.record()
            s.rare_counts(0, n, R.data_ptr(), ldr, st)
            e1.record()
            s.stripe_counts(0, n, out.data_ptr(), ldo, R.data_ptr(), ldr, st)
            e2.record()
            torch.cuda.synchronize()
            rare_ms, tile_ms = e0.elapsed_time(e1), e1.elapsed_time(e2)
            print(f"rare counts {rare_ms:.3f} ms  tile pass {tile_ms:.3f} ms  "
                  f"{info['n_rare'] / rare_ms * 1e3:.3e} rare pairs/s", flush=True)
        s.check()


def cli_timing(tch, synth, args):
    """--cli-timing: the command-line tool end to end on the long-tail profiles
    (--n x --L) written as a TSV (sample ids, '-' for missing calls): the table
    parsed on the GPU (the default) and on the host cores (--host-parse), the
    full matrix written as TSV to /dev/null; wall seconds, best of 3 each."""
    import tempfile

    A = synth.longtail(n=args.n, L=args.L)
    t0 = time.perf_counter()
    fd, path = tempfile.mkstemp(suffix=".tsv")
    with os.fdopen(fd, "w") as f:
        f.write("FILE\t" + "\t".join(f"locus{k}" for k in range(args.L)) + "\n")
        for i in range(len(A)):
            f.write(f"s{i}\t" + "\t".join("-" if v == 0 else str(v) for v in A[i].tolist()) + "\n")
    gen_s = time.perf_counter() - t0
    size = os.path.getsize(path)
    res = {}
    try:
        for name, extra in (("gpu_parse", []), ("host_parse", ["--host-parse"])):
            walls = []
            for _ in range(3):
                t0 = time.perf_counter()
                r = subprocess.run([tch.CLI_PATH, "-i", path, "-o", "/dev/null", *extra], capture_output=True,
                                   text=True)
                walls.append(time.perf_counter() - t0)
                if r.returncode:
                    raise RuntimeError(r.stderr[-2000:])
            res[name] = {"wall_s": min(walls), "samples_s": [round(w, 3) for w in walls],
                         "log": [ln for ln in r.stderr.splitlines() if ln.startswith(("Loaded", "Encoded",
                                                                                         "Computed"))]}
    finally:
        os.unlink(path)
    print(json.dumps({"cli": f"{args.n} x {args.L} long-tail profiles, {size / 1e9:.2f} GB of TSV in, "
                             f"the full matrix as TSV out", "generate_s": gen_s, **res}), flush=True)


def batch_sets(tch, count, device):
    """The batched leg's generator: count sets, n log-uniform in [50, 5 000],
    L from {1 142, 1 343, 2 794, 3 016}, Zipf s in [1.0, 1.4] over lognormal
    distinct counts, 0-8 % missing (seed 21), added to a new tch.Batch."""
    rng = np.random.default_rng(21)
    b = tch.Batch(device=device)
    shapes = []
    build_s = 0.0
    for _ in range(count):
        n = int(np.exp(rng.uniform(np.log(50), np.log(5000))))
        L = int(rng.choice([1142, 1343, 2794, 3016]))
        s = float(rng.uniform(1.0, 1.4))
        k = np.clip(np.rint(rng.lognormal(np.log(40.0), 1.0, L)), 2, 500).astype(np.int64)
        a = (rng.zipf(max(s, 1.01), size=(n, L)) - 1) % k[None, :]
        A = (np.arange(L, dtype=np.uint64)[None, :] << np.uint64(20)) + a.astype(np.uint64) + np.uint64(1)
        A[rng.random((n, L)) < rng.uniform(0.0, 0.08)] = 0
        t0 = time.perf_counter()
        b.add(A)  # device encoding (tau per matrix)
        build_s += time.perf_counter() - t0
        shapes.append((n, L))
    return b, shapes, build_s


def batch_timing(tch, args, device):
    """--batch-timing: one batched solve with a fixed schedule (--branches):
    CUDA-event time of a graph replay (median of 5 after 3
    untimed) and the largest sets with their tau."""
    import torch

    b, shapes, _ = batch_sets(tch, args.batch_count, device)
    off, _ = b.layout()
    out = torch.empty(int(off[-1]) + 8, dtype=torch.int16, device=f"cuda:{device}")
    st = torch.cuda.Stream(device=device)
    b.set_schedule(args.branches)
    for _ in range(3):
        b.run(out.data_ptr(), st.cuda_stream)
    ms = []
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        b.run(out.data_ptr(), st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    b.check()
    taus = b.info()["taus"]
    pairs = [n * (n - 1) // 2 for n, _ in shapes]
    print(f"ms per batch {sorted(ms)[len(ms) // 2]:.3f} ({sum(pairs)} pairs, {args.batch_count} sets, "
          f"{args.branches} branches)", flush=True)
    for i in sorted(range(len(shapes)), key=lambda i: -pairs[i])[:8]:
        print(f"  set {i}: n {shapes[i][0]} L {shapes[i][1]} tau {taus[i]}", flush=True)
    b.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--kernel", default="tc_f4")
    ap.add_argument("--tau", type=int, default=0, help="0 = the analytic GB300 model's choice")
    ap.add_argument("--stripe", type=int, default=4096, help="rows per stripe of the e2e tch_run call")
    ap.add_argument("--e2e-steps", type=int, default=7, help="timed e2e passes; the median is reported")
    ap.add_argument("--cpu-steps", type=int, default=4, help="CPU baseline: steps of the reference arm's sample")
    ap.add_argument("--n", type=int, default=63005)
    ap.add_argument("--L", type=int, default=1142)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--analytic-tau", action="store_true", help="ignore the shipped learned tau model")
    ap.add_argument("--no-tau-sweep", action="store_true")
    ap.add_argument("--no-serving", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-tsv", action="store_true")
    ap.add_argument("--no-big", action="store_true", help="skip the founders and zipf_big legs")
    ap.add_argument("--founders-chunk-mb", type=int, default=2048,
                    help="largest single allocation of the founders operand (K chunks)")
    ap.add_argument("--big-stripe", type=int, default=16384, help="rows per stripe of the zipf_big leg")
    ap.add_argument("--batch-count", type=int, default=512)
    ap.add_argument("--serve-db", type=int, default=200000)
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--serving-only", action="store_true", help="run the serving leg alone and print its JSON")
    ap.add_argument("--step-timing", action="store_true",
                    help="time the rare counts and the tile pass of one solve of --n profiles at --tau, --reps times")
    ap.add_argument("--cli-timing", action="store_true",
                    help="time the command-line tool on the long-tail profiles as a TSV (GPU and host parse)")
    ap.add_argument("--batch-timing", action="store_true",
                    help="time one batched replay of --batch-count sets with --branches")
    ap.add_argument("--linkage-timing", action="store_true",
                    help="time the minimum spanning tree and nearest neighbours on the full matrix")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--branches", type=int, default=32)
    ap.add_argument("--ref-stride", type=int, default=6,
                    help="reference arm: rows k, k + s, ... of the triangle per step")
    ap.add_argument("--parity-rows", type=int, default=256,
                    help="spread rows of the timed output compared with the oracle")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    ws, rank, local = dist_env()
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(reference_arm(args)), flush=True)
        return
    if ws > 1:
        log("bench.py: this build offers one-GPU runs only; run it without torchrun")
        sys.exit(2)

    tch = importlib.import_module(PKG)
    synth = importlib.import_module(PKG + ".synth")
    if args.serving_only:  # a service runs in its own process
        print(json.dumps(serving_bench(tch, synth, args, local)), flush=True)
        return
    if args.step_timing:
        step_timing(tch, synth, args, local)
        return
    if args.batch_timing:
        batch_timing(tch, args, local)
        return
    if args.linkage_timing:
        linkage_timing(tch, synth, args, local)
        return
    if args.cli_timing:
        cli_timing(tch, synth, args)
        return

    t0 = time.perf_counter()
    A = synth.longtail(n=args.n, L=args.L)
    x, nd = tch.dense_ranks(A)
    n, L = x.shape
    pairs_total = n * (n - 1) // 2
    workload = workload_config(n, L)
    log(f"generated + ranked {n}x{L} in {time.perf_counter() - t0:.1f}s")

    import torch

    device = local
    torch.cuda.set_device(device)
    assert tch.device_count() > 0

    # tau: the learned model shipped with the package picks it (the analytic
    # model's pick is timed beside it below)
    tau_pick = {}
    if not args.tau and not args.analytic_tau:
        tau_pick = picks(tch, A, device) or {}
    t0 = time.perf_counter()
    solver = tch.Solver.from_calls(A, tau=args.tau, kernel=args.kernel, device=device)  # device encoder
    info = solver.info()
    tau = info["tau"]
    log(f"device-encoded tau={tau}: D={info['d_onehot']} n_rare={info['n_rare']} in "
        f"{time.perf_counter() - t0:.1f}s", info)
    a, b = 0, n
    ldo = (n + 7) // 8 * 8
    out = torch.empty(((b - a), ldo), dtype=torch.int16, device=f"cuda:{device}")
    stream = torch.cuda.Stream(device=device)
    sp = stream.cuda_stream

    def step():
        solver.stripe(a, b - a, out.data_ptr(), ldo, sp)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    solver.check()
    torch.cuda.synchronize()
    clocks = Clocks(device)
    clocks.start()
    time.sleep(0.3)
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    launch_ms = []
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    ev0.record(stream)
    for k in range(args.steps):
        evs[k][0].record(stream)
        step()
        evs[k][1].record(stream)
    ev1.record(stream)
    torch.cuda.synchronize()
    ck = clocks.stop()
    solver.check()
    total_ms = ev0.elapsed_time(ev1)
    launch_ms = [s.elapsed_time(e) for s, e in evs]
    ms_per_step = total_ms / args.steps
    value = pairs_total / (ms_per_step / 1e3)
    # the last timed step's output against the oracle on spread rows
    parity = parity_rows(load_oracle().dense_ranks(A)[0], out, args.parity_rows) if args.parity_rows else None
    log("parity:", parity)

    # a dense-rare solver's step is two launches: the stripe's rare counts,
    # then the tile pass that subtracts them; time them apart for the roofline
    dense = bool(info.get("rare_dense"))
    launches_per_step = 2 if dense else 1
    split = None
    tc_ms = statistics.median(launch_ms)
    if dense:
        ldr = (n - a + 255) // 256 * 256
        rbuf = torch.empty(((b - a), ldr), dtype=torch.int16, device=f"cuda:{device}")
        trip = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(max(args.steps, 3))]
        for e0, e1, e2 in trip:
            e0.record(stream)
            solver.rare_counts(a, b - a, rbuf.data_ptr(), ldr, sp)
            e1.record(stream)
            solver.stripe_counts(a, b - a, out.data_ptr(), ldo, rbuf.data_ptr(), ldr, sp)
            e2.record(stream)
        torch.cuda.synchronize()
        solver.check()
        rare_ms = statistics.median(e0.elapsed_time(e1) for e0, e1, _ in trip)
        tc_ms = statistics.median(e1.elapsed_time(e2) for _, e1, e2 in trip)
        split = {"rare_counts_ms": rare_ms, "tile_pass_ms": tc_ms, "rare_pairs": int(info["n_rare"]),
                 "rare_pairs_per_s": info["n_rare"] * (b - a) / max(n, 1) / (rare_ms / 1e3)}
        del rbuf
        log("split:", split)

    # roofline of the tile-pass kernel (tc_stripe_kernel)
    k_alg = L + int(info["d_onehot"])
    my_pairs = sum(n - 1 - i for i in range(a, b))
    ops_per_launch = 2.0 * my_pairs * k_alg
    achieved = ops_per_launch / (tc_ms / 1e3) / 1e12
    peak_info = tc_peaks()
    mp = measured_peaks()
    peak = peak_info.get("tc_f4_tflops") if peak_info.get("tc_f4_tflops_check") == "exact" else None
    peak_src = "tch-peak tcgen05 kind::mxf4 probe on this GPU (same process)"
    if not peak:
        peak = 4 * (mp or {}).get("bf16_tflops", 1900.0)
        peak_src = "4 x measured bf16 (fp4 dense rate ratio)"
    roofline = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": peak_src,
                "algorithmic_ops_per_launch": ops_per_launch, "k_per_pair": k_alg,
                "k_padded_columns": info["k_presence"] + info["k_onehot"],
                "bf16_measured_tflops": (mp or {}).get("bf16_tflops"), "traffic": None}
    # DRAM bytes of one whole-triangle tile pass, from the ncu capture of this
    # workload (valid for the tau and row share it was taken at)
    prof = os.path.join(ROOT, "profiles", "tc_stripe_longtail_traffic.txt")
    if os.path.exists(prof):
        with open(prof) as f:
            kv = dict(line.split(":", 1) for line in f if ":" in line)
        if int(kv.get("tau", "0")) == tau and int(kv.get("n", "0")) == n:
            roofline["traffic"] = int(kv["bytes_per_launch"])
            roofline["traffic_source"] = kv.get("source", "").strip()

    # e2e through the C ABI with host buffers: tch_run (the reference's entry
    # point, host-encoded operands) and tch_run_calls (allele calls, device
    # encoder), first after the device-resident timing: copies from host memory
    # run slower after the legs that pin and release gigabytes of it
    e2e = None
    e2e_calls = None
    if args.e2e_steps > 0:
        import ctypes

        os.environ["TCH_VERBOSE"] = "1"  # phase breakdown on stderr
        tch.set_kernel(args.kernel)
        # the host path uploads every rare pair: its tau model charges the upload
        # (the tile pass's column MACs per second; pairs per second of the
        # upload at the host link's ~190 GB/s, 4 bytes each)
        tau_host = args.tau or tch.choose_tau(x, nd, args.stripe, tch.free_vram(device), 2.9e15, 4.5e10)
        enc = tch.encode_host(x, nd, tau_host)  # the reference host's encoding, outside the timed region
        h2d = enc.O.nbytes + enc.P.nbytes + enc.start.nbytes + enc.js.nbytes

        def pinned(a):
            """The step's input in page-locked host memory (the copy is made
            outside the timed region; the library copies it in every step)."""
            b = tch.pinned_empty(a.shape, a.dtype)
            np.copyto(b, a)
            return b

        hO, hP, hS, hJ, hA = pinned(enc.O), pinned(enc.P), pinned(enc.start), pinned(enc.js), pinned(A)
        d2h = sum(min(args.stripe, n - r0) * (n - r0) * 2 for r0 in range(0, n, args.stripe))

        def nop(ctx, r0, rows, w, ptr):
            pass

        cb = tch.CB(nop)
        link_before = host_link(device)
        times, times_calls = [], []
        for k in range(args.e2e_steps + 1):
            secs = ctypes.c_double(0)
            rg = ctypes.c_int(0)
            err = ctypes.create_string_buffer(512)
            t = time.perf_counter()
            rc = tch.lib().tch_run(device, enc.n, enc.n_pad, tch._ptr(hO), enc.K1, tch._ptr(hP), enc.K2,
                                   tch._ptr(hS), tch._ptr(hJ), enc.n_rare, args.stripe, cb, None,
                                   ctypes.byref(secs), ctypes.byref(rg), err, len(err))
            dt = time.perf_counter() - t
            if rc:
                raise RuntimeError(err.value.decode())
            tu = ctypes.c_int(0)
            t = time.perf_counter()
            rc = tch.lib().tch_run_calls(device, n, L, tch._ptr(hA), args.tau, args.stripe, cb, None,
                                         ctypes.byref(secs), ctypes.byref(tu), err, len(err))
            dt_calls = time.perf_counter() - t
            if rc:
                raise RuntimeError(err.value.decode())
            if k > 0:  # the first pass warms the context and the pinned stripe buffers
                times.append(dt)
                times_calls.append(dt_calls)
        os.environ.pop("TCH_VERBOSE", None)
        link = {"before": link_before, "after": host_link(device)}
        e2e_s = statistics.median(times)
        e2e = {"value": pairs_total / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "seconds_per_step": e2e_s, "tau": tau_host, "host_link_gbs": link,
               "samples_s": [round(t, 5) for t in times],
               "path": f"tch_run (the reference's C ABI): host O/P bits + rare CSR (page-locked host memory) "
                       f"uploaded, stripes of {args.stripe} rows copied back, no-op callback"}
        ec = statistics.median(times_calls)
        e2e_calls = {"value": pairs_total / ec, "unit": UNIT, "h2d_bytes_per_step": int(A.nbytes),
                     "d2h_bytes_per_step": int(d2h), "seconds_per_step": ec, "tau": int(tu.value), "host_link_gbs": link,
                     "samples_s": [round(t, 5) for t in times_calls],
                     "path": "tch_run_calls: allele calls (page-locked host memory) uploaded, device encoder, "
                             "same stripes and copy-back"}
        del hO, hP, hS, hJ, hA

    # serving: in a process of its own, as a service would run, after the e2e
    # legs and before the legs that churn host memory (large copies from host
    # memory slow down after them)
    serving = None
    if not args.no_serving:
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--serving-only",
                            "--serve-db", str(args.serve_db), "--serve-requests", str(args.serve_requests)],
                           capture_output=True, text=True, env=dict(os.environ, CUDA_VISIBLE_DEVICES=str(device)))
        if r.returncode:
            raise RuntimeError("serving leg failed: " + r.stderr[-2000:])
        serving = json.loads(r.stdout.strip().splitlines()[-1])
        serving["process"] = "separate (bench.py --serving-only)"
        log("serving:", serving)

    # learned vs analytic tau: whole-triangle device time at each pick and at
    # a sweep of taus around them (fresh solvers)
    tau_cmp = None
    if not args.no_tau_sweep:
        used = (int(tau), int(info.get("sub_rows", 0)), int(info.get("tile_group", 0)))
        swept = {used: ms_per_step}
        cands = {(t, 0, 0) for t in (512, 1024, 2048, 4096, 8192)} | set(tau_pick.values())
        for c in sorted(cands):
            if c not in swept:
                ms_t, _ = time_whole(tch, A, c[0], device, out, ldo, stream, sched=c[1:])
                swept[c] = ms_t
        best = min(swept, key=swept.get)
        key = lambda c: f"tau={c[0]} sub_rows={c[1]} group={c[2] or DEFAULT_GROUP}"  # noqa: E731
        tau_cmp = {"used": key(used), "swept_ms": {key(k): v for k, v in sorted(swept.items())},
                   "best_swept": {"candidate": key(best), "ms": swept[best]},
                   "note": "analytic: its tau with the default schedule; learned: the model's tau and schedule "
                           "(sub-stripe rows, raster group); whole-triangle device ms of fresh solvers"}
        for k, v in tau_pick.items():
            tau_cmp[k] = {"candidate": key(v), "ms": swept.get(v)}
        log("tau comparison:", tau_cmp)

    # the reference's TSV writer (main.rs:224-265) on the GPU: the full matrix
    # as text, delivered block by block to a callback that discards it
    tsv = None
    if not args.no_tsv:
        import ctypes

        nbytes = [0]

        def take(ctx, p, n):
            nbytes[0] += n

        cb = tch.TEXT_CB(take)
        ids = (ctypes.c_char_p * n)(*[f"sample{i:05d}".encode() for i in range(n)])
        err = ctypes.create_string_buffer(512)
        times = []
        for _ in range(2):
            nbytes[0] = 0
            t = time.perf_counter()
            rc = tch.lib().tch_solver_write_tsv(solver._h, ids, b"\t", b"cgmlst-hamming-gpu", 0, 0, 0, cb, None,
                                                err, len(err))
            times.append(time.perf_counter() - t)
            if rc:
                raise RuntimeError(err.value.decode())
        tsv = {"bytes": nbytes[0], "seconds": min(times), "gb_per_s": nbytes[0] / min(times) / 1e9,
               "pairs_per_s": pairs_total / min(times),
               "path": "tch_solver_write_tsv: whole triangle computed, mirrored, formatted on the GPU in blocks of "
                       "2048 rows, copied to pinned host memory, handed to a callback (full layout, tab)"}
        log("tsv writer:", tsv)

    batched = None
    if not args.no_batch:
        solver.close()
        del out
        torch.cuda.empty_cache()
        batched = batch_bench(tch, args, device)
        log("batched:", batched)

    big = None
    if not args.no_big:
        big = big_config_bench(tch, synth, args, device)

    cpu = None
    if not args.no_cpu:
        st = max(1, args.ref_stride)
        cpu_steps = max(1, min(st, args.cpu_steps))
        pairs, dt = cpu_count_steps(x, st, 0, cpu_steps)
        threads = load_oracle().lib().orc_num_threads()
        cpu = {"value": pairs / dt, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"oracle brute force (check.py:39-44 in C, OpenMP, {threads} threads) over rows k, k+{st}, "
                         f"... of the upper triangle for k = 0..{cpu_steps - 1}: {pairs} pairs in {dt:.1f} s"}

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": DTYPE,
            "data": "synthetic", "config": workload,
            "solver": {"tau": tau, "kernel": info["kernel"], "stripe_e2e": args.stripe, "rows_per_step": n},
            "gpu_launches": args.steps * launches_per_step, "step_split": split, "parity": parity,
            "clocks": ck, "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "e2e_device_encoder": e2e_calls, "tau_choice": tau_cmp, "tsv_writer": tsv, "batched": batched,
            "big_configs": big, "serving": serving, "peak_probe": peak_info}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
