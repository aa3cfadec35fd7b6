#!/usr/bin/env python3
"""Times one batched solve of uneven profile sets (tch_batch) with a fixed
schedule: [count] sets, n log-uniform in [50, 5 000], L from {1 142, 1 343,
2 794, 3 016}, Zipf s in [1.0, 1.4] over lognormal distinct counts, 0-8 %
missing — the generator and seed of the benchmark's batched leg.  Prints the
CUDA-event time of one graph replay (median of 5 after 3 untimed) and the
largest sets with the tau each got.

    python cgmlst-hamming-gpu_gb300/batch_timing.py [count] [branches] [cluster]
"""
import argparse
import importlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
PKG = os.path.basename(HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("count", type=int, nargs="?", default=512)
    ap.add_argument("branches", type=int, nargs="?", default=32)
    ap.add_argument("cluster", type=int, nargs="?", default=1)
    args = ap.parse_args()
    import numpy as np
    import torch

    tch = importlib.import_module(PKG)
    rng = np.random.default_rng(21)
    b = tch.Batch(device=0)
    shapes = []
    for _ in range(args.count):
        n = int(np.exp(rng.uniform(np.log(50), np.log(5000))))
        L = int(rng.choice([1142, 1343, 2794, 3016]))
        s = float(rng.uniform(1.0, 1.4))
        k = np.clip(np.rint(rng.lognormal(np.log(40.0), 1.0, L)), 2, 500).astype(np.int64)
        a = (rng.zipf(max(s, 1.01), size=(n, L)) - 1) % k[None, :]
        A = (np.arange(L, dtype=np.uint64)[None, :] << np.uint64(20)) + a.astype(np.uint64) + np.uint64(1)
        A[rng.random((n, L)) < rng.uniform(0.0, 0.08)] = 0
        b.add(A)
        shapes.append((n, L))
    off, _ = b.layout()
    out = torch.empty(int(off[-1]) + 8, dtype=torch.int16, device="cuda")
    st = torch.cuda.Stream()
    b.set_schedule(args.branches, args.cluster, args.cluster)
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
    print(f"ms per batch {sorted(ms)[len(ms) // 2]:.3f} ({sum(pairs)} pairs, {args.count} sets, "
          f"{args.branches} branches, cluster {args.cluster})", flush=True)
    for i in sorted(range(len(shapes)), key=lambda i: -pairs[i])[:8]:
        print(f"  set {i}: n {shapes[i][0]} L {shapes[i][1]} tau {taus[i]}", flush=True)
    b.close()


if __name__ == "__main__":
    main()
