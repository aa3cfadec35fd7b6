#!/usr/bin/env python3
"""Times the two passes of one whole-triangle solve apart, on the long-tail
profile generator: the dense rare counts (tch_solver_rare_counts) into a u16
block, then the tensor-core tile pass that subtracts them
(tch_solver_stripe_counts), with CUDA events on the launching stream.

    python cgmlst-hamming-gpu_gb300/step_timing.py [n] [tau] [reps]

n profiles x 1 142 loci (default 24 576), tau the rare threshold (default
2 048), reps the number of timed repetitions (default 3).  This is also the
small case the kernel profiles are captured on (one launch of each kernel per
repetition)."""
import argparse
import importlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
PKG = os.path.basename(HERE)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("n", type=int, nargs="?", default=24576)
    ap.add_argument("tau", type=int, nargs="?", default=2048)
    ap.add_argument("reps", type=int, nargs="?", default=3)
    args = ap.parse_args()
    import torch

    tch = importlib.import_module(PKG)
    synth = importlib.import_module(PKG + ".synth")
    n = args.n
    A = synth.longtail(n=n, L=1142)
    with tch.Solver.from_calls(A, tau=args.tau) as s:
        info = s.info()
        print(info, flush=True)
        ldr = (n + 255) // 256 * 256
        ldo = (n + 7) // 8 * 8
        R = torch.empty((n, ldr), dtype=torch.int16, device="cuda")
        out = torch.empty((n, ldo), dtype=torch.int16, device="cuda")
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


if __name__ == "__main__":
    main()
