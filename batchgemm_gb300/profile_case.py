"""Small, self-timed runs of one mode on a seeded workload, for profilers.

  python -m batchgemm_gb300.profile_case --mode tf32x3 --workload skewed --n 400 --reps 3

Builds one plan, runs ``reps`` warm executes, then ``reps`` timed executes
(CUDA events) and prints TFLOP/s.  Sized by --n so that a profiler capture of
one launch stays small (skewed with n = 400 holds about 2 GB on the device).
"""
from __future__ import annotations

import argparse
import os
import sys

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--mode", default="tf32x3")
    ap.add_argument("--workload", default="skewed",
                    choices=["skewed", "plain", "scale", "uneven", "cube"])
    ap.add_argument("--n", type=int, default=400, help="matrices (skewed, cube)")
    ap.add_argument("--size", type=int, default=1024, help="M = N = K of the cube workload")
    ap.add_argument("--force", type=int, default=-1, help="tile configuration id")
    ap.add_argument("--reps", type=int, default=3)
    a = ap.parse_args()
    import torch
    import batchgemm_gb300 as bg
    from batchgemm_gb300 import workloads
    from batchgemm_gb300.batch import DeviceBatch

    bg.lib()
    if a.workload == "skewed":
        w = workloads.skewed(0, a.n)
    elif a.workload == "cube":
        w = workloads.Workload("cube_%d_x%d" % (a.size, a.n), [a.size] * a.n, [a.size] * a.n,
                               [a.size] * a.n, 1.0, 0.0, "normal")
    else:
        w = {"plain": workloads.plain_fp32, "scale": workloads.simt_at_scale,
             "uneven": workloads.uneven_m}[a.workload](0)
    db = DeviceBatch(w.M, w.N, w.K).fill_fast(w.dist, 0)
    p = db.plan(a.mode, force_tile_config=a.force)
    for _ in range(a.reps):
        db.execute(p, w.alpha, w.beta)
    torch.cuda.synchronize()
    p.check_device()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        db.execute(p, w.alpha, w.beta)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / a.reps
    info = p.info()
    print("%s %s batch=%d gflop=%.2f ms=%.3f tflops=%.2f tiles=%d grid=%d" % (
        a.mode, w.name, w.batch, w.flops() / 1e9, ms, w.flops() / ms / 1e9, info["num_tiles"],
        info["grid"]))
    p.close()


if __name__ == "__main__":
    main()
