"""Measured tensor-pipe rates of this GPU, the denominators of the rooflines.

  python -m batchgemm_gb300.peaks [--sustained-s 4] [--cubes 32]

Prints one JSON line with
  * ``tf32_tflops``: cuBLAS TF32 GEMM (torch.matmul of FP32 8192 x 8192
    operands with TF32 allowed), 2 * 8192^3 flops, best of 10 launches by CUDA
    events (burst, the figure for a kernel timed alone);
  * ``tf32_tflops_sustained``: the same GEMM back to back for --sustained-s
    seconds (the figure under the power cap);
  * ``bf16_tflops``: the bf16 GEMM of the same size, best of 10, so the two
    can be compared on one box;
  * ``own_tf32_pair_tflops``: this library's single-product TF32 mode on
    --cubes matrices of 1024^3 (CTA-pair tiles), GEMM kernel alone (CUDA
    events the library records around its launch), best of 10;
  * the SM clocks sampled by nvidia-smi during the sustained loop;
  * ``hbm_mix_gbs``: HBM ceilings of four read:write mixes (one read and two
    writes -- the split pre-pass's mix --, copy, write only, read only) from
    the library's float4 streaming probe over 2 GiB buffers, best of two grid
    sizes and 5 launches each.

bench.py runs :func:`tf32_burst` itself on the box it measures on.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))

N_GEMM = 8192


def _matmul_rate(dtype, reps=10, n=N_GEMM):
    import torch
    a = torch.randn(n, n, device="cuda").to(dtype)
    b = torch.randn(n, n, device="cuda").to(dtype)
    for _ in range(3):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12, a, b


def tf32_burst(reps=10):
    """cuBLAS TF32 8192^3 GEMM, best of `reps` launches (TFLOP/s)."""
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        rate, a, b = _matmul_rate(torch.float32, reps)
        del a, b
        return rate
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


HBM_KINDS = {0: ("read1_write2", 3), 1: ("copy", 2), 2: ("write_only", 1), 3: ("read_only", 1)}


def hbm_mix(kinds=(0, 1, 2, 3), gib=2.0, reps=5):
    """GB/s of the library's streaming probe (bgemm_debug_hbm_probe) per
    read:write mix: algorithmic bytes over the best CUDA-event time."""
    import torch
    import batchgemm_gb300 as bg
    L = bg.lib()
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    n = int(gib * (1 << 30)) // 16 * 4  # floats, a whole number of float4 words
    x = torch.rand(n, device="cuda")
    y1 = torch.empty_like(x)
    y2 = torch.empty_like(x)
    st = torch.cuda.current_stream().cuda_stream
    out = {}
    try:
        for kind in kinds:
            name, words = HBM_KINDS[kind]
            best = float("inf")
            for grid in (8 * sms, 32 * sms):
                for r in range(reps + 2):
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record()
                    if L.bgemm_debug_hbm_probe(kind, x.data_ptr(), y1.data_ptr(), y2.data_ptr(),
                                               n // 4, grid, st) != 0:
                        raise RuntimeError("bgemm_debug_hbm_probe failed")
                    e1.record()
                    e1.synchronize()
                    if r >= 2:
                        best = min(best, e0.elapsed_time(e1))
            out[name] = round(words * n * 4 / (best * 1e-3) / 1e9, 1)
    finally:
        del x, y1, y2
        torch.cuda.empty_cache()
    return out


def _sustained(seconds):
    import torch
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    try:
        n = N_GEMM
        a = torch.randn(n, n, device="cuda")
        b = torch.randn(n, n, device="cuda")
        torch.matmul(a, b)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        # a first short loop sizes the number of launches to the duration
        e0.record()
        for _ in range(10):
            torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        per = e0.elapsed_time(e1) / 10
        reps = max(10, int(seconds * 1e3 / per))
        e0.record()
        for _ in range(reps):
            torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        return 2.0 * n ** 3 * reps / (e0.elapsed_time(e1) * 1e-3) / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def own_tf32_pair(cubes=32, size=1024, reps=10):
    """This library's TF32 mode on `cubes` matrices of size^3, GEMM kernel only."""
    import torch
    import batchgemm_gb300 as bg
    from batchgemm_gb300.batch import DeviceBatch
    bg.lib()
    db = DeviceBatch([size] * cubes, [size] * cubes, [size] * cubes).fill_fast("normal", 0)
    p = db.plan("tf32", kernel_family="pair")
    for _ in range(3):
        db.execute(p)
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()  # creates the CUDA events the library records into
        e1.record()
        p.set_kernel_events(e0, e1)
        db.execute(p)
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    p.set_kernel_events(None, None)
    p.check_device()
    hist = p.info()["tile_config_hist"]
    p.close()
    return 2.0 * size ** 3 * cubes / (best * 1e-3) / 1e12, best, hist


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--sustained-s", type=float, default=4.0)
    ap.add_argument("--cubes", type=int, default=32)
    a = ap.parse_args()
    import torch
    torch.cuda.init()
    out = {"gpu": torch.cuda.get_device_name(0), "gemm": "%d^3" % N_GEMM}
    out["tf32_tflops"] = round(tf32_burst(), 1)
    bf16, x, y = _matmul_rate(torch.bfloat16)
    del x, y
    out["bf16_tflops"] = round(bf16, 1)
    clk_path = os.path.join(tempfile.gettempdir(), "bgemm_peaks_clocks_%d.csv" % os.getpid())
    f = open(clk_path, "w")
    try:
        smi = subprocess.Popen(["nvidia-smi", "-i", "0", "--query-gpu=clocks.sm,clocks.max.sm,"
                                "power.draw,clocks_event_reasons.active",
                                "--format=csv,noheader,nounits", "-lms", "200"], stdout=f,
                               stderr=subprocess.DEVNULL)
    except OSError:
        smi = None
    time.sleep(0.3)
    out["tf32_tflops_sustained"] = round(_sustained(a.sustained_s), 1)
    if smi is not None:
        smi.terminate()
        smi.wait()
    f.close()
    sm, smax, pw = [], [], []
    for line in open(clk_path):
        p = [x.strip() for x in line.split(",")]
        try:
            sm.append(float(p[0]))
            smax.append(float(p[1]))
            pw.append(float(p[2]))
        except (ValueError, IndexError):
            continue
    if sm:
        busy = [s for s in sm if s > 0.5 * max(sm)] or sm
        out["sustained_clocks"] = {"sm_mhz_median": statistics.median(busy),
                                   "sm_max_mhz": max(smax), "power_w_max": max(pw),
                                   "samples": len(sm)}
    out["hbm_mix_gbs"] = hbm_mix()
    rate, ms, hist = own_tf32_pair(a.cubes)
    out["own_tf32_pair_tflops"] = round(rate, 1)
    out["own_tf32_pair"] = {"workload": "%d matrices 1024^3, TF32 mode, CTA-pair tiles" % a.cubes,
                            "gemm_ms_best": round(ms, 4),
                            "tile_config_hist": hist}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
