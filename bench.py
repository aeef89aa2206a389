"""Benchmark of variable-size batched SGEMM on GB300.

Headline workload: the skewed batch (4000 column-major matrices, 90 % with
M, N, K uniform in [8, 64] and 10 % uniform in [512, 2048], N(0, 1) entries,
alpha = 1, beta = 0), run by one persistent kernel per step from a
CUDA-graph replay.  ``value`` is useful TFLOP/s (sum 2MNK / time) with inputs
resident in HBM; ``e2e`` is the same metric through the one-shot C-ABI call
with host buffers (pinned host -> device copies of A and B, device -> host
copy of C inside the timed region).  The FP32 SIMT form is timed on the same
batch beside the headline mode.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--mode tf32x3|simt|tf32|bf16x3]
  python bench.py --impl reference ...   # the CPU loop on the host cores

N > 1 (torchrun, one rank per GPU) runs independent replicas: matrices of a
batch are independent, so each rank owns a whole batch and no collective
touches the data path (weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "vbatched SGEMM TFLOP/s: 3xTF32 persistent vs FP32-SIMT on GB300 at FP32-level err"
UNIT = "TFLOP/s"


L2_BYTES = 129 * 1000 * 1000
L2_FLUSH_BYTES = 512 << 20


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--mode", default=os.environ.get("BGEMM_BENCH_MODE", "tf32x3"))
    ap.add_argument("--workload", default="skewed_4000")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the other modes")
    ap.add_argument("--no-stream", action="store_true", help="skip the batch-stream leg")
    ap.add_argument("--stream-batches", type=int, default=200)
    return ap.parse_args()


# ------------------------------------------------------------------ dist --
def dist_init(n):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if os.environ.get("BGEMM_BENCH_BACKEND") != "gloo"
                                else "gloo")
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, device):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_tflops(flops_per_rank, ms_per_rank, world, device="cpu"):
    """Replicas: every rank runs the same batch; the job's throughput is all
    ranks' work over the slowest rank's time."""
    ms_max = max_over_ranks(ms_per_rank, world, device)
    return world * flops_per_rank / (ms_max * 1e-3) / 1e12, ms_max


# ---------------------------------------------------------------- clocks --
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        import tempfile
        self.path = os.path.join(tempfile.gettempdir(), "bgemm_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        busy = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def ncu_traffic(mode, workload):
    """DRAM bytes (read + write) of one launch of the dominant kernel, from the
    ncu capture summarised in profiles/ncu_traffic.txt (lines:
    `<mode> <workload> <bytes_per_launch> <how>`); None if not captured."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        p = line.split(None, 3)
        if len(p) >= 3 and p[0] == mode and p[1] == workload:
            try:
                return int(float(p[2]))
            except ValueError:
                return None
    return None


# ------------------------------------------------------------ CPU oracle --
def cpu_sample(w, budget_s=15.0, threads=None):
    """Times the CPU FP32 loop (the oracle port; the reference ships no CPU
    loop) on a bounded sample of the workload's matrices: all threads, whole
    matrices, largest-first pool.  Returns (TFLOP/s, cores, description)."""
    import oracle
    threads = threads or os.cpu_count() or 1
    rng = np.random.default_rng(123)
    order = [int(i) for i in rng.permutation(w.batch)]
    # whole matrices in random order, in chunks of growing size, until the
    # timed CPU work reaches the budget (data generation is not timed)
    fl_total, t_total, n_done, used, pos, chunk = 0.0, 0.0, 0, 1, 0, 8
    while t_total < budget_s and pos < len(order):
        sel = order[pos:pos + chunk]
        pos += len(sel)
        chunk *= 2
        Ms = [w.M[i] for i in sel]
        Ns = [w.N[i] for i in sel]
        Ks = [w.K[i] for i in sel]
        As = [rng.standard_normal(max(m * k, 1)).astype(np.float32) for m, k in zip(Ms, Ks)]
        Bs = [rng.standard_normal(max(k * n, 1)).astype(np.float32) for k, n in zip(Ks, Ns)]
        Cs = [np.zeros(max(m * n, 1), np.float32) for m, n in zip(Ms, Ns)]
        t0 = time.perf_counter()
        used = oracle.vbatched_f32(Ms, Ns, Ks, w.alpha, As, [max(1, m) for m in Ms], Bs,
                                   [max(1, k) for k in Ks], w.beta, Cs, [max(1, m) for m in Ms],
                                   nthreads=threads)
        t_total += time.perf_counter() - t0
        fl_total += sum(2.0 * m * n * k for m, n, k in zip(Ms, Ns, Ks))
        n_done += len(sel)
    rate = fl_total / max(t_total, 1e-9)
    desc = ("%d of %d matrices (%.1f GFLOP, random order, whole matrices), FP32 fma loop, "
            "%d threads, %.1f s timed" % (n_done, w.batch, fl_total / 1e9, used, t_total))
    return rate / 1e12, used, desc


# ---------------------------------------------------------------- GPU leg --
from batchgemm_gb300.accuracy import fp64_sampled_error  # noqa: E402
def gpu_leg(args, rank, world, local):
    import torch
    import batchgemm_gb300 as bg
    from batchgemm_gb300 import workloads
    from batchgemm_gb300.batch import DeviceBatch

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    bg.lib()
    w = workloads.CONFIGS[args.workload](0)
    flops = w.flops()
    db = DeviceBatch(w.M, w.N, w.K, device=str(dev)).fill_fast(w.dist, seed=rank)
    s = torch.cuda.Stream(device=dev)
    peaks = {}
    pk_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk_path):
        peaks = json.load(open(pk_path))
    num_sms = bg.device_info()["num_sms"]
    # inputs smaller than twice the 129 MB L2 get an L2 flush between timed steps
    flush = (torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
             if w.bytes() < 2 * L2_BYTES else None)

    def one_step_error(plan):
        """Error of one execute from a snapshot of C (the timed steps have
        accumulated beta * C into it)."""
        C0 = db.C.clone() if w.beta != 0 else None
        db.execute(plan, w.alpha, w.beta, stream=s)
        s.synchronize()
        return fp64_sampled_error(db, C0=C0, beta=w.beta, alpha=w.alpha)

    def time_mode(mode, steps, warmup, sample_clocks=False, **plan_kw):
        with torch.cuda.stream(s):
            plan = db.plan(mode, stream=s, **plan_kw)
        info = plan.info()
        # warm-up outside the graph, then capture one step
        for _ in range(max(1, min(warmup, 2))):
            db.execute(plan, w.alpha, w.beta, stream=s)
        s.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            db.execute(plan, w.alpha, w.beta, stream=s)
        with torch.cuda.stream(s):
            for _ in range(warmup):
                g.replay()
        s.synchronize()
        barrier(world)
        torch.cuda.synchronize(dev)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        clk = ClockSampler(local) if sample_clocks else None
        if clk:
            clk.__enter__()
            time.sleep(0.3)
        with torch.cuda.stream(s):
            if flush is None:
                ev0.record(s)
                for _ in range(steps):
                    g.replay()
                ev1.record(s)
            else:
                # inputs that fit in L2: a buffer larger than L2 is written
                # before every step, outside that step's events
                step_evs = []
                for _ in range(steps):
                    flush.zero_()
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(s)
                    g.replay()
                    b.record(s)
                    step_evs.append((a, b))
        s.synchronize()
        if clk:
            clk.__exit__(None, None, None)
        torch.cuda.synchronize(dev)
        barrier(world)
        if flush is None:
            ms = ev0.elapsed_time(ev1) / steps
        else:
            ms = sum(a.elapsed_time(b) for a, b in step_evs) / steps
        plan.check_device(stream=s)
        del g
        return plan, info, ms, (clk.summary() if clk else None)

    out = {}
    if args.mode in ("tf32", "tf32x3"):
        # the TF32 tensor rate of this GPU, measured before the timed region
        from batchgemm_gb300 import peaks as peaks_mod
        out["tf32_peak"] = peaks_mod.tf32_burst()
        torch.cuda.empty_cache()
    if args.mode in ("tf32", "tf32x3", "bf16x3"):
        # the HBM ceiling of the pre-pass's read:write mix (3xTF32: read 4 B,
        # write 8 B per element; TF32 and 3xBF16: read 4, write 4)
        from batchgemm_gb300 import peaks as peaks_mod
        out["pre_pass_mix"] = "read1_write2" if args.mode == "tf32x3" else "copy"
        out["pre_pass_peak"] = peaks_mod.hbm_mix(kinds=(0 if args.mode == "tf32x3" else 1,),
                                                 gib=1.0)[out["pre_pass_mix"]]
    plan, info, ms, clocks = time_mode(args.mode, args.steps, args.warmup, sample_clocks=True)
    value, ms_max = whole_job_tflops(flops, ms, world, dev)
    err_max, err_mean, nsamp = one_step_error(plan)
    out.update(value=value, ms=ms_max, info=info, clocks=clocks, err=(err_max, err_mean, nsamp),
               launches=info["kernels_per_execute"] * args.steps)
    # the dominant (GEMM) kernel alone: events recorded by the library around
    # its launch, on the stream it is launched on, over `steps` executes
    evs = []
    for _ in range(args.steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(s)
        b.record(s)
        evs.append((a, b))
    s.synchronize()
    with torch.cuda.stream(s):
        for a, b in evs:
            if flush is not None:
                flush.zero_()
            plan.set_kernel_events(a, b)
            db.execute(plan, w.alpha, w.beta, stream=s)
    s.synchronize()
    plan.set_kernel_events(None, None)
    out["kernel_ms"] = sum(a.elapsed_time(b) for a, b in evs) / len(evs)
    if args.mode != "simt":
        # load balance of the GEMM's static tile schedule: every persistent
        # CTA stamps the global timer when it starts and when it finishes
        stamps = torch.zeros(2 * info["grid"], dtype=torch.int64, device=dev)
        plan.set_cta_timer(stamps.data_ptr())
        with torch.cuda.stream(s):
            db.execute(plan, w.alpha, w.beta, stream=s)
        s.synchronize()
        plan.set_cta_timer(None)
        t = stamps.view(-1, 2).cpu().numpy().astype(np.float64)
        span = t[:, 1].max() - t[:, 0].min()
        out["cta_balance"] = {
            "span_us": round(span / 1e3, 1),
            "finish_spread_us": round((t[:, 1].max() - t[:, 1].min()) / 1e3, 1),
            "mean_busy_frac": round(float((t[:, 1] - t[:, 0]).mean() / span), 4),
            "how": "global-timer stamps of every persistent CTA at start and end of one GEMM "
                   "launch (bgemm_plan_set_cta_timer)"}
    plan.close()

    # other modes on the same batch (a few steps each)
    extra = {}
    if not args.no_extra:
        for mode in ("simt", "tf32x3", "tf32", "bf16x3"):
            if mode == args.mode:
                continue
            try:
                p2, inf2, ms2, _ = time_mode(mode, max(3, args.steps // 4), 3)
                e2 = one_step_error(p2)
                extra[mode] = {"tflops": round(flops / (ms2 * 1e-3) / 1e12, 3),
                               "ms_per_step": round(ms2, 4),
                               "err_vs_fp64_max": e2[0], "err_vs_fp64_mean": e2[1]}
                p2.close()
            except bg.BgemmError as e:
                extra[mode] = {"unavailable": e.message}
        # mixed plan: matrices with min(M, N, K) < 64 on the FP32 SIMT kernel,
        # the rest in 3xTF32 (two GEMM kernels per execute)
        try:
            p2, inf2, ms2, _ = time_mode("tf32x3", max(3, args.steps // 4), 3, simt_below=64)
            e2 = one_step_error(p2)
            extra["tf32x3_mixed_simt_below_64"] = {
                "tflops": round(flops / (ms2 * 1e-3) / 1e12, 3), "ms_per_step": round(ms2, 4),
                "err_vs_fp64_max": e2[0], "err_vs_fp64_mean": e2[1],
                "kernels_per_execute": inf2["kernels_per_execute"]}
            p2.close()
        except bg.BgemmError as e:
            extra["tf32x3_mixed_simt_below_64"] = {"unavailable": e.message}
        # the same batch through the device-size entry (sizes and pointers in
        # device arrays, tile queue / workspace / tensor maps built on the
        # device; C += A B, so C is read as well), one captured call per step
        dM, dN, dK = (torch.tensor(v, dtype=torch.int32, device=dev) for v in (w.M, w.N, w.K))
        max_dim, max_k = max(max(w.M), max(w.N)), max(w.K)
        elems = sum((m + n) * k for m, n, k in zip(w.M, w.N, w.K))
        fw_args = (dM.data_ptr(), dN.data_ptr(), dK.data_ptr(), db.pA.data_ptr(),
                   db.pB.data_ptr(), db.pC.data_ptr(), w.batch, max_dim, max_k, args.mode)
        with torch.cuda.stream(s):
            bg.framework_gemm_mode(*fw_args, stream=s, max_operand_elems=elems)
        s.synchronize()
        bg.framework_check_device(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            bg.framework_gemm_mode(*fw_args, stream=s, max_operand_elems=elems)
        fw_steps = max(3, args.steps // 4)
        fw_evs = []
        with torch.cuda.stream(s):
            for _ in range(3):
                g.replay()
            for _ in range(fw_steps):
                if flush is not None:
                    flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(s)
                g.replay()
                b.record(s)
                fw_evs.append((a, b))
        s.synchronize()
        bg.framework_check_device(s)
        fw_ms = sum(a.elapsed_time(b) for a, b in fw_evs) / fw_steps
        extra["device_sizes_" + args.mode] = {
            "api": "bgemm_framework_gemm_mode (C += A B, sizes on the device)",
            "tflops": round(flops / (fw_ms * 1e-3) / 1e12, 3), "ms_per_step": round(fw_ms, 4)}
        del g
        bg.framework_release()
    out["extra"] = extra

    # roofline of the dominant kernel: algorithmic flops of one launch over its
    # own CUDA-event duration (pack pre-pass excluded; it is HBM-bound and
    # reported separately as pre_pass_ms)
    mode = args.mode
    kms = out["kernel_ms"]
    clk_max = (clocks or {}).get("sm_max_mhz") or 2070.0
    traffic = ncu_traffic(mode, w.name)
    if mode == "simt":
        peak = num_sms * 128 * 2 * clk_max * 1e6 / 1e12
        ach = flops / (kms * 1e-3) / 1e12
        out["roofline"] = {"bound": "fp32_simt", "achieved": round(ach, 3),
                           "peak": round(peak, 2), "unit": "TFLOP/s",
                           "frac": round(ach / peak, 4), "traffic": traffic,
                           "kernel": "simt_persistent_kernel", "kernel_ms": round(kms, 4),
                           "algorithmic_flops_per_launch": flops,
                           "peak_source": "SMs x 128 FP32 lanes x 2 x max SM clock (device "
                                          "properties; MEASURED_PEAKS.json has no FP32 figure)"}
    else:
        mult = 3.0 if mode in ("tf32x3", "bf16x3") else 1.0
        if mode == "bf16x3":
            pipe_peak = peaks.get("bf16_tflops", 1900.0)
            src = ("of measured bf16 dense (MEASURED_PEAKS.json, cuBLAS bf16 8192^3, burst)"
                   if "bf16_tflops" in peaks else "of fallback bf16 dense 1.9 PFLOP/s")
        else:
            pipe_peak = out["tf32_peak"]
            src = ("of measured TF32 dense: cuBLAS TF32 GEMM 8192^3 (torch.matmul, FP32 "
                   "operands, TF32 allowed), best of 10 by CUDA events, measured in this run "
                   "before the timed region (batchgemm_gb300.peaks.tf32_burst)")
        ach = mult * flops / (kms * 1e-3) / 1e12
        step_ms = out["ms"]
        pre_ms = step_ms - kms
        pre_traffic = ncu_traffic(mode + "_pre_pass", w.name)
        out["roofline"] = {"bound": "tensor", "achieved": round(ach, 2),
                           "peak": round(pipe_peak, 1), "unit": "TFLOP/s",
                           "frac": round(ach / pipe_peak, 4), "traffic": traffic,
                           "kernel": "tc2_gemm_kernel / tc_gemm_kernel", "kernel_ms": round(kms, 4),
                           "pre_pass_ms": round(pre_ms, 4),
                           "algorithmic_flops_per_launch": mult * flops,
                           "peak_source": src + ("; achieved counts the 3 tensor products"
                                                 if mult > 1 else ""),
                           # the whole step (pre-pass + GEMM) against the same pipe:
                           # useful flops over (peak / products)
                           "step_frac": round(mult * flops / (step_ms * 1e-3) / 1e12 / pipe_peak,
                                              4),
                           "step_dram_bytes": (traffic + pre_traffic
                                               if traffic and pre_traffic else None),
                           "pre_pass_traffic": pre_traffic}
        elems = float(sum(m * k + k * n for m, n, k in zip(w.M, w.N, w.K)))
        pre_bytes = elems * (4 + {"tf32": 4, "tf32x3": 8, "bf16x3": 4}[mode])
        pre_ach = pre_bytes / (pre_ms * 1e-3) / 1e9
        out["roofline"]["pre_pass"] = {
            "bound": "hbm", "achieved": round(pre_ach, 1), "peak": out["pre_pass_peak"],
            "unit": "GB/s", "frac": round(pre_ach / out["pre_pass_peak"], 4),
            "algorithmic_bytes": pre_bytes,
            "peak_source": "measured in this run before the timed region: the library's float4 "
                           "streaming probe (bgemm_debug_hbm_probe) with the pre-pass's mix (%s), "
                           "1 GiB buffers, best of two grids" % out["pre_pass_mix"]}
        if mode != "bf16x3" and "bf16_tflops" in peaks:
            out["roofline"]["bf16_measured_tflops"] = peaks["bf16_tflops"]
        if "cta_balance" in out:
            out["roofline"]["cta_balance"] = out["cta_balance"]

    # end to end through the one-shot C-ABI call with host buffers.  Every
    # step copies its inputs in from pinned host memory, runs
    # bgemm_sgemm_vbatched and copies C out.  Steps are pipelined the way a
    # serving loop would run them: two device copies of the batch, one stream
    # each for copy-in, compute and copy-out, so step i+1's copy-in and step
    # i-1's copy-out overlap step i's compute (C2C is full duplex).
    if not args.no_e2e:
        hA = torch.empty(db.A.numel(), dtype=torch.float32, pin_memory=True)
        hB = torch.empty(db.B.numel(), dtype=torch.float32, pin_memory=True)
        hA.copy_(db.A)
        hB.copy_(db.B)
        hCin = torch.empty(db.C.numel(), dtype=torch.float32, pin_memory=True)
        hCin.copy_(db.C)
        hC = [torch.empty(db.C.numel(), dtype=torch.float32, pin_memory=True) for _ in range(2)]
        dbs = [db, DeviceBatch(w.M, w.N, w.K, device=str(dev))]
        s_in = torch.cuda.Stream(device=dev)
        s_out = torch.cuda.Stream(device=dev)
        h2d = (hA.numel() + hB.numel()) * 4
        if w.beta != 0:
            h2d += hCin.numel() * 4
        d2h = db.C.numel() * 4
        ev = {k: [torch.cuda.Event() for _ in range(2)] for k in ("in", "run", "out")}
        started = [False, False]

        def e2e_step(i):
            j = i % 2
            d = dbs[j]
            with torch.cuda.stream(s_in):
                if started[j]:  # buffers of step i-2 are free once it was copied out
                    s_in.wait_event(ev["out"][j])
                d.A.copy_(hA, non_blocking=True)
                d.B.copy_(hB, non_blocking=True)
                if w.beta != 0:
                    d.C.copy_(hCin, non_blocking=True)
                ev["in"][j].record(s_in)
            with torch.cuda.stream(s):
                s.wait_event(ev["in"][j])
                d.run(mode, w.alpha, w.beta, stream=s)
                ev["run"][j].record(s)
            with torch.cuda.stream(s_out):
                s_out.wait_event(ev["run"][j])
                hC[j].copy_(d.C, non_blocking=True)
                ev["out"][j].record(s_out)
            started[j] = True

        for i in range(2):
            e2e_step(i)
        torch.cuda.synchronize(dev)
        barrier(world)
        esteps = max(4, args.steps // 2)
        t0 = time.perf_counter()
        for i in range(esteps):
            e2e_step(i)
        torch.cuda.synchronize(dev)
        ems = (time.perf_counter() - t0) * 1e3 / esteps
        barrier(world)
        ems = max_over_ranks(ems, world, dev)
        out["e2e"] = {"value": round(world * flops / (ems * 1e-3) / 1e12, 4), "unit": UNIT,
                      "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                      "ms_per_step": round(ems, 3),
                      "api": "bgemm_sgemm_vbatched; pinned host buffers; copy-in, compute and "
                             "copy-out on three streams, two device copies (steps pipelined)",
                      "timing": "host wall clock over %d steps after 2 warm-up steps, device "
                                "synchronised before and after" % esteps}
        del dbs[1]
    if not args.no_stream:
        out["stream"] = stream_leg(args, dev, s)
    return w, out


# ------------------------------------------------------------ stream leg --
def stream_leg(args, dev, s):
    """The batch stream: successive batches (64..1024 matrices each, M, N, K
    log-uniform in [1, 4096], U[-1, 1] entries, alpha = beta = 1).  One plan
    per mode, created with the element-wise maximum of every batch's
    requirements as capacity; its execute is captured once in a CUDA graph,
    and each batch is uploaded with bgemm_plan_update (host planning of batch
    b+1 overlaps the GPU running batch b) before one graph replay.  Reports
    per-batch device latency (upload + kernels, CUDA events) p50/p99 and the
    aggregate useful TFLOP/s over the whole stream."""
    import types
    import torch
    import batchgemm_gb300 as bg
    from batchgemm_gb300 import workloads

    bs = workloads.stream_batches(0, args.stream_batches)
    nb = len(bs)
    al = lambda x: (x + 3) // 4 * 4  # 16-byte aligned starts
    dims = {"A": lambda w: zip(w.M, w.K), "B": lambda w: zip(w.K, w.N),
            "C": lambda w: zip(w.M, w.N)}
    # operand pools twice the largest batch; matrices are laid out from a
    # cursor that keeps moving (wrapping) across batches, so consecutive
    # batches touch different memory and no batch reads the previous one's
    # operands out of L2
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    pools, offs = {}, {}
    for key in "ABC":
        sizes = [[al(r * c) for r, c in dims[key](w)] for w in bs]
        pool_n = 2 * max(sum(v) for v in sizes) + 64
        cur, o_all = 0, []
        for v in sizes:
            o = []
            for n in v:
                if cur + n > pool_n:
                    cur = 0
                o.append(cur)
                cur += n
            o_all.append(o)
        offs[key] = o_all
        pools[key] = torch.empty(pool_n, dtype=torch.float32, device=dev).uniform_(
            -1, 1, generator=g)
    cap_batch = max(w.batch for w in bs)
    ptr_host = torch.zeros((nb, 3, cap_batch), dtype=torch.int64, pin_memory=True)
    for b, w in enumerate(bs):
        for j, key in enumerate("ABC"):
            base = pools[key].data_ptr()
            ptr_host[b, j, :w.batch] = torch.tensor([base + 4 * o for o in offs[key][b]],
                                                    dtype=torch.int64)
    arrs = []
    for w in bs:
        lda = [max(1, m) for m in w.M]
        ldb = [max(1, k) for k in w.K]
        arrs.append(tuple(bg.int_array(v) for v in (w.M, w.N, w.K, lda, ldb, lda)))
    flops = [w.flops() for w in bs]

    def run(mode, simt_below=0):
        opts = {"kernel_family": "pair"} if mode in ("tf32x3", "bf16x3") else {}
        if simt_below:
            opts["simt_below"] = simt_below
        t0 = time.perf_counter()
        reqs = [bg.plan_requirements(*arrs[b], mode=mode, **opts) for b in range(nb)]
        req_ms = (time.perf_counter() - t0) * 1e3 / nb
        cap = bg.max_requirements(reqs)
        ptr_dev = torch.zeros((3, cap_batch), dtype=torch.int64, device=dev)
        pA, pB, pC = (ptr_dev[j].data_ptr() for j in range(3))
        with torch.cuda.stream(s):
            plan = bg.Plan(*arrs[0], mode=mode, stream=s, capacity=cap, **opts)
            for b in range(3):  # warm-up outside the graph
                ptr_dev.copy_(ptr_host[b], non_blocking=True)
                plan.update(*arrs[b], stream=s)
                plan.execute(1.0, pA, pB, 1.0, pC, stream=s)
        s.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=s):
            plan.execute(1.0, pA, pB, 1.0, pC, stream=s)
        mk = lambda: torch.cuda.Event(enable_timing=True)
        evs = [(mk(), mk(), mk()) for _ in range(nb)]
        host_ms = []
        torch.cuda.synchronize(dev)
        with torch.cuda.stream(s):
            for b in range(nb):
                evs[b][0].record(s)
                ptr_dev.copy_(ptr_host[b], non_blocking=True)
                t0 = time.perf_counter()
                plan.update(*arrs[b], stream=s)
                host_ms.append((time.perf_counter() - t0) * 1e3)
                evs[b][1].record(s)  # uploads enqueued: the GPU part starts here
                graph.replay()
                evs[b][2].record(s)
        s.synchronize()
        plan.check_device(stream=s)
        lat = sorted(a.elapsed_time(c) for a, _, c in evs)
        gpu = sorted(r.elapsed_time(c) for _, r, c in evs)
        total_ms = evs[0][0].elapsed_time(evs[-1][2])
        # accuracy of the last batch, run again from a snapshot of C
        b = nb - 1
        w = bs[b]
        C0 = pools["C"].clone()
        with torch.cuda.stream(s):
            ptr_dev.copy_(ptr_host[b], non_blocking=True)
            plan.update(*arrs[b], stream=s)
            graph.replay()
        s.synchronize()
        view = types.SimpleNamespace(
            batch=w.batch, M=w.M, N=w.N, K=w.K, lda=[max(1, m) for m in w.M],
            ldb=[max(1, k) for k in w.K], ldc=[max(1, m) for m in w.M], offA=offs["A"][b],
            offB=offs["B"][b], offC=offs["C"][b], A=pools["A"], B=pools["B"], C=pools["C"])
        e_max, e_mean, n_s = fp64_sampled_error(view, per_matrix=2, C0=C0, beta=1.0)
        # and of ten more batches (each from a snapshot of C)
        errs = [(e_mean, e_max, n_s)]
        for b in range(max(0, nb - 11), nb - 1):
            w = bs[b]
            C0.copy_(pools["C"])
            with torch.cuda.stream(s):
                ptr_dev.copy_(ptr_host[b], non_blocking=True)
                plan.update(*arrs[b], stream=s)
                graph.replay()
            s.synchronize()
            view = types.SimpleNamespace(
                batch=w.batch, M=w.M, N=w.N, K=w.K, lda=[max(1, m) for m in w.M],
                ldb=[max(1, k) for k in w.K], ldc=[max(1, m) for m in w.M], offA=offs["A"][b],
                offB=offs["B"][b], offC=offs["C"][b], A=pools["A"], B=pools["B"], C=pools["C"])
            mx, mn, n_b = fp64_sampled_error(view, per_matrix=2, C0=C0, beta=1.0, seed=b)
            errs.append((mn, mx, n_b))
        n_all = sum(e[2] for e in errs)
        err_batches = {"batches": len(errs), "samples": n_all,
                       "mean": sum(e[0] * e[2] for e in errs) / max(n_all, 1),
                       "max": max(e[1] for e in errs)}
        del C0, graph
        info = plan.info()
        plan.close()
        pct = lambda q: lat[min(len(lat) - 1, int(round(q * (len(lat) - 1))))]
        gpct = lambda q: gpu[min(len(gpu) - 1, int(round(q * (len(gpu) - 1))))]
        return {"tflops": round(sum(flops) / (total_ms * 1e-3) / 1e12, 3),
                "total_ms": round(total_ms, 2),
                "latency_ms_p50": round(pct(0.50), 4), "latency_ms_p99": round(pct(0.99), 4),
                "latency_ms_max": round(lat[-1], 4),
                "gpu_replay_ms_p50": round(gpct(0.50), 4),
                "gpu_replay_ms_p99": round(gpct(0.99), 4),
                "gpu_replay_ms_sum": round(sum(gpu), 2),
                "host_update_ms_p50": round(statistics.median(host_ms), 4),
                "host_requirements_ms_mean": round(req_ms, 4),
                "kernels_per_batch": info["kernels_per_execute"] + (0 if mode == "simt" else 1),
                "capacity": cap,
                "err_vs_fp64_last_batch": {"max": e_max, "mean": e_mean, "samples": n_s},
                "err_vs_fp64_batches": err_batches}

    def run_device_sizes(mode):
        """The same stream through bgemm_framework_gemm_mode: per batch only the
        size and pointer arrays are copied to the device (padded to the
        largest batch with empty matrices) and one captured call replays; the
        tile choice, queue, split operands and tensor maps are built on the
        device, so there is no host planning at all."""
        cap = max(w.batch for w in bs)
        sz_host = torch.zeros((nb, 3, cap), dtype=torch.int32, pin_memory=True)
        for b, w in enumerate(bs):
            for j, v in enumerate((w.M, w.N, w.K)):
                sz_host[b, j, :w.batch] = torch.tensor(v, dtype=torch.int32)
        sz_dev = torch.zeros((3, cap), dtype=torch.int32, device=dev)
        ptr_dev = torch.zeros((3, cap_batch), dtype=torch.int64, device=dev)
        max_dim = max(max(max(w.M), max(w.N)) for w in bs)
        max_k = max(max(w.K) for w in bs)
        elems = max(sum((m + n) * k for m, n, k in zip(w.M, w.N, w.K)) for w in bs)
        fw = (sz_dev[0].data_ptr(), sz_dev[1].data_ptr(), sz_dev[2].data_ptr(),
              ptr_dev[0].data_ptr(), ptr_dev[1].data_ptr(), ptr_dev[2].data_ptr(), cap,
              max_dim, max_k)

        def upload(b):
            sz_dev.copy_(sz_host[b], non_blocking=True)
            ptr_dev.copy_(ptr_host[b], non_blocking=True)

        with torch.cuda.stream(s):
            for b in range(3):
                upload(b)
                bg.framework_gemm_mode(*fw, mode=mode, stream=s, max_operand_elems=elems)
        s.synchronize()
        bg.framework_check_device(s)
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=s):
            bg.framework_gemm_mode(*fw, mode=mode, stream=s, max_operand_elems=elems)
        mk = lambda: torch.cuda.Event(enable_timing=True)
        evs = [(mk(), mk(), mk()) for _ in range(nb)]
        torch.cuda.synchronize(dev)
        with torch.cuda.stream(s):
            for b in range(nb):
                evs[b][0].record(s)
                upload(b)
                evs[b][1].record(s)
                graph.replay()
                evs[b][2].record(s)
        s.synchronize()
        bg.framework_check_device(s)
        lat = sorted(a.elapsed_time(c) for a, _, c in evs)
        gpu = sorted(r.elapsed_time(c) for _, r, c in evs)
        total_ms = evs[0][0].elapsed_time(evs[-1][2])
        del graph
        bg.framework_release()
        pct = lambda v, q: v[min(len(v) - 1, int(round(q * (len(v) - 1))))]
        return {"api": "bgemm_framework_gemm_mode (device size arrays, C += A B)",
                "tflops": round(sum(flops) / (total_ms * 1e-3) / 1e12, 3),
                "total_ms": round(total_ms, 2),
                "latency_ms_p50": round(pct(lat, 0.5), 4),
                "latency_ms_p99": round(pct(lat, 0.99), 4),
                "gpu_replay_ms_p50": round(pct(gpu, 0.5), 4),
                "gpu_replay_ms_p99": round(pct(gpu, 0.99), 4),
                "host_planning_ms": 0.0,
                "bounds": {"batch": cap, "max_dim": max_dim, "max_k": max_k,
                           "max_operand_elems": elems}}

    out = {"workload": "stream_%d: %d successive batches, U{64..1024} matrices each, M, N, K "
                       "log-uniform in [1, 4096], U[-1,1], alpha = beta = 1" % (nb, nb),
           "useful_tflop_total": round(sum(flops) / 1e12, 3),
           "per_batch_gflop_p50": round(statistics.median(flops) / 1e9, 2),
           "timing": "per batch: CUDA events on the launching stream before the pointer "
                     "upload, after bgemm_plan_update's uploads (gpu_replay = from there to "
                     "the end of the graph replay: GPU work only) and after the replay "
                     "(latency); host_update = wall time of bgemm_plan_update on the host "
                     "(planning plus any wait for a staging buffer), host_requirements = "
                     "host planning alone; aggregate = all batches / first start to last "
                     "stop; operands rotate through pools twice the largest batch (no L2 "
                     "reuse between batches)"}
    for mode in (args.mode, "simt") if args.mode != "simt" else ("simt",):
        try:
            out[mode] = run(mode)
        except bg.BgemmError as e:
            out[mode] = {"unavailable": e.message}
        torch.cuda.empty_cache()
        if mode != "simt":
            # mixed plan: min(M, N, K) < 64 on FP32 SIMT, the rest on tensor cores
            try:
                out[mode + "_mixed_simt_below_64"] = run(mode, simt_below=64)
            except bg.BgemmError as e:
                out[mode + "_mixed_simt_below_64"] = {"unavailable": e.message}
        torch.cuda.empty_cache()
        try:
            out["device_sizes_" + mode] = run_device_sizes(mode)
        except bg.BgemmError as e:
            out["device_sizes_" + mode] = {"unavailable": e.message}
        torch.cuda.empty_cache()
    if args.mode != "simt" and "tflops" in out.get(args.mode, {}) and \
            "tflops" in out.get("simt", {}):
        out["ratio_vs_simt"] = round(out[args.mode]["tflops"] / out["simt"]["tflops"], 3)
        a, b = out.get("device_sizes_" + args.mode, {}), out.get("device_sizes_simt", {})
        if "tflops" in a and "tflops" in b:
            out["ratio_vs_simt_device_sizes"] = round(a["tflops"] / b["tflops"], 3)
        m = out.get(args.mode + "_mixed_simt_below_64", {})
        if "tflops" in m:
            out["ratio_vs_simt_mixed"] = round(m["tflops"] / out["simt"]["tflops"], 3)
    for key in list(pools):
        del pools[key]
    return out


def main():
    args = parse()
    rank, world, local = dist_init(args.gpus)
    from batchgemm_gb300 import workloads
    w = workloads.CONFIGS[args.workload](0)
    config = {"workload": w.name, "desc": w.desc, "batch": w.batch,
              "useful_gflop_per_step": round(w.flops() / 1e9, 3),
              "mode": args.mode if args.impl == "ours" else "fp32 CPU loop",
              "l2": ("inputs (%.1f GB) larger than the 129 MB L2; no flush" % (w.bytes() / 1e9)
                     if w.bytes() >= 2 * L2_BYTES else
                     "inputs (%.3f GB) fit in the 129 MB L2: %d MB written before every timed "
                     "step, outside its CUDA events" % (w.bytes() / 1e9, L2_FLUSH_BYTES >> 20)),
              "parallelism": "replicas x%d" % world}

    if args.impl == "reference":
        # the reference ships no CPU implementation; its stand-in is the CPU
        # restatement of its fma loop (oracle/), timed on the host cores.
        if rank != 0:
            return
        vals = []
        desc = ""
        cores = 0
        # warm-up: the same loop, untimed, on a short sample (thread pool,
        # page-in of the oracle library and of the generated operands)
        for _ in range(args.warmup):
            cpu_sample(w, budget_s=0.5)
        steps = max(1, min(args.steps, 3))
        for _ in range(steps):
            v, cores, desc = cpu_sample(w, budget_s=8.0)
            vals.append(v)
        value = statistics.median(vals)
        line = {"metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": world,
                "steps": steps, "warmup": args.warmup, "ms_per_step": round(
                    w.flops() / (value * 1e12) * 1e3, 3), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "impl": "reference", "config": config,
                "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": cores,
                                 "kind": "port", "sample": desc},
                "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return

    w, out = gpu_leg(args, rank, world, local)
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu:
        v, cores, desc = cpu_sample(w, budget_s=12.0)
        cpu = {"value": round(v, 6), "unit": UNIT, "cores": cores, "kind": "port", "sample": desc}
    dtype = {"simt": "f32", "tf32": "tf32", "tf32x3": "tf32x3 (f32 in/out)",
             "bf16x3": "bf16x3 (f32 in/out)"}[args.mode]
    line = {
        "metric": METRIC, "value": round(out["value"], 4), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(out["ms"], 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": dtype,
        "data": "synthetic (seeded on device)", "config": config,
        "roofline": out["roofline"], "cpu_baseline": cpu, "clocks": out["clocks"],
        "gpu_launches": out["launches"],
        "err_vs_fp64": {"max": out["err"][0], "mean": out["err"][1], "samples": out["err"][2],
                        "normalised_by": "sum_k |a_mk b_kn|"},
        "plan": {"tiles": out["info"]["num_tiles"], "grid": out["info"]["grid"],
                 "cfg_hist": out["info"]["tile_config_hist"]},
        "other_modes": out["extra"],
    }
    if "e2e" in out:
        line["e2e"] = out["e2e"]
    if "stream" in out:
        line["stream"] = out["stream"]
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
