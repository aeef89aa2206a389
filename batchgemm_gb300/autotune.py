"""Autotuner of the planners' tile cost table and of the tensor-core
promotion schedule.

Tile costs.  For every mode and every tile configuration it runs uniform
batches whose matrices are whole multiples of the tile (several waves of
persistent CTAs), at several K, with the configuration forced and the
rebalance off; the time of one tile, t = a + b*K, is fitted by least squares.

Promotion schedule (--schedule).  The split modes on CTA pairs accumulate a
group of 128-byte K slices in tensor memory before the epilogue promotes the
group into FP32 registers; longer groups drain tensor memory less often
(faster) but let the tensor core's truncating accumulation run longer (less
accurate).  For each bucket of K (K <= 64, then one octave per bucket) and
each candidate group length (0 = promote every MMA and keep lo*lo) it times
the GEMM kernel on 24 matrices of 1024 x 1024 x K (N(0, 1) entries) and
measures the normalised error against FP64 on fixed samples, next to the FP32
SIMT path's error on the same samples.  It keeps the fastest group whose mean
and maximum error are both no worse than FP32 SIMT's (3xBF16, whose split
error is far above FP32's: the fastest within 2 % of its most accurate
group's mean).

Compile-time parameters (--build-params).  Two schedule constants are
template arguments of the kernels: the SIMT kernel's cp.async ring cap (a
small tile takes as many 16-k stages as the CTA's shared memory holds, up to
the cap) and the CTA-pair kernel's C-prefetch lead for beta != 0.  For each
candidate the table is rewritten, the library rebuilt, and a child process
times the workloads the parameter affects (ring: the plain 256-matrix batch,
the 2048-matrix log-uniform batch and eight stream batches on SIMT; lead: the
2048-matrix batch and eight stream batches in 3xTF32, both beta != 0); the
candidate with the least geometric-mean time is kept,
one parameter after the other.

All results are written to ``csrc/tile_table_tuned.inc``, which the library
compiles in place of the analytic defaults of ``csrc/tile_table.h``; what a
run does not measure is copied from the library's current tables.

  python -m batchgemm_gb300.autotune                     # tile costs, print
  python -m batchgemm_gb300.autotune --write             # ... and write
  python -m batchgemm_gb300.autotune --schedule --write  # schedule, write
  python -m batchgemm_gb300.autotune --build-params      # rebuild per candidate, write

The split/pack pre-pass of the tensor-core modes does not depend on the tile
configuration; its time is estimated from its bytes (read 4 B, write 4 or 8
B per element at the device's copy bandwidth) and removed before fitting.
"""
from __future__ import annotations

import argparse
import datetime
import json
import math
import os
import subprocess
import sys

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(PKG))

SIMT_CFGS = [(16, 16), (32, 32), (64, 32), (32, 64), (64, 64), (128, 64), (64, 128), (128, 128),
             (8, 128), (128, 8)]
MODE_IDS = {"tf32": 1, "tf32x3": 2, "bf16x3": 3}


def tc_dims(cfg):
    """(A-side rows, B-side rows, swap, pair) of a tensor-core tile configuration."""
    pair = cfg >= 8
    bn = (64 << (cfg & 3)) if pair else (16 << (cfg & 3))
    return (256 if pair else 128), bn, bool(cfg & 4), pair


def valid_tc(mode, cfg):
    if cfg >= 8:
        return (cfg & 3) != 3
    return True


def measure(mode, cfg, K, slots, waves=6, reps=5, hbm_gbs=6000.0):
    import torch
    from batchgemm_gb300.batch import DeviceBatch
    if mode == "simt":
        bm, bn = SIMT_CFGS[cfg]
        swap = False
    else:
        bm, bn, swap, _ = tc_dims(cfg)
    # matrices of ta x tb tiles; enough of them for `waves` waves
    ta = max(1, min(8, 1024 // bm))
    tb = max(1, min(8, 1024 // bn))
    tiles_per = ta * tb
    n = max(1, -(-waves * slots // tiles_per))
    ra, rb = bm * ta, bn * tb
    M, N = (rb, ra) if swap else (ra, rb)
    db = DeviceBatch([M] * n, [N] * n, [K] * n).fill_fast("normal", 0)
    with db.plan(mode, force_tile_config=cfg, rebalance=False) as p:
        info = p.info()
        assert info["num_tiles"] == n * tiles_per, (info["num_tiles"], n * tiles_per)
        for _ in range(2):
            db.execute(p, 1.0, 0.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            db.execute(p, 1.0, 0.0)
        e1.record()
        torch.cuda.synchronize()
        p.check_device()
        ms = e0.elapsed_time(e1) / reps
        grid = info["grid"]
    t_gemm_ns = ms * 1e6
    if mode != "simt":
        elems = n * (M * K + N * K)
        wbytes = {"tf32": 4, "tf32x3": 8, "bf16x3": 4}[mode]
        t_pack_ns = elems * (4 + wbytes) / (hbm_gbs * 1e9) * 1e9
        t_gemm_ns = max(t_gemm_ns - t_pack_ns, 0.05 * t_gemm_ns)
    lanes = grid // 2 if (mode != "simt" and cfg >= 8) else grid
    per_tile = t_gemm_ns * lanes / (n * tiles_per)
    del db
    return per_tile, ms


def fit(Ks, ts):
    A = np.vstack([np.ones(len(Ks)), np.array(Ks, float)]).T
    w = 1.0 / np.array(ts)  # relative error weighting
    sol, *_ = np.linalg.lstsq(A * w[:, None], np.array(ts) * w, rcond=None)
    a, b = float(sol[0]), float(sol[1])
    return max(a, 50.0), max(b, 1e-3)


SCHED_BUCKET_K = [48, 96, 192, 384, 768, 1536, 3072, 6144]  # one K per bucket
SCHED_CANDIDATES = [0, 1, 2, 3, 4, 6, 8]


def sched_measure(mode, K, group, n=24, size=1024, reps=5, samples=128):
    """GEMM-kernel time (ms, best of reps) and sampled errors (numpy) of one
    promotion group length on n matrices of size x size x K."""
    import ctypes
    import torch
    import batchgemm_gb300 as bg
    from batchgemm_gb300.accuracy import fp64_sampled_error
    from batchgemm_gb300.batch import DeviceBatch
    L = bg.lib()
    mid = MODE_IDS[mode]
    prev = (ctypes.c_int * 8)()
    L.bgemm_debug_get_tc_schedule(mid, prev)
    g = list(prev)
    g[_bucket(K)] = group
    assert L.bgemm_debug_set_tc_schedule(mid, (ctypes.c_int * 8)(*g)) == 0
    try:
        db = DeviceBatch([size] * n, [size] * n, [K] * n).fill_fast("normal", 0)
        best = float("inf")
        with db.plan(mode, kernel_family="pair") as p:
            for _ in range(2):
                db.execute(p, 1.0, 0.0)
            torch.cuda.synchronize()
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                e1.record()
                p.set_kernel_events(e0, e1)
                db.execute(p, 1.0, 0.0)
                e1.synchronize()
                best = min(best, e0.elapsed_time(e1))
            p.set_kernel_events(None, None)
            p.check_device()
        err, _ = fp64_sampled_error(db, per_matrix=samples, seed=7, samples=True)
        db.C.zero_()
        with db.plan("simt") as ps:
            db.execute(ps, 1.0, 0.0)
        torch.cuda.synchronize()
        serr, _ = fp64_sampled_error(db, per_matrix=samples, seed=7, samples=True)
        del db
        torch.cuda.empty_cache()
        return best, err, serr
    finally:
        L.bgemm_debug_set_tc_schedule(mid, (ctypes.c_int * 8)(*list(prev)))


def _bucket(K):
    if K <= 64:
        return 0
    b, v = 0, (K - 1) >> 6
    while v > 1:
        v >>= 1
        b += 1
    return min(b + 1, 7)


def sweep_schedule(modes):
    """Per mode and bucket of K: the fastest group length within the error bar."""
    out = {}
    for mode in modes:
        row = []
        for b, K in enumerate(SCHED_BUCKET_K):
            nk = -(-K // (32 if mode != "bf16x3" else 64))  # 128-byte slices
            cands = [g for g in SCHED_CANDIDATES if g == 0 or g <= max(nk, 1)]
            if b > 0:
                cands = [g for g in cands if g != 0 or K <= 128]
            res = []
            for g in cands:
                ms, e, se = sched_measure(mode, K, g)
                res.append((g, ms, float(e.mean()), float(e.max()), float(se.mean()),
                            float(se.max())))
                print("schedule %-6s K=%-5d group %d  %.4f ms  err mean %.3g max %.3g  |  "
                      "simt mean %.3g max %.3g" % ((mode, K) + res[-1]), flush=True)
            if mode == "tf32x3":
                ok = [r for r in res if r[2] <= r[4] and r[3] <= r[5]]
            else:
                best_mean = min(r[2] for r in res)
                ok = [r for r in res if r[2] <= 1.02 * best_mean]
            pick = min(ok, key=lambda r: r[1]) if ok else min(res, key=lambda r: r[2])
            print("schedule %-6s K=%-5d -> group %d" % (mode, K, pick[0]), flush=True)
            row.append(pick[0])
        out[mode] = row
    return out


def current_tables():
    """The library's compiled cost tables and schedule (to fill in what a run
    does not measure)."""
    import ctypes
    import batchgemm_gb300 as bg
    L = bg.lib()
    a, b = ctypes.c_float(), ctypes.c_float()
    simt = []
    for c in range(len(SIMT_CFGS)):
        L.bgemm_debug_tile_cost(0, c, ctypes.byref(a), ctypes.byref(b))
        simt.append((a.value, b.value))
    tc = {}
    for mode, mid in MODE_IDS.items():
        row = []
        for c in range(16):
            L.bgemm_debug_tile_cost(mid, c, ctypes.byref(a), ctypes.byref(b))
            row.append((a.value, b.value) if b.value > 0 else None)
        tc[mode] = row
    sched = {}
    for mode, mid in MODE_IDS.items():
        g = (ctypes.c_int * 8)()
        L.bgemm_debug_get_tc_schedule(mid, g)
        sched[mode] = list(g)
    ring, lead = ctypes.c_int(), ctypes.c_int()
    L.bgemm_debug_build_params(ctypes.byref(ring), ctypes.byref(lead))
    params = {"simt_ring_cap": ring.value, "c_prefetch_lead": lead.value}
    return simt, tc, sched, params


BUILD_CANDIDATES = {"simt_ring_cap": [4, 6, 8], "c_prefetch_lead": [0, 1, 2, 3, 4]}


def measure_build_params(which, reps=5):
    """Child process: times (ms) of the workloads a compile-time parameter
    affects, on the library as built."""
    import torch
    from batchgemm_gb300 import workloads
    from batchgemm_gb300.batch import DeviceBatch

    def timed(w, mode, alpha, beta):
        db = DeviceBatch(w.M, w.N, w.K).fill_fast("uniform", 0)
        with db.plan(mode) as p:
            for _ in range(3):
                db.execute(p, alpha, beta)
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record()
                db.execute(p, alpha, beta)
                e1.record()
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            p.check_device()
        del db
        torch.cuda.empty_cache()
        return float(np.median(ts))

    stream = workloads.stream_batches(0, 8)
    out = {}
    if which == "simt_ring_cap":
        out["plain_fp32_256"] = timed(workloads.plain_fp32(0), "simt", 1.0, 0.0)
        out["simt_at_scale_2048"] = timed(workloads.simt_at_scale(0), "simt", 1.0, 0.5)
        out["stream8"] = sum(timed(w, "simt", 1.0, 1.0) for w in stream)
    else:
        out["simt_at_scale_2048"] = timed(workloads.simt_at_scale(0), "tf32x3", 1.0, 0.5)
        out["stream8"] = sum(timed(w, "tf32x3", 1.0, 1.0) for w in stream)
    return out


def sweep_build_params(args, tables, dev_name, num_sms):
    """Rebuild per candidate and keep the fastest value of each parameter."""
    simt, tc, sched, params = tables
    params = dict(params)
    root = os.path.dirname(PKG)
    result = {}
    for name, cands in BUILD_CANDIDATES.items():
        res = {}
        for v in cands:
            trial = dict(params, **{name: v})
            write_table(args.out, simt, tc, sched, dev_name, num_sms, trial)
            subprocess.check_call([sys.executable, "-c", "import batchgemm_gb300 as bg; bg.build()"],
                                  cwd=root, stdout=subprocess.DEVNULL)
            txt = subprocess.check_output([sys.executable, "-m", "batchgemm_gb300.autotune",
                                           "--measure-build-params", name], cwd=root)
            res[v] = json.loads(txt.decode().strip().splitlines()[-1])
            print("build param %s = %d: %s" % (name, v, json.dumps(res[v])), flush=True)
        # least geometric-mean time over the workloads
        score = {v: sum(math.log(t) for t in r.values()) for v, r in res.items()}
        params[name] = min(score, key=score.get)
        result[name] = {"times_ms": {str(v): r for v, r in res.items()}, "pick": params[name]}
        print("build param %s -> %d" % (name, params[name]), flush=True)
    write_table(args.out, simt, tc, sched, dev_name, num_sms, params)
    subprocess.check_call([sys.executable, "-c", "import batchgemm_gb300 as bg; bg.build()"],
                          cwd=root, stdout=subprocess.DEVNULL)
    return result


def write_table(out, simt, tc, sched, dev_name, num_sms, params):
    def row(v):
        return "{%.1ff, %.4ff}" % tuple(v) if v else "{0.f, 0.f}"
    lines = [
        "// Generated by batchgemm_gb300/autotune.py on %s (%s, %d SMs); do not edit." % (
            datetime.date.today().isoformat(), dev_name, num_sms),
        "// Per-tile time t = a + b*K in ns, measured with every persistent CTA busy.",
        "constexpr TileCost kSimtCost[%d] = {%s};" % (len(simt), ", ".join(row(v) for v in simt)),
        "constexpr TileCost kTcCost[3][16] = {\n%s};" % ",\n".join(
            "  {%s}" % ", ".join(row(v) for v in tc[m]) for m in ("tf32", "tf32x3", "bf16x3")),
        "// Promotion groups of the split modes on CTA pairs per bucket of K (128-byte",
        "// K slices; 0 = every MMA, lo*lo kept): the fastest within the error bar.",
        "#define BGEMM_TUNED_HAS_SCHEDULE 1",
        "constexpr unsigned char kTcGroupTable[3][8] = {%s};" % ", ".join(
            "{%s}" % ", ".join(str(int(x)) for x in sched[m]) for m in ("tf32", "tf32x3",
                                                                        "bf16x3")),
        "// Compile-time schedule parameters: SIMT ring cap, pair-kernel C-prefetch lead.",
        "#define BGEMM_TUNED_HAS_BUILD_PARAMS 1",
        "constexpr int kSimtRingCap = %d;" % int(params["simt_ring_cap"]),
        "constexpr int kTcCPrefetchLead = %d;" % int(params["c_prefetch_lead"]),
    ]
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", out)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--out", default=os.path.join(PKG, "csrc", "tile_table_tuned.inc"))
    ap.add_argument("--modes", default="simt,tf32,tf32x3,bf16x3")
    ap.add_argument("--schedule", action="store_true",
                    help="sweep the promotion schedule instead of the tile costs")
    ap.add_argument("--json", default=None, help="also dump raw measurements here")
    ap.add_argument("--build-params", action="store_true",
                    help="sweep the compile-time parameters (rebuilds the library), write")
    ap.add_argument("--measure-build-params", default=None, help=argparse.SUPPRESS)
    args = ap.parse_args()
    import torch
    import batchgemm_gb300 as bg
    bg.lib()
    if args.measure_build_params:
        print(json.dumps(measure_build_params(args.measure_build_params)), flush=True)
        return
    dev = bg.device_info()
    simt_cur, tc_cur, sched_cur, params_cur = current_tables()
    if args.build_params:
        res = sweep_build_params(args, (simt_cur, tc_cur, sched_cur, params_cur),
                                 torch.cuda.get_device_name(0), dev["num_sms"])
        if args.json:
            json.dump(res, open(args.json, "w"), indent=1)
        return
    if args.schedule:
        modes = [m for m in args.modes.split(",") if m in ("tf32x3", "bf16x3")]
        sched = dict(sched_cur)
        sched.update(sweep_schedule(modes))
        if args.json:
            json.dump(sched, open(args.json, "w"), indent=1)
        if args.write:
            write_table(args.out, simt_cur, tc_cur, sched, torch.cuda.get_device_name(0),
                        dev["num_sms"], params_cur)
        return
    peaks = {}
    pk = os.path.join(os.path.dirname(PKG), "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = float(peaks.get("hbm_gbs", 6000.0))
    simt_slots = dev["num_sms"] * dev["simt_ctas_per_sm"]
    tc_slots = dev["num_sms"] * dev["tc_ctas_per_sm"]
    raw = {}
    simt = list(simt_cur)
    tc = {m: list(v) for m, v in tc_cur.items()}
    for mode in args.modes.split(","):
        Ks = [16, 64, 256, 1024] if mode == "simt" else [32, 128, 512, 2048]
        cfgs = range(len(SIMT_CFGS)) if mode == "simt" else [c for c in range(16)
                                                               if valid_tc(mode, c)]
        for c in cfgs:
            slots = simt_slots if mode == "simt" else (tc_slots // 2 if c >= 8 else tc_slots)
            ts = []
            for K in Ks:
                t, ms = measure(mode, c, K, slots, hbm_gbs=hbm)
                ts.append(t)
                raw.setdefault(mode, {}).setdefault(str(c), []).append([K, t, ms])
            a, b = fit(Ks, ts)
            print("%-7s cfg %2d  a=%9.1f ns  b=%8.3f ns/K   per-tile %s" % (
                mode, c, a, b, " ".join("%.0f" % x for x in ts)), flush=True)
            if mode == "simt":
                simt[c] = (a, b)
            else:
                tc[mode][c] = (a, b)
    if args.json:
        json.dump(raw, open(args.json, "w"), indent=1)
    if args.write:
        write_table(args.out, simt, tc, sched_cur, torch.cuda.get_device_name(0),
                    dev["num_sms"], params_cur)


if __name__ == "__main__":
    main()
