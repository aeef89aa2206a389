"""Autotuner of the planners' tile cost table.

For every mode and every tile configuration it runs uniform batches whose
matrices are whole multiples of the tile (several waves of persistent CTAs),
at several K, with the configuration forced and the rebalance off; the time
of one tile, t = a + b*K, is fitted by least squares and written to
``csrc/tile_table_tuned.inc``, which the library compiles in place of the
analytic defaults of ``csrc/tile_table.h``.

  python -m batchgemm_gb300.autotune            # measure and print
  python -m batchgemm_gb300.autotune --write    # ... and write the table

The split/pack pre-pass of the tensor-core modes does not depend on the tile
configuration; its time is estimated from its bytes (read 4 B, write 4 or 8
B per element at the device's copy bandwidth) and removed before fitting.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os
import sys

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(PKG))

SIMT_CFGS = [(16, 16), (32, 32), (64, 32), (32, 64), (64, 64), (128, 64), (64, 128), (128, 128)]
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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--write", action="store_true")
    ap.add_argument("--out", default=os.path.join(PKG, "csrc", "tile_table_tuned.inc"))
    ap.add_argument("--modes", default="simt,tf32,tf32x3,bf16x3")
    ap.add_argument("--json", default=None, help="also dump raw measurements here")
    args = ap.parse_args()
    import torch
    import batchgemm_gb300 as bg
    bg.lib()
    dev = bg.device_info()
    peaks = {}
    pk = os.path.join(os.path.dirname(PKG), "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    hbm = float(peaks.get("hbm_gbs", 6000.0))
    simt_slots = dev["num_sms"] * dev["simt_ctas_per_sm"]
    tc_slots = dev["num_sms"] * dev["tc_ctas_per_sm"]
    raw = {}
    simt = [None] * 8
    tc = {m: [None] * 16 for m in MODE_IDS}
    for mode in args.modes.split(","):
        Ks = [16, 64, 256, 1024] if mode == "simt" else [32, 128, 512, 2048]
        cfgs = range(8) if mode == "simt" else [c for c in range(16) if valid_tc(mode, c)]
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
    if not args.write:
        return
    # keep analytic defaults for anything not measured in this run
    lines = [
        "// Generated by batchgemm_gb300/autotune.py on %s (%s, %d SMs); do not edit." % (
            datetime.date.today().isoformat(), torch.cuda.get_device_name(0), dev["num_sms"]),
        "// Per-tile time t = a + b*K in ns, measured with every persistent CTA busy.",
    ]
    def row(v):
        return "{%.1ff, %.4ff}" % v if v else "{0.f, 0.f}"
    if any(v is None for v in simt):
        sys.exit("the SIMT table needs every configuration measured (run with simt in --modes)")
    lines.append("constexpr TileCost kSimtCost[8] = {%s};" % ", ".join(row(v) for v in simt))
    rows = []
    for mode in ("tf32", "tf32x3", "bf16x3"):
        if all(v is None for v in tc[mode]):
            sys.exit("mode %s was not measured" % mode)
        rows.append("  {%s}" % ", ".join(row(v) for v in tc[mode]))
    lines.append("constexpr TileCost kTcCost[3][16] = {\n%s};" % ",\n".join(rows))
    out = args.out
    with open(out, "w") as f:
        f.write("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
