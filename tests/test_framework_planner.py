"""Host replays of the device-side planners of bgemm_framework_gemm_mode
(bgemm_debug_framework_tc_plan) and bgemm_framework_gemm
(bgemm_debug_framework_plan), without a GPU.

The same per-matrix decisions as fwtc_plan_kernel (tile configuration from the
cost table, bins, strips, workspace panels), reserved in matrix order instead
of by atomics.  For random batches with empty, K = 0, one-row and
out-of-bounds matrices, in every tensor-core mode:
  * every output tile of every in-bounds matrix is in the queue exactly once,
    a matrix's tiles adjacent;
  * every 32-row strip of A and B of a matrix with work is a pre-pass job
    exactly once, grouped by matrix, the longest K (quarter-octave bins) first;
  * the split-operand panels are 256-byte aligned, disjoint, and fit the
    scratch the entry sizes from max_dim / max_k or from the operand bound;
  * out-of-bounds sizes and a too small operand bound raise the error bits
    the device reports.
"""
import ctypes
import math

import numpy as np
import pytest

import batchgemm_gb300 as bg

MODES = {"tf32": 1, "tf32x3": 2, "bf16x3": 3}


def quarter_octave(x):
    """floor(4 log2 x) for x >= 1 from the float32 bits (the planners' bin
    function, restated), 0 below 1."""
    x = np.float32(x)
    if not x >= 1:
        return 0
    u = int(np.array([x], np.float32).view(np.uint32)[0])
    e = ((u >> 23) & 0xff) - 127
    m = np.array([(u & 0x7fffff) | 0x3f800000], np.uint32).view(np.float32)[0]
    edges = [np.float32(1.18920712), np.float32(1.41421356), np.float32(1.68179283)]
    return 4 * e + sum(int(m >= q) for q in edges)


def tile_bin(mode_id, cfg, K):
    """Quarter-octave bin of the modelled tile time a + b*K (float32, as the
    device computes it) of configuration cfg."""
    L = bg.lib()
    a, b = ctypes.c_float(), ctypes.c_float()
    assert L.bgemm_debug_tile_cost(mode_id, cfg, ctypes.byref(a), ctypes.byref(b)) == 0
    t = np.float32(a.value) + np.float32(b.value) * np.float32(K)
    return min(63, max(0, quarter_octave(t) - 24))


def assert_longest_first(items, cfgs, K, mode_id):
    """Along the queue the modelled tile time's bin never increases."""
    bins = [tile_bin(mode_id, cfgs[mat], K[mat]) for mat, _, _ in items]
    assert all(b0 >= b1 for b0, b1 in zip(bins, bins[1:])), "queue not longest-first"


def fw_plan(M, N, K, max_dim, max_k, mode, elems=0, with_cfg=False):
    L = bg.lib()
    n = len(M)
    ia = lambda v: (ctypes.c_int * max(n, 1))(*v)
    nj, used, cap, err = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
    f = L.bgemm_debug_framework_tc_plan
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_int] * 3 + [ctypes.c_longlong, ctypes.c_int,
                                                              ctypes.c_void_p, ctypes.c_int,
                                                              ctypes.c_void_p, ctypes.c_int] + \
        [ctypes.c_void_p] * 6
    cfg = (ctypes.c_int * max(n, 1))()
    args = lambda items, mi, jobs, mj, ws: (ia(M), ia(N), ia(K), n, max_dim, max_k, elems,
                                            MODES[mode], items, mi, jobs, mj, ws,
                                            ctypes.byref(nj), ctypes.byref(used),
                                            ctypes.byref(cap), ctypes.byref(err), cfg)
    cnt = f(*args(None, 0, None, 0, None))
    assert cnt >= 0
    items = (ctypes.c_int * max(3 * cnt, 1))()
    jobs = (ctypes.c_int * max(3 * nj.value, 1))()
    ws = (ctypes.c_longlong * max(5 * n, 1))()
    cnt2 = f(*args(items, cnt, jobs, nj.value, ws))
    assert cnt2 == cnt
    out = (np.array(items[:3 * cnt]).reshape(-1, 3), np.array(jobs[:3 * nj.value]).reshape(-1, 3),
           np.array(ws[:5 * n]).reshape(-1, 5), used.value, cap.value, err.value)
    return out + (list(cfg)[:n],) if with_cfg else out


def batch(seed, n=80, max_dim=900, max_k=700):
    rng = np.random.default_rng(seed)
    M = np.exp(rng.uniform(0, np.log(max_dim), n)).astype(int).tolist()
    N = np.exp(rng.uniform(0, np.log(max_dim), n)).astype(int).tolist()
    K = np.exp(rng.uniform(0, np.log(max_k), n)).astype(int).tolist()
    M[:6] = [0, 5, 1, max_dim, 2, 700]
    N[:6] = [9, 0, max_dim, 1, 3, 600]
    K[:6] = [4, 4, 17, max_k, 0, 300]
    return M, N, K


def check_plan(M, N, K, mode, items, jobs, ws, used, cap, in_bounds):
    # tiles: each exactly once, a matrix's tiles adjacent
    seen = set()
    order = []
    for mat, tm, tn in items:
        key = (mat, tm, tn)
        assert key not in seen
        seen.add(key)
        if not order or order[-1] != mat:
            assert mat not in order, "tiles of matrix %d are not adjacent" % mat
            order.append(mat)
    for i in range(len(M)):
        got = {k for k in seen if k[0] == i}
        if not (in_bounds[i] and M[i] and N[i]):
            assert not got
            continue
        # the tile grid is 256 rows on one side and 64/128/256 on the other
        sides = sorted((1 + max(k[1] for k in got), 1 + max(k[2] for k in got)))
        ok = False
        for bn in (64, 128, 256):
            for ra, rb in ((M[i], N[i]), (N[i], M[i])):
                if [-(-ra // 256), -(-rb // bn)] in ([sides[0], sides[1]], [sides[1], sides[0]]):
                    ok = True
        assert ok, "matrix %d (%dx%d): tile grid %s" % (i, M[i], N[i], sides)
        assert len(got) == sides[0] * sides[1]
    # strips: every 32-row strip once, grouped by matrix, longest K first
    strips = [tuple(j) for j in jobs]
    assert len(set(strips)) == len(strips)
    work = [i for i in range(len(M)) if in_bounds[i] and M[i] and N[i] and K[i]]
    want = {(i, 0, r) for i in work for r in range(0, M[i], 32)}
    want |= {(i, 1, r) for i in work for r in range(0, N[i], 32)}
    assert set(strips) == want
    mats = []
    for mat, _, _ in strips:
        if not mats or mats[-1] != mat:
            assert mat not in mats
            mats.append(mat)
    kbins = [min(63, quarter_octave(K[m])) for m in mats]
    assert kbins == sorted(kbins, reverse=True)
    # workspace panels: aligned, disjoint, inside the scratch
    esz = 2 if mode == "bf16x3" else 4
    split = mode != "tf32"
    spans = []
    for i in work:
        a_hi, a_lo, b_hi, b_lo, kpad = ws[i]
        assert kpad * esz % 16 == 0 and K[i] <= kpad < K[i] + 16 // esz
        for off, rows in ((a_hi, M[i]), (b_hi, N[i])) + (((a_lo, M[i]), (b_lo, N[i]))
                                                        if split else ()):
            assert off % 256 == 0
            spans.append((off, off + rows * kpad * esz))
    spans.sort()
    for (s0, e0), (s1, e1) in zip(spans, spans[1:]):
        assert e0 <= s1, "workspace panels overlap"
    assert not spans or spans[-1][1] <= used <= cap


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("seed", [1, 2])
def test_device_planner_replay_covers_everything(built_lib, mode, seed):
    M, N, K = batch(seed * 7 + len(mode))
    # the default bound (batch * 2 * max_dim * max_k) and the exact operand bound
    elems = sum((m + n) * k for m, n, k in zip(M, N, K))
    for bound in (0, elems):
        items, jobs, ws, used, cap, err, cfgs = fw_plan(M, N, K, 900, 700, mode, bound,
                                                        with_cfg=True)
        assert err == 0
        check_plan(M, N, K, mode, items, jobs, ws, used, cap, [True] * len(M))
        assert_longest_first(items, cfgs, K, MODES[mode])


def test_device_planner_replay_flags_out_of_bounds(built_lib):
    M, N, K = [40, 950, 30, 8], [33, 20, 30, 8], [17, 20, 701, 8]
    items, jobs, ws, used, cap, err = fw_plan(M, N, K, 900, 700, "tf32x3")
    assert err == 1
    check_plan(M, N, K, "tf32x3", items, jobs, ws, used, cap, [True, False, False, True])


def test_device_planner_replay_operand_bound_too_small(built_lib):
    M, N, K = batch(3)
    elems = sum((m + n) * k for m, n, k in zip(M, N, K))
    items, jobs, ws, used, cap, err = fw_plan(M, N, K, 900, 700, "tf32x3", elems // 4)
    assert err == 2 and len(items) == 0 and len(jobs) == 0 and used > cap


def test_device_planner_replay_prefers_pair_tiles_of_the_cost_table(built_lib):
    """Large square matrices take the 256 x 256 pair tile; a tiny M with large
    N is swapped so the 256-row side walks N."""
    items, *_ = fw_plan([2048] * 4, [2048] * 4, [2048] * 4, 2048, 2048, "tf32x3")
    assert len(items) == 4 * 8 * 8
    items, *_ = fw_plan([3] * 8, [2048] * 8, [1024] * 8, 2048, 1024, "tf32x3")
    tm_max = max(t[1] for t in items)
    assert tm_max == 7  # 2048 / 256 tiles along the MMA's M side: the operands are swapped


# ---- the SIMT entry (bgemm_framework_gemm) -------------------------------
SIMT_CFGS = [(16, 16), (32, 32), (64, 32), (32, 64), (64, 64), (128, 64), (64, 128), (128, 128),
             (8, 128), (128, 8)]


SLOTS = 304  # persistent SIMT CTAs on GB300 (152 SMs x 2)


def fw_simt_plan(M, N, K, max_dim, slots=SLOTS):
    L = bg.lib()
    n = len(M)
    ia = lambda v: (ctypes.c_int * max(n, 1))(*v)
    f = L.bgemm_debug_framework_plan
    f.restype = ctypes.c_int
    cfg = (ctypes.c_int * max(n, 1))()
    err = ctypes.c_int()
    cnt = f(ia(M), ia(N), ia(K), n, max_dim, slots, cfg, None, 0, ctypes.byref(err))
    assert cnt >= 0
    items = (ctypes.c_int * max(3 * cnt, 1))()
    assert f(ia(M), ia(N), ia(K), n, max_dim, slots, cfg, items, cnt, ctypes.byref(err)) == cnt
    return list(cfg)[:n], np.array(items[:3 * cnt]).reshape(-1, 3), err.value


@pytest.mark.parametrize("seed", [4, 5, 6])
def test_simt_device_planner_replay(built_lib, seed):
    """Every tile of every in-bounds matrix once, a matrix's tiles adjacent;
    out-of-bounds sizes flagged and skipped."""
    M, N, K = batch(seed, n=120, max_dim=800, max_k=800)
    M[6], N[7] = 900, 1000  # above max_dim: skipped and flagged
    cfgs, items, err = fw_simt_plan(M, N, K, 800)
    assert err == 1
    seen, order = set(), []
    for mat, tm, tn in items:
        assert (mat, tm, tn) not in seen
        seen.add((mat, tm, tn))
        if not order or order[-1] != mat:
            assert mat not in order
            order.append(mat)
    for i in range(len(M)):
        got = {k for k in seen if k[0] == i}
        if M[i] > 800 or N[i] > 800 or not (M[i] and N[i]):
            assert cfgs[i] == -1 and not got
            continue
        bm, bn = SIMT_CFGS[cfgs[i]]
        assert got == {(i, a, b) for a in range(-(-M[i] // bm)) for b in range(-(-N[i] // bn))}
    assert_longest_first(items, cfgs, K, 0)


def test_quarter_octave_bins_match_log2(built_lib):
    """The integer bin function agrees with floor(4 log2 x) away from the
    bin edges (where only the rounding of log2 could differ)."""
    rng = np.random.default_rng(0)
    for x in np.concatenate([np.exp(rng.uniform(0, 20, 2000)), np.arange(1, 3000)]):
        x32 = np.float32(x)
        v = 4 * math.log2(float(x32))
        if abs(v - round(v)) > 1e-5:
            assert quarter_octave(x32) == math.floor(v), x32


def test_simt_device_planner_rebalances_small_batches(built_lib):
    """The reference's small sweep batches (first 8 or 16 rows of its shape
    file): with one wave of persistent CTAs the rebalance splits the longest
    tiles, so the queue holds more, shorter tiles than the per-matrix choice
    alone; a batch with plenty of tiles is left alone."""
    from batchgemm_gb300 import workloads
    for B in (8, 16):
        w = workloads.ref_dataset(B)
        _, items_1, _ = fw_simt_plan(w.M, w.N, w.K, 512, slots=1)   # one CTA: no split helps
        cfgs, items, err = fw_simt_plan(w.M, w.N, w.K, 512)
        assert err == 0 and len(items) > len(items_1), (B, len(items), len(items_1))
        assert_longest_first(items, cfgs, w.K, 0)
    rng = np.random.default_rng(9)
    M = rng.integers(256, 1024, 600).tolist()
    _, a, _ = fw_simt_plan(M, M, M, 1024, slots=1)
    _, b, _ = fw_simt_plan(M, M, M, 1024)
    assert len(a) == len(b)  # thousands of tiles for 304 CTAs: nothing to rebalance



def test_thin_matrices_take_thin_tiles_within_16_bit_coordinates(built_lib):
    """M <= 8 (or N <= 8) matrices take the 8 x 128 (or 128 x 8) tiles; a
    matrix whose thin-tile grid would pass 65535 tiles along a side takes a
    configuration that fits the 16-bit tile coordinates, in both planners."""
    from test_abi import simt_queue
    M = [4, 2000, 8, 3000]
    N = [2000, 4, 3000, 8]
    K = [64, 64, 16, 16]
    # one CTA slot: no rebalance for parallelism splits the tiles further
    for cfgs, items in (fw_simt_plan(M, N, K, 4096, slots=1)[:2], simt_queue(M, N, K, slots=1)):
        assert cfgs == [8, 9, 8, 9], cfgs
    tall = [700000, 5]
    wide = [3, 700000]
    for cfgs, items in (fw_simt_plan(tall, wide, [2, 2], 1 << 20)[:2],
                        simt_queue(tall, wide, [2, 2])):
        for i in range(2):
            bm, bn = SIMT_CFGS[cfgs[i]]
            assert -(-tall[i] // bm) <= 65535 and -(-wide[i] // bn) <= 65535, cfgs
        assert items[:, 1].max() <= 65535 and items[:, 2].max() <= 65535
