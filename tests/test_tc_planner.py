"""Host logic of the tensor-core planner, without a GPU (bgemm_debug_tc_plan).

For random batches with empty, K = 0, tiny-by-huge and ordinary matrices, in
every tensor-core mode and kernel family:
  * every output tile of every matrix is in the queue exactly once, and a
    matrix's tiles are adjacent;
  * the pre-pass workspace gives each matrix four 256-byte aligned, disjoint
    panels of rows x kpad elements (kpad = K rounded up to 16 bytes);
  * the pre-pass strips cover every 32-row strip of A and B exactly once,
    grouped by matrix, matrices with the longest K first (load balance of
    the pre-pass kernel).
"""
import ctypes

import numpy as np
import pytest

import batchgemm_gb300 as bg

MODES = {"tf32": 1, "tf32x3": 2, "bf16x3": 3}


def tc_plan(M, N, K, mode, family, slots=152, clusters=76):
    L = bg.lib()
    n = len(M)
    ia = lambda v: (ctypes.c_int * max(n, 1))(*v)
    cfg = (ctypes.c_int * max(n, 1))()
    nj, wsb, fam = ctypes.c_int(), ctypes.c_longlong(), ctypes.c_int()
    L.bgemm_debug_tc_plan.restype = ctypes.c_int
    cnt = L.bgemm_debug_tc_plan(ia(M), ia(N), ia(K), n, MODES[mode], family, slots, clusters,
                                cfg, None, 0, None, None, 0, ctypes.byref(nj),
                                ctypes.byref(wsb), ctypes.byref(fam))
    assert cnt >= 0, bg.lib().bgemm_last_error_message()
    items = (ctypes.c_int * max(3 * cnt, 1))()
    ws = (ctypes.c_longlong * max(5 * n, 1))()
    jobs = (ctypes.c_int * max(3 * nj.value, 1))()
    cnt2 = L.bgemm_debug_tc_plan(ia(M), ia(N), ia(K), n, MODES[mode], family, slots, clusters,
                                 cfg, items, cnt, ws, jobs, nj.value, ctypes.byref(nj),
                                 ctypes.byref(wsb), ctypes.byref(fam))
    assert cnt2 == cnt
    return (list(cfg)[:n], np.array(items[:3 * cnt]).reshape(-1, 3),
            np.array(ws[:5 * n]).reshape(-1, 5), np.array(jobs[:3 * nj.value]).reshape(-1, 3),
            wsb.value, fam.value)


def tile_dims(cfg):
    swap = bool(cfg & (1 << 8))
    c = cfg & 0xff
    if c >= 8:
        return 256, 64 << (c & 3), swap, True
    return 128, 16 << (c & 3), swap, False


def batch(seed, n=60):
    rng = np.random.default_rng(seed)
    M = np.exp(rng.uniform(0, np.log(3000), n)).astype(int).tolist()
    N = np.exp(rng.uniform(0, np.log(3000), n)).astype(int).tolist()
    K = np.exp(rng.uniform(0, np.log(3000), n)).astype(int).tolist()
    M[:6] = [0, 5, 1, 3000, 2, 700]
    N[:6] = [9, 0, 2999, 1, 3, 700]
    K[:6] = [4, 4, 17, 64, 0, 700]
    return M, N, K


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("family", [0, 1, 2])
def test_tc_plan_covers_every_tile_and_strip(built_lib, mode, family):
    M, N, K = batch(list(MODES).index(mode) * 3 + family + 3)
    cfgs, items, ws, jobs, ws_bytes, fam = tc_plan(M, N, K, mode, family)
    if family:
        assert fam == family
    # tiles: each exactly once, a matrix's tiles adjacent
    seen = {}
    order = []
    for pos, (mat, tm, tn) in enumerate(items):
        assert (mat, tm, tn) not in seen
        seen[(mat, tm, tn)] = pos
        if not order or order[-1] != mat:
            assert mat not in order, "tiles of matrix %d are not adjacent" % mat
            order.append(mat)
    for i in range(len(M)):
        if not (M[i] and N[i]):
            assert cfgs[i] == -1
            continue
        bm, bn, swap, pair = tile_dims(cfgs[i])
        assert pair == (fam == 2)
        ra, rb = (N[i], M[i]) if swap else (M[i], N[i])
        want = {(i, a, b) for a in range(-(-ra // bm)) for b in range(-(-rb // bn))}
        got = {k for k in seen if k[0] == i}
        assert got == want, "matrix %d (%dx%dx%d, cfg %x)" % (i, M[i], N[i], K[i], cfgs[i])
    # workspace panels
    esz = 2 if mode == "bf16x3" else 4
    split = mode != "tf32"
    spans = []
    for i in range(len(M)):
        a_hi, a_lo, b_hi, b_lo, kpad = ws[i]
        assert kpad * esz % 16 == 0 and K[i] <= kpad < K[i] + 16 // esz
        if not (M[i] and N[i] and K[i]):
            continue
        for off, rows in ((a_hi, M[i]), (b_hi, N[i])) + (((a_lo, M[i]), (b_lo, N[i]))
                                                        if split else ()):
            assert off % 256 == 0
            spans.append((off, off + rows * kpad * esz))
        if not split:
            assert a_lo == a_hi and b_lo == b_hi
    spans.sort()
    for (s0, e0), (s1, e1) in zip(spans, spans[1:]):
        assert e0 <= s1, "workspace panels overlap"
    assert not spans or spans[-1][1] <= ws_bytes
    # pre-pass strips: every 32-row strip once, grouped by matrix, longest K first
    strips = [tuple(j) for j in jobs]
    assert len(set(strips)) == len(strips)
    want = {(i, 0, r) for i in range(len(M)) if M[i] and N[i] and K[i] for r in range(0, M[i], 32)}
    want |= {(i, 1, r) for i in range(len(M)) if M[i] and N[i] and K[i] for r in range(0, N[i], 32)}
    assert set(strips) == want
    job_mats = []
    for mat, _, _ in strips:
        if not job_mats or job_mats[-1] != mat:
            job_mats.append(mat)
    assert len(job_mats) == len(set(job_mats))
    ks = [K[m] for m in job_mats]
    assert ks == sorted(ks, reverse=True)


def test_tc_plan_without_pairs_uses_one_sm_tiles(built_lib):
    M, N, K = batch(1)
    cfgs, *_, fam = tc_plan(M, N, K, "tf32x3", 0, clusters=0)
    assert fam == 1
    assert all(c == -1 or (c & 0xff) < 8 for c in cfgs)


def test_tc_plan_swaps_small_m(built_lib):
    """Tiny M with large N and K runs with the operands swapped, so the MMA's
    M side walks N (the uneven-M grouped-shape case).  Enough matrices that
    every persistent CTA is busy: with only a few, the rebalance may prefer
    more, smaller tiles for parallelism."""
    M, N, K = [1, 3, 16] * 100, [1024] * 300, [1024] * 300
    for family in (1, 2):
        cfgs, *_ = tc_plan(M, N, K, "tf32x3", family)
        assert all(c & (1 << 8) for c in cfgs), [hex(c) for c in cfgs]
