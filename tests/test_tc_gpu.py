"""Tensor-core (tcgen05) modes on the GPU through the C ABI.

Two oracles per case:
  * the FP64 GEMM, with the sqrt(K)-scaled bound
        |c - c64| <= factor * u * sqrt(K) * (|alpha| sum|a b| + |beta c0|)
    (u = 2^-24 for TF32X3, 2^-16 for BF16X3, 2^-11 for TF32);
  * the exact FP64 value of the products the mode forms (hi*hi [+ hi*lo +
    lo*hi] of the same rounded halves), which leaves only the tensor core's
    FP32 accumulation as the gap -- a tight check that catches any layout,
    swizzle or operand mix-up.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
import oracle  # noqa: E402
from batchgemm_gb300 import workloads  # noqa: E402
from batchgemm_gb300.batch import DeviceBatch  # noqa: E402
from gpu_util import make_batch, f64_check  # noqa: E402

EDGE = [1, 2, 3, 7, 8, 9, 15, 16, 17, 31, 33, 63, 65, 127, 129, 200, 257]
MODES = {
    # mode: (oracle mode, FP64 factor, unit, split-exact factor)
    "tf32x3": (oracle.MODE_TF32X3, 32.0, 2.0 ** -24, 16.0),
    "bf16x3": (oracle.MODE_BF16X3, 8.0, 2.0 ** -16, 16.0),
    "tf32": (oracle.MODE_TF32, 4.0, 2.0 ** -11, 16.0),
}


def test_device_tensor_maps_match_host_encoding(cuda):
    """The tensor maps the device builds are byte-identical to the driver's
    host encoding of the same panels (runs before any GEMM of this file)."""
    import ctypes
    L = bg.lib()
    L.bgemm_debug_compare_tensor_maps.argtypes = [ctypes.c_void_p] * 2 + \
        [ctypes.POINTER(ctypes.c_int)] * 3
    rng = np.random.default_rng(17)
    # extents on both sides of 128 KiB, K above and below 256, tiny and wide
    M = [1, 17, 300, 129, 600, 64, 1024, 2000, 40, 5] + rng.integers(1, 3000, 10).tolist()
    N = [5, 64, 33, 250, 700, 2000, 1024, 3, 41, 4096] + rng.integers(1, 3000, 10).tolist()
    K = [3, 100, 64, 31, 333, 1, 1024, 2048, 257, 96] + rng.integers(1, 3000, 10).tolist()
    for mode in ("tf32", "tf32x3", "bf16x3"):
        forces = [-1, 0, 1, 2, 3, 4, 5, 6, 7] + ([8, 9, 10, 12, 13, 14] if mode != "tf32" else [])
        for f in forces:
            p = bg.Plan(M, N, K, M, K, M, mode=mode, force_tile_config=f)
            a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            rc = L.bgemm_debug_compare_tensor_maps(p._h, None, ctypes.byref(a), ctypes.byref(b),
                                                   ctypes.byref(c))
            p.close()
            assert rc == 0 and a.value == 4 * len(M), (mode, f, rc, a.value)
            assert b.value == 0, "%s cfg %d: %d of %d maps differ (first byte %d)" % (
                mode, f, b.value, a.value, c.value)


def split_check(db, host, got, alpha, beta, omode, factor):
    """|c - exact(split products)| <= factor * 2^-24 * sqrt(K) * bound."""
    hA, hB, hC0 = host
    worst = 0.0
    for i in range(db.batch):
        M, N, K = db.M[i], db.N[i], db.K[i]
        if not (M and N):
            continue
        want = oracle.sgemm_split_f64(omode, M, N, K, alpha, hA[db.offA[i]:], db.lda[i],
                                      hB[db.offB[i]:], db.ldb[i], beta, hC0[db.offC[i]:],
                                      db.ldc[i])
        _, bound = oracle.sgemm_f64(M, N, K, alpha, hA[db.offA[i]:], db.lda[i],
                                    hB[db.offB[i]:], db.ldb[i], beta, hC0[db.offC[i]:],
                                    db.ldc[i])
        ldc = db.ldc[i]
        g = got[db.offC[i]:db.offC[i] + ldc * N].reshape(N, ldc)[:, :M].reshape(-1)
        e = oracle.normalized_error(g, want, bound)
        lim = factor * 2.0 ** -24 * np.sqrt(max(K, 1))
        assert e.max() <= lim, "matrix %d (%dx%dx%d): split err %.3g > %.3g" % (
            i, M, N, K, e.max(), lim)
        worst = max(worst, float(e.max()))
    return worst


def guard_intact(db, host_c, got):
    """Everything outside the matrices (ld padding, guard bands) is untouched."""
    mask = np.ones(got.size, bool)
    for i in range(db.batch):
        M, N, ldc = db.M[i], db.N[i], db.ldc[i]
        if M and N:
            idx = db.offC[i] + np.arange(N)[:, None] * ldc + np.arange(M)[None, :]
            mask[idx.reshape(-1)] = False
    a = got[mask].view(np.uint32)
    b = host_c[mask].view(np.uint32)
    assert np.array_equal(a, b), "write outside a matrix"


def run_mode(mode, M, N, K, alpha, beta, offset=0, lda=None, ldb=None, ldc=None, seed=0,
             c_nan=False, dist="uniform", force=None):
    omode, fac, unit, sfac = MODES[mode]
    db, host = make_batch(M, N, K, lda, ldb, ldc, offset=offset, seed=seed, c_nan=c_nan,
                          dist=dist)
    if force is None:
        db.run(mode, alpha, beta)
    else:
        with db.plan(mode, force_tile_config=force) as p:
            db.execute(p, alpha, beta)
            torch.cuda.synchronize()
            p.check_device()
    torch.cuda.synchronize()
    got = db.C.cpu().numpy()
    guard_intact(db, host[2], got)
    host_in = (host[0], host[1], np.nan_to_num(host[2]) if c_nan else host[2])
    worst, mean = f64_check(db, host_in, got, alpha, beta, fac, unit)
    sworst = split_check(db, host_in, got, alpha, beta, omode, sfac)
    return worst, mean, sworst


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("offset", [0, 1])
def test_random_edge_shapes(cuda, mode, offset):
    rng = np.random.default_rng(offset + 7)
    n = 40
    M = rng.choice(EDGE, n).tolist()
    N = rng.choice(EDGE, n).tolist()
    K = rng.choice(EDGE, n).tolist()
    w, m, s = run_mode(mode, M, N, K, 1.0, 0.0, offset=offset, seed=n)
    print("%s offset %d: max err %.3g mean %.3g split-exact %.3g" % (mode, offset, w, m, s))


@pytest.mark.parametrize("mode", list(MODES))
def test_alpha_beta_and_ld(cuda, mode):
    rng = np.random.default_rng(3)
    n = 24
    M = rng.integers(1, 300, n).tolist()
    N = rng.integers(1, 300, n).tolist()
    K = rng.integers(1, 300, n).tolist()
    lda = [m + int(rng.integers(0, 5)) for m in M]
    ldb = [k + int(rng.integers(0, 5)) for k in K]
    ldc = [m + int(rng.integers(0, 5)) for m in M]
    run_mode(mode, M, N, K, 0.5, -1.5, lda=lda, ldb=ldb, ldc=ldc, seed=4)
    run_mode(mode, M, N, K, 1.0, 1.0, seed=5)


@pytest.mark.parametrize("mode", list(MODES))
def test_beta_zero_nan_c_and_k_zero(cuda, mode):
    run_mode(mode, [37, 64, 5, 9], [19, 64, 128, 4], [40, 8, 3, 0], 2.0, 0.0, c_nan=True)
    run_mode(mode, [4, 0, 9, 5], [6, 3, 0, 5], [0, 4, 4, 0], 1.0, 0.5)


@pytest.mark.parametrize("cfg", [c for c in range(16) if c < 8 or (c & 3) != 3])
def test_every_tile_config(cuda, cfg):
    """One-SM tiles (ids 0-7) and CTA-pair tiles (ids 8-14, cta_group::2)."""
    rng = np.random.default_rng(cfg + 50)
    M = rng.integers(1, 600, 10).tolist()
    N = rng.integers(1, 600, 10).tolist()
    K = rng.integers(1, 200, 10).tolist()
    for mode in ("tf32x3", "bf16x3"):
        run_mode(mode, M, N, K, 1.0, 0.25, force=cfg, seed=cfg)
    # beta = 0 runs the pair kernel's separate beta-free instantiation
    run_mode("tf32x3", M, N, K, 1.0, 0.0, force=cfg, seed=cfg + 1)
    run_mode("tf32", M, N, K, 0.5, 0.0, force=cfg, seed=cfg)


def test_pair_tiles_for_single_product(cuda):
    """The single-product TF32 mode runs on CTA pairs too (hi panels only,
    one accumulator per tile), including K = 0 and ragged edges."""
    M, N, K = [300, 1024, 17, 5], [300, 700, 1, 900], [300, 1024, 0, 77]
    for cfg in (8, 9, 10, 12, 13, 14):
        with bg.Plan(M, N, K, M, [max(1, k) for k in K], M, mode="tf32",
                     force_tile_config=cfg) as p:
            assert sum(p.info()["tile_config_hist"][8:]) == 4
        run_mode("tf32", M, N, K, 1.0, 0.5, force=cfg, seed=cfg)


def test_pair_mode_chosen_for_large_matrices(cuda):
    # many large matrices: the cost table prefers 256-row CTA-pair tiles
    M = [1024] * 48 + [700, 512, 33]
    p = bg.Plan(M, M, M, M, M, M, mode="tf32x3")
    info = p.info()
    p.close()
    assert sum(info["tile_config_hist"][8:]) == len(M), info
    assert info["grid"] % 2 == 0
    # a few tiny matrices: a 256-row pair tile would be mostly padding, so
    # the cost model keeps one-SM tiles
    few = [16, 8, 32, 20]
    p = bg.Plan(few, few, few, few, few, few, mode="tf32x3")
    assert sum(p.info()["tile_config_hist"][:8]) == 4
    p.close()
    run_mode("tf32x3", M[-4:], M[-4:], M[-4:], 1.0, 0.0, seed=12)


@pytest.mark.parametrize("force", [None, 4, 5, 7, 12, 13, 14])
def test_small_m_swapped_orientation(cuda, force):
    """Uneven-M shape class (tiny M, N = K = 1024): the planner's own choice,
    and every swapped configuration (C^T = B^T A^T, the long side on the MMA's
    M dimension; one-SM 4, 5, 7 and CTA-pair 12, 13, 14) forced."""
    M = [1, 3, 16, 40, 64, 200]
    run_mode("tf32x3", M, [1024] * 6, [1024] * 6, 1.0, 0.0, seed=9, force=force)


def test_tc_plan_graph_replay(cuda):
    rng = np.random.default_rng(21)
    M = rng.integers(1, 300, 30).tolist()
    N = rng.integers(1, 300, 30).tolist()
    K = rng.integers(1, 300, 30).tolist()
    db, host = make_batch(M, N, K, seed=1)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan = db.plan("tf32x3", stream=s)
        db.execute(plan, 1.0, 0.0, stream=s)
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        db.execute(plan, 1.0, 0.0, stream=s)
    for rep in range(3):
        db2, host2 = make_batch(M, N, K, seed=200 + rep)
        db.A.copy_(db2.A)
        db.B.copy_(db2.B)
        g.replay()
        torch.cuda.synchronize()
        f64_check(db, (host2[0], host2[1], host[2]), db.C.cpu().numpy(), 1.0, 0.0, 32.0,
                  2.0 ** -24)
    plan.check_device(stream=s)
    plan.close()


@pytest.mark.parametrize("mode", ["tf32x3", "bf16x3", "tf32"])
def test_skewed_full_size_error_vs_fp64(cuda, mode):
    """The skewed 4000-matrix batch, whole: sampled FP64 error within bound and
    (TF32X3) no worse than the FP32 SIMT path on the same samples."""
    import bench
    w = workloads.skewed(0)
    db = DeviceBatch(w.M, w.N, w.K).fill_fast(w.dist, seed=2)
    db.run(mode, 1.0, 0.0)
    torch.cuda.synchronize()
    emax, emean, n = bench.fp64_sampled_error(db, per_matrix=4, seed=1)
    unit = {"tf32x3": 2.0 ** -24, "bf16x3": 2.0 ** -16, "tf32": 2.0 ** -11}[mode]
    assert emax <= 32 * unit * np.sqrt(2048)
    db.run("simt", 1.0, 0.0)
    torch.cuda.synchronize()
    smax, smean, _ = bench.fp64_sampled_error(db, per_matrix=4, seed=1)
    print("%s: max %.3g mean %.3g | simt max %.3g mean %.3g" % (mode, emax, emean, smax, smean))
    # the strict comparison with FP32 SIMT (mean and max) is
    # test_error_bar_gpu.py::test_tf32x3_error_not_above_fp32_simt_skewed


def test_bounded_wait_expires_and_context_survives(cuda):
    """A device-side wait on a barrier that nothing completes gives up after
    its limit, raises the error word and returns; the context stays usable
    (the failure path of every tensor-core kernel, without a GPU fault)."""
    import ctypes
    L = bg.lib()
    L.bgemm_debug_bounded_wait_selftest.argtypes = [ctypes.c_ulonglong] + \
        [ctypes.POINTER(ctypes.c_int)] * 3
    err, ret, ok = ctypes.c_int(-1), ctypes.c_int(-1), ctypes.c_int(-1)
    rc = L.bgemm_debug_bounded_wait_selftest(2_000_000, ctypes.byref(err), ctypes.byref(ret),
                                             ctypes.byref(ok))
    assert rc == 0
    assert (err.value, ret.value, ok.value) == (1, 1, 0)
    run_mode("tf32x3", [64, 200], [64, 100], [64, 300], 1.0, 0.0, seed=3)
