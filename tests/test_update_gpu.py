"""Plans that take new batches (bgemm_plan_update) under one captured CUDA graph.

A plan is created with a capacity (the element-wise maximum of
bgemm_plan_requirements over the batches to come), its execute is captured
once, and every following batch is uploaded with bgemm_plan_update before a
replay.  Each replay is checked against the oracle: bit-exact for the SIMT
mode (alpha = beta = 1 is the reference's in-place fma chain), the
sqrt(K)-scaled FP64 bound for the tensor-core modes, and the device-built
tensor maps byte-identical to the host encoding after every update.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
import oracle  # noqa: E402
from gpu_util import make_batch, oracle_batch, assert_bits_equal, f64_check  # noqa: E402

FP64_BOUND = {"tf32x3": (32.0, 2.0 ** -24), "bf16x3": (8.0, 2.0 ** -16),
              "tf32": (4.0, 2.0 ** -11)}


def shapes(seed, n_batches, lo=3, hi=40, max_dim=300):
    rng = np.random.default_rng(seed)
    out = []
    for b in range(n_batches):
        n = int(rng.integers(lo, hi + 1))
        dims = lambda: np.exp(rng.uniform(0, np.log(max_dim), n)).astype(int).tolist()
        M, N, K = dims(), dims(), dims()
        if b == 1:  # empty and degenerate matrices inside a batch
            M[0], N[1 % n], K[2 % n] = 0, 0, 0
        out.append((M, N, K))
    return out


def compare_tmaps(plan):
    L = bg.lib()
    L.bgemm_debug_compare_tensor_maps.argtypes = [ctypes.c_void_p] * 2 + \
        [ctypes.POINTER(ctypes.c_int)] * 3
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = L.bgemm_debug_compare_tensor_maps(plan._h, None, ctypes.byref(a), ctypes.byref(b),
                                           ctypes.byref(c))
    assert rc == 0
    assert b.value == 0, "%d of %d maps differ (first byte %d)" % (b.value, a.value, c.value)
    return a.value


def check(mode, db, host, alpha, beta, what):
    got = db.C.cpu().numpy()
    if mode == "simt":
        assert_bits_equal(got, oracle_batch(db, host, alpha, beta), what)
    else:
        factor, unit = FP64_BOUND[mode]
        f64_check(db, host, got, alpha, beta, factor, unit)


@pytest.mark.parametrize("mode,family", [("simt", "auto"), ("tf32x3", "pair"),
                                         ("tf32x3", "single"), ("bf16x3", "pair"),
                                         ("tf32", "auto")])
def test_update_then_graph_replay(cuda, mode, family):
    batches = shapes(41, 5)
    opts = {} if mode == "simt" else {"kernel_family": family}
    reqs = [bg.plan_requirements(M, N, K, [max(1, m) for m in M], [max(1, k) for k in K],
                                 [max(1, m) for m in M], mode=mode, **opts)
            for M, N, K in batches]
    cap = bg.max_requirements(reqs)
    pA, pB, pC = (torch.zeros(cap["batch"], dtype=torch.int64, device=cuda) for _ in range(3))
    s = torch.cuda.Stream()
    M, N, K = batches[0]
    db, host = make_batch(M, N, K, seed=0)
    with torch.cuda.stream(s):
        plan = db.plan(mode, stream=s, capacity=cap, **opts)
        got_cap = plan.capacity()
        for k in ("batch", "tiles", "pack_jobs", "workspace_bytes"):
            assert got_cap[k] == cap[k], (k, got_cap, cap)
        if mode == "tf32":
            assert got_cap["kernel_family"] in (1, 2)  # chosen by the cost model
        elif mode != "simt":
            assert got_cap["kernel_family"] == {"pair": 2, "single": 1}[family]
        for dst, src in ((pA, db.pA), (pB, db.pB), (pC, db.pC)):
            dst[:len(M)].copy_(src)
        plan.execute(1.0, pA.data_ptr(), pB.data_ptr(), 1.0, pC.data_ptr(), stream=s)
    s.synchronize()
    check(mode, db, host, 1.0, 1.0, "before capture")
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.execute(1.0, pA.data_ptr(), pB.data_ptr(), 1.0, pC.data_ptr(), stream=s)
    order = list(range(1, len(batches))) + [0]
    for step, b in enumerate(order):
        M, N, K = batches[b]
        db, host = make_batch(M, N, K, seed=100 + step)
        with torch.cuda.stream(s):
            for dst, src in ((pA, db.pA), (pB, db.pB), (pC, db.pC)):
                dst[:len(M)].copy_(src)
            plan.update(M, N, K, db.lda, db.ldb, db.ldc, stream=s)
            g.replay()
        s.synchronize()
        plan.check_device(s)
        info = plan.info()
        assert info["batch"] == len(M)
        assert info["num_tiles"] == reqs[b]["tiles"]
        check(mode, db, host, 1.0, 1.0, "batch %d after update" % b)
        if mode != "simt":
            n_maps = compare_tmaps(plan)
            assert n_maps == 4 * sum(1 for i in range(len(M)) if M[i] and N[i] and K[i])


def test_back_to_back_updates_without_sync(cuda):
    """Several update + replay pairs queued before one synchronisation: the
    double-buffered staging keeps each batch's upload intact."""
    batches = shapes(7, 6, lo=10, hi=30, max_dim=200)
    lds = lambda M, K: ([max(1, m) for m in M], [max(1, k) for k in K], [max(1, m) for m in M])
    reqs = [bg.plan_requirements(M, N, K, *lds(M, K), mode="simt") for M, N, K in batches]
    cap = bg.max_requirements(reqs)
    s = torch.cuda.Stream()
    dbs = [make_batch(M, N, K, seed=300 + i) for i, (M, N, K) in enumerate(batches)]
    ptrs = [torch.zeros(cap["batch"] * 3, dtype=torch.int64, device=cuda)]
    pA, pB, pC = ptrs[0][:cap["batch"]], ptrs[0][cap["batch"]:2 * cap["batch"]], \
        ptrs[0][2 * cap["batch"]:]
    M, N, K = batches[0]
    with torch.cuda.stream(s):
        plan = bg.Plan(M, N, K, *lds(M, K), mode="simt", stream=s, capacity=cap)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.execute(1.0, pA.data_ptr(), pB.data_ptr(), 1.0, pC.data_ptr(), stream=s)
    with torch.cuda.stream(s):
        for i, (M, N, K) in enumerate(batches):
            db = dbs[i][0]
            pA[:len(M)].copy_(db.pA)
            pB[:len(M)].copy_(db.pB)
            pC[:len(M)].copy_(db.pC)
            plan.update(M, N, K, db.lda, db.ldb, db.ldc, stream=s)
            g.replay()
    s.synchronize()
    for i, (db, host) in enumerate(dbs):
        assert_bits_equal(db.C.cpu().numpy(), oracle_batch(db, host, 1.0, 1.0), "batch %d" % i)


@pytest.mark.parametrize("mode", ["simt", "tf32x3"])
def test_update_beyond_capacity_keeps_previous_batch(cuda, mode):
    M, N, K = [20, 33, 7], [18, 5, 64], [9, 70, 3]
    db, host = make_batch(M, N, K, seed=9)
    plan = db.plan(mode)
    big = [512] * 4
    with pytest.raises(bg.BgemmError) as ei:
        plan.update(big, big, big, big, big, big)
    assert ei.value.status == 2  # BGEMM_ERROR_NOT_SUPPORTED
    with pytest.raises(bg.BgemmError) as ei:  # same batch size, more tiles
        plan.update([600, 1, 1], [600, 1, 1], [600, 1, 1], [600, 1, 1], [600, 1, 1], [600, 1, 1])
    assert ei.value.status == 2
    db.execute(plan, 1.0, 1.0)
    torch.cuda.synchronize()
    check(mode, db, host, 1.0, 1.0, "previous batch kept")
    plan.close()


def test_update_to_empty_batch_and_back(cuda):
    """A batch without work still runs the captured launches (they find no
    tiles); C is untouched.  Then a real batch again."""
    M, N, K = [40, 9], [17, 64], [33, 5]
    db, host = make_batch(M, N, K, seed=21)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan = db.plan("tf32x3", stream=s)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        db.execute(plan, 1.0, 1.0, stream=s)
    before = db.C.clone()
    with torch.cuda.stream(s):
        plan.update([0, 40], [17, 0], [33, 5], [1, 40], [33, 5], [1, 40], stream=s)
        g.replay()
    s.synchronize()
    plan.check_device(s)
    assert torch.equal(db.C.isnan(), before.isnan())
    assert torch.equal(torch.nan_to_num(db.C), torch.nan_to_num(before))
    with torch.cuda.stream(s):
        plan.update(M, N, K, db.lda, db.ldb, db.ldc, stream=s)
        g.replay()
    s.synchronize()
    check("tf32x3", db, host, 1.0, 1.0, "after empty batch")
    plan.close()


def test_update_refused_while_capturing(cuda):
    M, N, K = [8, 8], [8, 8], [8, 8]
    db, _ = make_batch(M, N, K, seed=2)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan = db.plan("simt", stream=s)
    g = torch.cuda.CUDAGraph()
    err = None
    with torch.cuda.graph(g, stream=s):
        try:
            plan.update(M, N, K, db.lda, db.ldb, db.ldc, stream=s)
        except bg.BgemmError as e:
            err = e
        db.execute(plan, 1.0, 0.0, stream=s)
    assert err is not None and err.status == 1 and err.arg == 9
    plan.close()


def test_kernel_family_options(cuda):
    M, N, K = [256] * 8, [256] * 8, [64] * 8
    lda = M
    with bg.Plan(M, N, K, lda, K, lda, mode="tf32", kernel_family="pair") as p:
        assert p.capacity()["kernel_family"] == 2
    with pytest.raises(bg.BgemmError) as ei:
        bg.Plan(M, N, K, lda, K, lda, mode="tf32x3", kernel_family=3)
    assert ei.value.status == 1
    with pytest.raises(bg.BgemmError) as ei:  # a pair config with the one-SM family
        bg.Plan(M, N, K, lda, K, lda, mode="tf32x3", kernel_family="single", force_tile_config=9)
    assert ei.value.status == 1
    for fam, want in (("single", 1), ("pair", 2)):
        r = bg.plan_requirements(M, N, K, lda, K, lda, mode="tf32x3", kernel_family=fam)
        assert r["kernel_family"] == want
        p = bg.Plan(M, N, K, lda, K, lda, mode="tf32x3", kernel_family=fam)
        assert p.capacity() == r
        p.close()
