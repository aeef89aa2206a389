"""The one-shot entries' plan cache (bgemm_sgemm_vbatched) on the GPU.

The reference sorts its shape file offline by K and tile class so that its
dense grid meets similar tiles together (ROCm/data/sort.cpp:17-60).  Here the
planner orders the tile queue itself, and the plan cache is keyed by the
shape multiset, so:
  * the same batch in another order reuses the cached plan (re-planned into
    its buffers, no new plan) and every matrix's C is bit-identical;
  * the same batch on another stream reuses the plan, ordered after its
    previous use;
  * cycling more distinct large batches than the cache's byte limit holds
    evicts old plans instead of failing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
from gpu_util import make_batch, assert_bits_equal  # noqa: E402


def permuted(db, host, perm, seed):
    """The batch of `db` with its matrices in order `perm` (same data)."""
    M = [db.M[i] for i in perm]
    N = [db.N[i] for i in perm]
    K = [db.K[i] for i in perm]
    db2, _ = make_batch(M, N, K, seed=seed)
    hA, hB, hC = host
    for j, i in enumerate(perm):
        for dst, src, off_d, off_s, n in (
                (db2.A, hA, db2.offA[j], db.offA[i], db.lda[i] * db.K[i]),
                (db2.B, hB, db2.offB[j], db.offB[i], db.ldb[i] * db.N[i]),
                (db2.C, hC, db2.offC[j], db.offC[i], db.ldc[i] * db.N[i])):
            if n:
                dst[off_d:off_d + n].copy_(torch.from_numpy(src[off_s:off_s + n]))
    return db2


def c_of(db, i):
    n = db.ldc[i] * db.N[i]
    return db.C[db.offC[i]:db.offC[i] + n].cpu().numpy()


@pytest.mark.parametrize("mode", ["simt", "tf32x3"])
def test_permuted_batch_reuses_plan_bit_identical(cuda, mode):
    rng = np.random.default_rng(31)
    n = 40
    M = rng.integers(1, 700, n).tolist()
    N = rng.integers(1, 700, n).tolist()
    K = rng.integers(0, 900, n).tolist()
    db, host = make_batch(M, N, K, seed=4)
    perm = rng.permutation(n).tolist()
    db2 = permuted(db, host, perm, seed=4)
    s0 = bg.plan_cache_stats()
    db.run(mode, 1.0, 0.5)
    db2.run(mode, 1.0, 0.5)
    torch.cuda.synchronize()
    s1 = bg.plan_cache_stats()
    assert s1["misses"] - s0["misses"] == 1, (s0, s1)
    assert s1["reorders"] - s0["reorders"] == 1, (s0, s1)
    for j, i in enumerate(perm):
        assert_bits_equal(c_of(db2, j), c_of(db, i), "%s matrix %d (slot %d)" % (mode, i, j))
    # the first order again: re-planned back, same bits as the first run
    ref = db.C.clone()
    db.C.copy_(torch.from_numpy(host[2]))
    db.run(mode, 1.0, 0.5)
    torch.cuda.synchronize()
    s2 = bg.plan_cache_stats()
    assert s2["misses"] == s1["misses"] and s2["reorders"] - s1["reorders"] == 1
    assert_bits_equal(db.C.cpu().numpy(), ref.cpu().numpy(), mode + " back to the first order")


def test_other_stream_reuses_plan(cuda):
    rng = np.random.default_rng(32)
    M = rng.integers(1, 400, 20).tolist()
    db, host = make_batch(M, M, M, seed=6)
    db.run("tf32x3", 1.0, 0.0)
    torch.cuda.synchronize()
    want = db.C.cpu().numpy()
    s0 = bg.plan_cache_stats()
    side = torch.cuda.Stream()
    for _ in range(3):
        with torch.cuda.stream(side):
            db.run("tf32x3", 1.0, 0.0, stream=side)
        db.run("tf32x3", 1.0, 0.0)  # the default stream again
    torch.cuda.synchronize()
    s1 = bg.plan_cache_stats()
    assert s1["misses"] == s0["misses"] and s1["hits"] - s0["hits"] == 6
    assert_bits_equal(db.C.cpu().numpy(), want, "alternating streams")


def test_byte_limit_evicts_instead_of_failing(cuda):
    """Four distinct batches whose plans hold ~270 MB of split operands each,
    cycled twice under a limit of two plans' worth: every call succeeds, the
    cache stays under the limit, and old plans are evicted."""
    batches = []
    for j in range(4):
        sz = [2048 - 16 * j] * 4
        db, _ = make_batch(sz, sz, sz, seed=j)
        batches.append(db)
    bg.plan_cache_clear()
    s0 = bg.plan_cache_stats()
    p = batches[0].plan("tf32x3")
    one = p.info()["device_bytes"]
    p.close()
    try:
        bg.plan_cache_set_limit(int(2.2 * one))
        for _ in range(2):
            for db in batches:
                db.run("tf32x3", 1.0, 0.0)
                st = bg.plan_cache_stats()
                assert st["bytes"] <= int(2.2 * one), st
        torch.cuda.synchronize()
        s1 = bg.plan_cache_stats()
        assert s1["misses"] - s0["misses"] == 8 and s1["evictions"] - s0["evictions"] >= 6, s1
    finally:
        bg.plan_cache_set_limit(0)
        bg.plan_cache_clear()
