"""Mixed plans (plan option simt_below): in a tensor-core mode, matrices with
min(M, N, K) below the threshold run on the FP32 SIMT kernel in the same
execute, the rest on the tensor cores; both halves take the caller's full
pointer arrays.

Checks: every SIMT-routed matrix is bit-identical to the FP32 oracle (the
SIMT contract), every tensor-core matrix within the mode's FP64 bound, guard
bands untouched; a mixed plan created with the capacity of several batches
takes each of them through bgemm_plan_update."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
import oracle  # noqa: E402
from gpu_util import make_batch, oracle_batch, U  # noqa: E402

BELOW = 64


def shapes(seed, n=40):
    rng = np.random.default_rng(seed)
    M = np.exp(rng.uniform(0, np.log(900), n)).astype(int).tolist()
    N = np.exp(rng.uniform(0, np.log(900), n)).astype(int).tolist()
    K = np.exp(rng.uniform(0, np.log(900), n)).astype(int).tolist()
    M[:4], N[:4], K[:4] = [3, 600, 700, 0], [700, 5, 600, 9], [500, 400, 20, 30]
    return M, N, K


def check(db, host, got, alpha, beta):
    want32 = oracle_batch(db, host, alpha, beta)
    hA, hB, hC0 = host
    for i in range(db.batch):
        M, N, K = db.M[i], db.N[i], db.K[i]
        if not (M and N):
            continue
        ldc = db.ldc[i]
        sl = slice(db.offC[i], db.offC[i] + ldc * N)
        if min(M, N, K) < BELOW:
            g = np.ascontiguousarray(got[sl]).view(np.uint32)
            w = np.ascontiguousarray(want32[sl]).view(np.uint32)
            assert (g == w).all(), "SIMT-routed matrix %d (%dx%dx%d) not bit-exact" % (
                i, M, N, K)
        else:
            C64, bound = oracle.sgemm_f64(M, N, K, alpha, hA[db.offA[i]:], db.lda[i],
                                          hB[db.offB[i]:], db.ldb[i], beta, hC0[db.offC[i]:], ldc)
            g = got[sl].reshape(N, ldc)[:, :M].T.reshape(-1, order="F")
            e = oracle.normalized_error(g, C64, bound)
            assert e.max() <= 32 * U * np.sqrt(K), "tensor-core matrix %d: %.3g" % (i, e.max())
    # guard bands and ld padding untouched
    pad = np.isnan(host[2])
    assert np.isnan(got[pad]).all()


@pytest.mark.parametrize("mode", ["tf32x3", "bf16x3"])
def test_mixed_plan_routes_and_matches(cuda, mode):
    M, N, K = shapes(3)
    db, host = make_batch(M, N, K, seed=5)
    with bg.Plan(db.M, db.N, db.K, db.lda, db.ldb, db.ldc, mode=mode, simt_below=BELOW) as p:
        info = p.info()
        assert info["kernels_per_execute"] == 3
        db.execute(p, 1.0, 0.5)
        torch.cuda.synchronize()
        p.check_device()
    got = db.C.cpu().numpy()
    if mode == "tf32x3":
        check(db, host, got, 1.0, 0.5)
    else:  # 3xBF16: only the SIMT half has a bit-exact contract
        want32 = oracle_batch(db, host, 1.0, 0.5)
        for i in range(db.batch):
            if db.M[i] and db.N[i] and min(db.M[i], db.N[i], db.K[i]) < BELOW:
                sl = slice(db.offC[i], db.offC[i] + db.ldc[i] * db.N[i])
                assert (got[sl].view(np.uint32) == want32[sl].view(np.uint32)).all()


def test_mixed_plan_update_stream(cuda):
    batches = [shapes(s) for s in (11, 12, 13)]
    reqs = [bg.plan_requirements(M, N, K, [max(1, m) for m in M], [max(1, k) for k in K],
                                 [max(1, m) for m in M], mode="tf32x3", simt_below=BELOW)
            for M, N, K in batches]
    assert all(r["simt_tiles"] > 0 for r in reqs)
    cap = bg.max_requirements(reqs)
    M0, N0, K0 = batches[0]
    db0, _ = make_batch(M0, N0, K0, seed=1)
    with bg.Plan(db0.M, db0.N, db0.K, db0.lda, db0.ldb, db0.ldc, mode="tf32x3",
                 simt_below=BELOW, capacity=cap) as p:
        assert p.capacity()["simt_tiles"] == cap["simt_tiles"]
        for b, (M, N, K) in enumerate(batches):
            db, host = make_batch(M, N, K, seed=20 + b)
            p.update(db.M, db.N, db.K, db.lda, db.ldb, db.ldc)
            db.execute(p, 1.0, 1.0)
            torch.cuda.synchronize()
            p.check_device()
            check(db, host, db.C.cpu().numpy(), 1.0, 1.0)
