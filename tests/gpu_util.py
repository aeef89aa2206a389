"""Helpers shared by the GPU parity tests."""
import numpy as np
import torch

import oracle
from batchgemm_gb300.batch import DeviceBatch

U = 2.0 ** -24  # FP32 unit roundoff


def make_batch(M, N, K, lda=None, ldb=None, ldc=None, offset=0, seed=0, dist="uniform",
               c_nan=False):
    """DeviceBatch whose matrices hold seeded host-generated values; padding NaN."""
    db = DeviceBatch(M, N, K, lda, ldb, ldc, offset_floats=offset)
    rng = np.random.default_rng(seed)
    hA, hB, hC = db.host()

    def fill(flat, offs, rows, cols, ld, nan=False):
        for o, r, c, l in zip(offs, rows, cols, ld):
            if r and c:
                v = flat[o:o + l * c].reshape(c, l)
                if nan:
                    v[:, :r] = np.nan
                elif dist == "normal":
                    v[:, :r] = rng.standard_normal((c, r)).astype(np.float32)
                else:
                    v[:, :r] = rng.uniform(-1, 1, (c, r)).astype(np.float32)

    fill(hA, db.offA, db.M, db.K, db.lda)
    fill(hB, db.offB, db.K, db.N, db.ldb)
    fill(hC, db.offC, db.M, db.N, db.ldc, nan=c_nan)
    db.A.copy_(torch.from_numpy(hA))
    db.B.copy_(torch.from_numpy(hB))
    db.C.copy_(torch.from_numpy(hC))
    return db, (hA, hB, hC)


def oracle_batch(db, host, alpha, beta):
    """Runs the FP32 oracle on host copies; returns the expected flat C buffer."""
    hA, hB, hC = host
    C = hC.copy()
    for i in range(db.batch):
        if db.M[i] and db.N[i]:
            oracle.sgemm_f32(db.M[i], db.N[i], db.K[i], alpha, hA[db.offA[i]:], db.lda[i],
                             hB[db.offB[i]:], db.ldb[i], beta, C[db.offC[i]:], db.ldc[i])
    return C


def assert_bits_equal(got, want, what=""):
    g = np.ascontiguousarray(got).view(np.uint32)
    w = np.ascontiguousarray(want).view(np.uint32)
    bad = np.nonzero(g != w)[0]
    assert bad.size == 0, "%s: %d of %d words differ, first at %d: got %r want %r" % (
        what, bad.size, g.size, bad[0], got[bad[0]], want[bad[0]])


def f64_check(db, host_in, C_got, alpha, beta, factor, unit):
    """max / mean of the normalised error against the FP64 oracle; asserts the
    sqrt(K)-scaled bound  |c - c64| <= factor * unit * sqrt(K) * (|alpha| sum|ab| + |beta c0|)."""
    hA, hB, hC0 = host_in
    worst, tot, cnt = 0.0, 0.0, 0
    for i in range(db.batch):
        M, N, K = db.M[i], db.N[i], db.K[i]
        if not (M and N):
            continue
        C64, bound = oracle.sgemm_f64(M, N, K, alpha, hA[db.offA[i]:], db.lda[i],
                                      hB[db.offB[i]:], db.ldb[i], beta, hC0[db.offC[i]:],
                                      db.ldc[i])
        ldc = db.ldc[i]
        got = C_got[db.offC[i]:db.offC[i] + ldc * N].reshape(N, ldc)[:, :M].T.reshape(-1,
                                                                                      order="F")
        e = oracle.normalized_error(got, C64, bound)
        lim = factor * unit * np.sqrt(max(K, 1))
        assert np.isfinite(got).all(), "matrix %d has non-finite outputs" % i
        assert e.max() <= lim, "matrix %d (%dx%dx%d): err %.3g > %.3g" % (i, M, N, K, e.max(),
                                                                          lim)
        worst = max(worst, float(e.max()))
        tot += float(e.sum())
        cnt += e.size
    return worst, tot / max(cnt, 1)
