"""Accuracy of every mode against the FP64 oracle at full workload sizes.

The precision target: on the skewed 4000-matrix batch (90 % of matrices with
M, N, K in [8, 64], 10 % in [512, 2048], N(0, 1) entries) the 3xTF32
tensor-core form's normalised error against FP64,
    |c - c64| / (|alpha| sum_k |a b| + |beta c0|),
is no worse than the plain FP32 SIMT path's -- both its mean and its maximum
over the same fixed samples (4 entries per matrix, 16 000 in all).  Data and
kernels are deterministic, so the comparison is exact run to run.

The other workloads (plain 256, SIMT-at-scale 2048 with beta = 0.5, uneven-M
128, ten batches of the batch stream with alpha = beta = 1) check each mode
against its sqrt(K)-scaled bound entry by entry,
    err <= factor * u * sqrt(K),
u = 2^-24 (FP32 SIMT, 3xTF32), 2^-16 (3xBF16), 2^-11 (TF32).  Each test
prints a `ERRTABLE` line with the means and maxima it measured.
"""
import types

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import bench  # noqa: E402
from batchgemm_gb300 import workloads  # noqa: E402
from batchgemm_gb300.batch import DeviceBatch  # noqa: E402

BOUND = {  # mode: (factor, unit)
    "simt": (8.0, 2.0 ** -24),
    "tf32x3": (32.0, 2.0 ** -24),
    "bf16x3": (8.0, 2.0 ** -16),
    "tf32": (4.0, 2.0 ** -11),
}


def run_errors(db, mode, alpha, beta, C0host, seed=1, per_matrix=4):
    """One step of `mode` from the C snapshot C0host; per-sample errors and K."""
    db.C.copy_(C0host)
    db.run(mode, alpha, beta)
    torch.cuda.synchronize()
    return bench.fp64_sampled_error(db, per_matrix=per_matrix, seed=seed, C0=C0host,
                                    beta=beta, alpha=alpha, samples=True)


def check_bound(mode, e, K, what):
    f, u = BOUND[mode]
    lim = f * u * np.sqrt(np.maximum(K, 1.0))
    bad = np.nonzero(e > lim)[0]
    assert bad.size == 0, "%s %s: %d samples above the bound, worst %.3g (K=%d, bound %.3g)" % (
        what, mode, bad.size, e[bad[0]], K[bad[0]], lim[bad[0]])


def test_tf32x3_error_not_above_fp32_simt_skewed(cuda):
    """3xTF32 mean AND max error on the skewed batch <= FP32 SIMT's, same samples."""
    w = workloads.skewed(0)
    db = DeviceBatch(w.M, w.N, w.K).fill_fast(w.dist, seed=2)
    C0 = db.C.clone()
    res = {}
    for mode in ("simt", "tf32x3", "bf16x3", "tf32"):
        e, K = run_errors(db, mode, 1.0, 0.0, C0)
        check_bound(mode, e, K, w.name)
        res[mode] = (float(e.mean()), float(e.max()), e.size)
    for mode, (mean, mx, n) in res.items():
        print("ERRTABLE %s %s mean %.3g max %.3g samples %d" % (w.name, mode, mean, mx, n))
    assert res["tf32x3"][2] == 16000
    assert res["tf32x3"][0] <= res["simt"][0], "3xTF32 mean error above FP32 SIMT's"
    assert res["tf32x3"][1] <= res["simt"][1], "3xTF32 max error above FP32 SIMT's"


@pytest.mark.parametrize("name", ["plain_fp32_256", "simt_at_scale_2048", "uneven_m_128"])
def test_config_error_bounds(cuda, name):
    """The plain 256-matrix batch, the 2048-matrix log-uniform batch and the
    uneven-M 128-matrix batch whole, every mode within its bound on sampled
    entries."""
    w = workloads.CONFIGS[name](0)
    db = DeviceBatch(w.M, w.N, w.K).fill_fast(w.dist, seed=3)
    C0 = db.C.clone()
    for mode in ("simt", "tf32x3", "bf16x3", "tf32"):
        e, K = run_errors(db, mode, w.alpha, w.beta, C0, per_matrix=8)
        check_bound(mode, e, K, name)
        print("ERRTABLE %s %s mean %.3g max %.3g samples %d" % (name, mode, e.mean(), e.max(),
                                                               e.size))


def test_stream_batches_error_bounds(cuda):
    """Ten batches of the batch stream (alpha = beta = 1), every mode within
    its bound on every batch."""
    bs = workloads.stream_batches(0, 10)
    acc = {m: [] for m in BOUND}
    for b, w in enumerate(bs):
        db = DeviceBatch(w.M, w.N, w.K).fill_fast("uniform", seed=100 + b)
        C0 = db.C.clone()
        for mode in BOUND:
            e, K = run_errors(db, mode, 1.0, 1.0, C0, seed=b, per_matrix=2)
            check_bound(mode, e, K, w.name)
            acc[mode].append(e)
        del db, C0
        torch.cuda.empty_cache()
    for mode, es in acc.items():
        e = np.concatenate(es)
        print("ERRTABLE stream_10_batches %s mean %.3g max %.3g samples %d" % (
            mode, e.mean(), e.max(), e.size))
