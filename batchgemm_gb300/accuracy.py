"""Normalised error of computed C entries against an FP64 evaluation on the
GPU, on sampled entries (used by the benchmark, the autotuner and the
accuracy tests).

For a sampled entry (m, n) of matrix i the error is
    |c - c64| / (|alpha| sum_k |a_mk b_kn| + |beta c0|),
with c64 = alpha sum_k a_mk b_kn + beta c0 formed in FP64 from the FP32
inputs.  Samples are drawn from a seeded generator, so the same call on the
same batch picks the same entries whatever mode produced C.
"""
from __future__ import annotations

import numpy as np


def fp64_sampled_error(db, per_matrix=4, seed=0, C0=None, beta=0.0, alpha=1.0,
                       samples=False):
    """Normalised error |c - c64| / (|alpha| sum|a b| + |beta c0|) on sampled
    entries, FP64 on the GPU (C0: the C buffer before the step, when beta != 0).
    Returns (max, mean, count), or with samples=True (errors, K of each
    sample) as numpy arrays."""
    import torch
    rng = np.random.default_rng(seed)
    idx_m, idx_n, mats = [], [], []
    for i in range(db.batch):
        if db.M[i] and db.N[i] and db.K[i]:
            for _ in range(per_matrix):
                mats.append(i)
                idx_m.append(int(rng.integers(0, db.M[i])))
                idx_n.append(int(rng.integers(0, db.N[i])))
    if not mats:
        return (np.zeros(0), np.zeros(0)) if samples else (0.0, 0.0, 0)
    kmax = max(db.K[i] for i in mats)
    S = len(mats)
    dev = db.A.device
    errs = []
    chunk = max(1, (1 << 26) // kmax)
    for s0 in range(0, S, chunk):
        ss = range(s0, min(S, s0 + chunk))
        K = torch.tensor([db.K[mats[s]] for s in ss], device=dev)
        ar = torch.arange(kmax, device=dev)
        mask = ar[None, :] < K[:, None]
        ka = torch.where(mask, ar[None, :], 0)
        offA = torch.tensor([db.offA[mats[s]] + idx_m[s] for s in ss], device=dev)
        lda = torch.tensor([db.lda[mats[s]] for s in ss], device=dev)
        offB = torch.tensor([db.offB[mats[s]] + idx_n[s] * db.ldb[mats[s]] for s in ss],
                            device=dev)
        a = db.A[offA[:, None] + ka * lda[:, None]].double()
        b = db.B[offB[:, None] + ka].double()
        prod = torch.where(mask, a * b, torch.zeros_like(a))
        exact = alpha * prod.sum(1)
        absb = abs(alpha) * prod.abs().sum(1)
        offC = torch.tensor([db.offC[mats[s]] + idx_m[s] + idx_n[s] * db.ldc[mats[s]]
                             for s in ss], device=dev)
        c = db.C[offC].double()
        if C0 is not None and beta != 0.0:
            c0 = beta * C0[offC].double()
            exact = exact + c0
            absb = absb + c0.abs()
        errs.append(((c - exact).abs() / absb.clamp_min(1e-300)).cpu())
    e = torch.cat(errs)
    if samples:
        return e.numpy(), np.array([db.K[i] for i in mats], dtype=np.float64)
    return float(e.max()), float(e.mean()), S
