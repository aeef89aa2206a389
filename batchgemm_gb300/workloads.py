"""Seeded synthetic workloads of variable-size batched SGEMM.

Each workload is a list of (M, N, K) shapes plus the alpha/beta and value
distribution the benchmark uses for it.  The reference's only shape fixture
(CUDA/data/data_MN_K_512_128, first B rows form a batch of B) is available as
``ref_dataset`` through the copy kept in tests/golden/ref_dataset_shapes.npy.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import List

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@dataclass
class Workload:
    name: str
    M: List[int]
    N: List[int]
    K: List[int]
    alpha: float = 1.0
    beta: float = 0.0
    dist: str = "uniform"      # "uniform" in [-1, 1] or "normal" N(0, 1)
    desc: str = ""
    extra: dict = field(default_factory=dict)

    @property
    def batch(self) -> int:
        return len(self.M)

    def flops(self) -> float:
        return float(sum(2.0 * m * n * k for m, n, k in zip(self.M, self.N, self.K)))

    def bytes(self) -> float:
        per_c = 2 if self.beta != 0 else 1
        return float(sum(4.0 * (m * k + k * n + per_c * m * n)
                         for m, n, k in zip(self.M, self.N, self.K)))


def _log_uniform_int(rng, lo: int, hi: int, n: int) -> np.ndarray:
    x = np.exp(rng.uniform(np.log(lo), np.log(hi + 1), n))
    return np.clip(np.floor(x).astype(np.int64), lo, hi)


def plain_fp32(seed: int = 0) -> Workload:
    """256 matrices, M, N, K uniform integers in [16, 256], alpha = 1, beta = 0."""
    rng = np.random.default_rng(seed)
    s = rng.integers(16, 257, size=(256, 3))
    return Workload("plain_fp32_256", s[:, 0].tolist(), s[:, 1].tolist(), s[:, 2].tolist(),
                    1.0, 0.0, "uniform",
                    "256 mats, M,N,K~U{16..256}, U[-1,1], alpha=1, beta=0, lda=M, ldb=K, ldc=M")


def simt_at_scale(seed: int = 0) -> Workload:
    """2048 matrices, M, N, K log-uniform integers in [32, 1024], beta = 0.5."""
    rng = np.random.default_rng(seed)
    M, N, K = (_log_uniform_int(rng, 32, 1024, 2048) for _ in range(3))
    return Workload("simt_at_scale_2048", M.tolist(), N.tolist(), K.tolist(), 1.0, 0.5,
                    "uniform", "2048 mats, M,N,K log-uniform [32,1024], U[-1,1], alpha=1, "
                    "beta=0.5, C0~U[-1,1]")


def skewed(seed: int = 0, n: int = 4000) -> Workload:
    """4000 matrices: 90% with M, N, K uniform in [8, 64], 10% uniform in [512, 2048]."""
    rng = np.random.default_rng(seed)
    big = rng.random(n) < 0.10
    s = np.where(big[:, None], rng.integers(512, 2049, size=(n, 3)),
                 rng.integers(8, 65, size=(n, 3)))
    return Workload("skewed_4000", s[:, 0].tolist(), s[:, 1].tolist(), s[:, 2].tolist(),
                    1.0, 0.0, "normal",
                    "4000 mats, 90% M,N,K~U{8..64}, 10% U{512..2048}, N(0,1), alpha=1, beta=0",
                    {"n_big": int(big.sum())})


def uneven_m(seed: int = 0) -> Workload:
    """128 matrices with N = K = 1024 and M ~ Zipf(1.2) clipped to [1, 8192]."""
    rng = np.random.default_rng(seed)
    M = np.clip(rng.zipf(1.2, 128), 1, 8192)
    return Workload("uneven_m_128", M.tolist(), [1024] * 128, [1024] * 128, 1.0, 0.0,
                    "uniform", "128 mats, N=K=1024, M=clip(Zipf(1.2),1,8192), U[-1,1]")


def stream_batches(seed: int = 0, n_batches: int = 200) -> List[Workload]:
    """200 batches of U{64..1024} matrices, M, N, K log-uniform in [1, 4096], alpha = beta = 1."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(n_batches):
        n = int(rng.integers(64, 1025))
        M, N, K = (_log_uniform_int(rng, 1, 4096, n) for _ in range(3))
        out.append(Workload("stream_%03d" % b, M.tolist(), N.tolist(), K.tolist(), 1.0, 1.0,
                            "uniform", "stream batch %d" % b))
    return out


def ref_dataset(batch: int) -> Workload:
    """First `batch` rows of the reference's shape fixture; C += A*B as the reference does."""
    shapes = np.load(os.path.join(ROOT, "tests", "golden", "ref_dataset_shapes.npy")).astype(
        np.int64)
    s = shapes[:batch]
    return Workload("ref_dataset_%d" % batch, s[:, 0].tolist(), s[:, 1].tolist(),
                    s[:, 2].tolist(), 1.0, 1.0, "uniform",
                    "first %d rows of data_MN_K_512_128" % batch)


CONFIGS = {
    "plain_fp32_256": plain_fp32,
    "simt_at_scale_2048": simt_at_scale,
    "skewed_4000": skewed,
    "uneven_m_128": uneven_m,
}
