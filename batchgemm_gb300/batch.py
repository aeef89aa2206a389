"""Device storage of a batch of column-major matrices (PyTorch as the allocator).

All A matrices of a batch live in one flat float32 device buffer, likewise B
and C; each matrix starts at a 16-byte boundary plus an optional offset (so
tests can force misaligned operands).  The device arrays of per-matrix
pointers that the C ABI takes are int64 tensors.  Column padding (ld > rows)
and a guard band after every matrix are filled with NaN so tests can prove
that nothing outside a matrix is read into or written.
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np

try:
    import torch
except ImportError:  # the CPU-only tests do not need torch
    torch = None

from . import sgemm_vbatched, Plan, MODES

GUARD = 16  # floats of NaN after every matrix


def _layout(rows: Sequence[int], cols: Sequence[int], ld: Sequence[int], align: int,
            offset: int):
    offs, cur = [], 0
    for r, c, l in zip(rows, cols, ld):
        cur = (cur + align - 1) // align * align + offset
        offs.append(cur)
        cur += (l * c if (r > 0 and c > 0) else 0) + GUARD
    return offs, cur + align


class DeviceBatch:
    def __init__(self, M, N, K, lda=None, ldb=None, ldc=None, offset_floats: int = 0,
                 device: str = "cuda"):
        self.M = [int(x) for x in M]
        self.N = [int(x) for x in N]
        self.K = [int(x) for x in K]
        n = len(self.M)
        self.lda = [max(1, m) for m in self.M] if lda is None else [int(x) for x in lda]
        self.ldb = [max(1, k) for k in self.K] if ldb is None else [int(x) for x in ldb]
        self.ldc = [max(1, m) for m in self.M] if ldc is None else [int(x) for x in ldc]
        self.device = device
        self.offA, na = _layout(self.M, self.K, self.lda, 4, offset_floats)
        self.offB, nb = _layout(self.K, self.N, self.ldb, 4, offset_floats)
        self.offC, nc = _layout(self.M, self.N, self.ldc, 4, offset_floats)
        nan = float("nan")
        self.A = torch.full((na,), nan, dtype=torch.float32, device=device)
        self.B = torch.full((nb,), nan, dtype=torch.float32, device=device)
        self.C = torch.full((nc,), nan, dtype=torch.float32, device=device)
        self._ptrs()
        self.batch = n

    def _ptrs(self):
        bA, bB, bC = self.A.data_ptr(), self.B.data_ptr(), self.C.data_ptr()
        self.pA = torch.tensor([bA + 4 * o for o in self.offA], dtype=torch.int64,
                               device=self.device)
        self.pB = torch.tensor([bB + 4 * o for o in self.offB], dtype=torch.int64,
                               device=self.device)
        self.pC = torch.tensor([bC + 4 * o for o in self.offC], dtype=torch.int64,
                               device=self.device)

    # -- views ------------------------------------------------------------
    @staticmethod
    def _view(buf, off, rows, cols, ld):
        """(rows x cols) column-major view: element (r, c) at buf[off + r + c*ld]."""
        if rows == 0 or cols == 0:
            return torch.empty((rows, cols), dtype=buf.dtype, device=buf.device)
        return buf[off:off + ld * cols].view(cols, ld)[:, :rows].t()

    def a(self, i):
        return self._view(self.A, self.offA[i], self.M[i], self.K[i], self.lda[i])

    def b(self, i):
        return self._view(self.B, self.offB[i], self.K[i], self.N[i], self.ldb[i])

    def c(self, i):
        return self._view(self.C, self.offC[i], self.M[i], self.N[i], self.ldc[i])

    # -- filling ----------------------------------------------------------
    def fill(self, dist: str = "uniform", seed: int = 0, c0: bool = True) -> "DeviceBatch":
        """Fill every matrix (not the padding) from a seeded device generator."""
        g = torch.Generator(device=self.device)
        g.manual_seed(seed)
        for which, views in (("A", self.a), ("B", self.b), ("C", self.c)):
            if which == "C" and not c0:
                continue
            for i in range(self.batch):
                v = views(i)
                if v.numel() == 0:
                    continue
                if dist == "normal":
                    v.copy_(torch.randn(v.shape, generator=g, device=self.device))
                else:
                    v.copy_(torch.rand(v.shape, generator=g, device=self.device) * 2 - 1)
        return self

    def fill_fast(self, dist: str = "uniform", seed: int = 0) -> "DeviceBatch":
        """Fill whole buffers at once (padding included) -- for large benchmark batches."""
        g = torch.Generator(device=self.device)
        g.manual_seed(seed)
        for buf in (self.A, self.B, self.C):
            if dist == "normal":
                buf.normal_(generator=g)
            else:
                buf.uniform_(-1, 1, generator=g)
        return self

    def set_from_numpy(self, As, Bs, Cs) -> "DeviceBatch":
        """Copies in matrices given as 2-D arrays or flat column-major (ld = rows) data."""
        for i in range(self.batch):
            for v, arr in ((self.a(i), As[i]), (self.b(i), Bs[i]), (self.c(i), Cs[i])):
                if v.numel():
                    a = np.asarray(arr, np.float32)
                    if a.ndim == 1:
                        a = a.reshape(v.shape[1], v.shape[0]).T
                    v.copy_(torch.from_numpy(np.ascontiguousarray(a)).to(self.device))
        return self

    # -- running ----------------------------------------------------------
    def run(self, mode="simt", alpha: float = 1.0, beta: float = 0.0, stream=None) -> None:
        sgemm_vbatched(self.M, self.N, self.K, alpha, self.pA.data_ptr(), self.lda,
                       self.pB.data_ptr(), self.ldb, beta, self.pC.data_ptr(), self.ldc,
                       mode=mode, stream=stream)

    def plan(self, mode="simt", **kw) -> Plan:
        return Plan(self.M, self.N, self.K, self.lda, self.ldb, self.ldc, mode=mode, **kw)

    def execute(self, plan: Plan, alpha=1.0, beta=0.0, stream=None) -> None:
        plan.execute(alpha, self.pA.data_ptr(), self.pB.data_ptr(), beta, self.pC.data_ptr(),
                     stream=stream)

    # -- host copies for the oracle ---------------------------------------
    def host(self):
        """Flat host copies (numpy) of the A, B, C buffers."""
        return (self.A.cpu().numpy(), self.B.cpu().numpy(), self.C.cpu().numpy())
