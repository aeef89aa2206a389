"""CPU oracle for column-major variable-size batched SGEMM.

TEST INFRASTRUCTURE ONLY.  The tests, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` use it as the checker; the library never
imports it and has no CPU fallback.

The C restatement lives in ``oracle.c`` (semantics and reference citations in
its header).  ``build()`` compiles it with gcc into ``oracle/_build``;
``build_ref_emul()`` compiles the reference's own tile bodies into
``oracle/_ref/ref_emul`` when the reference checkout is present (golden-vector
generation only); ``build_ref_gpu()`` compiles the reference's GPU kernels
unchanged into ``oracle/_ref/ref_framework.cubin`` (GPU parity and timing).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build", __import__("platform").machine())
LIB_PATH = os.path.join(BUILD_DIR, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

MODE_SIMT_FP32, MODE_TF32, MODE_TF32X3, MODE_BF16X3 = 0, 1, 2, 3

_lib: Optional[ctypes.CDLL] = None


def build(force: bool = False) -> str:
    """Compile oracle.c into a shared library (gcc, no CUDA)."""
    src = os.path.join(HERE, "oracle.c")
    hdr = os.path.join(HERE, "oracle.h")
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= max(os.path.getmtime(src), os.path.getmtime(hdr))):
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    cmd = ["gcc", "-O3", "-std=c11", "-shared", "-fPIC", "-ffp-contract=off",
           "-fno-fast-math", "-pthread", src, "-o", tmp, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def reference_root() -> str:
    """Where the BatchGEMM reference checkout is read from when the test
    infrastructure builds from it: $BGEMM_REFERENCE_DIR, else the build
    container's read-only checkout.  It is absent on machines that only run
    the prebuilt files."""
    return os.environ.get("BGEMM_REFERENCE_DIR", "/root/reference")


def build_ref_emul(ref_root: Optional[str] = None) -> Optional[str]:
    """Build the reference-emulation binary (only where the reference exists)."""
    ref_root = ref_root or reference_root()
    if not os.path.isdir(os.path.join(ref_root, "CUDA", "batching")):
        return None
    subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref_emul"), "REF=" + ref_root,
                    "OUT=" + REF_DIR], check=True)
    return os.path.join(REF_DIR, "ref_emul")


def build_ref_gpu(ref_root: Optional[str] = None) -> Optional[str]:
    """Build the reference framework kernels' cubin (only where the reference
    exists); returns its path, or the prebuilt one, or None."""
    ref_root = ref_root or reference_root()
    out = os.path.join(REF_DIR, "ref_framework.cubin")
    if os.path.isdir(os.path.join(ref_root, "CUDA", "framework")):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref_gpu"), "REF=" + ref_root,
                        "OUT=" + REF_DIR], check=True)
    return out if os.path.exists(out) else None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        fp = ctypes.POINTER(ctypes.c_float)
        dp = ctypes.POINTER(ctypes.c_double)
        i = ctypes.c_int
        L.bgo_sgemm_f32.argtypes = [i, i, i, ctypes.c_float, fp, i, fp, i, ctypes.c_float, fp, i]
        L.bgo_sgemm_f64.argtypes = [i, i, i, ctypes.c_double, fp, i, fp, i, ctypes.c_double, fp,
                                    i, dp, dp]
        L.bgo_round_tf32.argtypes = [ctypes.c_float]
        L.bgo_round_tf32.restype = ctypes.c_float
        L.bgo_round_bf16.argtypes = [ctypes.c_float]
        L.bgo_round_bf16.restype = ctypes.c_float
        L.bgo_split.argtypes = [i, fp, ctypes.c_size_t, fp, fp]
        L.bgo_sgemm_split_f64.argtypes = [i, i, i, i, ctypes.c_double, fp, i, fp, i,
                                          ctypes.c_double, fp, i, dp]
        pp = ctypes.POINTER(fp)
        ip = ctypes.POINTER(ctypes.c_int)
        L.bgo_vbatched_f32.argtypes = [i, ip, ip, ip, ctypes.c_float, pp, ip, pp, ip,
                                       ctypes.c_float, pp, ip, i]
        L.bgo_vbatched_f32.restype = ctypes.c_int
        _lib = L
    return _lib


def _fp(a: np.ndarray):
    assert a.dtype == np.float32 and (a.flags["C_CONTIGUOUS"] or a.flags["F_CONTIGUOUS"])
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dp(a: Optional[np.ndarray]):
    if a is None:
        return None
    assert a.dtype == np.float64
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# Matrices are passed as flat float32 buffers holding column-major data
# (element (r, c) at buf[r + c*ld]).

def sgemm_f32(M, N, K, alpha, A, lda, B, ldb, beta, C, ldc) -> np.ndarray:
    """C <- alpha*A*B + beta*C in FP32 with the reference's fma order (in place)."""
    lib().bgo_sgemm_f32(M, N, K, alpha, _fp(A), lda, _fp(B), ldb, beta, _fp(C), ldc)
    return C


def sgemm_f64(M, N, K, alpha, A, lda, B, ldb, beta, C0, ldc, want_bound=True):
    """Returns (C64, bound): FP64 result (M x N, ld = M, flat) and
    |alpha|*sum|a||b| + |beta*c0| per element."""
    C64 = np.zeros(max(M * N, 1), np.float64)
    bound = np.zeros(max(M * N, 1), np.float64) if want_bound else None
    c0 = C0 if C0 is not None else np.zeros(1, np.float32)
    lib().bgo_sgemm_f64(M, N, K, alpha, _fp(A), lda, _fp(B), ldb, beta, _fp(c0), ldc,
                        _dp(C64), _dp(bound))
    return C64[:M * N], (bound[:M * N] if bound is not None else None)


def sgemm_split_f64(mode, M, N, K, alpha, A, lda, B, ldb, beta, C0, ldc) -> np.ndarray:
    C64 = np.zeros(max(M * N, 1), np.float64)
    c0 = C0 if C0 is not None else np.zeros(1, np.float32)
    lib().bgo_sgemm_split_f64(mode, M, N, K, alpha, _fp(A), lda, _fp(B), ldb, beta, _fp(c0),
                              ldc, _dp(C64))
    return C64[:M * N]


def split(mode: int, x: np.ndarray):
    x = np.ascontiguousarray(x, dtype=np.float32).reshape(-1)
    hi = np.empty_like(x)
    lo = np.empty_like(x)
    lib().bgo_split(mode, _fp(x), x.size, _fp(hi), _fp(lo))
    return hi, lo


def vbatched_f32(Ms: Sequence[int], Ns: Sequence[int], Ks: Sequence[int], alpha: float,
                 As, ldas, Bs, ldbs, beta: float, Cs, ldcs, nthreads: int = 1) -> int:
    """Batched FP32 oracle over a thread pool (largest matrix first). Returns threads used."""
    n = len(Ms)
    ia = lambda v: (ctypes.c_int * n)(*[int(x) for x in v])
    pa = lambda v: (ctypes.POINTER(ctypes.c_float) * n)(*[_fp(x) for x in v])
    return lib().bgo_vbatched_f32(n, ia(Ms), ia(Ns), ia(Ks), alpha, pa(As), ia(ldas), pa(Bs),
                                  ia(ldbs), beta, pa(Cs), ia(ldcs), nthreads)


def normalized_error(C: np.ndarray, C64: np.ndarray, bound: np.ndarray):
    """Per-element |c - c64| / (|alpha| sum|a||b| + |beta c0|) (0 where the bound is 0)."""
    err = np.abs(C.astype(np.float64) - C64)
    den = np.where(bound > 0, bound, 1.0)
    e = np.where(bound > 0, err / den, err)
    return e
