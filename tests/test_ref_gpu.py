"""The reference framework's own GPU kernel on the GB300, beside the drop-in.

oracle/_ref/ref_framework.cubin is the reference's CUDA/framework/kernel.h
compiled unchanged for sm_103a (oracle/ref_gpu/).  The test loads it with the
driver API and launches the reference's `gemm` kernel (kernel.h:11) the way
the reference's host code does (gemm.cu:181-200: a dense grid of
(max tiles along M, max tiles along N, batch) blocks, 16 KB of dynamic shared
memory), every matrix on the reference's column-major tile strategy 2
(32 x 32, kernel_128_new.h:131).  The other strategies mix row- and
column-major indexing as shipped, so they are not run.  Strategy 2 needs M and
N multiples of 32 and K a multiple of 8, and uses 128 of the block's threads:
the launch gives it exactly 128 threads, so every thread reaches its barriers.

The drop-in bgemm_framework_gemm must produce the same C, bit for bit, from
the same device arrays (the GPU pin of the oracle's fma order), and the
timings of both are printed (informational).
"""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_framework.cubin")
GEMM_SYMBOL = b"_Z4gemmPiS_S_PPfS1_S1_S_"  # gemm(int*, int*, int*, float**, float**, float**, int*)


class RefKernel:
    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        rc = self.cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode())
        assert rc == 0, "cuModuleLoad: %d" % rc
        self.fn = ctypes.c_void_p()
        rc = self.cu.cuModuleGetFunction(ctypes.byref(self.fn), self.mod, GEMM_SYMBOL)
        assert rc == 0, "cuModuleGetFunction: %d" % rc

    def launch(self, grid, dM, dN, dK, dA, dB, dC, dT, stream=0):
        args = [ctypes.c_void_p(x) for x in (dM, dN, dK, dA, dB, dC, dT)]
        params = (ctypes.c_void_p * 7)(*[ctypes.cast(ctypes.pointer(a), ctypes.c_void_p)
                                         for a in args])
        rc = self.cu.cuLaunchKernel(self.fn, ctypes.c_uint(grid[0]), ctypes.c_uint(grid[1]),
                                    ctypes.c_uint(grid[2]), ctypes.c_uint(128), ctypes.c_uint(1),
                                    ctypes.c_uint(1), ctypes.c_uint(4 * 4 * 128 * 8),
                                    ctypes.c_void_p(stream), params, None)
        assert rc == 0, "cuLaunchKernel: %d" % rc

    def close(self):
        self.cu.cuModuleUnload(self.mod)


@pytest.fixture(scope="module")
def ref_kernel(cuda):
    if not os.path.exists(CUBIN):
        pytest.skip("reference cubin not built (needs the reference checkout at build time)")
    torch.zeros(1, device="cuda")  # the runtime's primary context is current
    k = RefKernel()
    yield k
    k.close()


def batch_arrays(M, N, K, seed):
    rng = np.random.default_rng(seed)
    dev = "cuda"
    bufs = {}
    for name, rows, cols in (("A", M, K), ("B", K, N), ("C", M, N)):
        sizes = [r * c for r, c in zip(rows, cols)]
        offs = np.concatenate([[0], np.cumsum([(s + 3) // 4 * 4 for s in sizes])[:-1]]).astype(int)
        host = rng.uniform(-1, 1, int(offs[-1] + sizes[-1] + 4)).astype(np.float32)
        buf = torch.from_numpy(host).to(dev)
        ptrs = torch.tensor([buf.data_ptr() + 4 * int(o) for o in offs], dtype=torch.int64,
                            device=dev)
        bufs[name] = (buf, ptrs)
    ints = {k: torch.tensor(v, dtype=torch.int32, device=dev) for k, v in
            (("M", M), ("N", N), ("K", K), ("T", [2] * len(M)))}
    return bufs, ints


def shapes(seed, n):
    rng = np.random.default_rng(seed)
    M = (rng.integers(1, 17, n) * 32).tolist()
    N = (rng.integers(1, 17, n) * 32).tolist()
    K = (rng.integers(1, 65, n) * 8).tolist()
    return M, N, K


def run_both(ref, M, N, K, seed):
    bufs, ints = batch_arrays(M, N, K, seed)
    C0 = bufs["C"][0].clone()
    grid = (max(m // 32 for m in M), max(n // 32 for n in N), len(M))
    ref.launch(grid, ints["M"].data_ptr(), ints["N"].data_ptr(), ints["K"].data_ptr(),
               bufs["A"][1].data_ptr(), bufs["B"][1].data_ptr(), bufs["C"][1].data_ptr(),
               ints["T"].data_ptr())
    torch.cuda.synchronize()
    c_ref = bufs["C"][0].clone()
    bufs["C"][0].copy_(C0)
    bg.framework_gemm(ints["M"].data_ptr(), ints["N"].data_ptr(), ints["K"].data_ptr(),
                      bufs["A"][1].data_ptr(), bufs["B"][1].data_ptr(), bufs["C"][1].data_ptr(),
                      len(M), max(max(M), max(N)))
    torch.cuda.synchronize()
    bg.framework_check_device()
    return c_ref, bufs["C"][0].clone(), bufs, ints, grid, C0


def test_reference_kernel_matches_drop_in_bit_for_bit(ref_kernel):
    for seed, n in ((1, 8), (2, 64), (3, 256)):
        M, N, K = shapes(seed, n)
        c_ref, c_ours, *_ = run_both(ref_kernel, M, N, K, seed)
        a = c_ref.cpu().numpy().view(np.uint32)
        b = c_ours.cpu().numpy().view(np.uint32)
        bad = np.nonzero(a != b)[0]
        assert bad.size == 0, "batch %d: %d words differ" % (n, bad.size)


def test_reference_kernel_timing(ref_kernel):
    """Informational: the reference's dense-grid kernel vs the persistent
    drop-in on the same arrays (printed, not asserted)."""
    M, N, K = shapes(5, 2048)
    _, _, bufs, ints, grid, _ = run_both(ref_kernel, M, N, K, 5)
    flops = sum(2.0 * m * n * k for m, n, k in zip(M, N, K))
    e = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    reps = 10
    e[0].record()
    for _ in range(reps):
        ref_kernel.launch(grid, ints["M"].data_ptr(), ints["N"].data_ptr(), ints["K"].data_ptr(),
                          bufs["A"][1].data_ptr(), bufs["B"][1].data_ptr(),
                          bufs["C"][1].data_ptr(), ints["T"].data_ptr())
    e[1].record()
    e[2].record()
    for _ in range(reps):
        bg.framework_gemm(ints["M"].data_ptr(), ints["N"].data_ptr(), ints["K"].data_ptr(),
                          bufs["A"][1].data_ptr(), bufs["B"][1].data_ptr(),
                          bufs["C"][1].data_ptr(), len(M), max(max(M), max(N)))
    e[3].record()
    torch.cuda.synchronize()
    t_ref = e[0].elapsed_time(e[1]) / reps
    t_ours = e[2].elapsed_time(e[3]) / reps
    print("\nreference gemm (strategy 2): %.3f ms = %.2f TFLOP/s; drop-in: %.3f ms = %.2f TFLOP/s"
          % (t_ref, flops / t_ref / 1e9, t_ours, flops / t_ours / 1e9))


def _time(fn, reps=20, rounds=5, sync_each=False):
    """Median over `rounds` of the mean ms of `reps` calls (after a warm-up),
    CUDA events on the current stream; sync_each mirrors the reference's timed
    loop, which synchronises the device after every launch
    (CUDA/framework/gemm.cu:203-214).  Calls of tens of microseconds vary a
    lot from one round to the next, hence the median."""
    fn()
    torch.cuda.synchronize()
    out = []
    for _ in range(rounds):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
            if sync_each:
                torch.cuda.synchronize()
        e1.record()
        torch.cuda.synchronize()
        out.append(e0.elapsed_time(e1) / reps)
    return sorted(out)[len(out) // 2]


def test_reference_sweep_table(ref_kernel):
    """Informational: the reference's published sweep (CUDA/framework/run.sh:
    14-24, ./gemm B 512 6000 for B = 8 .. 256 over the first B rows of
    data_MN_K_512_128; log-test-verify3:1-6) on this GPU.  GFLOP/s count
    sum(2MNK + 2MN) as the reference does (gemm.cu:84-85), 10 launches each.

    Columns: the reference kernel on strategy-2-compatible shapes (M, N of
    the shape file rounded up to multiples of 32; its other tile bodies are
    wrong as shipped and are not run), timed like the reference (device sync
    after every launch) and back to back; the drop-in bgemm_framework_gemm
    on the same arrays; the drop-in and the 3xTF32 mode on the shape file's
    own sizes (C += A B)."""
    from batchgemm_gb300 import workloads
    rows = []
    for B in (8, 16, 32, 64, 128, 256):
        w = workloads.ref_dataset(B)
        M32 = [(m + 31) // 32 * 32 for m in w.M]
        N32 = [(n + 31) // 32 * 32 for n in w.N]
        fl32 = sum(2.0 * m * n * k + 2.0 * m * n for m, n, k in zip(M32, N32, w.K))
        bufs, ints = batch_arrays(M32, N32, w.K, B)
        grid = (max(m // 32 for m in M32), max(n // 32 for n in N32), B)
        args = (ints["M"].data_ptr(), ints["N"].data_ptr(), ints["K"].data_ptr(),
                bufs["A"][1].data_ptr(), bufs["B"][1].data_ptr(), bufs["C"][1].data_ptr())
        ref = lambda: ref_kernel.launch(grid, *args, ints["T"].data_ptr())
        ours = lambda: bg.framework_gemm(*args, B, max(max(M32), max(N32)))
        t_ref_sync = _time(ref, sync_each=True)
        t_ref = _time(ref)
        t_ours32 = _time(ours)
        # the shape file's own sizes
        fl = sum(2.0 * m * n * k + 2.0 * m * n for m, n, k in zip(w.M, w.N, w.K))
        bufs2, ints2 = batch_arrays(w.M, w.N, w.K, B + 1)
        args2 = (ints2["M"].data_ptr(), ints2["N"].data_ptr(), ints2["K"].data_ptr(),
                 bufs2["A"][1].data_ptr(), bufs2["B"][1].data_ptr(), bufs2["C"][1].data_ptr())
        t_ours = _time(lambda: bg.framework_gemm(*args2, B, max(max(w.M), max(w.N))))
        ld = lambda v: bg.int_array([max(1, x) for x in v])
        Mi, Ni, Ki = bg.int_array(w.M), bg.int_array(w.N), bg.int_array(w.K)
        lda, ldb = ld(w.M), ld(w.K)
        t_x3 = _time(lambda: bg.sgemm_vbatched(Mi, Ni, Ki, 1.0, args2[3], lda, args2[4], ldb,
                                               1.0, args2[5], lda, mode="tf32x3"))
        bg.framework_check_device()
        rows.append((B, fl32 / t_ref_sync / 1e6, fl32 / t_ref / 1e6, fl32 / t_ours32 / 1e6,
                     fl / t_ours / 1e6, fl / t_x3 / 1e6))
    print("\nSWEEP | B | ref kernel s2, sync each | ref kernel s2 | drop-in (same) | "
          "drop-in, file shapes | 3xTF32, file shapes |  (GFLOP/s, sum 2MNK + 2MN)")
    for r in rows:
        print("SWEEP | %d | %.1f | %.1f | %.1f | %.1f | %.1f |" % r)
