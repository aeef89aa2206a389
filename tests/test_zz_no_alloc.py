"""bgemm_framework_gemm_noalloc, the allocation-free variant of the device-queue
FP32 entry point.

Some callers cannot allocate device memory while they run: a real-time loop
that must not risk the device-wide synchronisation an allocation can cause,
or a plug-in whose host application owns the device memory budget through its
own pool.  For them the library keeps the tile queue in a fixed __device__
array instead of allocating it.  This file checks, through the C ABI, that two
calls in a row give the same bits as the regular entry point (the FP32 SIMT
tests' tolerance is bit-exactness), and that calls beyond the array's limits
are refused before any work.  It is named to run last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
from batchgemm_gb300 import workloads  # noqa: E402
from gpu_util import make_batch, oracle_batch, assert_bits_equal  # noqa: E402


def _dev(v):
    return torch.tensor(v, dtype=torch.int32, device="cuda")


def test_noalloc_matches_regular_entry_twice(cuda):
    L = bg.lib()
    w = workloads.ref_dataset(64)  # the reference's own shapes, sizes up to 512
    rng = np.random.default_rng(5)
    M = w.M + rng.integers(1, 200, 16).tolist()
    N = w.N + rng.integers(1, 200, 16).tolist()
    K = w.K + rng.integers(0, 200, 16).tolist()
    db, host = make_batch(M, N, K, seed=9)
    dM, dN, dK = _dev(M), _dev(N), _dev(K)
    n = len(M)
    want = oracle_batch(db, host, 1.0, 1.0)

    # the regular entry point
    st = L.bgemm_framework_gemm(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(), db.pA.data_ptr(),
                                db.pB.data_ptr(), db.pC.data_ptr(), None, n, 512, None)
    assert st == 0
    torch.cuda.synchronize()
    regular = db.C.cpu().numpy()
    assert_bits_equal(regular, want, "regular entry")

    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    for call in range(2):  # the shared array keeps the last call's contents
        db.C.copy_(torch.from_numpy(host[2]))
        st = L.bgemm_framework_gemm_noalloc(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(),
                                            db.pA.data_ptr(), db.pB.data_ptr(),
                                            db.pC.data_ptr(), n, 512, info.data_ptr(), None)
        assert st == 0, bg.lib().bgemm_last_error_message()
        torch.cuda.synchronize()
        assert_bits_equal(db.C.cpu().numpy(), regular, "no-alloc call %d" % call)
    assert int(info.item()) == 0


def test_noalloc_refuses_sizes_beyond_its_array(cuda):
    L = bg.lib()
    d = _dev([1])
    # more matrices than the array holds
    st = L.bgemm_framework_gemm_noalloc(d.data_ptr(), d.data_ptr(), d.data_ptr(), 1, 1, 1,
                                        5000, 16, None, None)
    assert st == 2
    assert b"4096" in L.bgemm_last_error_message()
    # worst-case tile count beyond the array
    st = L.bgemm_framework_gemm_noalloc(d.data_ptr(), d.data_ptr(), d.data_ptr(), 1, 1, 1,
                                        64, 4096, None, None)
    assert st == 2
    assert b"262144" in L.bgemm_last_error_message()


def test_noalloc_reports_oversized_matrix(cuda):
    L = bg.lib()
    db, host = make_batch([8, 40], [8, 40], [8, 8], seed=1)
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    dM, dN, dK = _dev([8, 40]), _dev([8, 40]), _dev([8, 8])  # keep them alive
    st = L.bgemm_framework_gemm_noalloc(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(),
                                        db.pA.data_ptr(), db.pB.data_ptr(), db.pC.data_ptr(), 2,
                                        32, info.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    assert int(info.item()) & 1  # 40 > max_dim: skipped and flagged
    want = oracle_batch(db, host, 1.0, 1.0)
    got = db.C.cpu().numpy()
    assert_bits_equal(got[db.offC[0]:db.offC[0] + 64], want[db.offC[0]:db.offC[0] + 64], "m0")
    assert_bits_equal(got[db.offC[1]:db.offC[1] + 1600], host[2][db.offC[1]:db.offC[1] + 1600],
                      "skipped matrix untouched")
