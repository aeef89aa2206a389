"""bgemm_framework_gemm_mode: the device-size entry (the reference framework
kernel's arguments, C_i += A_i B_i column-major, lda = M_i, ldb = K_i,
ldc = M_i) in the tensor-core modes, where tile choice, queue, split-operand
workspace, pre-pass strips and tensor maps are all built on the device.

Each case is checked against the FP64 oracle with the sqrt(K)-scaled bound of
its mode; the SIMT mode must equal bgemm_framework_gemm bit for bit.  A
captured graph replays with new sizes written into the device arrays, and
sizes outside max_dim / max_k are skipped and reported.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
from gpu_util import make_batch, oracle_batch, assert_bits_equal, f64_check  # noqa: E402

FP64_BOUND = {"tf32x3": (32.0, 2.0 ** -24), "bf16x3": (8.0, 2.0 ** -16),
              "tf32": (4.0, 2.0 ** -11)}


def dev(v):
    return torch.tensor(v, dtype=torch.int32, device="cuda")


def shapes(seed, n, max_dim=700, max_k=900):
    rng = np.random.default_rng(seed)
    M = np.exp(rng.uniform(0, np.log(max_dim), n)).astype(int).tolist()
    N = np.exp(rng.uniform(0, np.log(max_dim), n)).astype(int).tolist()
    K = np.exp(rng.uniform(0, np.log(max_k), n)).astype(int).tolist()
    # empty, K = 0, one row / column, swapped-operand shapes, the limits
    M[:7] = [0, 12, 1, max_dim, 3, max_dim, 65]
    N[:7] = [9, 40, max_dim, 1, max_dim - 60, max_dim, 0]
    K[:7] = [5, 0, 300, 77, max_k, max_k, 8]
    return M, N, K


def run(db, M, N, K, max_dim, max_k, mode, stream=None):
    dM, dN, dK = dev(M), dev(N), dev(K)
    bg.framework_gemm_mode(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(), db.pA.data_ptr(),
                           db.pB.data_ptr(), db.pC.data_ptr(), len(M), max_dim, max_k, mode,
                           stream=stream)
    return dM, dN, dK


@pytest.mark.parametrize("mode", ["tf32x3", "bf16x3", "tf32"])
def test_framework_mode_parity(cuda, mode):
    M, N, K = shapes(5 + len(mode), 90)
    db, host = make_batch(M, N, K, seed=17)
    run(db, M, N, K, 700, 900, mode)
    torch.cuda.synchronize()
    bg.framework_check_device()
    factor, unit = FP64_BOUND[mode]
    worst, mean = f64_check(db, host, db.C.cpu().numpy(), 1.0, 1.0, factor, unit)
    print("\n%s: max err %.3g, mean %.3g" % (mode, worst, mean))
    # a second call runs on the same scratch (queue counters reset themselves)
    db.C.copy_(torch.from_numpy(host[2]))
    run(db, M, N, K, 700, 900, mode)
    torch.cuda.synchronize()
    bg.framework_check_device()
    f64_check(db, host, db.C.cpu().numpy(), 1.0, 1.0, factor, unit)


def test_framework_mode_simt_is_the_drop_in(cuda):
    M, N, K = shapes(3, 40, max_dim=300, max_k=300)
    db, host = make_batch(M, N, K, seed=4)
    run(db, M, N, K, 300, 300, "simt")
    torch.cuda.synchronize()
    bg.framework_check_device()
    assert_bits_equal(db.C.cpu().numpy(), oracle_batch(db, host, 1.0, 1.0), "simt mode")


@pytest.mark.parametrize("mode", ["tf32x3", "bf16x3"])
def test_framework_mode_graph_replay_with_new_sizes(cuda, mode):
    """One capture; every replay reads whatever the size and pointer arrays
    hold.  The first call (outside capture) sizes the library's scratch."""
    n_cap = 64
    s = torch.cuda.Stream()
    dM, dN, dK = (torch.zeros(n_cap, dtype=torch.int32, device="cuda") for _ in range(3))
    pA, pB, pC = (torch.zeros(n_cap, dtype=torch.int64, device="cuda") for _ in range(3))
    args = lambda: (dM.data_ptr(), dN.data_ptr(), dK.data_ptr(), pA.data_ptr(), pB.data_ptr(),
                    pC.data_ptr(), n_cap, 512, 512, mode)

    def load(seed, n):
        M, N, K = shapes(seed, n, max_dim=512, max_k=512)
        # the tail of the arrays holds empty matrices
        M, N, K = M + [0] * (n_cap - n), N + [0] * (n_cap - n), K + [0] * (n_cap - n)
        db, host = make_batch(M, N, K, seed=seed)
        with torch.cuda.stream(s):
            dM.copy_(dev(M))
            dN.copy_(dev(N))
            dK.copy_(dev(K))
            pA.copy_(db.pA)
            pB.copy_(db.pB)
            pC.copy_(db.pC)
        return db, host

    db0, host0 = load(50, 30)
    with torch.cuda.stream(s):
        bg.framework_gemm_mode(*args(), stream=s)
    s.synchronize()
    bg.framework_check_device()
    factor, unit = FP64_BOUND[mode]
    f64_check(db0, host0, db0.C.cpu().numpy(), 1.0, 1.0, factor, unit)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        bg.framework_gemm_mode(*args(), stream=s)
    for seed, n in ((51, 64), (52, 7), (53, 40)):
        db, host = load(seed, n)
        with torch.cuda.stream(s):
            g.replay()
        s.synchronize()
        bg.framework_check_device()
        f64_check(db, host, db.C.cpu().numpy(), 1.0, 1.0, factor, unit)


def test_framework_mode_rejects_oversized_on_device(cuda):
    M, N, K = [40, 20, 30], [33, 20, 30], [17, 20, 30]
    db, host = make_batch(M, N, K, seed=8)
    before = [db.c(i).clone() for i in range(3)]
    bad_M, bad_K = [40, 200, 30], [17, 20, 900]  # matrix 1: M > max_dim; matrix 2: K > max_k
    run(db, bad_M, N, bad_K, 64, 64, "tf32x3")
    torch.cuda.synchronize()
    with pytest.raises(bg.BgemmError) as ei:
        bg.framework_check_device()
    assert ei.value.status == 1
    bg.framework_check_device()  # the flag is cleared once reported
    for i in (1, 2):  # skipped matrices are untouched
        assert torch.equal(db.c(i), before[i])
    # matrix 0 was computed
    want = before[0].double() + db.a(0).double() @ db.b(0).double()
    assert torch.allclose(db.c(0).double(), want, rtol=0, atol=1e-5)


def test_framework_mode_argument_errors(cuda):
    z = dev([1])
    p = torch.zeros(1, dtype=torch.int64, device="cuda")
    ptrs = (z.data_ptr(),) * 3 + (p.data_ptr(),) * 3
    with pytest.raises(bg.BgemmError) as ei:
        bg.framework_gemm_mode(*ptrs, 1, 0, 16, "tf32x3")
    assert (ei.value.status, ei.value.arg) == (1, 8)
    with pytest.raises(bg.BgemmError) as ei:
        bg.framework_gemm_mode(*ptrs, 1, 16, 0, "tf32x3")
    assert (ei.value.status, ei.value.arg) == (1, 9)
    with pytest.raises(bg.BgemmError) as ei:
        bg.framework_gemm_mode(*ptrs, 1, 16, 16, "tf32x3", max_operand_elems=-1)
    assert (ei.value.status, ei.value.arg) == (1, 10)
    with pytest.raises(bg.BgemmError) as ei:
        bg.framework_gemm_mode(*ptrs, 1, 16, 16, 7)
    assert (ei.value.status, ei.value.arg) == (1, 11)
    bg.framework_gemm_mode(*ptrs, 0, 16, 16, "tf32x3")  # empty batch: nothing to do


def test_framework_mode_operand_bound(cuda):
    """max_operand_elems sizes the split-operand workspace from the batch's
    actual sum of (M + N) * K instead of the batch * max_dim * max_k worst
    case; a batch above the bound is not computed and is reported."""
    M, N, K = shapes(77, 60, max_dim=600, max_k=800)
    elems = sum((m + n) * k for m, n, k in zip(M, N, K))
    db, host = make_batch(M, N, K, seed=31)
    dM, dN, dK = dev(M), dev(N), dev(K)
    call = lambda e: bg.framework_gemm_mode(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(),
                                            db.pA.data_ptr(), db.pB.data_ptr(),
                                            db.pC.data_ptr(), len(M), 600, 800, "tf32x3",
                                            max_operand_elems=e)
    call(elems)
    torch.cuda.synchronize()
    bg.framework_check_device()
    f64_check(db, host, db.C.cpu().numpy(), 1.0, 1.0, *FP64_BOUND["tf32x3"])
    # scratch released, then sized for a tenth of the batch: nothing computed
    bg.framework_release()
    before = db.C.clone()
    bg.framework_gemm_mode(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(), db.pA.data_ptr(),
                           db.pB.data_ptr(), db.pC.data_ptr(), len(M), 600, 800, "bf16x3",
                           max_operand_elems=elems // 10)
    torch.cuda.synchronize()
    with pytest.raises(bg.BgemmError) as ei:
        bg.framework_check_device()
    assert ei.value.status == 2
    assert torch.equal(db.C.isnan(), before.isnan())
    assert torch.equal(torch.nan_to_num(db.C), torch.nan_to_num(before))
    bg.framework_release()  # the next call sizes the scratch again
    db.C.copy_(torch.from_numpy(host[2]))
    call(elems)
    torch.cuda.synchronize()
    bg.framework_check_device()
    f64_check(db, host, db.C.cpu().numpy(), 1.0, 1.0, *FP64_BOUND["tf32x3"])
