"""FP32 SIMT path on the GPU: bit-exact with the oracle and with the
reference's own tile-body outputs, called through the C ABI."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
import oracle  # noqa: E402
from batchgemm_gb300 import workloads  # noqa: E402
from gpu_util import make_batch, oracle_batch, assert_bits_equal, f64_check, U  # noqa: E402

EDGE = [1, 2, 3, 7, 8, 9, 15, 16, 17, 31, 33, 63, 65, 127, 129, 200]


def run_case(M, N, K, alpha, beta, offset=0, lda=None, ldb=None, ldc=None, seed=0,
             c_nan=False, dist="uniform"):
    db, host = make_batch(M, N, K, lda, ldb, ldc, offset=offset, seed=seed, c_nan=c_nan,
                          dist=dist)
    want = oracle_batch(db, host, alpha, beta)
    db.run("simt", alpha, beta)
    torch.cuda.synchronize()
    got = db.C.cpu().numpy()
    assert_bits_equal(got, want, "SIMT vs oracle")
    return db


@pytest.mark.parametrize("offset", [0, 1, 2])
@pytest.mark.parametrize("alpha,beta", [(1.0, 0.0), (1.0, 1.0), (0.5, -2.0), (-1.25, 0.5)])
def test_random_edge_shapes(cuda, offset, alpha, beta):
    rng = np.random.default_rng(offset * 10 + int(alpha * 4) + 100)
    n = 48
    M = rng.choice(EDGE, n).tolist()
    N = rng.choice(EDGE, n).tolist()
    K = rng.choice(EDGE + [0], n).tolist()
    run_case(M, N, K, alpha, beta, offset=offset, seed=n)


def test_padded_leading_dimensions(cuda):
    rng = np.random.default_rng(7)
    n = 30
    M = rng.integers(1, 150, n).tolist()
    N = rng.integers(1, 150, n).tolist()
    K = rng.integers(1, 150, n).tolist()
    lda = [m + int(rng.integers(0, 9)) for m in M]
    ldb = [k + int(rng.integers(0, 9)) for k in K]
    ldc = [m + int(rng.integers(0, 9)) for m in M]
    run_case(M, N, K, 0.75, 0.25, lda=lda, ldb=ldb, ldc=ldc)
    # aligned leading dimensions (vector paths) with ragged M
    lda = [(m + 3) // 4 * 4 for m in M]
    ldb = [(k + 3) // 4 * 4 for k in K]
    ldc = [(m + 3) // 4 * 4 for m in M]
    run_case(M, N, K, 1.0, 0.0, lda=lda, ldb=ldb, ldc=ldc)


def test_beta_zero_does_not_read_c(cuda):
    run_case([37, 64, 5], [19, 64, 128], [40, 8, 3], 1.5, 0.0, c_nan=True)


def test_zero_and_empty_matrices(cuda):
    # K = 0 -> C = beta*C (or unchanged in place); M or N = 0 -> nothing
    run_case([4, 0, 9, 5], [6, 3, 0, 5], [0, 4, 4, 0], 1.0, 0.5)
    run_case([4, 5], [6, 5], [0, 0], 1.0, 1.0)


@pytest.mark.parametrize("cfg", range(10))
def test_every_tile_config(cuda, cfg):
    rng = np.random.default_rng(cfg)
    M = rng.integers(1, 300, 12).tolist()
    N = rng.integers(1, 300, 12).tolist()
    K = rng.integers(0, 70, 12).tolist()
    for off in (0, 1):
        db, host = make_batch(M, N, K, offset=off, seed=cfg)
        want = oracle_batch(db, host, 1.0, 0.5)
        with db.plan("simt", force_tile_config=cfg) as p:
            assert p.info()["tile_config_hist"][cfg] == 12
            db.execute(p, 1.0, 0.5)
            torch.cuda.synchronize()
        assert_bits_equal(db.C.cpu().numpy(), want, "config %d" % cfg)


def test_reference_kernel_outputs_bit_exact(cuda):
    """The reference's own tile-body outputs (golden fixture) reproduced on the GPU."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.npz"))
    n = int(z["ncases"])
    M, N, K, As, Bs, Cs, Cref = [], [], [], [], [], [], []
    for i in range(n):
        p = "c%02d_" % i
        m, nn, k = (int(v) for v in z[p + "mnk"])
        M.append(m); N.append(nn); K.append(k)
        As.append(z[p + "A"]); Bs.append(z[p + "B"]); Cs.append(z[p + "C0"]); Cref.append(z[p + "C"])
    from batchgemm_gb300.batch import DeviceBatch
    db = DeviceBatch(M, N, K)
    db.set_from_numpy(As, Bs, Cs)
    db.run("simt", 1.0, 1.0)
    torch.cuda.synchronize()
    for i in range(n):
        got = db.c(i).t().contiguous().cpu().numpy().reshape(-1)
        assert_bits_equal(got, Cref[i], str(z["c%02d_kernel" % i]))


def test_framework_drop_in_golden_and_dataset(cuda):
    """bgemm_framework_gemm: device size arrays, C += A*B, bit-exact."""
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.npz"))
    from batchgemm_gb300.batch import DeviceBatch
    n = int(z["ncases"])
    dims = [tuple(int(v) for v in z["c%02d_mnk" % i]) for i in range(n)]
    M, N, K = [d[0] for d in dims], [d[1] for d in dims], [d[2] for d in dims]
    db = DeviceBatch(M, N, K)
    db.set_from_numpy([z["c%02d_A" % i] for i in range(n)], [z["c%02d_B" % i] for i in range(n)],
                      [z["c%02d_C0" % i] for i in range(n)])
    dev = lambda v: torch.tensor(v, dtype=torch.int32, device="cuda")
    dM, dN, dK = dev(M), dev(N), dev(K)
    bg.framework_gemm(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(), db.pA.data_ptr(),
                      db.pB.data_ptr(), db.pC.data_ptr(), n, 256)
    bg.framework_check_device()
    for i in range(n):
        got = db.c(i).t().contiguous().cpu().numpy().reshape(-1)
        assert_bits_equal(got, z["c%02d_C" % i], "framework " + str(z["c%02d_kernel" % i]))
    # the reference's own shape fixture, B = 64 (sizes up to 512)
    w = workloads.ref_dataset(64)
    db, host = make_batch(w.M, w.N, w.K, seed=3)
    want = oracle_batch(db, host, 1.0, 1.0)
    dM, dN, dK = dev(w.M), dev(w.N), dev(w.K)
    for _ in range(2):  # the queue resets itself between calls
        db.C.copy_(torch.from_numpy(host[2]))
        bg.framework_gemm(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(), db.pA.data_ptr(),
                          db.pB.data_ptr(), db.pC.data_ptr(), w.batch, 512)
        bg.framework_check_device()
        assert_bits_equal(db.C.cpu().numpy(), want, "framework dataset")


def test_framework_thin_matrices_bit_exact(cuda):
    """bgemm_framework_gemm on thin matrices (M <= 8 or N <= 8, long K), where
    the device planner can choose the thin tiles: C += A*B stays bit-exact."""
    rng = np.random.default_rng(17)
    n = 24
    thin = rng.integers(1, 9, n)
    wide = rng.integers(200, 1500, n)
    M = [int(t) if i % 2 == 0 else int(w) for i, (t, w) in enumerate(zip(thin, wide))]
    N = [int(w) if i % 2 == 0 else int(t) for i, (t, w) in enumerate(zip(thin, wide))]
    K = rng.integers(100, 700, n).tolist()
    db, host = make_batch(M, N, K, seed=8)
    want = oracle_batch(db, host, 1.0, 1.0)
    dev = lambda v: torch.tensor(v, dtype=torch.int32, device="cuda")
    dM, dN, dK = dev(M), dev(N), dev(K)
    bg.framework_gemm(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(), db.pA.data_ptr(),
                      db.pB.data_ptr(), db.pC.data_ptr(), n, 2048)
    bg.framework_check_device()
    assert_bits_equal(db.C.cpu().numpy(), want, "framework thin")


def test_framework_rejects_oversized_on_device(cuda):
    dev = lambda v: torch.tensor(v, dtype=torch.int32, device="cuda")
    from batchgemm_gb300.batch import DeviceBatch
    db = DeviceBatch([8, 8], [8, 8], [8, 8]).fill()
    before = db.c(1).clone()
    dM = dev([8, 600])  # 600 > max_dim: skipped and reported
    dN, dK = dev([8, 8]), dev([8, 8])
    bg.framework_gemm(dM.data_ptr(), dN.data_ptr(), dK.data_ptr(),
                      db.pA.data_ptr(), db.pB.data_ptr(), db.pC.data_ptr(), 2, 64)
    with pytest.raises(bg.BgemmError):
        bg.framework_check_device()
    bg.framework_check_device()  # the flag is cleared once reported


def test_plan_graph_replay(cuda):
    """Plan execute inside a captured CUDA graph; replays see fresh inputs."""
    rng = np.random.default_rng(11)
    M = rng.integers(1, 260, 40).tolist()
    N = rng.integers(1, 260, 40).tolist()
    K = rng.integers(1, 260, 40).tolist()
    db, host = make_batch(M, N, K, seed=5)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        plan = db.plan("simt", stream=s)
        db.execute(plan, 1.0, 0.0, stream=s)  # warm up outside capture
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        db.execute(plan, 1.0, 0.0, stream=s)
    for rep in range(3):
        db2, host2 = make_batch(M, N, K, seed=100 + rep)
        db.A.copy_(db2.A)
        db.B.copy_(db2.B)
        g.replay()
        torch.cuda.synchronize()
        want = oracle_batch(db, (host2[0], host2[1], host[2]), 1.0, 0.0)
        assert_bits_equal(db.C.cpu().numpy(), want, "replay %d" % rep)
    plan.close()


def test_plain_fp32_256_full(cuda):
    """The 256-matrix plain FP32 workload, whole, bit-exact and within the FP64 bound."""
    w = workloads.plain_fp32(0)
    db, host = make_batch(w.M, w.N, w.K, seed=0)
    hA, hB, hC = host
    want = hC.copy()
    Cs = [want[o:] for o in db.offC]
    oracle.vbatched_f32(w.M, w.N, w.K, 1.0, [hA[o:] for o in db.offA], db.lda,
                        [hB[o:] for o in db.offB], db.ldb, 0.0, Cs, db.ldc,
                        nthreads=os.cpu_count() or 4)
    db.run("simt", 1.0, 0.0)
    torch.cuda.synchronize()
    got = db.C.cpu().numpy()
    assert_bits_equal(got, want, "plain_fp32_256")
    worst, mean = f64_check(db, host, got, 1.0, 0.0, 8.0, U)
    assert worst < 8 * U * 16


def sampled_bit_exact(db, host, got, alpha, beta, per_matrix=4, seed=0):
    """Re-derives sampled entries with the oracle (1x1 GEMMs) and compares bits."""
    hA, hB, hC0 = host
    rng = np.random.default_rng(seed)
    checked = 0
    for i in range(db.batch):
        M, N, K = db.M[i], db.N[i], db.K[i]
        if not (M and N):
            continue
        for _ in range(per_matrix):
            m, n = int(rng.integers(0, M)), int(rng.integers(0, N))
            c = np.array([hC0[db.offC[i] + m + n * db.ldc[i]]], np.float32)
            oracle.sgemm_f32(1, 1, K, alpha, hA[db.offA[i] + m:], db.lda[i],
                             hB[db.offB[i] + n * db.ldb[i]:], db.ldb[i], beta, c, 1)
            g = got[db.offC[i] + m + n * db.ldc[i]]
            assert c.view(np.uint32)[0] == np.float32(g).view(np.uint32), (i, m, n, g, c[0])
            checked += 1
    return checked


@pytest.mark.parametrize("name", ["simt_at_scale_2048", "skewed_4000", "uneven_m_128"])
def test_full_size_sampled_bit_exact(cuda, name):
    w = workloads.CONFIGS[name](0)
    from batchgemm_gb300.batch import DeviceBatch
    db = DeviceBatch(w.M, w.N, w.K).fill_fast(w.dist, seed=1)
    host = tuple(x.cpu().numpy() for x in (db.A, db.B, db.C))
    db.run("simt", w.alpha, w.beta)
    torch.cuda.synchronize()
    got = db.C.cpu().numpy()
    n = sampled_bit_exact(db, host, got, w.alpha, w.beta, per_matrix=3)
    assert n > 100
