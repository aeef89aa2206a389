"""The CPU oracle, pinned against the reference's own outputs (CPU only)."""
import numpy as np
import pytest

import oracle

GOLD = None


def gold():
    global GOLD
    if GOLD is None:
        import os
        GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "ref_kernels.npz"))
    return GOLD


def cases():
    z = gold()
    for i in range(int(z["ncases"])):
        p = "c%02d_" % i
        yield str(z[p + "kernel"]), tuple(int(v) for v in z[p + "mnk"]), z[p + "A"], z[p + "B"], \
            z[p + "C0"], z[p + "C"]


def test_golden_fixture_complete():
    kernels = {c[0] for c in cases()}
    # the framework's column-major body and every correct Li body are pinned
    assert "fw_128_32x32" in kernels
    assert {"li_256_16x16", "li_256_32x32", "li_256_64x64", "li_256_128x64", "li_256_64x128",
            "li_256_128x128"} <= kernels
    assert {"li_128_16x16", "li_128_32x32", "li_128_64x64", "li_128_64x128",
            "li_128_128x64"} <= kernels


@pytest.mark.parametrize("idx", range(13))
def test_oracle_bit_exact_vs_reference_kernels(idx):
    """alpha = beta = 1 is the reference's in-place chain: identical bits."""
    kern, (M, N, K), A, B, C0, Cref = list(cases())[idx]
    C = C0.copy()
    oracle.sgemm_f32(M, N, K, 1.0, A, M, B, K, 1.0, C, M)
    assert np.array_equal(C.view(np.uint32), Cref.view(np.uint32)), kern


def test_oracle_f64_bound_on_golden():
    for kern, (M, N, K), A, B, C0, Cref in cases():
        C64, bound = oracle.sgemm_f64(M, N, K, 1.0, A, M, B, K, 1.0, C0, M)
        e = oracle.normalized_error(Cref, C64, bound)
        assert e.max() <= 8 * 2.0 ** -24 * np.sqrt(K), kern


def _rand(rng, *shape):
    return rng.uniform(-1, 1, shape).astype(np.float32)


def test_beta_zero_never_reads_c():
    rng = np.random.default_rng(1)
    M, N, K = 7, 5, 9
    A, B = _rand(rng, M * K), _rand(rng, K * N)
    C = np.full(M * N, np.nan, np.float32)
    oracle.sgemm_f32(M, N, K, 2.0, A, M, B, K, 0.0, C, M)
    assert np.isfinite(C).all()


def test_alpha_beta_formula():
    rng = np.random.default_rng(2)
    M, N, K = 6, 4, 11
    A, B, C0 = _rand(rng, M * K), _rand(rng, K * N), _rand(rng, M * N)
    C = C0.copy()
    oracle.sgemm_f32(M, N, K, 0.75, A, M, B, K, -0.5, C, M)
    # restate the formula with numpy's float32 fma-free arithmetic per step
    Am, Bm = A.reshape(K, M).T, B.reshape(N, K).T
    for n in range(N):
        for m in range(M):
            acc = np.float32(0)
            for k in range(K):
                acc = np.float32(np.float64(Am[m, k]) * np.float64(Bm[k, n]) + np.float64(acc))
            want = np.float32(0.75 * np.float64(acc) + np.float64(np.float32(-0.5 * C0[n * M + m])))
            assert C[n * M + m] == want


def test_k_zero_and_empty():
    C0 = np.arange(12, dtype=np.float32)
    C = C0.copy()
    oracle.sgemm_f32(3, 4, 0, 1.0, np.zeros(1, np.float32), 3, np.zeros(1, np.float32), 1, 0.5,
                     C, 3)
    assert np.array_equal(C, np.float32(0.5) * C0)
    C = C0.copy()
    oracle.sgemm_f32(3, 4, 0, 1.0, np.zeros(1, np.float32), 3, np.zeros(1, np.float32), 1, 1.0,
                     C, 3)
    assert np.array_equal(C, C0)


def test_leading_dimensions_respected():
    rng = np.random.default_rng(3)
    M, N, K, lda, ldb, ldc = 5, 3, 4, 8, 6, 7
    A, B = _rand(rng, lda * K), _rand(rng, ldb * N)
    C = np.full(ldc * N, 123.0, np.float32)
    oracle.sgemm_f32(M, N, K, 1.0, A, lda, B, ldb, 0.0, C, ldc)
    Am = A.reshape(K, lda).T[:M]
    Bm = B.reshape(N, ldb).T[:K]
    ref = Am.astype(np.float64) @ Bm.astype(np.float64)
    Cm = C.reshape(N, ldc).T
    assert np.allclose(Cm[:M], ref, atol=1e-5)
    assert (Cm[M:] == 123.0).all()


def test_split_tf32_bf16_properties():
    rng = np.random.default_rng(4)
    x = rng.standard_normal(10000).astype(np.float32)
    for mode, drop in ((oracle.MODE_TF32X3, 13), (oracle.MODE_BF16X3, 16)):
        hi, lo = oracle.split(mode, x)
        assert ((hi.view(np.uint32) & ((1 << drop) - 1)) == 0).all()
        assert ((lo.view(np.uint32) & ((1 << drop) - 1)) == 0).all()
        resid = np.abs(x.astype(np.float64) - hi - lo) / np.abs(x)
        bound = 2.0 ** -(2 * (23 - drop) + 2) * 1.01
        assert resid.max() <= bound, (mode, resid.max(), bound)
    hi, lo = oracle.split(oracle.MODE_TF32, x)
    assert (lo == 0).all()


def test_round_ties_to_even():
    lib = oracle.lib()
    # 1 + 2^-11 is exactly half an ulp of TF32 at 1.0: ties to even -> 1.0
    assert lib.bgo_round_tf32(np.float32(1.0 + 2.0 ** -11)) == 1.0
    # 1 + 3*2^-11 ties up to 1 + 2^-9
    assert lib.bgo_round_tf32(np.float32(1.0 + 3 * 2.0 ** -11)) == np.float32(1.0 + 2.0 ** -9)
    assert lib.bgo_round_bf16(np.float32(1.0 + 2.0 ** -8)) == 1.0
    assert np.isinf(lib.bgo_round_tf32(np.float32(np.inf)))


def test_split_f64_matches_mode_definition():
    rng = np.random.default_rng(5)
    M, N, K = 9, 7, 33
    A, B = _rand(rng, M * K), _rand(rng, K * N)
    exact, _ = oracle.sgemm_f64(M, N, K, 1.0, A, M, B, K, 0.0, None, M)
    s3 = oracle.sgemm_split_f64(oracle.MODE_TF32X3, M, N, K, 1.0, A, M, B, K, 0.0, None, M)
    s1 = oracle.sgemm_split_f64(oracle.MODE_TF32, M, N, K, 1.0, A, M, B, K, 0.0, None, M)
    assert np.abs(s3 - exact).max() < 1e-5
    assert np.abs(s1 - exact).max() > np.abs(s3 - exact).max()


def test_vbatched_threads_equal_single():
    rng = np.random.default_rng(6)
    Ms, Ns, Ks = [5, 17, 33, 1], [3, 9, 2, 4], [7, 0, 12, 5]
    As = [_rand(rng, max(m * k, 1)) for m, k in zip(Ms, Ks)]
    Bs = [_rand(rng, max(k * n, 1)) for k, n in zip(Ks, Ns)]
    C0 = [_rand(rng, m * n) for m, n in zip(Ms, Ns)]
    C1 = [c.copy() for c in C0]
    C2 = [c.copy() for c in C0]
    oracle.vbatched_f32(Ms, Ns, Ks, 1.5, As, Ms, Bs, [max(k, 1) for k in Ks], 0.25, C1, Ms,
                        nthreads=3)
    for i in range(4):
        oracle.sgemm_f32(Ms[i], Ns[i], Ks[i], 1.5, As[i], Ms[i], Bs[i], max(Ks[i], 1), 0.25,
                         C2[i], Ms[i])
        assert np.array_equal(C1[i], C2[i])
