"""Row-major storage and transposed operands (BLAS / magma vbatched surface).

Every case draws op(A) (M x K), op(B) (K x N) and C0 (M x N), stores A, B and
C in the requested layout and transposition with padded leading dimensions,
runs the library, and compares with the oracle on the column-major NN problem
of the same op(A), op(B), C0: bit-exact for the FP32 SIMT mode (the fma chain
over k does not depend on storage), the sqrt(K)-scaled FP64 bound for the
tensor-core modes.  The padding is NaN and must stay untouched.
"""
import itertools

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
import oracle  # noqa: E402

BOUND = {"tf32x3": (32.0, 2.0 ** -24), "bf16x3": (8.0, 2.0 ** -16), "tf32": (4.0, 2.0 ** -11)}


def store(X, layout, ld):
    """Flat storage of matrix X (r x c) in `layout` with leading dimension ld,
    padding NaN."""
    r, c = X.shape
    if layout == "col":
        buf = np.full((c, ld), np.nan, np.float32)
        buf[:, :r] = X.T
    else:
        buf = np.full((r, ld), np.nan, np.float32)
        buf[:, :c] = X
    return buf.reshape(-1)


def load(flat, layout, r, c, ld):
    if layout == "col":
        return flat[:c * ld].reshape(c, ld)[:, :r].T
    return flat[:r * ld].reshape(r, ld)[:, :c]


class Case:
    def __init__(self, layout, ta, tb, M, N, K, seed, pad=3):
        rng = np.random.default_rng(seed)
        self.layout, self.ta, self.tb = layout, ta, tb
        self.M, self.N, self.K = M, N, K
        self.opA = [rng.uniform(-1, 1, (m, k)).astype(np.float32) for m, k in zip(M, K)]
        self.opB = [rng.uniform(-1, 1, (k, n)).astype(np.float32) for k, n in zip(K, N)]
        self.C0 = [rng.uniform(-1, 1, (m, n)).astype(np.float32) for m, n in zip(M, N)]
        sA = [a.T if ta == "T" else a for a in self.opA]       # stored matrices
        sB = [b.T if tb == "T" else b for b in self.opB]
        ext = lambda X: X.shape[0] if layout == "col" else X.shape[1]
        self.lda = [max(1, ext(x)) + pad * (i % 2) for i, x in enumerate(sA)]
        self.ldb = [max(1, ext(x)) + pad * ((i + 1) % 2) for i, x in enumerate(sB)]
        self.ldc = [max(1, ext(x)) + pad for x in self.C0]
        self.dev = {}
        for name, mats, lds in (("A", sA, self.lda), ("B", sB, self.ldb), ("C", self.C0, self.ldc)):
            flats = [store(x, layout, l) for x, l in zip(mats, lds)]
            offs, cur = [], 0
            for f in flats:
                cur = (cur + 3) // 4 * 4
                offs.append(cur)
                cur += f.size + 8
            host = np.full(cur + 8, np.nan, np.float32)
            for o, f in zip(offs, flats):
                host[o:o + f.size] = f
            buf = torch.from_numpy(host).cuda()
            ptrs = torch.tensor([buf.data_ptr() + 4 * o for o in offs], dtype=torch.int64,
                                device="cuda")
            self.dev[name] = (buf, ptrs, offs, host)

    def ptrs(self):
        return tuple(self.dev[k][1].data_ptr() for k in "ABC")

    def result(self):
        buf, _, offs, host0 = self.dev["C"]
        got = buf.cpu().numpy()
        # everything outside the matrices (padding, gaps) is untouched
        mask = np.isnan(host0)
        for i, o in enumerate(offs):
            r, c = self.M[i], self.N[i]
            if self.layout == "col":
                idx = o + np.add.outer(np.arange(r), np.arange(c) * self.ldc[i])
            else:
                idx = o + np.add.outer(np.arange(r) * self.ldc[i], np.arange(c))
            mask[idx] = False
        pad_got = got[mask]
        assert np.isnan(pad_got).all(), "padding written"
        return [load(got[o:], self.layout, m, n, l)
                for o, m, n, l in zip(offs, self.M, self.N, self.ldc)]

    def expected_f32(self, alpha, beta):
        out = []
        for a, b, c0, m, n, k in zip(self.opA, self.opB, self.C0, self.M, self.N, self.K):
            C = np.asfortranarray(c0).reshape(-1, order="F").copy()
            if m and n:
                oracle.sgemm_f32(m, n, k, alpha, np.asfortranarray(a).reshape(-1, order="F"),
                                 max(1, m), np.asfortranarray(b).reshape(-1, order="F"),
                                 max(1, k), beta, C, max(1, m))
            out.append(C.reshape(n, m).T if m and n else c0)
        return out

    def check_fp64(self, got, alpha, beta, mode):
        factor, unit = BOUND[mode]
        for g, a, b, c0, m, n, k in zip(got, self.opA, self.opB, self.C0, self.M, self.N, self.K):
            if not (m and n):
                continue
            C64, bound = oracle.sgemm_f64(m, n, k, alpha,
                                          np.asfortranarray(a).reshape(-1, order="F"), max(1, m),
                                          np.asfortranarray(b).reshape(-1, order="F"), max(1, k),
                                          beta, np.asfortranarray(c0).reshape(-1, order="F"),
                                          max(1, m))
            e = oracle.normalized_error(np.asfortranarray(g).reshape(-1, order="F"), C64, bound)
            assert e.max() <= factor * unit * np.sqrt(max(k, 1)), (m, n, k, e.max())


def shapes(seed, n=14):
    rng = np.random.default_rng(seed)
    M = rng.integers(1, 200, n).tolist() + [0, 1, 129]
    N = rng.integers(1, 200, n).tolist() + [5, 1, 257]
    K = rng.integers(0, 200, n).tolist() + [3, 1, 64]
    return M, N, K


COMBOS = list(itertools.product(["col", "row"], ["N", "T"], ["N", "T"]))


@pytest.mark.parametrize("layout,ta,tb", COMBOS)
def test_simt_bit_exact(cuda, layout, ta, tb):
    M, N, K = shapes(COMBOS.index((layout, ta, tb)))
    for alpha, beta in ((1.0, 1.0), (0.5, -1.5), (2.0, 0.0)):
        c = Case(layout, ta, tb, M, N, K, seed=len(M))
        pA, pB, pC = c.ptrs()
        bg.sgemm_vbatched_ex(layout, ta, tb, M, N, K, alpha, pA, c.lda, pB, c.ldb, beta, pC,
                             c.ldc, mode="simt")
        torch.cuda.synchronize()
        for i, (g, w) in enumerate(zip(c.result(), c.expected_f32(alpha, beta))):
            np.testing.assert_array_equal(np.ascontiguousarray(g).view(np.uint32),
                                          np.ascontiguousarray(w).view(np.uint32),
                                          err_msg="matrix %d %s" % (i, (layout, ta, tb)))


@pytest.mark.parametrize("mode", list(BOUND))
@pytest.mark.parametrize("layout,ta,tb", COMBOS)
def test_tensor_core_modes(cuda, mode, layout, ta, tb):
    M, N, K = shapes(7)
    c = Case(layout, ta, tb, M, N, K, seed=3)
    pA, pB, pC = c.ptrs()
    bg.sgemm_vbatched_ex(layout, ta, tb, M, N, K, 0.75, pA, c.lda, pB, c.ldb, 0.5, pC, c.ldc,
                         mode=mode)
    torch.cuda.synchronize()
    c.check_fp64(c.result(), 0.75, 0.5, mode)


@pytest.mark.parametrize("layout,ta,tb", [("row", "N", "N"), ("col", "T", "T"), ("row", "T", "N")])
def test_plan_with_layout_and_update(cuda, layout, ta, tb):
    """Plan options carry the storage order and ops; updates keep them."""
    M, N, K = shapes(11)
    c = Case(layout, ta, tb, M, N, K, seed=5)
    pA, pB, pC = c.ptrs()
    M2, N2, K2 = shapes(12)
    c2 = Case(layout, ta, tb, M2, N2, K2, seed=6)
    reqs = [bg.plan_requirements(x.M, x.N, x.K, x.lda, x.ldb, x.ldc, mode="tf32x3", layout=layout,
                                 trans_a=ta, trans_b=tb) for x in (c, c2)]
    with bg.Plan(c.M, c.N, c.K, c.lda, c.ldb, c.ldc, mode="tf32x3", layout=layout, trans_a=ta,
                 trans_b=tb, capacity=bg.max_requirements(reqs)) as p:
        p.execute(1.0, pA, pB, 1.0, pC)
        torch.cuda.synchronize()
        c.check_fp64(c.result(), 1.0, 1.0, "tf32x3")
        p.update(c2.M, c2.N, c2.K, c2.lda, c2.ldb, c2.ldc)
        qA, qB, qC = c2.ptrs()
        p.execute(1.0, qA, qB, 1.0, qC)
        torch.cuda.synchronize()
        p.check_device()
    c2.check_fp64(c2.result(), 1.0, 1.0, "tf32x3")


@pytest.mark.parametrize("layout,ta,tb", COMBOS)
def test_thin_tiles_bit_exact(cuda, layout, ta, tb):
    """The thin SIMT tiles (8 x 128 for M <= 8, 128 x 8 for N <= 8), forced,
    in every storage order and transposition: bit-exact with the oracle,
    ragged edges and padding included."""
    rng = np.random.default_rng(40 + COMBOS.index((layout, ta, tb)))
    for cfg, thin in ((8, "M"), (9, "N")):
        n = 6
        small = rng.integers(1, 9, n).tolist()
        big = rng.integers(1, 300, n).tolist()
        M, N = (small, big) if thin == "M" else (big, small)
        K = rng.integers(0, 90, n).tolist()
        c = Case(layout, ta, tb, M, N, K, seed=cfg)
        pA, pB, pC = c.ptrs()
        with bg.Plan(M, N, K, c.lda, c.ldb, c.ldc, mode="simt", layout=layout, trans_a=ta,
                     trans_b=tb, force_tile_config=cfg) as p:
            assert p.info()["tile_config_hist"][cfg] == n
            p.execute(0.5, pA, pB, -1.5, pC)
            torch.cuda.synchronize()
        for i, (g, w) in enumerate(zip(c.result(), c.expected_f32(0.5, -1.5))):
            np.testing.assert_array_equal(np.ascontiguousarray(g).view(np.uint32),
                                          np.ascontiguousarray(w).view(np.uint32),
                                          err_msg="cfg %d matrix %d %s" % (cfg, i, (layout, ta, tb)))
