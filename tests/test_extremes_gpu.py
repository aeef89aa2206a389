"""Extreme shapes: very tall, very wide, very long K, many tiny matrices, and
the tile-index limit (a matrix needing more than 65535 tiles along one side
with the largest tile is refused with BGEMM_ERROR_NOT_SUPPORTED, no launch)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

import batchgemm_gb300 as bg  # noqa: E402
from gpu_util import make_batch, oracle_batch, assert_bits_equal, f64_check  # noqa: E402

BOUND = {"tf32x3": (32.0, 2.0 ** -24), "bf16x3": (8.0, 2.0 ** -16), "tf32": (4.0, 2.0 ** -11)}
TALL = (1 << 20) + 3

CASES = {
    "tall": ([TALL, 7], [1, 3], [5, 9]),
    "wide": ([1, 3], [TALL, 7], [5, 9]),
    "long_k": ([33, 1, 130], [33, 2, 5], [(1 << 16) + 7, (1 << 15) + 1, 40000]),
}


@pytest.mark.parametrize("mode", ["simt", "tf32x3", "bf16x3", "tf32"])
@pytest.mark.parametrize("case", list(CASES))
def test_extreme_aspect_and_long_k(cuda, mode, case):
    M, N, K = CASES[case]
    db, host = make_batch(M, N, K, seed=4)
    alpha, beta = 1.0, 0.5
    db.run(mode, alpha, beta)
    torch.cuda.synchronize()
    got = db.C.cpu().numpy()
    if mode == "simt":
        assert_bits_equal(got, oracle_batch(db, host, alpha, beta), case)
    else:
        factor, unit = BOUND[mode]
        f64_check(db, host, got, alpha, beta, factor, unit)


@pytest.mark.parametrize("mode", ["simt", "tf32x3"])
def test_many_tiny_matrices(cuda, mode):
    rng = np.random.default_rng(8)
    n = 20000
    M = rng.integers(0, 9, n).tolist()
    N = rng.integers(0, 9, n).tolist()
    K = rng.integers(0, 9, n).tolist()
    db, host = make_batch(M, N, K, seed=2)
    db.run(mode, 1.0, 1.0)
    torch.cuda.synchronize()
    got = db.C.cpu().numpy()
    if mode == "simt":
        assert_bits_equal(got, oracle_batch(db, host, 1.0, 1.0), "tiny")
    else:
        f64_check(db, host, got, 1.0, 1.0, *BOUND[mode])


@pytest.mark.parametrize("mode,rows", [("simt", (1 << 23) + 129),     # > 65535 tiles of 128
                                       ("tf32x3", (1 << 24) + 257)])  # > 65535 tiles of 256
def test_tile_index_limit_is_an_error(cuda, mode, rows):
    M = [rows]
    with pytest.raises(bg.BgemmError) as ei:
        bg.Plan(M, [1], [1], M, [1], M, mode=mode)
    assert ei.value.status == 2
    # one tile size down still fits (CTA-pair tiles of 256 rows for the tensor cores)
    ok = [(1 << 23) + 129]
    if mode != "simt":
        bg.Plan(ok, [1], [1], ok, [1], ok, mode=mode).close()
