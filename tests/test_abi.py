"""The C ABI and the host planner, without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

import batchgemm_gb300 as bg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SIMT_CFGS = [(16, 16), (32, 32), (64, 32), (32, 64), (64, 64), (128, 64), (64, 128), (128, 128),
             (8, 128), (128, 8)]


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if h.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", h)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(bgemm_\w+)\s*\(", txt))
    return names


def test_exports_every_declared_symbol(built_lib):
    names = declared_symbols()
    assert len(names) >= 15
    for n in sorted(names):
        assert hasattr(built_lib, n), n


def test_status_strings(built_lib):
    built_lib.bgemm_status_string.restype = ctypes.c_char_p
    assert built_lib.bgemm_status_string(0) == b"BGEMM_SUCCESS"
    assert built_lib.bgemm_status_string(5) == b"BGEMM_ERROR_DEVICE_TIMEOUT"
    assert built_lib.bgemm_version() >= 100


@pytest.mark.parametrize("field,argpos", [("M", 1), ("N", 2), ("K", 3), ("lda", 6), ("ldb", 8),
                                          ("ldc", 11)])
def test_invalid_arguments_blas_numbering(built_lib, field, argpos):
    """Negative sizes and short leading dimensions are rejected before any
    device work, naming the argument (1-based) and the matrix."""
    sh = {"M": [4, 5, 6], "N": [3, 3, 3], "K": [2, 2, 2]}
    ld = {"lda": [4, 5, 6], "ldb": [2, 2, 2], "ldc": [4, 5, 6]}
    if field in sh:
        sh[field][1] = -1
    else:
        ld[field][1] = 0 if field != "lda" else 4  # lda < M = 5
    with pytest.raises(bg.BgemmError) as ei:
        bg.sgemm_vbatched(sh["M"], sh["N"], sh["K"], 1.0, 1, ld["lda"], 1, ld["ldb"], 0.0, 1,
                          ld["ldc"], mode="simt")
    assert ei.value.status == 1
    assert ei.value.arg == argpos
    assert ei.value.matrix == 1


def test_unknown_mode_rejected(built_lib):
    with pytest.raises(bg.BgemmError) as ei:
        bg.sgemm_vbatched([1], [1], [1], 1.0, 1, [1], 1, [1], 0.0, 1, [1], mode=9)
    assert ei.value.arg == 13


def test_null_pointer_arrays_rejected(built_lib):
    with pytest.raises(bg.BgemmError) as ei:
        bg.sgemm_vbatched([2], [2], [2], 1.0, None, [2], 1, [2], 0.0, 1, [2])
    assert ei.value.arg == 5
    with pytest.raises(bg.BgemmError) as ei:
        bg.sgemm_vbatched([2], [2], [2], 1.0, 1, [2], 1, [2], 0.0, None, [2])
    assert ei.value.arg == 10


def test_empty_batches_are_noops(built_lib):
    bg.sgemm_vbatched([], [], [], 1.0, None, [], None, [], 0.0, None, [])
    # matrices with M or N = 0 produce no work and need no pointers
    bg.sgemm_vbatched([0, 3], [5, 0], [2, 2], 1.0, None, [1, 3], None, [2, 2], 0.0, None, [1, 3])


def test_no_cpu_fallback_without_gpu(built_lib):
    """On a machine without an sm_103 device, real work fails loudly."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    with pytest.raises(bg.BgemmError) as ei:
        bg.sgemm_vbatched([8], [8], [8], 1.0, 1, [8], 1, [8], 0.0, 1, [8])
    assert ei.value.status in (2, 4)


def test_framework_mode_argument_checks_without_gpu(built_lib):
    """The device-size entry checks its arguments before touching a device:
    BLAS-style numbers (dM 1 .. max_operand_elems 10, mode 11); an empty
    batch is a no-op."""
    p = 8  # any non-null address: never dereferenced by the checks
    args = lambda **kw: [kw.get(k, d) for k, d in (
        ("dM", p), ("dN", p), ("dK", p), ("dA", p), ("dB", p), ("dC", p), ("batch", 1),
        ("max_dim", 16), ("max_k", 16), ("mode", "tf32x3"))]
    for kw, argpos in ((dict(mode=9), 11), (dict(batch=-1), 7), (dict(dK=None), 3),
                       (dict(dC=None), 6), (dict(max_dim=0), 8), (dict(max_k=0), 9)):
        with pytest.raises(bg.BgemmError) as ei:
            bg.framework_gemm_mode(*args(**kw))
        assert (ei.value.status, ei.value.arg) == (1, argpos), kw
    with pytest.raises(bg.BgemmError) as ei:
        bg.framework_gemm_mode(*args(), max_operand_elems=-5)
    assert ei.value.arg == 10
    bg.framework_gemm_mode(*args(batch=0))


def simt_queue(M, N, K, slots=304, force=-1, rebalance=True):
    L = bg.lib()
    n = len(M)
    ia = lambda v: (ctypes.c_int * max(n, 1))(*v)
    cfg = (ctypes.c_int * max(n, 1))()
    cnt = L.bgemm_debug_simt_queue(ia(M), ia(N), ia(K), n, slots, force, int(rebalance), cfg,
                                   None, 0)
    assert cnt >= 0
    items = (ctypes.c_int * max(3 * cnt, 1))()
    cnt2 = L.bgemm_debug_simt_queue(ia(M), ia(N), ia(K), n, slots, force, int(rebalance), cfg,
                                    items, cnt)
    assert cnt2 == cnt
    return list(cfg)[:n], np.array(items[:3 * cnt]).reshape(-1, 3)


def coverage_ok(M, N, cfgs, items):
    seen = {}
    for mat, tm, tn in items:
        bm, bn = SIMT_CFGS[cfgs[mat]]
        assert tm * bm < M[mat] and tn * bn < N[mat]
        key = (mat, tm, tn)
        assert key not in seen, key
        seen[key] = 1
    for i in range(len(M)):
        if M[i] and N[i]:
            bm, bn = SIMT_CFGS[cfgs[i]]
            want = -(-M[i] // bm) * -(-N[i] // bn)
            got = sum(1 for k in seen if k[0] == i)
            assert got == want
        else:
            assert cfgs[i] == -1


@pytest.mark.parametrize("seed", range(4))
def test_queue_covers_every_tile_once(built_lib, seed):
    rng = np.random.default_rng(seed)
    n = 60
    M = rng.integers(0, 300, n).tolist()
    N = rng.integers(0, 300, n).tolist()
    K = rng.integers(0, 300, n).tolist()
    cfgs, items = simt_queue(M, N, K)
    coverage_ok(M, N, cfgs, items)


def test_queue_is_longest_first(built_lib):
    from batchgemm_gb300 import workloads
    w = workloads.skewed(0, 400)
    cfgs, items = simt_queue(w.M, w.N, w.K)
    coverage_ok(w.M, w.N, cfgs, items)
    # modelled tile time is non-increasing along the queue: K and tile area of
    # consecutive matrices never grow together
    mats = [items[0][0]]
    for m in items[:, 0]:
        if m != mats[-1]:
            mats.append(m)
    assert len(mats) == len(set(mats)), "a matrix's tiles are contiguous"
    big = set(i for i in range(w.batch) if max(w.M[i], w.N[i], w.K[i]) >= 512)
    first = mats[:len(big)]
    assert sum(1 for m in first if m in big) >= 0.9 * len(big)


def test_rebalance_splits_tiles_for_small_batches(built_lib):
    # one 1024^3 matrix: 64 tiles of 128x128 leave most of 304 CTA slots idle
    cfg_nr, it_nr = simt_queue([1024], [1024], [1024], rebalance=False)
    cfg_rb, it_rb = simt_queue([1024], [1024], [1024], rebalance=True)
    assert cfg_nr[0] == 7
    assert len(it_rb) > len(it_nr)
    coverage_ok([1024], [1024], cfg_rb, it_rb)


def test_forced_config(built_lib):
    for c in range(len(SIMT_CFGS)):
        cfgs, items = simt_queue([100, 7], [90, 300], [5, 5], force=c)
        assert cfgs == [c, c]
        coverage_ok([100, 7], [90, 300], cfgs, items)


def test_reference_dataset_planned(built_lib):
    shapes = np.load(os.path.join(ROOT, "tests", "golden", "ref_dataset_shapes.npy")).astype(int)
    for b in (8, 16, 32, 64, 128, 256):
        M, N, K = shapes[:b, 0].tolist(), shapes[:b, 1].tolist(), shapes[:b, 2].tolist()
        cfgs, items = simt_queue(M, N, K)
        coverage_ok(M, N, cfgs, items)


def test_option_structs_match_the_header(tmp_path):
    """ctypes mirrors of the option / requirement / info structs have the C
    header's sizes and field offsets (gcc compiles a probe of the header)."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("no gcc")
    structs = {"bgemm_plan_options_t": bg.PlanOptions,
               "bgemm_plan_requirements_t": bg.PlanRequirements,
               "bgemm_plan_info_t": bg.PlanInfo}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "bgemm.h"', 'int main(void){']
    for cname, py in structs.items():
        lines.append('printf("%s sizeof %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f[0], cname,
                                                                          f[0]))
    lines.append("return 0;}")
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "probe"
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    out = subprocess.check_output([str(exe)]).decode().split("\n")
    got = {}
    for line in out:
        if line:
            c, f, v = line.split()
            got[(c, f)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "sizeof")] == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, (cname, f[0])


@pytest.mark.parametrize("layout,ta,tb,bad,argpos", [
    ("col", "T", "N", "lda", 9),   # A stored K x M: lda >= K
    ("col", "N", "T", "ldb", 11),  # B stored N x K: ldb >= N
    ("row", "N", "N", "lda", 9),   # row-major A (M x K): lda >= K
    ("row", "N", "N", "ldc", 14),  # row-major C (M x N): ldc >= N
    ("row", "T", "T", "ldb", 11),  # row-major B^T stored N x K: ldb >= K
])
def test_layout_trans_leading_dimension_rules(built_lib, layout, ta, tb, bad, argpos):
    """bgemm_sgemm_vbatched_ex checks each leading dimension against the extent
    it spans for the given storage order and op, before any device work."""
    M, N, K = [7, 9], [5, 30], [11, 20]
    ext = {"col": {"lda": lambda i: K[i] if ta == "T" else M[i],
                   "ldb": lambda i: N[i] if tb == "T" else K[i], "ldc": lambda i: M[i]},
           "row": {"lda": lambda i: M[i] if ta == "T" else K[i],
                   "ldb": lambda i: K[i] if tb == "T" else N[i], "ldc": lambda i: N[i]}}[layout]
    ld = {k: [ext[k](i) for i in range(2)] for k in ("lda", "ldb", "ldc")}
    ld[bad][1] -= 1
    with pytest.raises(bg.BgemmError) as ei:
        bg.sgemm_vbatched_ex(layout, ta, tb, M, N, K, 1.0, 1, ld["lda"], 1, ld["ldb"], 0.0, 1,
                             ld["ldc"])
    assert ei.value.status == 1 and ei.value.arg == argpos and ei.value.matrix == 1


def test_layout_trans_enum_values_rejected(built_lib):
    L = bg.lib()
    one = bg.int_array([1])
    assert L.bgemm_sgemm_vbatched_ex(2, 0, 0, one, one, one, 1.0, None, one, None, one, 0.0,
                                     None, one, 1, 0, None) == 1
    assert L.bgemm_last_error_arg(None) == 1
    assert L.bgemm_sgemm_vbatched_ex(0, 0, 5, one, one, one, 1.0, None, one, None, one, 0.0,
                                     None, one, 1, 0, None) == 1
    assert L.bgemm_last_error_arg(None) == 3
