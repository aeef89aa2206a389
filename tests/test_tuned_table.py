"""The autotuned tables the planners and kernels compile in (csrc/
tile_table_tuned.inc, written by batchgemm_gb300/autotune.py): shape and
bounds, read back through the library's debug entries.  No GPU needed."""
import ctypes
import os
import re

import batchgemm_gb300 as bg
from batchgemm_gb300 import autotune

INC = os.path.join(os.path.dirname(bg.__file__), "csrc", "tile_table_tuned.inc")


def test_schedule_table_shape_and_bounds(built_lib):
    L = bg.lib()
    text = open(INC).read()
    m = re.search(r"kTcGroupTable\[3\]\[8\] = \{(.*)\};", text)
    assert m, "the tuned table carries a promotion schedule"
    rows = re.findall(r"\{([^{}]*)\}", m.group(1))
    assert len(rows) == 3 and all(len(r.split(",")) == 8 for r in rows)
    for mode in (2, 3):
        g = (ctypes.c_int * 8)()
        assert L.bgemm_debug_get_tc_schedule(mode, g) == 0
        vals = list(g)
        assert vals == [int(x) for x in rows[mode - 1].split(",")]
        for b, v in enumerate(vals):
            assert v in autotune.SCHED_CANDIDATES, (mode, b, v)
            assert b <= 1 or v != 0, "the every-MMA path is only for K <= 128"


def test_schedule_override_round_trip(built_lib):
    L = bg.lib()
    orig = (ctypes.c_int * 8)()
    L.bgemm_debug_get_tc_schedule(2, orig)
    try:
        want = [0, 1, 2, 3, 4, 6, 8, 2]
        assert L.bgemm_debug_set_tc_schedule(2, (ctypes.c_int * 8)(*want)) == 0
        got = (ctypes.c_int * 8)()
        L.bgemm_debug_get_tc_schedule(2, got)
        assert list(got) == want
        assert L.bgemm_debug_set_tc_schedule(2, (ctypes.c_int * 8)(*([99] * 8))) == -1
        assert L.bgemm_debug_set_tc_schedule(7, (ctypes.c_int * 8)()) == -1
    finally:
        L.bgemm_debug_set_tc_schedule(2, None)
    back = (ctypes.c_int * 8)()
    L.bgemm_debug_get_tc_schedule(2, back)
    assert list(back) == list(orig)


def test_k_buckets():
    """K <= 64, then one octave per bucket, capped at the last bucket."""
    cases = {1: 0, 64: 0, 65: 1, 128: 1, 129: 2, 256: 2, 257: 3, 512: 3, 1024: 4, 1025: 5,
             2048: 5, 4096: 6, 4097: 7, 100000: 7}
    for K, b in cases.items():
        assert autotune._bucket(K) == b, K
    for b, K in enumerate(autotune.SCHED_BUCKET_K):
        assert autotune._bucket(K) == b


def test_cost_table_positive_for_every_runnable_configuration(built_lib):
    L = bg.lib()
    a, b = ctypes.c_float(), ctypes.c_float()
    for c in range(10):
        assert L.bgemm_debug_tile_cost(0, c, ctypes.byref(a), ctypes.byref(b)) == 0
        assert a.value > 0 and b.value > 0
    for mode in (1, 2, 3):
        for c in range(16):
            assert L.bgemm_debug_tile_cost(mode, c, ctypes.byref(a), ctypes.byref(b)) == 0
            if c >= 8 and (c & 3) == 3:
                continue  # no such CTA-pair tile
            assert a.value > 0 and b.value > 0, (mode, c)


def test_build_params_in_table_and_library(built_lib):
    """The compile-time schedule parameters the autotuner sweeps with a
    rebuild per candidate: written in the table, compiled into the library,
    and one of the candidates."""
    L = bg.lib()
    text = open(INC).read()
    ring = int(re.search(r"kSimtRingCap = (\d+);", text).group(1))
    lead = int(re.search(r"kTcCPrefetchLead = (\d+);", text).group(1))
    r, c = ctypes.c_int(), ctypes.c_int()
    assert L.bgemm_debug_build_params(ctypes.byref(r), ctypes.byref(c)) == 0
    assert (r.value, c.value) == (ring, lead)
    assert ring in autotune.BUILD_CANDIDATES["simt_ring_cap"]
    assert lead in autotune.BUILD_CANDIDATES["c_prefetch_lead"]
    assert L.bgemm_debug_build_params(None, ctypes.byref(c)) == -1


def test_write_table_round_trip(tmp_path):
    """autotune.write_table emits every table the library compiles in; the
    values read back from the text are the ones written."""
    simt = [(1000.0 + c, 10.0 + c) for c in range(len(autotune.SIMT_CFGS))]
    tc = {m: [((2000.0 + c, 5.0 + c) if c != 11 else None) for c in range(16)]
          for m in ("tf32", "tf32x3", "bf16x3")}
    sched = {"tf32": [0, 2, 2, 2, 2, 2, 2, 2], "tf32x3": [0, 1, 1, 1, 2, 3, 4, 4],
             "bf16x3": [0, 0, 3, 3, 4, 4, 4, 4]}
    params = {"simt_ring_cap": 6, "c_prefetch_lead": 0}
    out = tmp_path / "t.inc"
    autotune.write_table(str(out), simt, tc, sched, "test device", 152, params)
    text = out.read_text()
    rows = re.findall(r"\{([\d.]+)f, ([\d.]+)f\}", text.split("kSimtCost")[1].split(";")[0])
    assert [(float(a), float(b)) for a, b in rows] == simt
    tc_text = text.split("kTcCost")[1].split(";")[0]
    vals = re.findall(r"\{([\d.]+)f, ([\d.]+)f\}", tc_text)
    assert len(vals) == 48
    assert (float(vals[16 + 11][0]), float(vals[16 + 11][1])) == (0.0, 0.0)  # no such tile
    assert (float(vals[16 + 3][0]), float(vals[16 + 3][1])) == (2003.0, 8.0)
    g = re.search(r"kTcGroupTable\[3\]\[8\] = \{(.*)\};", text).group(1)
    assert [[int(x) for x in r.split(",")] for r in re.findall(r"\{([^{}]*)\}", g)] == [
        sched["tf32"], sched["tf32x3"], sched["bf16x3"]]
    assert "kSimtRingCap = 6;" in text and "kTcCPrefetchLead = 0;" in text
    assert "#define BGEMM_TUNED_HAS_SCHEDULE 1" in text
    assert "#define BGEMM_TUNED_HAS_BUILD_PARAMS 1" in text
