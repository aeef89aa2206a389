"""The HBM streaming probe behind the pre-pass roofline
(bgemm_debug_hbm_probe): its kernels move the bytes they are credited with,
and invalid arguments are refused before any launch."""
import ctypes

import pytest

import batchgemm_gb300 as bg


def test_probe_rejects_invalid_arguments(built_lib):
    L = bg.lib()
    buf = (ctypes.c_float * 64)()
    p = ctypes.addressof(buf)
    assert L.bgemm_debug_hbm_probe(4, p, p, p, 4, 1, None) == -1      # no such kind
    assert L.bgemm_debug_hbm_probe(0, p, p, None, 4, 1, None) == -1   # kind 0 needs y2
    assert L.bgemm_debug_hbm_probe(1, None, p, p, 4, 1, None) == -1   # kind 1 needs x
    assert L.bgemm_debug_hbm_probe(2, p, None, p, 4, 1, None) == -1   # every kind needs y1
    assert L.bgemm_debug_hbm_probe(1, p + 4, p, p, 4, 1, None) == -1  # not 16-byte aligned
    assert L.bgemm_debug_hbm_probe(1, p, p, p, 0, 1, None) == -1      # empty
    assert L.bgemm_debug_hbm_probe(1, p, p, p, 4, 0, None) == -1      # no CTA


@pytest.mark.gpu
def test_probe_kernels_move_their_bytes(cuda):
    torch = pytest.importorskip("torch")
    L = bg.lib()
    n = (1 << 20) + 4  # floats; not a multiple of the grid
    x = torch.rand(n, device="cuda")
    y1 = torch.zeros_like(x)
    y2 = torch.zeros_like(x)
    st = torch.cuda.current_stream().cuda_stream
    assert L.bgemm_debug_hbm_probe(0, x.data_ptr(), y1.data_ptr(), y2.data_ptr(), n // 4, 37,
                                   st) == 0
    torch.cuda.synchronize()
    assert torch.equal(y1, x) and torch.equal(y2, x * 0.5)
    y1.zero_()
    assert L.bgemm_debug_hbm_probe(1, x.data_ptr(), y1.data_ptr(), None, n // 4, 5, st) == 0
    assert L.bgemm_debug_hbm_probe(2, None, y2.data_ptr(), None, n // 4, 5, st) == 0
    assert L.bgemm_debug_hbm_probe(3, x.data_ptr(), y2.data_ptr(), None, n // 4, 5, st) == 0
    torch.cuda.synchronize()
    assert torch.equal(y1, x)
    assert torch.equal(y2[:8], torch.tensor([1.0, 2.0, 3.0, 4.0] * 2, device="cuda"))
