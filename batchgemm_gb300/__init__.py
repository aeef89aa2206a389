"""GB300-native variable-size batched SGEMM.

Python mirror of the C ABI in ``include/bgemm.h`` (``libbgemm_gb300.so``),
bound with ctypes exactly as a user of the shared library would bind it.  The
library is the product; this module only loads it, converts arguments and
raises on non-success statuses.  There is no Python or CPU fallback: if the
shared library is missing, :func:`lib` raises.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional, Sequence

__all__ = [
    "BgemmError", "MODES", "lib", "build", "sgemm_vbatched", "sgemm_vbatched_ex", "Plan",
    "plan_requirements", "max_requirements", "framework_gemm", "framework_gemm_mode",
    "framework_release", "framework_check_device", "device_info", "LIB_PATH",
    "plan_cache_set_limit", "plan_cache_clear", "plan_cache_stats",
]

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libbgemm_gb300.so")

MODES = {"simt": 0, "tf32": 1, "tf32x3": 2, "bf16x3": 3}
MODE_NAMES = {v: k for k, v in MODES.items()}

STATUS = {
    0: "BGEMM_SUCCESS", 1: "BGEMM_ERROR_INVALID_VALUE", 2: "BGEMM_ERROR_NOT_SUPPORTED",
    3: "BGEMM_ERROR_ALLOC", 4: "BGEMM_ERROR_CUDA", 5: "BGEMM_ERROR_DEVICE_TIMEOUT",
    6: "BGEMM_ERROR_INTERNAL",
}

_lib: Optional[ctypes.CDLL] = None


class BgemmError(RuntimeError):
    def __init__(self, status: int, arg: int, matrix: int, message: str):
        self.status, self.arg, self.matrix, self.message = status, arg, matrix, message
        super().__init__("%s (arg %d, matrix %d): %s" % (STATUS.get(status, status), arg,
                                                         matrix, message))


class PlanInfo(ctypes.Structure):
    _fields_ = [
        ("batch", ctypes.c_int), ("mode", ctypes.c_int), ("num_tiles", ctypes.c_int),
        ("grid", ctypes.c_int), ("tile_config_hist", ctypes.c_int * 16),
        ("useful_flops", ctypes.c_double), ("min_bytes", ctypes.c_double),
        ("device_bytes", ctypes.c_size_t), ("workspace_bytes", ctypes.c_size_t),
        ("kernels_per_execute", ctypes.c_int), ("reserved", ctypes.c_int * 7),
    ]

    def as_dict(self):
        return {
            "batch": self.batch, "mode": self.mode, "num_tiles": self.num_tiles,
            "grid": self.grid, "tile_config_hist": list(self.tile_config_hist),
            "useful_flops": self.useful_flops, "min_bytes": self.min_bytes,
            "device_bytes": self.device_bytes, "workspace_bytes": self.workspace_bytes,
            "kernels_per_execute": self.kernels_per_execute,
        }


class PlanRequirements(ctypes.Structure):
    """bgemm_plan_requirements_t: device sizes of a batch inside a plan."""
    _fields_ = [("batch", ctypes.c_int), ("tiles", ctypes.c_int), ("pack_jobs", ctypes.c_int),
                ("kernel_family", ctypes.c_int), ("workspace_bytes", ctypes.c_size_t),
                ("simt_tiles", ctypes.c_int), ("reserved", ctypes.c_int * 3)]
    KEYS = ("batch", "tiles", "pack_jobs", "kernel_family", "workspace_bytes", "simt_tiles")

    def as_dict(self):
        return {k: getattr(self, k) for k in self.KEYS}

    @classmethod
    def from_dict(cls, d):
        r = cls()
        for k in cls.KEYS:
            setattr(r, k, int(d.get(k, 0)))
        return r


KERNEL_FAMILIES = {"auto": 0, "single": 1, "pair": 2}


class PlanOptions(ctypes.Structure):
    _fields_ = [("force_tile_config", ctypes.c_int), ("max_ctas", ctypes.c_int),
                ("disable_rebalance", ctypes.c_int), ("host_tensor_maps", ctypes.c_int),
                ("kernel_family", ctypes.c_int),
                ("layout", ctypes.c_int), ("trans_a", ctypes.c_int), ("trans_b", ctypes.c_int),
                ("simt_below", ctypes.c_int), ("reserved", ctypes.c_int * 2),
                ("capacity", PlanRequirements)]


LAYOUTS = {"col": 0, "row": 1}


def _layout(v) -> int:
    return LAYOUTS[v] if isinstance(v, str) else int(v)


def _op(v) -> int:
    if isinstance(v, str):
        return {"N": 0, "T": 1, "n": 0, "t": 1}[v]
    return int(bool(v))


def _options(force_tile_config=-1, max_ctas=0, rebalance=True, host_tensor_maps=False,
             kernel_family="auto", capacity=None, layout="col",
             trans_a=False, trans_b=False, simt_below=0) -> PlanOptions:
    opt = PlanOptions()
    opt.simt_below = int(simt_below)
    opt.layout = _layout(layout)
    opt.trans_a = _op(trans_a)
    opt.trans_b = _op(trans_b)
    opt.force_tile_config = force_tile_config
    opt.max_ctas = max_ctas
    opt.disable_rebalance = 0 if rebalance else 1
    opt.host_tensor_maps = 1 if host_tensor_maps else 0
    opt.kernel_family = (KERNEL_FAMILIES[kernel_family] if isinstance(kernel_family, str)
                         else int(kernel_family))
    if capacity is not None:
        opt.capacity = (capacity if isinstance(capacity, PlanRequirements)
                        else PlanRequirements.from_dict(capacity))
    return opt


def build(**kw) -> str:
    """Compile libbgemm_gb300.so for sm_103a (see builder.py)."""
    from . import builder
    return builder.build(**kw)


def lib() -> ctypes.CDLL:
    """Load libbgemm_gb300.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libbgemm_gb300.so is not built (run __graft_entry__.build() or "
                           "python -m batchgemm_gb300.build)")
    L = ctypes.CDLL(LIB_PATH)
    i, f, vp = ctypes.c_int, ctypes.c_float, ctypes.c_void_p
    ip = ctypes.POINTER(ctypes.c_int)
    L.bgemm_sgemm_vbatched.argtypes = [ip, ip, ip, f, vp, ip, vp, ip, f, vp, ip, i, i, vp]
    L.bgemm_sgemm_vbatched_ex.argtypes = [i, i, i, ip, ip, ip, f, vp, ip, vp, ip, f, vp, ip, i, i,
                                          vp]
    L.bgemm_plan_create.argtypes = [ctypes.POINTER(vp), ip, ip, ip, ip, ip, ip, i, i, vp]
    L.bgemm_plan_create_ex.argtypes = [ctypes.POINTER(vp), ip, ip, ip, ip, ip, ip, i, i, vp,
                                       ctypes.POINTER(PlanOptions)]
    L.bgemm_plan_execute.argtypes = [vp, f, vp, vp, f, vp, vp]
    L.bgemm_plan_info.argtypes = [vp, ctypes.POINTER(PlanInfo)]
    L.bgemm_plan_requirements.argtypes = [ip, ip, ip, ip, ip, ip, i, i,
                                          ctypes.POINTER(PlanOptions),
                                          ctypes.POINTER(PlanRequirements)]
    L.bgemm_plan_update.argtypes = [vp, ip, ip, ip, ip, ip, ip, i, vp]
    L.bgemm_plan_capacity.argtypes = [vp, ctypes.POINTER(PlanRequirements)]
    L.bgemm_plan_check_device.argtypes = [vp, vp]
    L.bgemm_plan_set_kernel_events.argtypes = [vp, vp, vp]
    L.bgemm_plan_set_cta_timer.argtypes = [vp, vp]
    L.bgemm_plan_destroy.argtypes = [vp]
    L.bgemm_framework_gemm.argtypes = [vp, vp, vp, vp, vp, vp, vp, i, i, vp]
    L.bgemm_framework_check_device.argtypes = [vp]
    L.bgemm_framework_release.argtypes = []
    L.bgemm_framework_gemm_noalloc.argtypes = [vp, vp, vp, vp, vp, vp, i, i, vp, vp]
    L.bgemm_framework_gemm_mode.argtypes = [vp, vp, vp, vp, vp, vp, i, i, i, ctypes.c_longlong,
                                            i, vp]
    L.bgemm_last_error_arg.argtypes = [ip]
    L.bgemm_last_error_arg.restype = i
    L.bgemm_last_error_message.restype = ctypes.c_char_p
    L.bgemm_status_string.argtypes = [i]
    L.bgemm_status_string.restype = ctypes.c_char_p
    L.bgemm_device_info.argtypes = [ip, ip, ip]
    L.bgemm_version.restype = i
    L.bgemm_plan_cache_set_limit.argtypes = [ctypes.c_size_t]
    L.bgemm_plan_cache_clear.argtypes = []
    ll = ctypes.POINTER(ctypes.c_longlong)
    L.bgemm_debug_plan_cache_stats.argtypes = [ll] * 7
    L.bgemm_debug_plan_cache_stats.restype = i
    L.bgemm_debug_set_tc_schedule.argtypes = [i, vp]
    L.bgemm_debug_get_tc_schedule.argtypes = [i, vp]
    L.bgemm_debug_tile_cost.argtypes = [i, i, ctypes.POINTER(f), ctypes.POINTER(f)]
    L.bgemm_debug_build_params.argtypes = [ctypes.POINTER(i), ctypes.POINTER(i)]
    L.bgemm_debug_hbm_probe.argtypes = [i, vp, vp, vp, ctypes.c_longlong, i, vp]
    for name in ("bgemm_sgemm_vbatched", "bgemm_plan_create", "bgemm_plan_create_ex",
                 "bgemm_plan_execute", "bgemm_plan_info", "bgemm_plan_check_device",
                 "bgemm_plan_destroy", "bgemm_framework_gemm", "bgemm_framework_check_device",
                 "bgemm_framework_gemm_noalloc", "bgemm_framework_gemm_mode", "bgemm_framework_release",
                 "bgemm_device_info",
                 "bgemm_plan_set_kernel_events", "bgemm_plan_set_cta_timer",
                 "bgemm_plan_requirements",
                 "bgemm_plan_update", "bgemm_plan_capacity", "bgemm_sgemm_vbatched_ex",
                 "bgemm_plan_cache_set_limit", "bgemm_plan_cache_clear"):
        getattr(L, name).restype = i
    _lib = L
    return L


def _check(status: int) -> None:
    if status != 0:
        L = lib()
        m = ctypes.c_int(-1)
        arg = L.bgemm_last_error_arg(ctypes.byref(m))
        msg = (L.bgemm_last_error_message() or b"").decode(errors="replace")
        raise BgemmError(status, arg, m.value, msg)


def _iarr(v: Sequence[int]):
    if isinstance(v, ctypes.Array):  # already converted (hot loops convert once)
        return v
    n = len(v)
    return (ctypes.c_int * max(n, 1))(*[int(x) for x in v])


def int_array(v: Sequence[int]):
    """A ctypes int array for the size arguments (convert once, reuse in loops)."""
    return _iarr(v)


def _mode(mode) -> int:
    return MODES[mode] if isinstance(mode, str) else int(mode)


def _stream(stream) -> Optional[int]:
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream or None
    return int(stream) or None


def sgemm_vbatched(M, N, K, alpha, dA, lda, dB, ldb, beta, dC, ldc, mode="simt",
                   stream=None) -> None:
    """bgemm_sgemm_vbatched: host size arrays, device addresses of the pointer arrays."""
    _check(lib().bgemm_sgemm_vbatched(_iarr(M), _iarr(N), _iarr(K), float(alpha), dA,
                                      _iarr(lda), dB, _iarr(ldb), float(beta), dC, _iarr(ldc),
                                      len(M), _mode(mode), _stream(stream)))


def plan_requirements(M, N, K, lda, ldb, ldc, mode="simt", **options) -> dict:
    """bgemm_plan_requirements: the device sizes a batch needs in a plan made
    with these options (host-only planning, nothing allocated)."""
    opt = _options(**options)
    out = PlanRequirements()
    _check(lib().bgemm_plan_requirements(_iarr(M), _iarr(N), _iarr(K), _iarr(lda), _iarr(ldb),
                                         _iarr(ldc), len(M), _mode(mode), ctypes.byref(opt),
                                         ctypes.byref(out)))
    return out.as_dict()


def max_requirements(reqs) -> dict:
    """Element-wise maximum of requirement dicts (a capacity for all of them)."""
    out = {k: 0 for k in PlanRequirements.KEYS}
    for r in reqs:
        for k in out:
            out[k] = max(out[k], int(r[k]))
    return out


def sgemm_vbatched_ex(layout, trans_a, trans_b, M, N, K, alpha, dA, lda, dB, ldb, beta, dC,
                      ldc, mode="simt", stream=None) -> None:
    """bgemm_sgemm_vbatched_ex: storage order ("col"/"row") and op(A), op(B) ("N"/"T")."""
    _check(lib().bgemm_sgemm_vbatched_ex(_layout(layout), _op(trans_a), _op(trans_b), _iarr(M),
                                         _iarr(N), _iarr(K), float(alpha), dA, _iarr(lda), dB,
                                         _iarr(ldb), float(beta), dC, _iarr(ldc), len(M),
                                         _mode(mode), _stream(stream)))


class Plan:
    """bgemm_plan_create / execute / update / destroy."""

    def __init__(self, M, N, K, lda, ldb, ldc, mode="simt", stream=None,
                 force_tile_config: int = -1, max_ctas: int = 0, rebalance: bool = True,
                 host_tensor_maps: bool = False, kernel_family="auto", capacity=None,
                 layout="col", trans_a=False, trans_b=False, simt_below: int = 0):
        self._h = ctypes.c_void_p()
        self.batch = len(M)
        opt = _options(force_tile_config, max_ctas, rebalance, host_tensor_maps,
                       kernel_family, capacity, layout, trans_a, trans_b, simt_below)
        _check(lib().bgemm_plan_create_ex(ctypes.byref(self._h), _iarr(M), _iarr(N), _iarr(K),
                                          _iarr(lda), _iarr(ldb), _iarr(ldc), len(M),
                                          _mode(mode), _stream(stream), ctypes.byref(opt)))

    def execute(self, alpha, dA, dB, beta, dC, stream=None) -> None:
        _check(lib().bgemm_plan_execute(self._h, float(alpha), dA, dB, float(beta), dC,
                                        _stream(stream)))

    def update(self, M, N, K, lda, ldb, ldc, stream=None) -> None:
        """bgemm_plan_update: re-plan a new batch into this plan's buffers."""
        n = len(M)
        _check(lib().bgemm_plan_update(self._h, _iarr(M), _iarr(N), _iarr(K), _iarr(lda),
                                       _iarr(ldb), _iarr(ldc), n, _stream(stream)))
        self.batch = n

    def capacity(self) -> dict:
        out = PlanRequirements()
        _check(lib().bgemm_plan_capacity(self._h, ctypes.byref(out)))
        return out.as_dict()

    def info(self) -> dict:
        inf = PlanInfo()
        _check(lib().bgemm_plan_info(self._h, ctypes.byref(inf)))
        return inf.as_dict()

    def check_device(self, stream=None) -> None:
        _check(lib().bgemm_plan_check_device(self._h, _stream(stream)))

    def set_kernel_events(self, start=None, stop=None) -> None:
        """Record these torch.cuda.Event objects around the plan's GEMM kernel
        in every following execute (they must have been recorded once, so that
        the CUDA event exists)."""
        h = lambda e: None if e is None else (e.cuda_event or None)
        _check(lib().bgemm_plan_set_kernel_events(self._h, h(start), h(stop)))

    def set_cta_timer(self, d_times=None) -> None:
        """Per-CTA start/end global-timer stamps of the GEMM kernel into the
        device buffer at address d_times (2 x grid uint64), or stop (None)."""
        _check(lib().bgemm_plan_set_cta_timer(self._h, d_times))

    def close(self) -> None:
        if self._h:
            _check(lib().bgemm_plan_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def framework_gemm(dM, dN, dK, dA, dB, dC, batch: int, max_dim: int, stream=None,
                   dT=None) -> None:
    """Reference drop-in: device size arrays, C_i += A_i B_i (lda=M, ldb=K, ldc=M)."""
    _check(lib().bgemm_framework_gemm(dM, dN, dK, dA, dB, dC, dT, int(batch), int(max_dim),
                                      _stream(stream)))


def framework_gemm_mode(dM, dN, dK, dA, dB, dC, batch: int, max_dim: int, max_k: int,
                        mode="tf32x3", stream=None, max_operand_elems: int = 0) -> None:
    """The same device-size entry in any mode: for the tensor-core modes the
    tile queue, split operands and tensor maps are built on the device.
    max_dim bounds every M and N, max_k every K, max_operand_elems the sum of
    (M + N) * K over the batch (0: batch * 2 * max_dim * max_k); they size
    the library's scratch."""
    _check(lib().bgemm_framework_gemm_mode(dM, dN, dK, dA, dB, dC, int(batch), int(max_dim),
                                           int(max_k), int(max_operand_elems), _mode(mode),
                                           _stream(stream)))


def framework_release() -> None:
    """Free the framework entries' scratch on the current device."""
    _check(lib().bgemm_framework_release())


def framework_check_device(stream=None) -> None:
    _check(lib().bgemm_framework_check_device(_stream(stream)))


def plan_cache_set_limit(nbytes: int) -> None:
    """Device bytes the one-shot entries' cached plans may hold (0: default)."""
    _check(lib().bgemm_plan_cache_set_limit(int(nbytes)))


def plan_cache_clear() -> None:
    """Free every evictable cached plan of the current device."""
    _check(lib().bgemm_plan_cache_clear())


def plan_cache_stats() -> dict:
    """Counters of the plan cache on the current device."""
    v = [ctypes.c_longlong() for _ in range(7)]
    lib().bgemm_debug_plan_cache_stats(*[ctypes.byref(x) for x in v])
    keys = ("entries", "bytes", "hits", "reorders", "misses", "evictions", "limit")
    return {k: x.value for k, x in zip(keys, v)}


def device_info() -> dict:
    a, b, c = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    _check(lib().bgemm_device_info(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
    return {"num_sms": a.value, "simt_ctas_per_sm": b.value, "tc_ctas_per_sm": c.value}
