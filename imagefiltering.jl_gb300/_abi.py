"""ctypes binding of the C ABI in ``include/ifx_gb300.h``.

This is the same binding a Julia ``ccall`` layer makes; here it serves the
Python mirror of the reference API and the tests.  Loading fails loudly when
the CUDA library has not been built: there is no CPU fallback.
"""
import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libifx_gb300.so")

# ifx_eltype
F32, F64, N0F8, U8, I16 = 0, 1, 2, 3, 4
I8, U16, I32, I64, N0F16 = 5, 6, 7, 8, 9
# ifx_style
STYLES = {"replicate": 0, "circular": 1, "symmetric": 2, "reflect": 3, "fill": 4}
MAX_DIMS = 4
MAX_TAPS = 129


class ArgumentError(ValueError):
    """The reference's ArgumentError."""


class DimensionMismatch(ValueError):
    """The reference's DimensionMismatch."""


class ErrorException(RuntimeError):
    """The reference's error(...) / DivideError."""


class CudaError(RuntimeError):
    pass


class OutOfMemory(MemoryError):
    pass


class Unsupported(NotImplementedError):
    """A case the GB300 path does not implement (no CPU fallback exists)."""


class Cancelled(RuntimeError):
    """A served request cancelled before it ran."""


class InexactError(ValueError):
    """Julia's InexactError: a value does not fit the target eltype."""


_EXC = {1: ArgumentError, 2: DimensionMismatch, 3: ErrorException, 4: CudaError, 5: OutOfMemory,
        6: TimeoutError, 7: Unsupported, 8: Cancelled}


class IfxArray(C.Structure):
    _fields_ = [("data", C.c_void_p), ("eltype", C.c_int32), ("ndim", C.c_int32),
                ("size", C.c_int64 * 4), ("stride", C.c_int64 * 4), ("first", C.c_int64 * 4)]


class IfxBorder(C.Structure):
    _fields_ = [("style", C.c_int32), ("explicit_pad", C.c_int32), ("lo", C.c_int64 * 4),
                ("hi", C.c_int64 * 4), ("fill_value", C.c_double)]


class IfxFactor(C.Structure):
    _fields_ = [("axis", C.c_int32), ("length", C.c_int32), ("first", C.c_int64),
                ("weights", C.POINTER(C.c_double))]


class IfxIir(C.Structure):
    _fields_ = [("axis", C.c_int32), ("coef_f32", C.c_int32), ("a", C.c_double * 3), ("b", C.c_double * 3),
                ("scale", C.c_double), ("M", C.c_double * 9), ("asum", C.c_double), ("bsum", C.c_double)]


class IfxRequest(C.Structure):
    _fields_ = [("op", C.c_int32), ("window", C.c_int32), ("img", IfxArray), ("out", IfxArray * 2),
                ("border", IfxBorder), ("taps", C.c_int32 * 2), ("first", C.c_int64 * 2),
                ("weights", C.POINTER(C.c_double) * 2)]


OP_FACTORED2D, OP_GRADIENTS2D, OP_LAPLACIAN2D, OP_MEDIAN2D = 1, 2, 3, 4


class IfxTuneChoice(C.Structure):
    _fields_ = [("variant", C.c_int32), ("x_first", C.c_int32), ("tile_w", C.c_int32), ("tile_h", C.c_int32),
                ("depth", C.c_int32), ("ms", C.c_double)]


TUNE_SEP2D, TUNE_SEP3D = 0, 1


class IfxServerConfig(C.Structure):
    _fields_ = [("hbm_cap_bytes", C.c_int64), ("max_batch", C.c_int32), ("max_inflight", C.c_int32)]


class IfxServerMetrics(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("batches", C.c_uint64), ("pixels", C.c_uint64), ("p50_latency_s", C.c_double),
                ("p99_latency_s", C.c_double), ("max_latency_s", C.c_double), ("busy_s", C.c_double),
                ("hbm_in_use", C.c_int64), ("hbm_peak", C.c_int64), ("queue_depth", C.c_int32),
                ("deferred_free", C.c_uint64)]

SYMBOLS = ["ifx_abi_version", "ifx_create", "ifx_destroy", "ifx_last_error", "ifx_launch_count",
           "ifx_synchronize", "ifx_padarray", "ifx_imfilter_factored", "ifx_imfilter_dense",
           "ifx_imfilter_laplacian", "ifx_imgradients", "ifx_mapwindow_median",
           "ifx_mapwindow_extrema", "ifx_batch_run", "ifx_batch_plan_create", "ifx_batch_plan_launch",
           "ifx_batch_plan_destroy", "ifx_server_create", "ifx_server_submit",
           "ifx_server_wait", "ifx_server_drain", "ifx_server_metrics", "ifx_server_reset_metrics",
           "ifx_server_destroy", "ifx_noalloc_scratch_bytes", "ifx_imfilter_factored_noalloc",
           "ifx_na_prepare", "ifx_na_divide", "ifx_na_normalize_separable",
           "ifx_imfilter_factored_sum", "ifx_findlocalextrema", "ifx_maxabs", "ifx_imfilter_fft",
           "ifx_imfilter_iir", "ifx_autotune", "ifx_autotune_choice", "ifx_server_cancel",
           "ifx_server_inject_launch_error", "ifx_server_pause", "ifx_debug_force_wait_timeout", "ifx_convert",
           "ifx_autotune_lookup", "ifx_autotune_pin", "ifx_autotune_clear", "ifx_batch_autotune_lookup",
           "ifx_batch_autotune_pin"]

_lib = None
_lock = threading.Lock()


def load(path: str = LIB_PATH):
    """Load the shared library and declare its prototypes."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(path):
            raise RuntimeError("libifx_gb300.so is not built (run __graft_entry__.build()); the "
                               "GB300 path has no CPU fallback")
        lib = C.CDLL(path)
        P = C.POINTER
        vp = C.c_void_p
        lib.ifx_abi_version.restype = C.c_int
        lib.ifx_create.argtypes = [P(vp), C.c_int]
        lib.ifx_destroy.argtypes = [vp]
        lib.ifx_last_error.restype = C.c_char_p
        lib.ifx_launch_count.restype = C.c_uint64
        lib.ifx_synchronize.argtypes = [vp, vp]
        lib.ifx_debug_force_wait_timeout.argtypes = [vp, C.c_int32]
        lib.ifx_convert.argtypes = [vp, P(IfxArray), P(IfxArray), vp]
        lib.ifx_padarray.argtypes = [vp, P(IfxArray), P(IfxArray), P(IfxBorder), vp]
        lib.ifx_imfilter_factored.argtypes = [vp, P(IfxArray), P(IfxArray), C.c_int32,
                                              P(IfxFactor), P(IfxBorder), vp]
        lib.ifx_imfilter_dense.argtypes = [vp, P(IfxArray), P(IfxArray), P(C.c_double),
                                           P(C.c_int64), P(C.c_int64), P(IfxBorder), C.c_int32, vp]
        lib.ifx_imfilter_laplacian.argtypes = [vp, P(IfxArray), P(IfxArray), P(C.c_int32),
                                               P(IfxBorder), vp]
        lib.ifx_imgradients.argtypes = [vp, P(IfxArray), P(IfxArray), P(C.c_double),
                                        P(C.c_double), C.c_int32, C.c_int64, P(C.c_int32),
                                        P(IfxBorder), vp]
        lib.ifx_mapwindow_median.argtypes = [vp, P(IfxArray), P(IfxArray), P(C.c_int64),
                                             P(C.c_int64), P(IfxBorder), vp]
        lib.ifx_mapwindow_extrema.argtypes = [vp, P(IfxArray), P(IfxArray), P(C.c_int64),
                                              P(C.c_int64), P(IfxBorder), C.c_int32, vp]
        lib.ifx_batch_run.argtypes = [vp, P(IfxRequest), C.c_int32, P(C.c_int64), vp]
        lib.ifx_batch_plan_create.argtypes = [vp, P(IfxRequest), C.c_int32, P(vp)]
        lib.ifx_batch_plan_launch.argtypes = [vp, P(C.c_int64), vp]
        lib.ifx_batch_plan_destroy.argtypes = [vp]
        lib.ifx_server_create.argtypes = [vp, P(IfxServerConfig), P(vp)]
        lib.ifx_server_submit.argtypes = [vp, P(IfxRequest), P(C.c_uint64)]
        lib.ifx_server_wait.argtypes = [vp, C.c_uint64, C.c_double, P(C.c_int32)]
        lib.ifx_server_drain.argtypes = [vp, C.c_double]
        lib.ifx_server_cancel.argtypes = [vp, C.c_uint64]
        lib.ifx_server_inject_launch_error.argtypes = [vp, C.c_int32]
        lib.ifx_server_pause.argtypes = [vp, C.c_int32]
        lib.ifx_server_metrics.argtypes = [vp, P(IfxServerMetrics)]
        lib.ifx_server_reset_metrics.argtypes = [vp]
        lib.ifx_server_destroy.argtypes = [vp]
        lib.ifx_na_prepare.argtypes = [vp, P(IfxArray), P(IfxArray), P(IfxArray), C.c_int32,
                                       P(C.c_int32), vp]
        lib.ifx_na_divide.argtypes = [vp, P(IfxArray), P(IfxArray), vp]
        lib.ifx_na_normalize_separable.argtypes = [vp, P(IfxArray), P(IfxArray), vp]
        lib.ifx_imfilter_factored_sum.argtypes = [vp, P(IfxArray), P(IfxArray), C.c_int32, C.c_int32,
                                                  P(IfxFactor), C.c_double, P(IfxBorder), vp]
        lib.ifx_findlocalextrema.argtypes = [vp, P(IfxArray), P(C.c_int32), P(C.c_int32), C.c_int32,
                                             P(C.c_int64), P(C.c_double), C.c_int64, P(C.c_int64), vp]
        lib.ifx_maxabs.argtypes = [vp, P(IfxArray), P(C.c_double), vp]
        lib.ifx_autotune.argtypes = [vp, C.c_int32, C.c_char_p]
        lib.ifx_autotune_choice.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64,
                                            C.c_int64, P(C.c_int32), P(C.c_int32), P(C.c_double)]
        lib.ifx_autotune_lookup.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, P(C.c_int32), C.c_int32,
                                            P(C.c_int64), P(IfxTuneChoice)]
        lib.ifx_autotune_pin.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, P(C.c_int32), C.c_int32,
                                         P(C.c_int64), P(IfxTuneChoice)]
        lib.ifx_autotune_clear.argtypes = [vp]
        lib.ifx_batch_autotune_lookup.argtypes = [vp] + [C.c_int32] * 6 + [P(IfxTuneChoice)]
        lib.ifx_batch_autotune_pin.argtypes = [vp] + [C.c_int32] * 6 + [P(IfxTuneChoice)]
        lib.ifx_imfilter_iir.argtypes = [vp, P(IfxArray), P(IfxArray), C.c_int32, P(IfxIir), P(IfxBorder), vp]
        lib.ifx_imfilter_fft.argtypes = [vp, P(IfxArray), P(IfxArray), P(C.c_double), P(C.c_int64),
                                         P(C.c_int64), P(IfxBorder), vp]
        lib.ifx_noalloc_scratch_bytes.restype = C.c_uint64
        lib.ifx_imfilter_factored_noalloc.argtypes = [P(IfxArray), P(IfxArray), C.c_int32, P(IfxFactor),
                                                      P(IfxBorder), vp]
        for name in SYMBOLS:
            getattr(lib, name)          # every declared entry point must be exported
        _lib = lib
        return lib


def check(rc: int) -> None:
    if rc != 0:
        msg = load().ifx_last_error().decode(errors="replace")
        raise _EXC.get(rc, RuntimeError)(msg)


class Context:
    """One library context (device, stream, scratch buffers)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.ifx_create(C.byref(h), int(device)))
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.ifx_destroy(self.handle)
            self.handle = None

    def synchronize(self, stream=None):
        check(self.lib.ifx_synchronize(self.handle, stream))


_ctx = None


def context() -> Context:
    """The process-wide default context (device from IFX_DEVICE, default 0)."""
    global _ctx
    if _ctx is None:
        _ctx = Context(int(os.environ.get("IFX_DEVICE", "0")))
    return _ctx


def launch_count() -> int:
    return int(load().ifx_launch_count())


# ----------------------------------------------------------------- descriptors
def eltype_code(kind: str) -> int:
    return {"F32": F32, "F64": F64, "N0F8": N0F8, "U8": U8, "I16": I16, "I8": I8, "U16": U16, "I32": I32,
            "I64": I64, "N0F16": N0F16}[kind]


def describe(data_ptr: int, kind: str, shape, strides=None, first=None) -> IfxArray:
    a = IfxArray()
    a.data = data_ptr
    a.eltype = eltype_code(kind)
    a.ndim = len(shape)
    if not 1 <= a.ndim <= MAX_DIMS:
        raise Unsupported("arrays of %d dimensions (1..4 supported)" % a.ndim)
    s = 1
    for d, n in enumerate(shape):
        a.size[d] = int(n)
        a.stride[d] = int(strides[d]) if strides is not None else s
        a.first[d] = int(first[d]) if first is not None else 1
        s *= int(n)
    return a


def border_struct(style: str, lo=None, hi=None, fill=0.0) -> IfxBorder:
    b = IfxBorder()
    b.style = STYLES[style]
    b.fill_value = float(fill)
    if lo is not None:
        b.explicit_pad = 1
        for d, v in enumerate(lo):
            b.lo[d] = int(v)
        for d, v in enumerate(hi):
            b.hi[d] = int(v)
    return b


def dptr(arr: np.ndarray):
    return C.cast(arr.ctypes.data, C.POINTER(C.c_double))
