"""The batched engine from Python: many device-resident 2-D requests of
different sizes, ops and borders in one persistent launch
(``ifx_batch_run``).

Each request mirrors one reference call:
    ("gaussian", sigma)  imfilter(img, KernelFactors.gaussian((σ,σ)), border)
    ("factored", kx, ky) imfilter(img, (kx, ky), border) with 1-D factors of <= 33 taps
    ("sobel",) etc.      imgradients(img, KernelFactors.sobel, border)
    ("laplacian",)       imfilter(img, Kernel.Laplacian(), border)
    ("median", w)        mapwindow(median!, img, (w,w); border)
"""
import ctypes as C

import numpy as np

from . import _abi
from .arrays import DeviceArray, kind_of, ptr_strides, stream_for
from .borders import border_struct
from .kernels import KernelFactors

GRADIENTS = ("sobel", "prewitt", "scharr", "bickley", "ando3")
MEDIAN_OUT = {"N0F8": "F32", "U8": "F64", "F32": "F32"}


def out_kinds(op):
    name = op[0]
    if name in ("gaussian", "factored"):
        return ["F64"]
    if name in GRADIENTS:
        return ["F64", "F64"]
    return ["F32"]


class Batch:
    """A list of requests; keeps the host-side weight arrays alive."""

    def __init__(self):
        self.reqs = []
        self._keep = []

    def __len__(self):
        return len(self.reqs)

    def add(self, op, img, outs, border="replicate"):
        """op: a tuple as in the module docstring; img/outs: DeviceArray."""
        q = _abi.IfxRequest()
        kind = kind_of(img)
        p, st = ptr_strides(img)
        q.img = _abi.describe(p, kind, img.shape, st)
        for i, o in enumerate(outs):
            po, so = ptr_strides(o)
            q.out[i] = _abi.describe(po, kind_of(o), o.shape, so)
        q.border = border_struct(border, 2, kind)
        name = op[0]
        if name in ("gaussian", "factored"):
            if name == "gaussian":
                g = KernelFactors.gaussian(float(op[1]))
                fx = fy = (g.first[0], np.ascontiguousarray(g.data, dtype=np.float64))
            else:
                fx = (op[1].first[0], np.ascontiguousarray(op[1].data, dtype=np.float64))
                fy = (op[2].first[0], np.ascontiguousarray(op[2].data, dtype=np.float64))
            q.op = _abi.OP_FACTORED2D
            for a, (first, w) in enumerate((fx, fy)):
                q.taps[a] = w.size
                q.first[a] = first
                q.weights[a] = _abi.dptr(w)
                self._keep.append(w)
        elif name in GRADIENTS:
            d, s = getattr(KernelFactors, name).gradient_pair
            d = np.ascontiguousarray(d, dtype=np.float64)
            s = np.ascontiguousarray(s, dtype=np.float64)
            q.op = _abi.OP_GRADIENTS2D
            q.taps[0] = q.taps[1] = 3
            q.first[0] = q.first[1] = -1
            q.weights[0] = _abi.dptr(d)
            q.weights[1] = _abi.dptr(s)
            self._keep += [d, s]
        elif name == "laplacian":
            q.op = _abi.OP_LAPLACIAN2D
        elif name == "median":
            q.op = _abi.OP_MEDIAN2D
            q.window = int(op[1])
        else:
            raise _abi.Unsupported("batched op %r" % (name,))
        self.reqs.append(q)
        self._keep += [img, outs]
        return q

    def run(self, stream=None):
        """Enqueue the whole batch; returns the number of tiles."""
        ctx = _abi.context()
        arr = (_abi.IfxRequest * max(1, len(self.reqs)))(*self.reqs)
        tiles = C.c_int64()
        if stream is None and self._keep:
            stream = stream_for(*[k for k in self._keep if isinstance(k, DeviceArray)])
        _abi.check(ctx.lib.ifx_batch_run(ctx.handle, arr, len(self.reqs), C.byref(tiles), stream))
        self._arr = arr
        return tiles.value


class Plan:
    """A batch validated once (ifx_batch_plan_create); launch() replays it."""

    def __init__(self, batch):
        self.batch = batch
        self.ctx = _abi.context()
        self._arr = (_abi.IfxRequest * max(1, len(batch.reqs)))(*batch.reqs)
        h = C.c_void_p()
        _abi.check(self.ctx.lib.ifx_batch_plan_create(self.ctx.handle, self._arr, len(batch.reqs),
                                                      C.byref(h)))
        self.handle = h

    def launch(self, stream=None):
        tiles = C.c_int64()
        if stream is None:
            stream = stream_for(*[k for k in self.batch._keep if isinstance(k, DeviceArray)])
        _abi.check(self.ctx.lib.ifx_batch_plan_launch(self.handle, C.byref(tiles), stream))
        return tiles.value

    def close(self):
        if self.handle:
            self.ctx.lib.ifx_batch_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def outputs_for(op, img):
    """Device outputs with the eltypes the reference returns."""
    kinds = out_kinds(op)
    if op[0] == "median":
        kinds = [MEDIAN_OUT[kind_of(img)]]
    return [DeviceArray.empty(img.shape, k, img.tensor.device) for k in kinds]


_KIND_CODE = {"F32": 0, "F64": 1, "N0F8": 2, "U8": 3}
_OP_CODE = {"factored": 1, "gradients": 2, "laplacian": 3, "median": 4}


def autotune_lookup(op, in_kind, out_kind, kx=0, ky=0, window=0):
    """The batched engine's cached tile for a key, {"tile_w", "tile_h", "ms"},
    or None.  op: "factored" (kx, ky = the factors' taps), "gradients",
    "laplacian" or "median" (window 3 or 5)."""
    ctx = _abi.context()
    ch = _abi.IfxTuneChoice()
    rc = ctx.lib.ifx_batch_autotune_lookup(ctx.handle, _OP_CODE[op], _KIND_CODE[in_kind], _KIND_CODE[out_kind],
                                           int(kx), int(ky), int(window), C.byref(ch))
    if rc:
        return None
    return {"tile_w": ch.tile_w, "tile_h": ch.tile_h, "ms": ch.ms}


def autotune_pin(op, in_kind, out_kind, tile_w, tile_h, kx=0, ky=0, window=0):
    """Pin the batched engine's tile for a key (batches described after this
    use it; a tile the engine cannot take runs as the default)."""
    ctx = _abi.context()
    ch = _abi.IfxTuneChoice(0, 0, int(tile_w), int(tile_h), 0, 0.0)
    _abi.check(ctx.lib.ifx_batch_autotune_pin(ctx.handle, _OP_CODE[op], _KIND_CODE[in_kind], _KIND_CODE[out_kind],
                                              int(kx), int(ky), int(window), C.byref(ch)))
