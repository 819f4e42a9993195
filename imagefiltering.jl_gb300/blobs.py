"""blob_LoG, multiLoG, findlocalmaxima / findlocalminima (src/extrema.jl)
on the GB300 path: the Laplacian-of-Gaussian stack, the local-extrema search
and maximum(abs, img) run as library kernels; this module builds the LoG terms
and formats the results as the reference does.
"""
import ctypes as C
import math
from collections.abc import Sequence

import numpy as np

from . import _abi
from .arrays import DeviceArray, alloc_like, host_view, kind_of, ptr_strides, stream_for
from .borders import border_struct


class BlobLoG:
    """BlobLoG (src/extrema.jl:1-22): location (1-based index tuple), sigma
    (per-axis tuple) and amplitude of a peak of the -LoG-filtered image."""

    __slots__ = ("location", "sigma", "amplitude")

    def __init__(self, location, sigma, amplitude):
        self.location = tuple(int(i) for i in location)
        self.sigma = tuple(float(s) for s in sigma)
        self.amplitude = float(amplitude)

    @classmethod
    def _fast(cls, location, sigma, amplitude):
        b = cls.__new__(cls)
        b.location, b.sigma, b.amplitude = location, sigma, amplitude
        return b

    def __eq__(self, other):
        return (isinstance(other, BlobLoG) and self.location == other.location and self.sigma == other.sigma
                and self.amplitude == other.amplitude)

    def __repr__(self):
        return "BlobLoG(location=CartesianIndex%s, σ=%s, amplitude=%r)" % (
            self.location if len(self.location) > 1 else "(%d,)" % self.location[0], self.sigma, self.amplitude)


class BlobList(Sequence):
    """The blobs of one blob_LoG call, kept as arrays (1-based locations, scale
    indices, amplitudes); a BlobLoG is built only when an element is read, so
    finding thousands of blobs costs no per-blob host objects."""

    def __init__(self, locations, scales, amplitudes, sigmas):
        self.locations = locations              # (n, N) int64, 1-based
        self.scales = scales                    # (n,) index into sigmas
        self.amplitudes = amplitudes            # (n,) float64
        self.sigmas = sigmas                    # per-scale sigma tuples

    def __len__(self):
        return int(self.amplitudes.size)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[j] for j in range(*i.indices(len(self)))]
        if i < 0:
            i += len(self)
        if not 0 <= i < len(self):
            raise IndexError(i)
        return BlobLoG._fast(tuple(int(v) for v in self.locations[i]), self.sigmas[int(self.scales[i])],
                             float(self.amplitudes[i]))

    def __eq__(self, other):
        return list(self) == list(other)

    def __repr__(self):
        return "BlobList(%d blobs)" % len(self)


def _desc(a, kind):
    p, st = ptr_strides(a)
    return _abi.describe(p, kind, a.shape, st)


def log_terms(sigmas):
    """Kernel.LoG(σs) (src/kernel.jl:325-339) as a sum over axes d of separable
    terms: C (x_d^2/σ_d^4 - 1/σ_d^2) exp(-x_d^2/2σ_d^2) along d times
    exp(-x_e^2/2σ_e^2) along every other axis e, C = 1/(Π σ (2π)^(N/2)),
    half-widths ceil(8.5σ)>>1.  Returns the (first, weights) of the factor of
    each (term, axis)."""
    N = len(sigmas)
    ws = [int(math.ceil(8.5 * s)) >> 1 for s in sigmas]
    Cn = 1.0 / (float(np.prod(sigmas)) * (2 * math.pi) ** (N / 2))
    terms = []
    for d in range(N):
        facs = []
        for e in range(N):
            x = np.arange(-ws[e], ws[e] + 1, dtype=np.float64)
            s2 = float(sigmas[e]) ** 2
            g = np.exp(-x * x / (2 * s2))
            w = Cn * (x * x / (s2 * s2) - 1.0 / s2) * g if e == d else g
            facs.append((e, -ws[e], w))
        terms.append(facs)
    return terms


def _float_kind(kind):
    return {"F32": "F32", "F64": "F64", "N0F8": "F32", "U8": "F64"}[kind]


def multiLoG(img, sigmas, sigma_shape=None):
    """multiLoG (src/extrema.jl:87-98): the stack (σ first) of -σ LoG(σ σshape)
    filters of img with Pad(:reflect), in float(eltype(img))."""
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    sigmas = [float(s) for s in sigmas]
    if sigmas != sorted(sigmas):
        raise _abi.ErrorException("sigmas must be sorted")
    N = img.ndim
    shape = tuple(float(s) for s in (sigma_shape or (1,) * N))
    okind = _float_kind(kind)
    stack = alloc_like(img, (len(sigmas),) + tuple(img.shape), okind)
    ctx = _abi.context()
    b = border_struct("reflect", N, kind)
    slice_out = alloc_like(img, img.shape, okind)
    for i, s in enumerate(sigmas):
        terms = log_terms([s * f for f in shape])
        arr = (_abi.IfxFactor * (N * N))()
        keep = []
        for t, facs in enumerate(terms):
            for e, (ax, first, w) in enumerate(facs):
                w = np.ascontiguousarray(w)
                keep.append(w)
                f = arr[t * N + e]
                f.axis, f.length, f.first, f.weights = ax, w.size, first, _abi.dptr(w)
        _abi.check(ctx.lib.ifx_imfilter_factored_sum(ctx.handle, _desc(slice_out, okind), _desc(img, kind), N, N,
                                                     arr, -s, b, stream_for(img, slice_out)))
        if isinstance(stack, DeviceArray):
            stack.tensor[i] = slice_out.tensor
        else:
            stack[i] = slice_out
    return stack


def _localextrema_raw(img, window, edges, minima):
    """(column-major linear indices, values) of the strict local extrema."""
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    nd = img.ndim
    if nd > _abi.MAX_DIMS:
        raise _abi.Unsupported("at most %d dimensions" % _abi.MAX_DIMS)
    if window is None:
        window = (3,) * nd                     # default_window: every axis of an Array is spatial
    if isinstance(edges, bool):
        edges = (edges,) * nd
    if len(window) != nd or len(edges) != nd:
        raise _abi.DimensionMismatch("window and edges need one entry per dimension")
    win = (C.c_int32 * 4)(*[int(w) for w in window])
    edg = (C.c_int32 * 4)(*[int(bool(e)) for e in edges])
    ctx = _abi.context()
    total = int(np.prod(img.shape))
    cap = max(1, min(total, 1 << 18))
    while True:
        idx = np.empty(cap, dtype=np.int64)
        val = np.empty(cap, dtype=np.float64)
        count = C.c_int64(0)
        _abi.check(ctx.lib.ifx_findlocalextrema(ctx.handle, _desc(img, kind), win, edg, int(minima),
                                                idx.ctypes.data_as(C.POINTER(C.c_int64)),
                                                val.ctypes.data_as(C.POINTER(C.c_double)), cap, C.byref(count),
                                                stream_for(img)))
        if count.value <= cap:
            break
        cap = count.value
    n = count.value
    return idx[:n], val[:n]


def _localextrema(img, window, edges, minima):
    idx, val = _localextrema_raw(img, window, edges, minima)
    coords = np.unravel_index(idx, tuple(img.shape), order="F")
    return [tuple(int(c[k]) + 1 for c in coords) for k in range(idx.size)], val


def findlocalmaxima(img, window=None, edges=True):
    """findlocalmaxima (src/extrema.jl:109-111): 1-based index tuples of the
    elements larger than every neighbour of the window, in column-major order."""
    return _localextrema(img, window, edges, False)[0]


def findlocalminima(img, window=None, edges=True):
    """findlocalminima (src/extrema.jl:118-120)."""
    return _localextrema(img, window, edges, True)[0]


def blob_LoG(img, sigmas, edges=None, sigma_shape=None, rthresh=0.001):
    """blob_LoG(img, σscales; edges, σshape, rthresh) (src/extrema.jl:72-85)."""
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    N = img.ndim
    if edges is None:
        edges = (True,) + (False,) * N
    elif isinstance(edges, bool):
        edges = (edges,) * (N + 1)
    if len(edges) != N + 1:
        raise _abi.DimensionMismatch("edges needs N+1 entries")
    shape = tuple(float(s) for s in (sigma_shape or (1,) * N))
    sig = sorted(float(s) for s in sigmas)
    stack = multiLoG(img, sig, shape)
    idx, vals = _localextrema_raw(stack, (3,) * (N + 1), tuple(edges), False)
    coords = np.unravel_index(idx, tuple(stack.shape), order="F")
    if rthresh != 0:
        athresh = np.array([rthresh / (s ** N * float(np.prod(shape))) for s in sig])
        imgmax = C.c_double(0)
        ctx = _abi.context()
        _abi.check(ctx.lib.ifx_maxabs(ctx.handle, _desc(img, kind), C.byref(imgmax), stream_for(img)))
        # the same comparison per maximum, vectorised: v > athresh[scale] * maximum(abs, img)
        keep = vals > athresh[coords[0]] * imgmax.value
    else:
        keep = np.ones(vals.size, dtype=bool)
    sel = np.nonzero(keep)[0]
    locs = np.stack([c[sel] for c in coords[1:]], axis=1).astype(np.int64) + 1
    sigt = [tuple(s * f for f in shape) for s in sig]
    return BlobList(locs, coords[0][sel], vals[sel].astype(np.float64), sigt)


__all__ = ["BlobLoG", "BlobList", "blob_LoG", "multiLoG", "findlocalmaxima", "findlocalminima", "log_terms"]
