"""mapwindow / mapwindow! for the rank functions the GB300 path implements:
median (median!, median), extrema, minimum and maximum
(src/mapwindow.jl).  An arbitrary Julia/Python function cannot cross the C
ABI, so other functions raise.

Dispatch mirrors the reference: ``mapwindow(extrema, A, window::Dims)``
without keywords is the Lemire filter (even windows allowed, edges truncated,
src/mapwindow.jl:337-338); any call with a border -- and every median /
minimum / maximum call -- goes through the generic window path with
``border="replicate"`` by default (src/mapwindow.jl:75-85), which requires odd
Dims windows (resolve_window, 133-137).
"""
import ctypes as C

import numpy as np

from . import _abi
from .arrays import DeviceArray, N0f8Array, alloc_like, host_view, kind_of, ptr_strides, stream_for
from .borders import Inner, border_struct, borderinstance


def median(v):
    """Marker for Statistics.median / median! in mapwindow."""
    raise TypeError("use mapwindow(median, img, window)")


median_ = median


def extrema(v):
    """Marker for Base.extrema in mapwindow."""
    raise TypeError("use mapwindow(extrema, img, window)")


def minimum(v):
    raise TypeError("use mapwindow(minimum, img, window)")


def maximum(v):
    raise TypeError("use mapwindow(maximum, img, window)")


def _fname(f):
    if f in (median, median_, np.median) or f == "median":
        return "median"
    if f is extrema or f == "extrema":
        return "extrema"
    if f in (minimum, np.min, np.amin, min) or f == "minimum":
        return "minimum"
    if f in (maximum, np.max, np.amax, max) or f == "maximum":
        return "maximum"
    raise _abi.Unsupported("mapwindow with an arbitrary function cannot run on the GB300 path; "
                           "median, extrema, minimum and maximum are supported")


def _is_dims(window):
    if isinstance(window, (int, np.integer)):
        return True
    return isinstance(window, (tuple, list)) and all(isinstance(w, (int, np.integer))
                                                      for w in window)


def resolve_window(window, nd, allow_even=False):
    """src/mapwindow.jl:133-148 -> (first offsets, lengths)."""
    if isinstance(window, (tuple, list)) and len(window) == 0:
        raise _abi.ArgumentError("empty window")
    if isinstance(window, (int, np.integer)):
        window = (int(window),)
    if isinstance(window, range):
        window = (window,)
    if _is_dims(window):
        if not allow_even and not all(w % 2 == 1 for w in window):
            raise _abi.ErrorException("entries in window must be odd, got %s" % (tuple(window),))
        wf = [-(int(w) >> 1) for w in window]
        wl = [int(w) for w in window]
    else:
        wf, wl = [], []
        for r in window:
            if isinstance(r, range):
                if r.step != 1:
                    raise _abi.ArgumentError("window ranges must be unit ranges")
                wf.append(r.start)
                wl.append(len(r))
            else:                                   # (first, last) pair
                wf.append(int(r[0]))
                wl.append(int(r[1]) - int(r[0]) + 1)
    if len(wl) != nd:
        raise _abi.DimensionMismatch("window has %d entries for a %d-d image" % (len(wl), nd))
    return wf, wl


_MEDIAN_OUT = {"N0F8": "F32", "U8": "F64", "F32": "F32", "F64": "F64"}


def mapwindow(f, img, window, border=None, indices=None):
    """mapwindow(f, img, window; border="replicate") (src/mapwindow.jl:75-85).

    extrema returns an array of shape (2,) + img.shape in Julia order
    (the Tuple{T,T} layout: min at [0], max at [1])."""
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    name = _fname(f)
    if isinstance(border, Inner):
        return _mapwindow_inner(f, img, window, name)
    if name == "extrema":
        shape = (2,) + tuple(img.shape)
        if isinstance(img, DeviceArray):
            out = DeviceArray.empty(shape, kind, img.tensor.device)
        else:
            out = np.empty(shape, dtype=np.asarray(img).dtype, order="F")
            if kind == "N0F8":
                out = out.view(N0f8Array)
    elif name == "median":
        out = alloc_like(img, img.shape, _MEDIAN_OUT[kind])
    else:
        out = alloc_like(img, img.shape, kind)
    return mapwindow_(f, out, img, window, border, indices)


def _mapwindow_inner(f, img, window, name):
    """border=Inner() (default_imginds, src/mapwindow.jl:95-100): only the
    indices whose whole window lies in the image, with their own axes; a window
    longer than an axis is a DimensionMismatch.  Those windows read inside the
    image, so any Pad style gives the same values there."""
    nd = img.ndim
    wf, wl = resolve_window(window, nd, allow_even=False)
    inds = [(1 - f0, n - (f0 + l - 1)) for f0, l, n in zip(wf, wl, img.shape)]
    if any(a > b for a, b in inds):
        raise _abi.DimensionMismatch("the window is larger than the array: no interior")
    full = mapwindow(f, img, window, border="replicate")
    lead = (slice(None),) if name == "extrema" else ()
    sl = lead + tuple(slice(a - 1, b) for a, b in inds)
    first = tuple(a for a, _ in inds)
    if isinstance(full, DeviceArray):
        r = DeviceArray(full.tensor[sl].contiguous(), full.kind, first)
    else:
        from .filtering import OffsetResult
        r = np.asfortranarray(full[sl]).view(OffsetResult)
        r.first = first
    return r


def mapwindow_(f, out, img, window, border=None, indices=None):
    """mapwindow!(f, out, img, window; border) (src/mapwindow.jl:113-121)."""
    if indices is not None:
        raise _abi.Unsupported("mapwindow indices= is not part of the GB300 path")
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    name = _fname(f)
    nd = img.ndim
    lemire = name == "extrema" and border is None and _is_dims(window)
    wf, wl = resolve_window(window, nd, allow_even=lemire)
    ip, ist = ptr_strides(img)
    ai = _abi.describe(ip, kind, img.shape, ist)
    ctx = _abi.context()
    wfa = (C.c_int64 * 4)(*wf)
    wla = (C.c_int64 * 4)(*wl)
    if name == "median":
        b = border_struct(borderinstance(border or "replicate"), nd, kind)
        okind = kind_of(out)
        op, ost = ptr_strides(out)
        ao = _abi.describe(op, okind, out.shape, ost)
        _abi.check(ctx.lib.ifx_mapwindow_median(ctx.handle, ao, ai, wfa, wla, b,
                                                stream_for(img, out)))
        return out
    which = {"extrema": 0, "minimum": 1, "maximum": 2}[name]
    if which == 0:
        op, ost = ptr_strides(out, values_per_elem=1)
        ost = tuple(s // 2 for s in ost[1:])     # strides in pairs over the image axes
        ao = _abi.describe(op, kind, img.shape, ost)
    else:
        op, ost = ptr_strides(out)
        ao = _abi.describe(op, kind, img.shape, ost)
    b = None if lemire else border_struct(borderinstance(border or "replicate"), nd, kind)
    _abi.check(ctx.lib.ifx_mapwindow_extrema(ctx.handle, ao, ai, wfa, wla,
                                             C.byref(b) if b is not None else None, which,
                                             stream_for(img, out)))
    return out
