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
from .arrays import (INT_KINDS, NATIVE_KINDS, DeviceArray, N0f8Array, N0f16Array, alloc_like, host_view,
                     kind_of, ptr_strides, stream_for)
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


# eltype of Statistics.middle of one value: Float64 for integers, Float32 for
# the 8/16-bit Normed types (taken as Float32, like Float32(::N0f8)), the float itself
_MEDIAN_OUT = {"N0F8": "F32", "N0F16": "F32", "U8": "F64", "F32": "F32", "F64": "F64", "I8": "F64",
               "I16": "F64", "U16": "F64", "I32": "F64", "I64": "F64"}


def _index_sel(indices, shape):
    """Julia index ranges per axis (1-based values: range(1, 11, 2) is 1:2:10,
    or a list of indices) -> numpy/torch selectors and the result's shape."""
    if not isinstance(indices, (tuple, list)) or (len(indices) and isinstance(indices[0], (int, np.integer))):
        indices = (indices,)
    if len(indices) != len(shape):
        raise _abi.DimensionMismatch("indices need one range per axis")
    sel, out_shape = [], []
    for r, n in zip(indices, shape):
        vals = list(r) if not isinstance(r, (int, np.integer)) else [int(r)]
        if any(v < 1 or v > n for v in vals):
            raise _abi.DimensionMismatch("indices outside the image's axes")
        if len(vals) >= 2 and all(b - a == vals[1] - vals[0] for a, b in zip(vals, vals[1:])) and vals[1] > vals[0]:
            sel.append(slice(vals[0] - 1, vals[-1], vals[1] - vals[0]))
        elif len(vals) == 1:
            sel.append(slice(vals[0] - 1, vals[0]))
        else:
            sel.append(np.asarray(vals, dtype=np.int64) - 1)
        out_shape.append(len(vals))
    return tuple(sel), tuple(out_shape)


def _take(full, sel, lead):
    """full[lead + sel] as a new array on the same side."""
    if isinstance(full, DeviceArray):
        t = full.tensor
        for ax, s_ in enumerate(lead + sel):
            if isinstance(s_, slice):
                idx = [slice(None)] * t.dim()
                idx[ax] = s_
                t = t[tuple(idx)]
            else:
                import torch
                t = t.index_select(ax, torch.as_tensor(s_, device=t.device))
        r = DeviceArray.empty(tuple(t.shape), full.kind, t.device)
        r.tensor.copy_(t)
        return r
    a = full
    for ax, s_ in enumerate(lead + sel):
        idx = [slice(None)] * a.ndim
        idx[ax] = s_
        a = a[tuple(idx)]
    return np.asfortranarray(a).view(type(full)) if isinstance(full, np.ndarray) else a


def _converted_rank(f, img, window, border, kind, name):
    """Rank filters of Int8..Int64, UInt16 and N0f16 images: the values (for
    N0f16 the codes, whose order is the values') are converted exactly to
    Float64 on the GPU, filtered there, and converted to the result's eltype
    (the image's for extrema / minimum / maximum)."""
    from .filtering import convert_, maxabs
    codes = img
    if kind == "N0F16":                      # the codes, as UInt16
        codes = DeviceArray(img.tensor, "U16") if isinstance(img, DeviceArray) else np.asarray(img).view(np.uint16)
    tmp = alloc_like(img, img.shape, "F64")
    convert_(tmp, codes)
    if kind == "I64" and not maxabs(tmp) < 2.0 ** 53:
        raise _abi.Unsupported("Int64 rank filters with values beyond 2^53")
    b = border
    if b is not None:
        from .filtering import _fill_in_eltype
        from .borders import Fill
        bi = borderinstance(b)
        if isinstance(bi, Fill):
            v = _fill_in_eltype(bi, kind)
            b = Fill(round(v * 65535) if kind == "N0F16" else v, bi.lo, bi.hi) if bi.lo is not None \
                else Fill(round(v * 65535) if kind == "N0F16" else v)
    res = mapwindow(f, tmp, window, border=b)
    if name == "median":
        if kind != "N0F16":
            return res                        # Float64 (middle of an integer)
        c16 = alloc_like(img, res.shape, "U16")
        convert_(c16, res)
        out = alloc_like(img, res.shape, "F32")
        convert_(out, DeviceArray(c16.tensor, "N0F16") if isinstance(c16, DeviceArray) else c16.view(N0f16Array))
        return out
    back = alloc_like(img, res.shape, "U16" if kind == "N0F16" else kind)
    convert_(back, res)
    if kind == "N0F16":
        return DeviceArray(back.tensor, "N0F16") if isinstance(back, DeviceArray) else back.view(N0f16Array)
    return back


def mapwindow(f, img, window, border=None, indices=None):
    """mapwindow(f, img, window; border="replicate") (src/mapwindow.jl:75-85).

    extrema returns an array of shape (2,) + img.shape in Julia order
    (the Tuple{T,T} layout: min at [0], max at [1])."""
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    name = _fname(f)
    if indices is not None:
        # mapwindow(f, img, window; indices) == mapwindow(f, img, window)[indices...]
        # (src/mapwindow.jl:95-121, test/mapwindow.jl:131-150)
        full = mapwindow(f, img, window, border=border)
        sel, _ = _index_sel(indices, img.shape)
        return _take(full, sel, (slice(None),) if name == "extrema" else ())
    if isinstance(border, Inner):
        return _mapwindow_inner(f, img, window, name)
    if kind not in NATIVE_KINDS:
        return _converted_rank(f, img, window, border, kind, name)
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
    """mapwindow!(f, out, img, window; border, indices) (src/mapwindow.jl:113-121)."""
    if indices is not None or kind_of(img) not in NATIVE_KINDS:
        res = mapwindow(f, img, window, border=border, indices=indices)
        if isinstance(out, DeviceArray):
            out.tensor.copy_(res.tensor)
        else:
            out[...] = np.asarray(res).view(np.asarray(out).dtype) if np.asarray(res).dtype == np.asarray(out).dtype \
                else np.asarray(res)
        return out
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
