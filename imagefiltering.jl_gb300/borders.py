"""Border specifications (src/border.jl) and ``padarray`` on the GPU.

``Pad`` and ``Fill`` mirror the reference types: without sizes they are
``Pad{0}`` / ``Fill{T,0}`` and the amount of padding comes from the kernel
(src/border.jl:236-237, 614-621); with sizes they are fully specified.
"""
from . import _abi
from .arrays import alloc_like, kind_of, ptr_strides, host_view, DeviceArray, stream_for

VALID_BORDERS = ("replicate", "circular", "reflect", "symmetric")


class Pad:
    """Pad(style), Pad(style, m, n, ...), Pad(style, (m,n)), Pad(style, lo, hi)
    (src/border.jl:136-248)."""

    def __init__(self, style="replicate", *sizes):
        if isinstance(style, int):
            sizes = (style,) + sizes
            style = "replicate"
        style = str(style).lstrip(":")
        if style not in VALID_BORDERS:
            raise _abi.ErrorException("border style %s unrecognized" % style)
        self.style = style
        self.lo = self.hi = None
        if len(sizes) == 1 and isinstance(sizes[0], (tuple, list)):
            self.lo = self.hi = tuple(int(x) for x in sizes[0])
        elif len(sizes) == 2 and all(isinstance(s, (tuple, list)) for s in sizes):
            lo, hi = tuple(sizes[0]), tuple(sizes[1])
            n = max(len(lo), len(hi))
            self.lo = tuple(int(x) for x in lo) if lo else (0,) * n
            self.hi = tuple(int(x) for x in hi) if hi else (0,) * n
        elif sizes:
            self.lo = self.hi = tuple(int(x) for x in sizes)

    def __repr__(self):
        return "Pad(:%s, %s, %s)" % (self.style, self.lo, self.hi)


class Fill:
    """Fill(value), Fill(value, (m,n)), Fill(value, lo, hi) (src/border.jl:465-555)."""

    def __init__(self, value, lo=None, hi=None):
        self.style = "fill"
        self.value = value
        if lo is not None and hi is None:
            hi = lo
        self.lo = tuple(int(x) for x in lo) if lo is not None else None
        self.hi = tuple(int(x) for x in hi) if hi is not None else None

    def __repr__(self):
        return "Fill(%r, %s, %s)" % (self.value, self.lo, self.hi)


class Inner:
    """Inner(), Inner(lo, hi) (src/border.jl:356-386): edges are discarded and
    only the interior of the result is returned -- the indices where the whole
    kernel support lies inside the image (Inner()), or inner.(lo, axes(img),
    hi) for explicit widths.  Results carry their first indices (`first`)."""

    def __init__(self, lo=None, hi=None):
        if lo is not None and hi is None:
            hi = lo
        self.lo = tuple(int(x) for x in lo) if lo is not None else None
        self.hi = tuple(int(x) for x in hi) if hi is not None else None
        if self.lo is not None and len(self.lo) != len(self.hi):
            raise _abi.ArgumentError("Inner: lo and hi need the same number of dimensions")

    def __repr__(self):
        return "Inner(%s, %s)" % (self.lo, self.hi)


class NA:
    """NA(na="isnan") (src/border.jl:388-405): output = (filtered array with
    Fill(0)) / (filtered ones with Fill(0)); elements for which `na` holds are
    also outside the image.  The predicate is one of "isnan" (the default),
    "notfinite" (NA(!isfinite)) or "none" (NA(x -> false)): a Julia closure
    cannot cross the C ABI."""

    CODES = {"isnan": 0, "notfinite": 1, "none": 2}

    def __init__(self, na="isnan"):
        if na not in self.CODES:
            raise _abi.ArgumentError("NA predicate must be one of %s" % sorted(self.CODES))
        self.na = na

    def __repr__(self):
        return "NA(%r)" % self.na


class NoPad:
    """NoPad(border=None) (src/border.jl:7-30): the image needs no padding --
    every index the requested outputs read lies inside it (imfilter_ with
    `inds`)."""

    def __init__(self, border=None):
        self.border = border

    def __repr__(self):
        return "NoPad(%r)" % (self.border,)


def borderinstance(border):
    """src/border.jl:147-156."""
    if isinstance(border, str):
        if border in VALID_BORDERS:
            return Pad(border)
        if border == "inner":
            raise _abi.ArgumentError("specifying Inner as a string is deprecated, use "
                                     "`imfilter(img, kern, Inner())` instead")
        raise _abi.ArgumentError("%s not a recognized border" % border)
    return border


def fill_value_for(border, kind):
    """convert(eltype(img), border.value) (src/borderarray.jl:11-20)."""
    if not isinstance(border, Fill):
        return 0.0
    v = border.value
    try:
        v = float(v)
    except (TypeError, ValueError):
        raise _abi.ArgumentError("Cannot convert elements of border=%r to eltype(inner)" % (border,))
    if kind == "U8":
        if v != int(v) or not 0 <= v <= 255:
            raise _abi.ArgumentError("Cannot convert elements of border=%r to eltype(inner)=UInt8"
                                     % (border,))
    elif kind == "N0F8":
        if not 0.0 <= v <= 1.0:
            raise _abi.ArgumentError("Cannot convert elements of border=%r to eltype(inner)=N0f8"
                                     % (border,))
        v = round(v * 255) / 255.0
    elif kind == "F32":
        import numpy as np
        v = float(np.float32(v))
    return v


def border_struct(border, ndim, kind):
    """The C descriptor of a border for an image of element kind `kind`."""
    border = borderinstance(border)
    if isinstance(border, (Inner, NA, NoPad)):
        raise _abi.ArgumentError("%r is not a padding border" % (border,))
    fill = fill_value_for(border, kind)
    if border.lo is not None and (len(border.lo) != ndim or len(border.hi) != ndim):
        raise _abi.ArgumentError("%r lacks the proper padding sizes for an array with %d "
                                 "dimensions" % (border, ndim))
    return _abi.border_struct(border.style, border.lo, border.hi, fill)


def padarray(img, border, T=None):
    """padarray([T], img, border) (src/border.jl:324-331) on the GPU.

    Returns ``(padded, first)``: the padded array and the first index of each
    of its axes (the reference returns an OffsetArray with those axes)."""
    border = borderinstance(border)
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    nd = img.ndim
    if border.lo is None or len(border.lo) != nd:
        raise _abi.ArgumentError("%r lacks the proper padding sizes for an array with %d "
                                 "dimensions" % (border, nd))
    okind = kind if T is None else T
    shape = tuple(n + l + h for n, l, h in zip(img.shape, border.lo, border.hi))
    out = alloc_like(img, shape, okind)
    ip, ist = ptr_strides(img)
    op, ost = ptr_strides(out)
    ai = _abi.describe(ip, kind, img.shape, ist)
    first = tuple(1 - l for l in border.lo)
    ao = _abi.describe(op, okind, shape, ost, first)
    b = border_struct(border, nd, kind)
    ctx = _abi.context()
    _abi.check(ctx.lib.ifx_padarray(ctx.handle, ao, ai, b, stream_for(img, out)))
    return out, first
