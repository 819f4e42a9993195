"""imfilter / imfilter! / imgradients on the GB300 path.

Host-side steps 1-4 of the reference's dispatch (src/imfilter.jl:1-49,
204-254) run here unchanged in meaning -- output eltype (filter_type,
1131-1154), kernel factoring (factorkernel, 1156-1184), border resolution
(borderinstance) and output allocation -- and then one C-ABI call does the
padding and filtering on the GPU.  ``Algorithm.GB300`` is the algorithm tag
of this backend; asking for the reference's CPU algorithms raises, because
this package has no CPU compute path.
"""
import ctypes as C

import numpy as np

from . import _abi
from .arrays import (INT_KINDS, NATIVE_KINDS, RGB, DeviceArray, alloc_like, host_view, kind_of, ptr_strides,
                     stream_for)
from .borders import Fill, Inner, NA, NoPad, border_struct, borderinstance
from .kernels import (Kernel, KernelFactors, LaplacianKernel, OffsetKernel, ReshapedOneD, TriggsSdika,
                      iscopy)


class Algorithm:
    """Algorithm tags (src/ImageFiltering.jl:52-65) plus this backend's GB300."""

    class Alg:
        pass

    class FIR(Alg):
        pass

    class FIRTiled(Alg):
        def __init__(self, tilesize=()):
            self.tilesize = tilesize

    class FFT(Alg):
        """Correlation through real FFTs on the GPU (cuFFT) over the padfft
        sizes of the reference (src/imfilter.jl:776-884)."""

    class IIR(Alg):
        pass

    class Mixed(Alg):
        pass

    class GB300(Alg):
        """Direct (FIR) filtering by the sm_103a kernels of this package.

        ``method``: "auto", "cuda_cores" or "tensor_cores" (dense kernels), or
        "fft" (the same as Algorithm.FFT())."""

        def __init__(self, method="auto"):
            self.method = method


_METHOD = {"auto": 0, "cuda_cores": 1, "tensor_cores": 2}


# ------------------------------------------------------------------ eltypes
def _kernel_dtype(k):
    if isinstance(k, LaplacianKernel):
        return None
    return np.dtype(k.dtype)


_INT_OF_DTYPE = {np.dtype(np.int8): "I8", np.dtype(np.uint8): "U8", np.dtype(np.int16): "I16",
                 np.dtype(np.uint16): "U16", np.dtype(np.int32): "I32", np.dtype(np.int64): "I64"}
_INT_BITS = {"I8": (8, True), "U8": (8, False), "I16": (16, True), "U16": (16, False), "I32": (32, True),
             "I64": (64, True)}


def _promote_int(a, b):
    """Julia's promote_type of two integer eltypes: the wider one; between a
    signed and an unsigned type of the same width (or a wider unsigned one),
    the unsigned one."""
    (na, sa), (nb, sb) = _INT_BITS[a], _INT_BITS[b]
    if sa == sb:
        return a if na >= nb else b
    s_, u_ = (a, b) if sa else (b, a)
    return s_ if _INT_BITS[s_][0] > _INT_BITS[u_][0] else u_


def _promote_one(img_kind, kdt):
    """typeof(zero(S)*zero(T) + ...) for the supported (S, T) pairs
    (src/imfilter.jl:1133; Float32 for Normed and Int, Float64 wins)."""
    if kdt is None:
        return None
    if img_kind == "F64" or kdt == np.float64:
        return "F64"
    if kdt == np.float32:
        return "F32"
    if kdt == np.bool_:
        kdt = np.dtype(np.int8) if img_kind in INT_KINDS else kdt
        if kdt == np.bool_:
            return "F32"
    if np.issubdtype(kdt, np.integer):
        if img_kind in ("F32", "N0F8", "N0F16"):
            return "F32"
        if img_kind in INT_KINDS:
            kk = _INT_OF_DTYPE.get(np.dtype(kdt))
            if kk is None:
                raise _abi.Unsupported("kernel eltype %s" % kdt)
            return img_kind if np.dtype(kdt) == np.bool_ else _promote_int(img_kind, kk)
    raise _abi.Unsupported("kernel eltype %s" % kdt)


def filter_type(img_kind, kernel):
    """src/imfilter.jl:1131-1154."""
    if isinstance(kernel, LaplacianKernel):
        # float32 for Normed, the type itself for signed integers, signed_type for unsigned
        return {"F32": "F32", "F64": "F64", "N0F8": "F32", "N0F16": "F32", "U8": "I16", "U16": "I32",
                "I8": "I8", "I16": "I16", "I32": "I32", "I64": "I64"}[img_kind]
    if isinstance(kernel, tuple):
        kinds = [filter_type(img_kind, k) for k in kernel]
        if "F64" in kinds:
            return "F64"
        if kinds and all(k in INT_KINDS for k in kinds):
            r = kinds[0]
            for k in kinds[1:]:
                r = _promote_int(r, k)
            return r
        if "F32" in kinds:
            return "F32"
        return kinds[0] if kinds else {"F64": "F64"}.get(img_kind, "F32")
    return _promote_one(img_kind, _kernel_dtype(kernel))


# ------------------------------------------------------------------ factoring
def factorkernel(kernel):
    """src/imfilter.jl:1156-1184: a 2-D dense kernel is tested for separability
    with an SVD (threshold sqrt(eps)); other kernels become 1-tuples."""
    if isinstance(kernel, tuple):
        return kernel
    if isinstance(kernel, (LaplacianKernel, ReshapedOneD, TriggsSdika)):
        return (kernel,)
    if not isinstance(kernel, OffsetKernel):
        raise _abi.ArgumentError("kernel must be an OffsetKernel (use centered(...))")
    if kernel.ndim != 2:
        return (kernel,)
    K = np.asarray(kernel.data)
    kf = np.asarray(K, dtype=np.float64 if K.dtype != np.float32 else np.float32)
    U, S, Vt = np.linalg.svd(kf)
    eps = np.finfo(S.dtype).eps
    separable = all(abs(s) < np.sqrt(eps) for s in S[1:])
    if not separable:
        dummy = OffsetKernel(np.ones((1, 1), dtype=K.dtype), (0, 0))
        return (dummy, kernel)
    ss = np.sqrt(S[0])
    u = (ss * U[:, 0]).astype(kf.dtype)
    v = (ss * Vt[0, :]).astype(kf.dtype)
    return (OffsetKernel(u.reshape(-1, 1, order="F"), (kernel.first[0], 0)),
            OffsetKernel(v.reshape(1, -1, order="F"), (0, kernel.first[1])))


def _as_factor(k, nd):
    """(axis, first, weights) when `k` filters along a single axis, else None."""
    if isinstance(k, ReshapedOneD):
        if k.axis >= nd:
            raise _abi.DimensionMismatch("factor along axis %d of a %d-d image" % (k.axis + 1, nd))
        return (k.axis, k.data.first[0], np.asarray(k.data.data, dtype=np.float64).reshape(-1))
    if isinstance(k, OffsetKernel):
        if k.ndim > nd:
            raise _abi.DimensionMismatch("kernel has more dimensions than the image")
        ext = [d for d in range(k.ndim) if k.shape[d] > 1]
        if len(ext) > 1:
            return None
        if any(k.first[d] != 0 for d in range(k.ndim) if d not in ext):
            return None
        ax = ext[0] if ext else 0
        return (ax, k.first[ax], np.asarray(k.data, dtype=np.float64).reshape(-1))
    return None


def _dense_of(k, nd):
    """N-d dense OffsetKernel (float64) for any kernel object."""
    if isinstance(k, (ReshapedOneD, LaplacianKernel)):
        k = k.dense()
    data = np.asarray(k.data, dtype=np.float64)
    first = list(k.first)
    while data.ndim < nd:
        data = data.reshape(data.shape + (1,), order="F")
        first.append(0)
    return OffsetKernel(data, first)


def _kernelconv(ks, nd):
    """kernelconv (src/imfilter.jl:1257-1270): the composite of a cascade.
    Pad-then-cascade equals one pass of the composite over the same padded
    image, so mixed cascades run as one dense filter."""
    acc = _dense_of(ks[0], nd)
    for k in ks[1:]:
        b = _dense_of(k, nd)
        shape = [sa + sb - 1 for sa, sb in zip(acc.shape, b.shape)]
        out = np.zeros(shape)
        for idx in np.ndindex(*b.shape):
            sl = tuple(slice(i, i + s) for i, s in zip(idx, acc.shape))
            out[sl] += acc.data * b.data[idx]
        acc = OffsetKernel(out, [fa + fb for fa, fb in zip(acc.first, b.first)])
    return acc


# ------------------------------------------------------------------ entry points
def _ctx():
    return _abi.context()


def _check_alg(alg):
    if isinstance(alg, (Algorithm.IIR, Algorithm.Mixed)):
        # the recursive filters run on the GPU whatever the tag; FIR factors
        # of the same call take the direct kernels
        alg = Algorithm.GB300()
    if alg is None or isinstance(alg, Algorithm.GB300):
        alg = alg or Algorithm.GB300()
        if alg.method not in _METHOD and alg.method != "fft":
            raise _abi.ArgumentError("unknown GB300 method %r" % (alg.method,))
        return Algorithm.FFT() if alg.method == "fft" else alg
    if isinstance(alg, Algorithm.FFT):
        return alg
    if isinstance(alg, Algorithm.Alg):
        raise _abi.Unsupported("%s runs on the CPU in the reference; this package implements "
                               "Algorithm.GB300() only" % type(alg).__name__)
    raise _abi.ArgumentError("unknown algorithm %r" % (alg,))


def _desc(a, kind, first=None):
    p, st = ptr_strides(a)
    return _abi.describe(p, kind, a.shape, st, first)


# ------------------------------------------------------------------ Inner / NA / NoPad
def kernel_support(kernel, nd):
    """calculate_padding / accumulate_padding (src/border.jl:640-652): the
    lowest and highest offset each axis of the processed kernel reads."""
    lo, hi = [0] * nd, [0] * nd
    for k in kernel:
        if iscopy(k) or _is_iir(k):                   # IIR filters have axes 0:0
            continue
        if isinstance(k, LaplacianKernel):
            for d, f in enumerate(k.flags[:nd]):
                if f:
                    lo[d] -= 1
                    hi[d] += 1
        elif isinstance(k, ReshapedOneD):
            n = np.asarray(k.data.data).size
            lo[k.axis] += k.data.first[0]
            hi[k.axis] += k.data.first[0] + n - 1
        else:
            for d in range(min(k.ndim, nd)):
                lo[d] += k.first[d]
                hi[d] += k.first[d] + k.shape[d] - 1
    return lo, hi


class OffsetResult(np.ndarray):
    """A host result whose axes do not start at 1 (an OffsetArray of the
    reference): `first` holds each axis' first index."""

    def __array_finalize__(self, obj):
        self.first = getattr(obj, "first", None)


def _region(a, first, inds):
    """a[inds] where a's axes start at `first` and inds are 1-based ranges (lo, hi)."""
    return tuple(slice(l - f, h - f + 1) for (l, h), f in zip(inds, first))


def _with_first(a, first):
    if isinstance(a, DeviceArray):
        t = a.tensor
        return DeviceArray(t if t.is_contiguous() else t.contiguous(), a.kind, first)
    r = np.asfortranarray(a).view(OffsetResult)
    r.first = tuple(first)
    return r


def _check_reads(inds, kernel, img_shape, what):
    lo, hi = kernel_support(kernel, len(img_shape))
    for d, ((a, b), n) in enumerate(zip(inds, img_shape)):
        if a > b:
            continue
        if a + lo[d] < 1 or b + hi[d] > n:
            raise _abi.ArgumentError("BoundsError: %s on axis %d reads indices %d:%d of an axis 1:%d"
                                     % (what, d + 1, a + lo[d], b + hi[d], n))


def _imfilter_inner(img, kernel, border, alg, T, kind):
    nd = img.ndim
    if any(_is_iir(k) for k in kernel):
        raise _abi.ArgumentError("IIR filters take NA(), Pad or Fill borders, not Inner()")
    if border.lo is None:
        lo, hi = kernel_support(kernel, nd)
        inds = [(max(1, 1 - l), min(n, n - h)) for l, h, n in zip(lo, hi, img.shape)]
    else:
        if len(border.lo) != nd:
            raise _abi.DimensionMismatch("dimensionality of img and the border must agree, got %d "
                                         "and %d" % (nd, len(border.lo)))
        inds = [(1 + l, n - h) for l, h, n in zip(border.lo, border.hi, img.shape)]
        _check_reads(inds, kernel, img.shape, "Inner()")
    # every output in `inds` reads inside the image: the border style is moot
    full = imfilter(img, kernel, "replicate", alg, T)
    sl = _region(full, (1,) * nd, inds)
    part = full.tensor[sl] if isinstance(full, DeviceArray) else full[sl]
    if isinstance(full, DeviceArray):
        part = DeviceArray(part, full.kind)
    return _with_first(part, tuple(a for a, _ in inds))


def _is_iir(k):
    return isinstance(k, TriggsSdika) or (isinstance(k, ReshapedOneD) and isinstance(k.data, TriggsSdika))


def _iir_factors(kernel, nd):
    """(factors, bare) for a cascade of Triggs-Sdika filters: factors are
    (axis, TriggsSdika) without the copies.  A tuple of bare TriggsSdika
    filters takes the axes in order (_imfilter_inplace_tuple!,
    src/imfilter.jl:892-953); ReshapedOneD factors their own axes.  None when
    the cascade holds no IIR filter."""
    ks = list(kernel)
    if not any(_is_iir(k) for k in ks):
        return None
    if all(isinstance(k, TriggsSdika) for k in ks):
        if len(ks) > nd:
            raise _abi.DimensionMismatch("cannot have more kernels than dimensions")
        facs, bare = list(enumerate(ks)), True
    else:
        facs, bare = [], False
        for k in ks:
            if iscopy(k):
                continue
            if not (isinstance(k, ReshapedOneD) and isinstance(k.data, TriggsSdika)):
                return "mixed", False
            if k.axis >= nd:
                raise _abi.DimensionMismatch("factor along axis %d of a %d-d image" % (k.axis + 1, nd))
            facs.append((k.axis, k.data))
    return [(ax, t) for ax, t in facs if not iscopy(t)], bare


def _imfilter_iir(out, img, facs, border, bare, kind, okind):
    """Triggs-Sdika cascades (src/imfilter.jl:892-1092) through ifx_imfilter_iir."""
    if isinstance(border, (Inner, NoPad)):
        raise _abi.ArgumentError("IIR filters take NA(), Pad or Fill borders, not %r" % (border,))
    if bare and not isinstance(border, Fill) and border.style != "replicate":
        raise _abi.ArgumentError('only "replicate" is supported')
    if okind not in ("F32", "F64"):
        raise _abi.Unsupported("IIR filtering writes Float32 or Float64 outputs")
    nd = img.ndim
    b = border_struct(border, nd, okind)
    arr = (_abi.IfxIir * max(len(facs), 1))()
    for i, (ax, t) in enumerate(facs):
        f = arr[i]
        f.axis = ax
        f.coef_f32 = int(t.dtype == np.float32)
        for j in range(3):
            f.a[j] = float(t.a[j])
            f.b[j] = float(t.b[j])
        for j in range(9):
            f.M[j] = float(t.M[j // 3, j % 3])
        f.scale = float(t.scale)
        f.asum = float(t.asum)
        f.bsum = float(t.bsum)
    ctx = _ctx()
    _abi.check(ctx.lib.ifx_imfilter_iir(ctx.handle, _desc(out, okind), _desc(img, kind), len(facs), arr, b,
                                        stream_for(img, out)))
    return out


def _colmajor(t):
    """A dense column-major copy of a (strided) torch view."""
    rev = list(reversed(range(t.dim())))
    return t.permute(*rev).contiguous().permute(*rev)


def _imfilter_mixed(out, img, kernel, border, alg, kind, okind):
    """Algorithm.Mixed: a cascade of Triggs-Sdika and FIR filters
    (src/imfilter.jl:385-457 with the padding of src/border.jl:614-662).  The
    image is padded (in the output eltype) by twice the accumulated FIR
    padding; stage k filters over indsstep_k -- the padded range shrunk by the
    first filter, then by each next one (next_shrink) -- so an IIR stage has
    its boundary values at the edges of its range; the image's indices are
    kept.  Every stage is a GPU call: FIR stages are Inner() filters of the
    stage's input box, IIR stages ifx_imfilter_iir passes over theirs."""
    import torch
    from .borders import padarray as _padarray
    nd = img.ndim
    if isinstance(border, (Inner, NoPad)):
        raise _abi.ArgumentError("IIR filters take NA(), Pad or Fill borders, not %r" % (border,))
    if okind not in ("F32", "F64"):
        raise _abi.Unsupported("IIR filtering writes Float32 or Float64 outputs")
    stages = []
    for k in kernel:
        if iscopy(k):
            continue
        if isinstance(k, TriggsSdika):
            if nd != 1:
                raise _abi.Unsupported("a bare TriggsSdika in a mixed cascade filters vectors only")
            stages.append(("iir", 0, k, [(0, 0)]))
        elif _is_iir(k):
            stages.append(("iir", k.axis, k.data, [(0, 0)] * nd))
        else:
            lo, hi = kernel_support((k,), nd)
            stages.append(("fir", k, None, list(zip(lo, hi))))
    for st in stages:
        if len(st[3]) < nd:
            st[3].extend([(0, 0)] * (nd - len(st[3])))
    pf, pl = kernel_support(kernel, nd)               # accumulate_padding (IIR filters 0:0)
    pf = [2 * f if f < 0 else f for f in pf]          # doublepadding: IIR and FIR together
    pl = [2 * l if l > 0 else l for l in pl]
    lo = tuple(max(-f, 0) for f in pf)
    hi = tuple(max(l, 0) for l in pl)
    dimg = img if isinstance(img, DeviceArray) else DeviceArray.from_host(host_view(img, kind))
    pb = Fill(border.value, lo, hi) if isinstance(border, Fill) else type(border)(border.style, lo, hi)
    buf, _ = _padarray(dimg, pb, okind)               # image index i (0-based) at i + lo
    R = [(f, n - 1 + l) for f, l, n in zip(pf, pl, img.shape)]

    def shrink(R, st):
        return [(r0 - f, r1 - l) for (r0, r1), (f, l) in zip(R, st[3])]

    def sl(R):
        return tuple(slice(r0 + o, r1 + o + 1) for (r0, r1), o in zip(R, lo))

    R = shrink(R, stages[0])
    for i, st in enumerate(stages):
        nxt = DeviceArray(torch.empty_like(buf.tensor), okind)
        if st[0] == "iir":
            sub = DeviceArray(_colmajor(buf.tensor[sl(R)]), okind)
            res = DeviceArray(_colmajor(torch.empty_like(sub.tensor)), okind)
            _imfilter_iir(res, sub, [(st[1], st[2])], border, False, okind, okind)
        else:
            E = [(r0 + f, r1 + l) for (r0, r1), (f, l) in zip(R, st[3])]
            sub = DeviceArray(_colmajor(buf.tensor[sl(E)]), okind)
            res = imfilter(sub, (st[1],), Inner(), alg, okind)
        nxt.tensor[sl(R)] = res.tensor.to(nxt.tensor.dtype)
        buf = nxt
        if i + 1 < len(stages):
            R = shrink(R, stages[i + 1])
    I = [(max(r0, 0), min(r1, n - 1)) for (r0, r1), n in zip(R, img.shape)]
    region = tuple(slice(i0, i1 + 1) for i0, i1 in I)
    vals = buf.tensor[sl(I)]
    if isinstance(out, DeviceArray):
        out.tensor[region] = vals.to(out.tensor.dtype)
    else:
        np.asarray(out).view(np.ndarray)[region] = vals.cpu().numpy()
    return out


def _separable_factors(kernel, nd):
    """isseparable (src/imfilter.jl:1218-1219: every factor has one extended
    dimension) with N factors for N dimensions, as normalize_separable!
    (1234-1239) needs: factor d's 1-D data (_vec) with its first index, which
    normalize_separable! pairs with axis d by position."""
    if len(kernel) != nd:
        return None
    out = []
    for k in kernel:
        if _is_iir(k):                                # isseparable: any IIR tuple (1218)
            out.append((None, k if isinstance(k, TriggsSdika) else k.data))
        elif isinstance(k, ReshapedOneD):
            out.append((k.data.first[0], np.asarray(k.data.data, dtype=np.float64).reshape(-1)))
        elif isinstance(k, OffsetKernel):
            ext = [d for d in range(k.ndim) if k.shape[d] > 1]
            if len(ext) != 1:
                return None
            out.append((k.first[ext[0]], np.asarray(k.data, dtype=np.float64).reshape(-1)))
        else:
            return None
    return out


def _imfilter_na(out, img, kernel, border, alg, kind, okind):
    """_imfilter_na! (src/imfilter.jl:280-318) with imfilter_na_separable! and
    imfilter_na_inseparable! (1094-1130): the filters are the library's Fill(0)
    filters, the NA mask and the divisions are ifx_na_* kernels."""
    if okind not in ("F32", "F64"):
        raise _abi.Unsupported("NA filtering writes Float32 or Float64 outputs")
    ctx = _ctx()
    nd = img.ndim
    na = border.na if kind in ("F32", "F64") else "none"
    zeroed = alloc_like(img, img.shape, okind)
    valid = alloc_like(img, img.shape, okind)
    has = C.c_int32(0)
    _abi.check(ctx.lib.ifx_na_prepare(ctx.handle, _desc(zeroed, okind), _desc(valid, okind),
                                      _desc(img, kind), NA.CODES[na], C.byref(has),
                                      stream_for(img, zeroed)))
    seps = _separable_factors(kernel, nd)
    if seps is not None and not has.value:
        imfilter_(out, img, kernel, Fill(0), alg)
        sums, keep = [], []
        for d, (first, w) in enumerate(seps):
            ones = alloc_like(img, (img.shape[d],), "F64")
            if isinstance(ones, DeviceArray):
                ones.tensor.fill_(1.0)
            else:
                ones[...] = 1.0
            k1 = (w,) if first is None else (ReshapedOneD(OffsetKernel(w, (first,)), 1, 0),)
            sd = imfilter(ones, k1, Fill(0), alg)
            keep.append(sd)
            sums.append(_desc(sd, "F64"))
        arr = (_abi.IfxArray * nd)(*sums)
        _abi.check(ctx.lib.ifx_na_normalize_separable(ctx.handle, _desc(out, okind), arr,
                                                      stream_for(out, img)))
        return out
    imfilter_(out, zeroed, kernel, Fill(0), alg)
    vp = imfilter(valid, kernel, Fill(0), alg)
    _abi.check(ctx.lib.ifx_na_divide(ctx.handle, _desc(out, okind), _desc(vp, kind_of(vp)),
                                     stream_for(out, vp)))
    return out


def convert_(out, img):
    """out .= convert.(eltype(out), img) on the GPU (ifx_convert): integer,
    N0f16 and other eltypes to Float32/Float64, and Float64 to integers (a value
    that is not an integer of the target's range raises InexactError, as the
    reference does when it stores a result)."""
    kind, okind = kind_of(img), kind_of(out)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    ctx = _ctx()
    try:
        _abi.check(ctx.lib.ifx_convert(ctx.handle, _desc(out, okind), _desc(img, kind), stream_for(img, out)))
    except _abi.ArgumentError as e:
        if "InexactError" in str(e):
            raise _abi.InexactError(str(e))
        raise
    return out


def _fill_in_eltype(border, kind):
    """Fill(v) holds v converted to the image eltype (src/borderarray.jl:11-20):
    an integer for integer images (InexactError otherwise), the nearest code
    for N0f16."""
    v = float(border.value)
    if kind in INT_KINDS:
        if v != int(v):
            raise _abi.InexactError("Fill value %r for an integer image" % (border.value,))
        return float(int(v))
    if kind == "N0F16":
        return round(v * 65535) / 65535.0
    return v


def _bound_sum_abs(kernel):
    """An upper bound of sum |weights| over the (cascaded) kernel."""
    b = 1.0
    for k in kernel:
        if iscopy(k):
            continue
        if isinstance(k, LaplacianKernel):
            b *= 4.0 * sum(1 for f in k.flags if f)
        elif isinstance(k, ReshapedOneD):
            b *= float(np.sum(np.abs(np.asarray(k.data.data, np.float64))))
        else:
            b *= float(np.sum(np.abs(np.asarray(getattr(k, "data", k), np.float64))))
    return b


def _imfilter_converted(out, img, kernel, border, alg, kind, okind):
    """Images the filters do not take directly (Int8..Int64, UInt16, N0f16) and
    integer results: the image is converted on the GPU to a compute eltype that
    holds its values exactly -- Float32 for 8- and 16-bit values, Float64 for
    32- and 64-bit integers and whenever the result is an integer (integer
    kernels on integer images accumulate exactly in Float64 while every partial
    sum stays below 2^53, checked from max|img| and sum |k|) -- filtered there,
    and an integer result is converted back (InexactError when it does not fit,
    as the reference's store would raise)."""
    int_out = okind in INT_KINDS
    ct = "F64" if (int_out or kind in ("I32", "I64")) else "F32"
    if kind in ("F32", "F64") and not int_out:
        ct = kind
    tmp = alloc_like(img, img.shape, ct)
    convert_(tmp, img)
    if int_out:
        m = maxabs(tmp)
        if not m * _bound_sum_abs(kernel) < 2.0 ** 53:
            raise _abi.Unsupported("integer filtering whose partial sums may exceed 2^53")
    if isinstance(border, Fill):
        border = Fill(_fill_in_eltype(border, kind), border.lo, border.hi) if border.lo is not None \
            else Fill(_fill_in_eltype(border, kind))
    res = alloc_like(img, img.shape, "F64") if int_out else out
    imfilter_(res, tmp, kernel, border, alg)
    if int_out:
        convert_(out, res)
    return out


def maxabs(img):
    """maximum(abs, img) on the GPU (ifx_maxabs)."""
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    r = C.c_double(0)
    ctx = _ctx()
    _abi.check(ctx.lib.ifx_maxabs(ctx.handle, _desc(img, kind), C.byref(r), stream_for(img)))
    return r.value


def _shift_kernel(kernel):
    """A processed kernel of the image axes as a kernel of the (channel, image
    axes...) array: nothing along the channel axis."""
    out = []
    for k in kernel:
        if isinstance(k, ReshapedOneD):
            out.append(ReshapedOneD(k.data, k.N + 1, k.axis + 1))
        elif isinstance(k, LaplacianKernel):
            out.append(LaplacianKernel((False,) + k.flags))
        elif isinstance(k, OffsetKernel):
            out.append(OffsetKernel(np.asarray(k.data)[None], (0,) + tuple(k.first)))
        else:
            raise _abi.Unsupported("kernel %r on an RGB image" % (k,))
    return tuple(out)


def _shift_border(border):
    if isinstance(border, (NA, Inner, NoPad)):
        raise _abi.Unsupported("%r borders of RGB images" % (border,))
    if getattr(border, "lo", None) is not None:
        lo, hi = (0,) + tuple(border.lo), (0,) + tuple(border.hi)
        return Fill(border.value, lo, hi) if isinstance(border, Fill) else type(border)(border.style, lo, hi)
    return border


def _imfilter_rgb(img, kernel, border, alg, T, out=None):
    """imfilter of an RGB image: the channel planes as one array with the
    channel axis first, filtered along the image axes only."""
    kind = kind_of(img.data)
    kernel = factorkernel(kernel)
    if T is None:
        T = filter_type(kind, kernel)
    if T in INT_KINDS:
        raise _abi.Unsupported("RGB images with integer results")
    k3 = _shift_kernel(kernel)
    b3 = _shift_border(borderinstance(border))
    if out is None:
        out = RGB(alloc_like(img.data, img.data.shape, T))
    imfilter_(out.data, img.data, k3, b3, alg)
    return out


def imfilter(img, kernel, border="replicate", alg=None, T=None):
    """imfilter([T], img, kernel, [border="replicate"], [alg]) (src/imfilter.jl:1-27).
    With Inner() the result covers only the interior and carries `first`."""
    if isinstance(img, RGB):
        return _imfilter_rgb(img, kernel, border, alg, T)
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    alg = _check_alg(alg)
    kernel = factorkernel(kernel)
    if T is None:
        T = filter_type(kind, kernel)
    border = borderinstance(border)
    if isinstance(border, Inner):
        return _imfilter_inner(img, kernel, border, alg, T, kind)
    out = alloc_like(img, img.shape, T)
    return imfilter_(out, img, kernel, border, alg)


def imfilter_(out, img, kernel, border="replicate", alg=None, inds=None):
    """imfilter!(out, img, kernel, [border], [alg]) (src/imfilter.jl:204-254);
    imfilter!(out, img, kernel, NoPad(), inds) computes only out[inds] (1-based
    (first, last) per axis), reading only inside img (src/imfilter.jl:367-404)."""
    if isinstance(img, RGB):
        if not isinstance(out, RGB):
            raise _abi.ArgumentError("an RGB image needs an RGB output")
        return _imfilter_rgb(img, kernel, border, alg, kind_of(out.data), out)
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    if isinstance(kernel, TriggsSdika) and isinstance(border, int) and not isinstance(border, bool):
        # imfilter!(r, out, img, kernel::TriggsSdika, dim, border) (src/imfilter.jl:922-933):
        # one pass along dimension `dim` (1-based), any Pad style or Fill
        dim, border = border, borderinstance("replicate" if alg is None else alg)
        if not 1 <= dim <= img.ndim:
            raise _abi.DimensionMismatch("dimension %d of a %d-d image" % (dim, img.ndim))
        facs = [] if iscopy(kernel) else [(dim - 1, kernel)]
        return _imfilter_iir(out, img, facs, border, False, kind, kind_of(out))
    alg = _check_alg(alg)
    okind = kind_of(out)
    kernel = factorkernel(kernel)
    nd = img.ndim
    border = borderinstance(border)
    lap_u8 = kind == "U8" and okind == "I16" and all(isinstance(k, LaplacianKernel) or iscopy(k) for k in kernel)
    if kind not in NATIVE_KINDS or (okind in INT_KINDS and not lap_u8):
        if isinstance(border, (NA, Inner)) or inds is not None or isinstance(border, NoPad):
            raise _abi.Unsupported("NA/Inner/NoPad filtering of %s images" % kind)
        return _imfilter_converted(out, img, kernel, border, alg, kind, okind)
    if isinstance(alg, Algorithm.FFT) and inds is None and isinstance(border, NoPad):
        # _imfilter_fft! with NoPad (src/imfilter.jl:819-841): the circular
        # correlation over the unpadded image, which is what a circular
        # border padded to any larger size gives
        border = borderinstance("circular")
    if (inds is not None or isinstance(border, NoPad)) and any(_is_iir(k) for k in kernel):
        raise _abi.Unsupported("IIR filters over a NoPad() subregion are not part of the GB300 path")
    if inds is not None or isinstance(border, NoPad):
        if not isinstance(border, NoPad):
            raise _abi.ErrorException("Invalid border strategy `%r`: only `NoPad()` is supported." % (border,))
        if inds is None:
            inds = [(1, n) for n in out.shape]
        inds = [(int(a), int(b)) for a, b in inds]
        if len(inds) != nd or any(b > n for (a, b), n in zip(inds, out.shape)):
            raise _abi.DimensionMismatch("inds must lie within the axes of out")
        _check_reads(inds, kernel, img.shape, "NoPad()")
        full = imfilter(img, kernel, "replicate", alg, okind)
        sl = _region(out, (1,) * nd, inds)
        if isinstance(out, DeviceArray):
            out.tensor[sl] = full.tensor[sl]
        else:
            out[sl] = full[sl]
        return out
    if isinstance(border, NA):
        return _imfilter_na(out, img, kernel, border, alg, kind, okind)
    if isinstance(border, Inner):
        raise _abi.ArgumentError("imfilter! with Inner(): allocate the interior with imfilter")
    iir = _iir_factors(kernel, nd)
    if iir is not None:
        if iir[0] == "mixed":
            return _imfilter_mixed(out, img, kernel, border, alg, kind, okind)
        return _imfilter_iir(out, img, iir[0], border, iir[1], kind, okind)
    b = border_struct(border, nd, kind)
    ai = _desc(img, kind)
    ao = _desc(out, okind)
    ctx = _ctx()
    ks = [k for k in kernel if not iscopy(k)]
    if isinstance(alg, Algorithm.FFT):
        return _imfilter_fft(ctx, out, ao, img, ai, ks, b, nd)
    if len(ks) == 1 and isinstance(ks[0], LaplacianKernel):
        L = ks[0]
        if L.N != nd:
            raise _abi.DimensionMismatch("Laplacian of %d dims on a %d-d image" % (L.N, nd))
        flags = (C.c_int32 * 4)(*[int(f) for f in L.flags])
        _abi.check(ctx.lib.ifx_imfilter_laplacian(ctx.handle, ao, ai, flags, b, stream_for(img, out)))
        return out
    facs = [_as_factor(k, nd) for k in ks]
    if all(f is not None for f in facs):
        keep = []
        arr = (_abi.IfxFactor * max(len(facs), 1))()
        for i, (ax, first, w) in enumerate(facs):
            w = np.ascontiguousarray(w, dtype=np.float64)
            keep.append(w)
            arr[i].axis = ax
            arr[i].length = w.size
            arr[i].first = first
            arr[i].weights = _abi.dptr(w)
        _abi.check(ctx.lib.ifx_imfilter_factored(ctx.handle, ao, ai, len(facs), arr, b,
                                                 stream_for(img, out)))
        return out
    K = ks[0] if len(ks) == 1 and isinstance(ks[0], OffsetKernel) else _kernelconv(ks, nd)
    K = _dense_of(K, nd)
    if K.ndim != nd:
        raise _abi.DimensionMismatch("kernel has %d dimensions, image %d" % (K.ndim, nd))
    data = np.asfortranarray(K.data, dtype=np.float64)
    ksz = (C.c_int64 * 4)(*K.shape)
    kf = (C.c_int64 * 4)(*K.first)
    _abi.check(ctx.lib.ifx_imfilter_dense(ctx.handle, ao, ai, _abi.dptr(data), ksz, kf, b,
                                          _METHOD[alg.method], stream_for(img, out)))
    return out


def _imfilter_fft(ctx, out, ao, img, ai, ks, b, nd):
    """_imfilter_fft! (src/imfilter.jl:819-841): the cascade's composite
    (kernelconv) correlated with the image padded to the padfft sizes
    (src/border.jl:239-248)."""
    if not ks:
        K = OffsetKernel(np.ones((1,) * nd), (0,) * nd)
    else:
        K = _dense_of(ks[0], nd) if len(ks) == 1 else _kernelconv(ks, nd)
    if K.ndim != nd:
        raise _abi.DimensionMismatch("kernel has %d dimensions, image %d" % (K.ndim, nd))
    data = np.asfortranarray(K.data, dtype=np.float64)
    ksz = (C.c_int64 * 4)(*K.shape)
    kf = (C.c_int64 * 4)(*K.first)
    _abi.check(ctx.lib.ifx_imfilter_fft(ctx.handle, ao, ai, _abi.dptr(data), ksz, kf, b,
                                        stream_for(img, out)))
    return out


def autotune(enable=True, cache=None):
    """Enable (or disable) the autotuner of the separable paths: the first
    device-array call per (eltypes, taps, Fill/Pad, size class) times the
    candidates -- for 2-D filters the tile kernel, pass order and output tile
    width and height; for 3-D filters the split sweeps (with their x/y tile)
    or the fused z-marching kernel (with its z chunk depth) -- and keeps the
    fastest; `cache` is a text file the choices persist in (loaded now,
    appended as keys are tuned)."""
    ctx = _ctx()
    _abi.check(ctx.lib.ifx_autotune(ctx.handle, int(bool(enable)),
                                    None if cache is None else str(cache).encode()))


_KIND_CODE = {"F32": 0, "F64": 1, "N0F8": 2, "U8": 3}


def autotune_choice(in_kind, out_kind, kx, ky, fill, shape):
    """The cached choice for a key: (x_first, variant, ms) with variant 1 the
    TMA tile kernel and 2 the gather kernel; None when the key is not tuned."""
    ctx = _ctx()
    xf, var, ms = C.c_int32(), C.c_int32(), C.c_double()
    rc = ctx.lib.ifx_autotune_choice(ctx.handle, _KIND_CODE[in_kind], _KIND_CODE[out_kind], int(kx), int(ky),
                                     int(bool(fill)), int(shape[0]), int(shape[1]) if len(shape) > 1 else 1,
                                     C.byref(xf), C.byref(var), C.byref(ms))
    if rc:
        return None
    return xf.value, var.value, ms.value


_TUNE_FIELDS = ("variant", "x_first", "tile_w", "tile_h", "depth", "ms")


def _tune_key(in_kind, out_kind, taps, shape):
    taps = tuple(int(t) for t in taps) + (1,) * (3 - len(taps))
    shape = tuple(int(n) for n in shape) + (1,) * (3 - len(shape))
    path = _abi.TUNE_SEP3D if len(shape) == 3 and shape[2] > 1 and taps[2] > 0 else _abi.TUNE_SEP2D
    return path, (C.c_int32 * 3)(*taps), (C.c_int64 * 3)(*shape)


def autotune_lookup(in_kind, out_kind, taps, fill, shape, path=None):
    """The cached choice for a key as a dict (variant, x_first, tile_w,
    tile_h, depth, ms), or None.  `taps` and `shape` are per axis (2 for the
    2-D path, 3 for the 3-D path); `path` defaults to 3-D for 3-D shapes."""
    ctx = _ctx()
    p, t, n = _tune_key(in_kind, out_kind, taps, shape)
    if path is not None:
        p = path
    ch = _abi.IfxTuneChoice()
    rc = ctx.lib.ifx_autotune_lookup(ctx.handle, p, _KIND_CODE[in_kind], _KIND_CODE[out_kind], t,
                                     int(bool(fill)), n, C.byref(ch))
    if rc:
        return None
    return {f: getattr(ch, f) for f in _TUNE_FIELDS}


def autotune_pin(in_kind, out_kind, taps, fill, shape, path=None, **choice):
    """Pin the choice for a key (fields as autotune_lookup returns them; the
    ones not given are 0 / the defaults): the next calls with the key run it."""
    ctx = _ctx()
    p, t, n = _tune_key(in_kind, out_kind, taps, shape)
    if path is not None:
        p = path
    unknown = set(choice) - set(_TUNE_FIELDS)
    if unknown:
        raise ArgumentError(f"unknown tuner fields {sorted(unknown)}")
    ch = _abi.IfxTuneChoice(**{"variant": 1, "x_first": 1, **choice})
    _abi.check(ctx.lib.ifx_autotune_pin(ctx.handle, p, _KIND_CODE[in_kind], _KIND_CODE[out_kind], t,
                                        int(bool(fill)), n, C.byref(ch)))


def autotune_clear():
    """Forget every cached and pinned choice (the cache file stays)."""
    ctx = _ctx()
    _abi.check(ctx.lib.ifx_autotune_clear(ctx.handle))


def imgradients(img, kernelfun=None, border="replicate"):
    """imgradients(img, kernelfun=KernelFactors.ando3, border="replicate")
    (src/specialty.jl:39-53): one output per dimension."""
    if kernelfun is None:
        kernelfun = KernelFactors.ando3
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    nd = img.ndim
    extended = [n > 1 for n in img.shape]
    if isinstance(borderinstance(border), Inner):
        # each gradient's interior: its kernel reads inside the image there
        grads = imgradients(img, kernelfun, "replicate")
        pair = getattr(kernelfun, "gradient_pair", None)
        if pair is not None:
            first = 1 - (np.asarray(pair[0]).size + 1) // 2
            lo = [first if e else 0 for e in extended]
            hi = [first + np.asarray(pair[0]).size - 1 if e else 0 for e in extended]
        else:
            k = _dense_of(kernelfun(tuple(extended), 1), nd)
            lo, hi = list(k.first), [f + n - 1 for f, n in zip(k.first, k.shape)]
        inds = [(max(1, 1 - l), min(n, n - h)) for l, h, n in zip(lo, hi, img.shape)]
        out = []
        for g in grads:
            sl = _region(g, (1,) * nd, inds)
            part = DeviceArray(g.tensor[sl], g.kind) if isinstance(g, DeviceArray) else g[sl]
            out.append(_with_first(part, tuple(a for a, _ in inds)))
        return tuple(out)
    if getattr(kernelfun, "dense_of", None):          # Kernel.sobel & co: dense 1-tuples
        outs = []
        for d in range(1, nd + 1):
            k = kernelfun(tuple(extended), d)
            outs.append(imfilter(img, k, border))
        return tuple(outs)
    pair = getattr(kernelfun, "gradient_pair", None)
    if pair is None:
        raise _abi.Unsupported("imgradients needs a KernelFactors or Kernel gradient function")
    if kernelfun.__name__ in ("ando4", "ando5") and not (nd == 2 and all(extended)):
        raise _abi.ErrorException("dimensions other than 2 are not yet supported")
    deriv = np.ascontiguousarray(pair[0], dtype=np.float64)
    smooth = np.ascontiguousarray(pair[1], dtype=np.float64)
    first = 1 - (deriv.size + 1) // 2
    T = "F64" if kind in ("F32", "F64", "N0F8", "U8") else None
    outs = [alloc_like(img, img.shape, T) for _ in range(nd)]
    descs = (_abi.IfxArray * nd)(*[_desc(o, T) for o in outs])
    ext = (C.c_int32 * 4)(*[int(e) for e in extended])
    b = border_struct(border, nd, kind)
    ctx = _ctx()
    _abi.check(ctx.lib.ifx_imgradients(ctx.handle, descs, _desc(img, kind), _abi.dptr(deriv),
                                       _abi.dptr(smooth), deriv.size, first, ext, b,
                                       stream_for(img)))
    return tuple(outs)


__all__ = ["Algorithm", "imfilter", "imfilter_", "imgradients", "filter_type", "factorkernel", "autotune",
           "autotune_choice", "autotune_lookup", "autotune_pin", "autotune_clear",
           "Kernel", "KernelFactors"]
