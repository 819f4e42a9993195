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
from .arrays import DeviceArray, alloc_like, host_view, kind_of, ptr_strides, stream_for
from .borders import border_struct, borderinstance
from .kernels import (Kernel, KernelFactors, LaplacianKernel, OffsetKernel, ReshapedOneD,
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
        pass

    class IIR(Alg):
        pass

    class Mixed(Alg):
        pass

    class GB300(Alg):
        """Direct (FIR) filtering by the sm_103a kernels of this package.

        ``method``: "auto", "cuda_cores" or "tensor_cores" (dense kernels)."""

        def __init__(self, method="auto"):
            self.method = method


_METHOD = {"auto": 0, "cuda_cores": 1, "tensor_cores": 2}


# ------------------------------------------------------------------ eltypes
def _kernel_dtype(k):
    if isinstance(k, LaplacianKernel):
        return None
    return np.dtype(k.dtype)


def _promote_one(img_kind, kdt):
    """typeof(zero(S)*zero(T) + ...) for the supported (S, T) pairs."""
    if kdt is None:
        return None
    if img_kind == "F64" or kdt == np.float64:
        return "F64"
    if kdt == np.float32:
        return "F32"
    if np.issubdtype(kdt, np.integer) or kdt == np.bool_:
        if img_kind in ("F32", "N0F8"):
            return "F32"
        raise _abi.Unsupported("integer kernels on integer images (integer arithmetic) are not "
                               "part of the GB300 path")
    raise _abi.Unsupported("kernel eltype %s" % kdt)


def filter_type(img_kind, kernel):
    """src/imfilter.jl:1131-1154."""
    if isinstance(kernel, LaplacianKernel):
        return {"F32": "F32", "F64": "F64", "N0F8": "F32", "U8": "I16"}[img_kind]
    if isinstance(kernel, tuple):
        kinds = [filter_type(img_kind, k) for k in kernel]
        if "F64" in kinds:
            return "F64"
        return kinds[0] if kinds else {"F64": "F64"}.get(img_kind, "F32")
    return _promote_one(img_kind, _kernel_dtype(kernel))


# ------------------------------------------------------------------ factoring
def factorkernel(kernel):
    """src/imfilter.jl:1156-1184: a 2-D dense kernel is tested for separability
    with an SVD (threshold sqrt(eps)); other kernels become 1-tuples."""
    if isinstance(kernel, tuple):
        return kernel
    if isinstance(kernel, (LaplacianKernel, ReshapedOneD)):
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
    if alg is None or isinstance(alg, Algorithm.GB300):
        return alg or Algorithm.GB300()
    if isinstance(alg, Algorithm.Alg):
        raise _abi.Unsupported("%s runs on the CPU in the reference; this package implements "
                               "Algorithm.GB300() only" % type(alg).__name__)
    raise _abi.ArgumentError("unknown algorithm %r" % (alg,))


def _desc(a, kind, first=None):
    p, st = ptr_strides(a)
    return _abi.describe(p, kind, a.shape, st, first)


def imfilter(img, kernel, border="replicate", alg=None, T=None):
    """imfilter([T], img, kernel, [border="replicate"], [alg]) (src/imfilter.jl:1-27)."""
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    alg = _check_alg(alg)
    kernel = factorkernel(kernel)
    if T is None:
        T = filter_type(kind, kernel)
    out = alloc_like(img, img.shape, T)
    return imfilter_(out, img, kernel, border, alg)


def imfilter_(out, img, kernel, border="replicate", alg=None):
    """imfilter!(out, img, kernel, [border], [alg]) (src/imfilter.jl:204-254)."""
    kind = kind_of(img)
    if not isinstance(img, DeviceArray):
        img = host_view(img, kind)
    alg = _check_alg(alg)
    okind = kind_of(out)
    kernel = factorkernel(kernel)
    nd = img.ndim
    b = border_struct(border, nd, kind)
    ai = _desc(img, kind)
    ao = _desc(out, okind)
    ctx = _ctx()
    ks = [k for k in kernel if not iscopy(k)]
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


__all__ = ["Algorithm", "imfilter", "imfilter_", "imgradients", "filter_type", "factorkernel",
           "Kernel", "KernelFactors"]
