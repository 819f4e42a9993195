"""Kernel weights, host side: ``Kernel`` (dense) and ``KernelFactors``
(separable), mirroring src/kernel.jl and src/kernelfactors.jl.

Weights are computed on the host in the kernel's own eltype (Float64 unless
Float32 standard deviations are passed, as in the reference) and are passed to
the GB300 library unchanged.

Representation (Julia -> Python):
  * ``OffsetArray`` kernel  -> ``OffsetKernel(data, first)``; data is a
    Fortran-ordered numpy array, ``first[d]`` the first index of axis d.
  * ``ReshapedOneD{N,Npre}`` -> ``ReshapedOneD(vec, N, axis=Npre)``.
  * ``Kernel.Laplacian``     -> ``LaplacianKernel(flags)``.
"""
import math

import numpy as np


class OffsetKernel:
    """An N-d kernel with arbitrary first indices (OffsetArrays.OffsetArray)."""

    def __init__(self, data, first):
        self.data = np.asfortranarray(np.asarray(data))
        if self.data.ndim == 0:
            self.data = self.data.reshape(1)
        self.first = tuple(int(f) for f in first)
        assert len(self.first) == self.data.ndim

    @property
    def ndim(self):
        return self.data.ndim

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def shape(self):
        return self.data.shape

    def axes(self):
        return [range(f, f + n) for f, n in zip(self.first, self.data.shape)]

    def last(self):
        return tuple(f + n - 1 for f, n in zip(self.first, self.data.shape))

    def __getitem__(self, idx):
        if not isinstance(idx, tuple):
            idx = (idx,)
        return self.data[tuple(i - f for i, f in zip(idx, self.first))]

    def __len__(self):
        return self.data.size

    def __repr__(self):
        return "OffsetKernel(first=%s, %r)" % (self.first, self.data)


def centered(a):
    """OffsetArrays.centered: axis of length n gets first index 1-(n+1)//2."""
    a = np.asarray(a)
    return OffsetKernel(a, [1 - (n + 1) // 2 for n in a.shape])


def iscopy(k) -> bool:
    """src/imfilter.jl:1252-1255: all axes 0:0 and the value 1."""
    if isinstance(k, ReshapedOneD):
        return iscopy(k.data)
    if isinstance(k, OffsetKernel):
        return all(n == 1 for n in k.shape) and all(f == 0 for f in k.first) and \
            k.data.reshape(-1)[0] == 1
    return False


class ReshapedOneD:
    """A 1-D factor filtering along ``axis`` of an ``N``-d array
    (src/kernelfactors.jl:52-131)."""

    def __init__(self, data, N, axis):
        if not isinstance(data, OffsetKernel):
            data = centered(data)
        if data.ndim != 1:
            raise ValueError("ReshapedOneD data must be one dimensional")
        self.data = data
        self.N = int(N)
        self.axis = int(axis)

    @property
    def dtype(self):
        return self.data.dtype

    def dense(self):
        """convert(AbstractArray, ...) as an N-d OffsetKernel."""
        shape = [1] * self.N
        first = [0] * self.N
        shape[self.axis] = len(self.data)
        first[self.axis] = self.data.first[0]
        return OffsetKernel(self.data.data.reshape(shape, order="F"), first)

    def __repr__(self):
        return "ReshapedOneD(N=%d, axis=%d, %r)" % (self.N, self.axis, self.data)


class LaplacianKernel:
    """Kernel.Laplacian(flags) (src/kernel.jl:341-391)."""

    def __init__(self, flags=(True, True)):
        self.flags = tuple(bool(f) for f in flags)
        self.N = len(self.flags)

    def dense(self):
        shape = [3 if f else 1 for f in self.flags]
        first = [-1 if f else 0 for f in self.flags]
        A = np.zeros(shape, dtype=np.int64, order="F")
        c = tuple(1 if f else 0 for f in self.flags)
        for d, f in enumerate(self.flags):
            if f:
                for s in (0, 2):
                    i = list(c)
                    i[d] = s
                    A[tuple(i)] = 1
        A[c] = -2 * sum(self.flags)
        return OffsetKernel(A, first)


def kernelfactors(factors):
    """kernelfactors(factors::NTuple{N,AbstractVector}) (src/kernelfactors.jl:586-591)."""
    N = len(factors)
    return tuple(ReshapedOneD(f, N, d) for d, f in enumerate(factors))


def _as_f(sigma):
    return np.float32 if isinstance(sigma, np.float32) else np.float64


class KernelFactors:
    """Separable kernels (src/kernelfactors.jl)."""

    @staticmethod
    def gaussian(sigma, l=None):
        """gaussian(σ, l=4*ceil(Int,σ)+1) (src/kernelfactors.jl:438-443), or the
        tuple form gaussian((σ1,σ2,...), [(l1,l2,...)]) (449-454)."""
        if isinstance(sigma, (tuple, list)):
            ls = l if l is not None else [None] * len(sigma)
            return kernelfactors([KernelFactors.gaussian(s, li) for s, li in zip(sigma, ls)])
        T = _as_f(sigma)
        s = T(sigma)
        if l is None:
            l = 4 * int(math.ceil(float(sigma))) + 1
        if l % 2 == 0:
            raise ValueError("ArgumentError: length must be odd")
        w = l >> 1
        if s == 0:
            g = np.array([1.0], dtype=T)
        else:
            x = np.arange(-w, w + 1, dtype=T)
            g = np.exp(-(x * x) / (T(2) * s * s)).astype(T)
        return centered((g / g.sum(dtype=T)).astype(T))

    @staticmethod
    def box(*sz):
        """box((m,n,...)) (src/kernelfactors.jl:172-176)."""
        if len(sz) == 1 and isinstance(sz[0], (tuple, list)):
            sz = tuple(sz[0])
        if not all(s % 2 == 1 for s in sz):
            raise ValueError("ArgumentError: kernel dimensions must be odd, got %s" % (sz,))
        return kernelfactors([centered(np.full(s, 1.0 / s)) for s in sz])

    # gradient factor pairs (derivative, smoothing), src/kernelfactors.jl:192-427
    _GRAD = {
        "sobel": (np.array([-1.0, 0.0, 1.0]) / 2, np.array([1.0, 2.0, 1.0]) / 4),
        "prewitt": (np.array([-1.0, 0.0, 1.0]) / 2, np.array([1.0, 1.0, 1.0]) / 3),
        "scharr": (np.array([-1.0, 0.0, 1.0]) / 2, np.array([3.0 / 32.0, 5.0 / 16.0, 3.0 / 32.0]) * 2),
        "bickley": (np.array([-1.0, 0.0, 1.0]) / 2, np.array([1.0 / 12.0, 1.0 / 3.0, 1.0 / 12.0]) * 2),
        "ando3": (np.array([-1.0, 0.0, 1.0]) / 2, 2 * np.array([0.112737, 0.274526, 0.112737])),
        "ando4": (1.46205884 * np.array([-0.0919833, -0.408017, 0.408017, 0.0919833]),
                  np.array([0.0919833, 0.408017, 0.408017, 0.0919833])),
        "ando5": (0.784406 * np.array([-0.137424, -0.362576, 0.0, 0.362576, 0.137424]),
                  np.array([0.0357338, 0.248861, 0.43081, 0.248861, 0.0357338])),
    }

    @staticmethod
    def gradfactors(extended, d, k1, k2):
        """gradfactors / kdim (src/kernelfactors.jl:598-604); d is 1-based."""
        N = len(extended)
        fs = []
        for i in range(N):
            if extended[i]:
                fs.append(centered(k1 if i == d - 1 else k2))
            else:
                fs.append(OffsetKernel(np.ones(1), [0]))
        return kernelfactors(fs)


def _make_grad(name):
    def grad(extended=None, d=None):
        k1, k2 = KernelFactors._GRAD[name]
        if extended is None:                      # the 2-D pair form, e.g. sobel()
            return (kernelfactors([centered(k1), centered(k2)]),
                    kernelfactors([centered(k2), centered(k1)]))
        if name in ("ando4", "ando5") and not (len(extended) == 2 and all(extended)):
            raise RuntimeError("dimensions other than 2 are not yet supported")
        return KernelFactors.gradfactors(extended, d, k1, k2)
    grad.__name__ = name
    grad.gradient_pair = KernelFactors._GRAD[name]
    return grad


for _n in KernelFactors._GRAD:
    setattr(KernelFactors, _n, staticmethod(_make_grad(_n)))


def _outer(factors):
    """broadcast(*, factors...) of ReshapedOneD factors -> dense OffsetKernel."""
    N = factors[0].N
    data = np.ones([1] * N)
    first = [0] * N
    for f in factors:
        dk = f.dense()
        data = data * dk.data
        first = [a + b for a, b in zip(first, dk.first)]
    return OffsetKernel(data, first)


class Kernel:
    """Dense kernels (src/kernel.jl)."""

    @staticmethod
    def gaussian(sigma, l=None):
        """Kernel.gaussian (src/kernel.jl:275-287): product of the factors."""
        if not isinstance(sigma, (tuple, list)):
            sigma = (sigma, sigma)
        if len(sigma) == 1:
            return KernelFactors.gaussian(sigma[0], None if l is None else l[0])
        return _outer(KernelFactors.gaussian(tuple(sigma), l))

    @staticmethod
    def DoG(sp, sm=None, l=None):
        """Kernel.DoG (src/kernel.jl:305-313)."""
        if not isinstance(sp, (tuple, list)):
            sp = (sp, sp)
        if sm is None:
            sm = tuple(s * math.sqrt(2) for s in sp)
            neg = Kernel.gaussian(tuple(sm))
            l = neg.shape
        a = Kernel.gaussian(tuple(sp), tuple(l))
        b = Kernel.gaussian(tuple(sm), tuple(l))
        return OffsetKernel(a.data - b.data, a.first)

    @staticmethod
    def LoG(sigma):
        """Kernel.LoG (src/kernel.jl:325-339): dense, half-width ceil(8.5σ)>>1."""
        if not isinstance(sigma, (tuple, list)):
            sigma = (sigma, sigma)
        sig = np.array(sigma, dtype=np.float64)
        N = len(sigma)
        ws = [int(math.ceil(8.5 * s)) >> 1 for s in sigma]
        grids = np.meshgrid(*[np.arange(-w, w + 1, dtype=np.float64) for w in ws], indexing="ij")
        C = 1.0 / (np.prod(sig) * (2 * math.pi) ** (N / 2))
        s2 = sig ** 2
        s2i = np.sum(1.0 / s2)
        xs = [g ** 2 / s2[d] for d, g in enumerate(grids)]
        val = (sum(x / s2[d] for d, x in enumerate(xs)) - s2i) * np.exp(-sum(xs) / 2)
        return OffsetKernel(C * val, [-w for w in ws])

    @staticmethod
    def Laplacian(flags=(True, True), N=None):
        """Kernel.Laplacian(flags) or Laplacian(dims, N) (src/kernel.jl:359-380)."""
        if N is not None:
            dims = flags
            flags = [False] * N
            for d in dims:
                flags[d - 1] = True
        return LaplacianKernel(flags)

    @staticmethod
    def laplacian2d(alpha=0):
        """Kernel.laplacian2d (src/kernel.jl:421-426)."""
        lc = alpha / (1 + alpha)
        lb = (1 - alpha) / (1 + alpha)
        lm = -4 / (1 + alpha)
        return centered(np.array([[lc, lb, lc], [lb, lm, lb], [lc, lb, lc]], dtype=np.float64))

    @staticmethod
    def box(sz):
        return _outer(KernelFactors.box(tuple(sz)))

    @staticmethod
    def reflect(k):
        """Kernel.reflect (src/kernel.jl:520-529): K'[-I] = K[I]."""
        data = k.data[tuple(slice(None, None, -1) for _ in range(k.ndim))]
        return OffsetKernel(data, [-(f + n - 1) for f, n in zip(k.first, k.shape)])


def _make_dense_grad(name):
    def grad(extended=None, d=None):
        if extended is None:
            a, b = getattr(KernelFactors, name)()
            return _outer(a), _outer(b)
        return (_outer(getattr(KernelFactors, name)(extended, d)),)
    grad.__name__ = name
    grad.dense_of = name
    return grad


for _n in KernelFactors._GRAD:
    setattr(Kernel, _n, staticmethod(_make_dense_grad(_n)))
