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
  * ``KernelFactors.TriggsSdika`` -> ``TriggsSdika(a, b, scale, M)``; a
    ``ReshapedOneD`` may wrap one (an IIR factor of an N-d cascade).
"""
import warnings
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
    """src/imfilter.jl:1252-1255: all axes 0:0 and the value 1; a Triggs-Sdika
    filter with zero coefficients and unit scale (1254)."""
    if isinstance(k, ReshapedOneD):
        return iscopy(k.data)
    if isinstance(k, TriggsSdika):
        return all(x == 0 for x in k.a) and all(x == 0 for x in k.b) and k.scale == 1
    if isinstance(k, OffsetKernel):
        return all(n == 1 for n in k.shape) and all(f == 0 for f in k.first) and \
            k.data.reshape(-1)[0] == 1
    return False


class TriggsSdika:
    """KernelFactors.TriggsSdika (src/kernelfactors.jl:462-505): an order-3
    forward filter ``a``, an order-3 backward filter ``b``, the right-edge
    matrix ``M`` (3x3) and the final ``scale``, all of one float type.

    ``TriggsSdika(a, b, scale, M)`` takes them as given; ``TriggsSdika(ab,
    scale)`` is the symmetric filter a = b = ab with M from Triggs & Sdika
    (2006) (src/kernelfactors.jl:497-505)."""

    def __init__(self, a, b, scale=None, M=None):
        if M is None:                                 # the symmetric form (ab, scale)
            if scale is not None:
                raise TypeError("TriggsSdika(a, b, scale, M) or TriggsSdika(ab, scale)")
            ab = np.asarray(a)
            T = ab.dtype.type if ab.dtype in (np.float32, np.float64) else np.float64
            self.a = ab.astype(T)
            self.b = ab.astype(T)
            self.scale = T(b)
            self.M = self._symmetric_M(self.a)
        else:
            aa = np.asarray(a)
            T = aa.dtype.type if aa.dtype in (np.float32, np.float64) else np.float64
            self.a = aa.astype(T)
            self.b = np.asarray(b).astype(T)
            self.scale = T(scale)
            self.M = np.asarray(M).astype(T).reshape(3, 3)
        if self.a.size != 3 or self.b.size != 3:
            raise ValueError("only order-3 Triggs-Sdika filters are supported")
        a1, a2, a3 = self.a
        b1, b2, b3 = self.b
        self.asum = (a1 + a2) + a3                    # sum(a) in the coefficients' type
        self.bsum = (b1 + b2) + b3

    @staticmethod
    def _symmetric_M(a):
        a1, a2, a3 = a
        one = type(a1)(1)
        den = (one + a1 - a2 + a3) * (one - a1 - a2 - a3) * (one + a2 + (a1 - a3) * a3)
        M = [[-a3 * a1 + one - a3 * a3 - a2, (a3 + a1) * (a2 + a3 * a1), a3 * (a1 + a3 * a2)],
             [a1 + a3 * a2, -(a2 - one) * (a2 + a3 * a1), -(a3 * a1 + a3 * a3 + a2 - one) * a3],
             [a3 * a1 + a2 + a1 * a1 - a2 * a2,
              a1 * a2 + a3 * a2 * a2 - a1 * a3 * a3 - a3 * a3 * a3 - a3 * a2 + a3, a3 * (a1 + a3 * a2)]]
        return np.array([[m / den for m in row] for row in M], dtype=type(a1))

    @property
    def dtype(self):
        return self.a.dtype

    def __repr__(self):
        return "TriggsSdika(a=%s, b=%s, scale=%r)" % (self.a, self.b, self.scale)


class ReshapedOneD:
    """A 1-D factor filtering along ``axis`` of an ``N``-d array
    (src/kernelfactors.jl:52-131); ``data`` is a 1-D kernel or a TriggsSdika."""

    def __init__(self, data, N, axis):
        if isinstance(data, TriggsSdika):
            self.data = data
            self.N = int(N)
            self.axis = int(axis)
            return
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
    def IIRGaussian(sigma, T=None, emit_warning=True):
        """IIRGaussian([T], σ; emit_warning=true) (src/kernelfactors.jl:527-569):
        the recursive approximation of a Gaussian of Young, van Vliet and van
        Ginkel (2002) as a symmetric TriggsSdika filter; a tuple of σs gives
        one ReshapedOneD factor per dimension.  T defaults to σ's float type
        (Float64 for integers)."""
        if isinstance(sigma, (tuple, list)):
            if T is None:
                T = np.float32 if sigma and all(isinstance(s, np.float32) for s in sigma) else np.float64
            N = len(sigma)
            return tuple(ReshapedOneD(KernelFactors.IIRGaussian(s, T, emit_warning), N, d)
                         for d, s in enumerate(sigma))
        if T is None:
            T = _as_f(sigma)
        T = np.dtype(T).type
        s = float(sigma)
        if emit_warning and s < 1 and s != 0:
            warnings.warn("σ is too small for accuracy")
        m0, m1, m2 = T(1.16680), T(1.10783), T(1.40586)
        q = T(1.31564 * (math.sqrt(1 + 0.490811 * s * s) - 1))
        two, three, four = T(2), T(3), T(4)
        ascale = (m0 + q) * (m1 * m1 + m2 * m2 + two * m1 * q + q * q)
        Bb = m0 * (m1 * m1 + m2 * m2) / ascale
        B = Bb * Bb
        a1 = q * (two * m0 * m1 + m1 * m1 + m2 * m2 + (two * m0 + four * m1) * q + three * q * q) / ascale
        a2 = -q * q * (m0 + two * m1 + three * q) / ascale
        a3 = q * q * q / ascale
        return TriggsSdika(np.array([a1, a2, a3], dtype=T), B)

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
