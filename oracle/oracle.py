"""Python face of the CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this module, and only as the checker.  The product
(the CUDA library and its host layer) never imports it.

Arrays follow Julia's memory order: numpy arrays in Fortran (column-major)
order whose axis 0 is Julia's axis 1.  All arithmetic is FP64 unless a routine
says otherwise.  Each wrapper names the reference lines its C routine restates
(paths relative to the ImageFiltering.jl v0.7.12 source tree).

``np_padarray`` is an independent numpy cross-check of the border maps: numpy's
``np.pad`` modes edge / wrap / symmetric / reflect / constant coincide with the
reference's replicate / circular / symmetric / reflect / Fill (the reference's
docstrings for symmetric and reflect are swapped relative to its code,
src/border.jl:107-130 vs 574-586; the code and test/border.jl:67-86 win).
"""
import ctypes as C

import numpy as np

from . import build as _build

STYLES = {"replicate": 0, "circular": 1, "symmetric": 2, "reflect": 3, "fill": 4}
_ERRS = {1: "ArgumentError", 2: "DimensionMismatch", 3: "Error", 5: "OutOfMemory"}

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build())
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="F")
        f64c = np.ctypeslib.ndpointer(np.float64, flags="C")
        i32p = np.ctypeslib.ndpointer(np.int32, flags="C")
        _lib.ora_padindex.argtypes = [C.c_int, C.c_int64, C.c_int64, C.c_int64, i64p]
        _lib.ora_padarray.argtypes = [C.c_int, i64p, f64p, C.c_int, C.c_double, i64p, i64p, f64p]
        _lib.ora_imfilter_cascade.argtypes = [C.c_int, i64p, f64p, C.c_int, i32p, i64p, i64p,
                                              f64c, C.c_int, C.c_double, f64p]
        _lib.ora_imfilter_dense.argtypes = [C.c_int, i64p, f64p, i64p, i64p, f64p,
                                            C.c_int, C.c_double, f64p]
        for nm in ("ora_laplacian_f64", "ora_laplacian_f32", "ora_laplacian_i64"):
            getattr(_lib, nm).argtypes = [C.c_int, i64p, f64p, i32p, C.c_int, C.c_double, f64p]
        _lib.ora_mapwindow_median.argtypes = [C.c_int, i64p, f64p, i64p, i64p, C.c_int,
                                              C.c_double, f64p]
        _lib.ora_mapwindow_extrema.argtypes = [C.c_int, i64p, f64p, i64p, i64p, C.c_int,
                                               C.c_double, f64p, f64p]
        _lib.ora_extrema_trunc.argtypes = [C.c_int, i64p, f64p, i64p, f64p, f64p]
        u8p = np.ctypeslib.ndpointer(np.uint8, flags="F")
        _lib.ora_mapwindow_median_u8_mt.argtypes = [i64p, u8p, i64p, i64p, C.c_int, C.c_double,
                                                    u8p, C.c_int64, C.c_int64]
        _lib.ora_imfilter_iir.argtypes = [C.c_int, i64p, f64p, C.c_int, i32p, f64c, f64c, f64c,
                                          C.c_int, C.c_double, C.c_int, C.c_int, f64p]
        _lib.ora_set_threads.argtypes = [C.c_int]
    return _lib


def set_threads(n: int) -> None:
    lib().ora_set_threads(int(n))


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle: %s" % _ERRS.get(rc, "status %d" % rc))


def _f64(a):
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def _dims(a):
    return np.array(a.shape, dtype=np.int64)


def padindex(style, lo, n, hi):
    """0-based source indices for padded positions -lo .. n-1+hi
    (src/border.jl:564-596)."""
    out = np.zeros(max(lo + n + hi, 1), dtype=np.int64)
    _check(lib().ora_padindex(STYLES[style], lo, n, hi, out))
    return out[: lo + n + hi]


def padarray(img, style, lo, hi, fill=0.0):
    """padarray(img, Pad(style, lo, hi)) or Fill(fill, lo, hi)
    (src/border.jl:324-352); returns the padded array (axis d starts at -lo[d])."""
    a = _f64(img)
    lo = np.array(lo, dtype=np.int64)
    hi = np.array(hi, dtype=np.int64)
    out = np.zeros(tuple(int(x) for x in lo + np.array(a.shape) + hi), dtype=np.float64, order="F")
    _check(lib().ora_padarray(a.ndim, _dims(a), a, STYLES[style], float(fill), lo, hi, out))
    return out


def imfilter_cascade(img, factors, style, fill=0.0):
    """imfilter with a tuple of 1-D factors, pad-then-cascade
    (src/imfilter.jl:331-341, 385-457, 671-739).  ``factors`` is a list of
    (axis, first_index, weights)."""
    a = _f64(img)
    nf = len(factors)
    axis = np.array([f[0] for f in factors], dtype=np.int32)
    first = np.array([f[1] for f in factors], dtype=np.int64)
    klen = np.array([len(f[2]) for f in factors], dtype=np.int64)
    kdata = np.ascontiguousarray(np.concatenate([np.asarray(f[2], np.float64) for f in factors])
                                 if nf else np.zeros(1))
    out = np.zeros(a.shape, dtype=np.float64, order="F")
    _check(lib().ora_imfilter_cascade(a.ndim, _dims(a), a, nf, axis, first, klen, kdata,
                                      STYLES[style], float(fill), out))
    return out


def imfilter_dense(img, K, kfirst, style, fill=0.0):
    """Dense N-d correlation, K[0,...] at index kfirst (src/imfilter.jl:624-669)."""
    a = _f64(img)
    k = _f64(K)
    assert k.ndim == a.ndim
    out = np.zeros(a.shape, dtype=np.float64, order="F")
    _check(lib().ora_imfilter_dense(a.ndim, _dims(a), a, _dims(k),
                                    np.array(kfirst, dtype=np.int64), k,
                                    STYLES[style], float(fill), out))
    return out


def laplacian(img, flags, style, fill=0.0, arith="f64"):
    """Laplacian stencil (src/specialty.jl:3-17) computed in the output eltype:
    arith 'f64', 'f32' (inputs must already be Float32 values) or 'int'."""
    a = _f64(img)
    out = np.zeros(a.shape, dtype=np.float64, order="F")
    fn = {"f64": lib().ora_laplacian_f64, "f32": lib().ora_laplacian_f32,
          "int": lib().ora_laplacian_i64}[arith]
    _check(fn(a.ndim, _dims(a), a, np.array(flags, dtype=np.int32), STYLES[style],
              float(fill), out))
    return out


def mapwindow_median(img, wfirst, wlen, style, fill=0.0):
    """mapwindow(median!, img, window; border) (src/mapwindow.jl:123-131, 270-333)."""
    a = _f64(img)
    out = np.zeros(a.shape, dtype=np.float64, order="F")
    _check(lib().ora_mapwindow_median(a.ndim, _dims(a), a, np.array(wfirst, np.int64),
                                      np.array(wlen, np.int64), STYLES[style], float(fill), out))
    return out


def mapwindow_extrema(img, wfirst, wlen, style, fill=0.0):
    """mapwindow(extrema, img, window; border) through the generic window path
    (src/mapwindow.jl:75-85, 270-333); returns (min, max)."""
    a = _f64(img)
    mn = np.zeros(a.shape, dtype=np.float64, order="F")
    mx = np.zeros(a.shape, dtype=np.float64, order="F")
    _check(lib().ora_mapwindow_extrema(a.ndim, _dims(a), a, np.array(wfirst, np.int64),
                                       np.array(wlen, np.int64), STYLES[style], float(fill),
                                       mn, mx))
    return mn, mx


def extrema_trunc(img, w):
    """mapwindow(extrema, A, window::Dims) without keywords -> Lemire filter with
    windows truncated at the edges (src/mapwindow.jl:337-338, 388-473)."""
    a = _f64(img)
    mn = np.zeros(a.shape, dtype=np.float64, order="F")
    mx = np.zeros(a.shape, dtype=np.float64, order="F")
    _check(lib().ora_extrema_trunc(a.ndim, _dims(a), a, np.array(w, np.int64), mn, mx))
    return mn, mx


def median_u8_rows(img_u8, wfirst, wlen, style, fill, row0, row1):
    """Threaded 8-bit median over rows [row0,row1) of a 2-D image (CPU-baseline
    timing helper; same window semantics as mapwindow_median)."""
    a = np.asfortranarray(img_u8, dtype=np.uint8)
    out = np.zeros(a.shape, dtype=np.uint8, order="F")
    _check(lib().ora_mapwindow_median_u8_mt(_dims(a), a, np.array(wfirst, np.int64),
                                            np.array(wlen, np.int64), STYLES[style], float(fill),
                                            out, int(row0), int(row1)))
    return out


_NP_MODES = {"replicate": "edge", "circular": "wrap", "symmetric": "symmetric",
             "reflect": "reflect"}


def np_padarray(img, style, lo, hi, fill=0.0):
    """Independent numpy restatement of padarray for cross-checking the C maps."""
    a = np.asarray(img, dtype=np.float64)
    widths = [(int(l), int(h)) for l, h in zip(lo, hi)]
    if style == "fill":
        return np.pad(a, widths, mode="constant", constant_values=fill)
    return np.pad(a, widths, mode=_NP_MODES[style])


# ------------------------------------------------------------------- IIR (Triggs-Sdika)
def triggs_sdika_M(a):
    """The right-edge matrix of a symmetric Triggs-Sdika filter
    (TriggsSdika(a, scale), src/kernelfactors.jl:497-505), row-major, in the
    coefficients' own float type."""
    a1, a2, a3 = a
    one = type(a1)(1)
    den = (one + a1 - a2 + a3) * (one - a1 - a2 - a3) * (one + a2 + (a1 - a3) * a3)
    M = [[-a3 * a1 + one - a3 * a3 - a2, (a3 + a1) * (a2 + a3 * a1), a3 * (a1 + a3 * a2)],
         [a1 + a3 * a2, -(a2 - one) * (a2 + a3 * a1), -(a3 * a1 + a3 * a3 + a2 - one) * a3],
         [a3 * a1 + a2 + a1 * a1 - a2 * a2, a1 * a2 + a3 * a2 * a2 - a1 * a3 * a3 - a3 * a3 * a3 - a3 * a2 + a3,
          a3 * (a1 + a3 * a2)]]
    return [[m / den for m in row] for row in M]


def iir_gaussian(sigma, T=np.float64):
    """IIRGaussian(T, σ) (src/kernelfactors.jl:527-545, Young, van Vliet and
    van Ginkel 2002): (a, b, scale, M) with a == b, every step in T."""
    T = np.dtype(T).type
    m0, m1, m2 = T(1.16680), T(1.10783), T(1.40586)
    q = T(1.31564 * (np.sqrt(1 + 0.490811 * float(sigma) * float(sigma)) - 1))
    ascale = (m0 + q) * (m1 * m1 + m2 * m2 + T(2) * m1 * q + q * q)
    B = (m0 * (m1 * m1 + m2 * m2) / ascale) ** 2
    a1 = q * (T(2) * m0 * m1 + m1 * m1 + m2 * m2 + (T(2) * m0 + T(4) * m1) * q + T(3) * q * q) / ascale
    a2 = -q * q * (m0 + T(2) * m1 + T(3) * q) / ascale
    a3 = q * q * q / ascale
    a = [T(a1), T(a2), T(a3)]
    return a, list(a), T(B), triggs_sdika_M(a)


def imfilter_iir(img, factors, edge="pad", fill=0.0, arith="f64", c32=False):
    """A cascade of Triggs-Sdika passes (src/imfilter.jl:961-1092): factors are
    (axis, a, b, scale, M); edge "pad" takes the boundary values from the
    lines' end elements (every Pad style, whose padding is empty for IIR
    filters), "fill" uses `fill`.  arith: "f64" (Float64 arithmetic and
    results), "f32" (Float32 arithmetic and results) or "f64/f32" (Float64
    arithmetic, Float32 results); c32: Float32 coefficients.  `img` must hold
    the values of the output eltype (Float32 values for the "f32" forms)."""
    a = _f64(img)
    nf = len(factors)
    axis = np.array([f[0] for f in factors], dtype=np.int32)
    ab = np.ascontiguousarray(np.concatenate([np.r_[np.asarray(f[1], np.float64), np.asarray(f[2], np.float64)]
                                              for f in factors]) if nf else np.zeros(1))
    sc = np.ascontiguousarray(np.array([float(f[3]) for f in factors] or [1.0]))
    M = np.ascontiguousarray(np.concatenate([np.asarray(f[4], np.float64).reshape(-1) for f in factors])
                             if nf else np.zeros(9))
    out = np.zeros(a.shape, dtype=np.float64, order="F")
    rc = lib().ora_imfilter_iir(a.ndim, _dims(a), a, nf, axis, ab, sc, M, 1 if edge == "fill" else 0,
                                float(fill), {"f64": 0, "f32": 1, "f64/f32": 2}[arith], int(bool(c32)), out)
    if rc == 2:
        raise ValueError("DimensionMismatch")
    _check(rc)
    return out


def imfilter_mixed(img, stages, style, fill=0.0):
    """A cascade of Triggs-Sdika and FIR filters (Algorithm.Mixed), FP64:
    src/imfilter.jl:385-457 over the padding of src/border.jl:614-662.  The
    image is padded by twice the accumulated FIR padding (doublepadding);
    stage k filters over indsstep_k, which starts as the padded range shrunk
    by the first filter and shrinks by each next filter (next_shrink); an IIR
    stage filters its whole range with its boundary values at the range's
    edges; the image's indices are kept.  stages: ("fir", K, first) with an
    N-d dense K, or ("iir", axis, (a, b, scale, M))."""
    a = _f64(img)
    nd = a.ndim

    def kax(st):
        if st[0] == "iir":
            return [(0, 0)] * nd
        K, first = np.asarray(st[1]), st[2]
        return [(first[d], first[d] + K.shape[d] - 1) for d in range(nd)]

    pf, pl = [0] * nd, [0] * nd
    for st in stages:
        for d, (f, l) in enumerate(kax(st)):
            pf[d] += f
            pl[d] += l
    pf = [2 * f if f < 0 else f for f in pf]
    pl = [2 * l if l > 0 else l for l in pl]
    lo = [max(-f, 0) for f in pf]
    hi = [max(l, 0) for l in pl]
    buf = padarray(a, style, lo, hi, fill)            # image index i (0-based) at i + lo
    R = [(f, n - 1 + l) for f, l, n in zip(pf, pl, a.shape)]      # expand(axes, padding), 0-based

    def shrink(R, st):
        return [(r0 - f, r1 - l) for (r0, r1), (f, l) in zip(R, kax(st))]

    def sl(R):
        return tuple(slice(r0 + o, r1 + o + 1) for (r0, r1), o in zip(R, lo))

    R = shrink(R, stages[0])
    for k, st in enumerate(stages):
        nxt = np.full(buf.shape, np.nan, order="F")
        if st[0] == "iir":
            ax, (ca, cb, sc, M) = st[1], st[2]
            nxt[sl(R)] = imfilter_iir(np.asfortranarray(buf[sl(R)]), [(ax, ca, cb, sc, M)],
                                      "fill" if style == "fill" else "pad", fill)
        else:
            K, first = np.asarray(st[1], np.float64), st[2]
            E = [(r0 + f, r1 + l) for (r0, r1), (f, l) in zip(R, kax(st))]
            full = imfilter_dense(np.asfortranarray(buf[sl(E)]), K, first, "replicate")
            inner = tuple(slice(-f, -f + (r1 - r0 + 1)) for (r0, r1), (f, l) in zip(R, kax(st)))
            nxt[sl(R)] = full[inner]
        buf = nxt
        if k + 1 < len(stages):
            R = shrink(R, stages[k + 1])
    out = np.full(a.shape, np.nan, order="F")
    I = [(max(r0, 0), min(r1, n - 1)) for (r0, r1), n in zip(R, a.shape)]
    out[tuple(slice(i0, i1 + 1) for i0, i1 in I)] = buf[sl(I)]
    return out


# ------------------------------------------------------------------- Algorithm.FFT()
def nextprod23(n):
    """nextprod([2, 3], n): the smallest 2^a 3^b >= n."""
    best, p2 = None, 1
    while p2 < 2 * max(n, 1):
        p = p2
        while p < 2 * max(n, 1):
            if p >= n and (best is None or p < best):
                best = p
            p *= 3
        p2 *= 2
    return best


def padfft(lo, hi, n):
    """padfft (src/border.jl:245-248): the kernel range lo:hi of an axis of
    length n becomes lo : lo + nextprod([2,3], n + hi - lo + 1) - n; returns
    the padding widths (before, after)."""
    P = nextprod23(n + hi - lo + 1)
    return -lo, lo + P - n


def imfilter_fft(img, K, kfirst, style, fill=0.0):
    """The FFT algorithm (src/imfilter.jl:819-870): pad with the border to the
    padfft sizes (src/border.jl:239-243, 551-555), place the kernel at the
    origin of a zero array of the padded size, correlate circularly through
    real FFTs (filtfft: irfft(rfft(A) .* conj(rfft(krn)))) and keep the
    image's indices.  FP64 (numpy's pocketfft)."""
    a = _f64(img)
    k = _f64(K)
    assert k.ndim == a.ndim
    widths = [padfft(f, f + m - 1, n) for f, m, n in zip(kfirst, k.shape, a.shape)]
    A = padarray(a, style, [w[0] for w in widths], [w[1] for w in widths], fill)
    krn = np.zeros(A.shape)
    krn[tuple(slice(0, m) for m in k.shape)] = k
    ax = list(range(A.ndim))
    R = np.fft.irfftn(np.fft.rfftn(A) * np.conj(np.fft.rfftn(krn)), s=A.shape, axes=ax)
    return np.asfortranarray(R[tuple(slice(0, n) for n in a.shape)])


# ------------------------------------------------------------------- NA() and Inner()
def naflag(img, na="isnan"):
    """na.(img) for the predicates the GB300 path takes (src/border.jl:388-405)."""
    a = np.asarray(img)
    if na == "isnan":
        return np.isnan(a)
    if na == "notfinite":
        return ~np.isfinite(a)
    return np.zeros(a.shape, dtype=bool)


def imfilter_na(img, filt, seps, na="isnan"):
    """_imfilter_na! (src/imfilter.jl:280-318) in FP64.  `filt(a)` is the filter
    with a Fill(0) border; `seps` lists (first, weights) of factor d for axis d
    -- or, for an IIR factor, a function that filters a vector of ones with it
    and Fill(0) -- when the kernel is separable with one factor per dimension
    (isseparable, 1218-1219), else None.  Separable and no NA element: the Fill(0) filter
    divided by the per-axis filters of ones, in axis order (normalize_dims!,
    1241-1250); otherwise the filter of the image with NA elements zeroed
    divided by the filter of the valid-pixel mask (imfilter_na_inseparable!,
    1110-1121)."""
    img = np.asfortranarray(np.asarray(img, dtype=np.float64))
    flag = naflag(img, na)
    with np.errstate(divide="ignore", invalid="ignore"):     # 0/0 -> NaN, as in Julia
        return _imfilter_na(img, filt, seps, flag)


def _imfilter_na(img, filt, seps, flag):
    if seps is not None and not flag.any():
        out = np.asarray(filt(img), dtype=np.float64)
        for d, sep in enumerate(seps):
            ones = np.asfortranarray(np.ones(img.shape[d]))
            if callable(sep):                      # an IIR factor: its filter of ones (1222-1228)
                sd = sep(ones)
            else:
                first, w = sep
                sd = imfilter_cascade(ones, [(0, first, np.asarray(w, np.float64))], "fill", 0.0)
            shape = [1] * img.ndim
            shape[d] = -1
            out = out / np.asarray(sd).reshape(shape)
        return out
    z = np.asfortranarray(np.where(flag, 0.0, img))
    v = np.asfortranarray((~flag).astype(np.float64))
    return np.asarray(filt(z), np.float64) / np.asarray(filt(v), np.float64)


def interior(shape, lo, hi):
    """_interior (src/border.jl:650-655): per axis the 1-based (first, last)
    where an offset range lo..hi stays inside 1..n."""
    return [(max(1, 1 - l), min(n, n - h)) for n, l, h in zip(shape, lo, hi)]


# ------------------------------------------------------------------- blob_LoG
def findlocalextrema(img, window, edges, minima=False):
    """findlocalextrema (src/extrema.jl:125-159): for every index i left in by
    the `edges` flags, i is kept when img[i] > img[i+j] (< for minima) for every
    j != 0 of the window (window >> 1 each side) with i+j inside the array.
    Returns 1-based index tuples in column-major order."""
    a = np.asarray(img, dtype=np.float64)
    nd = a.ndim
    half = [w >> 1 for w in window]
    out = []
    for lin in range(a.size):
        i = np.unravel_index(lin, a.shape, order="F")
        if any((not edges[d]) and (i[d] == 0 or i[d] == a.shape[d] - 1) for d in range(nd)):
            continue
        v = a[i]
        ok = True
        for off in np.ndindex(*[2 * h + 1 for h in half]):
            j = tuple(o - h for o, h in zip(off, half))
            if all(x == 0 for x in j):
                continue
            k = tuple(x + y for x, y in zip(i, j))
            if any(x < 0 or x >= n for x, n in zip(k, a.shape)):
                continue
            if not ((v < a[k]) if minima else (v > a[k])):
                ok = False
                break
        if ok:
            out.append(tuple(int(x) + 1 for x in i))
    return out


def log_kernel(sigmas):
    """Kernel.LoG(σs) (src/kernel.jl:325-339), dense, FP64: half-widths
    ceil(8.5σ)>>1, C (Σ x_d^2/σ_d^4 - Σ 1/σ_d^2) exp(-Σ x_d^2/2σ_d^2),
    C = 1/(Π σ (2π)^(N/2)).  Returns (K, first)."""
    import math
    N = len(sigmas)
    ws = [int(math.ceil(8.5 * s)) >> 1 for s in sigmas]
    s2 = np.array([float(s) ** 2 for s in sigmas])
    Cn = 1.0 / (float(np.prod(sigmas)) * (2 * math.pi) ** (N / 2))
    grids = np.meshgrid(*[np.arange(-w, w + 1, dtype=np.float64) for w in ws], indexing="ij")
    xs = sum(g * g / s for g, s in zip(grids, s2))
    xs4 = sum(g * g / (s * s) for g, s in zip(grids, s2))
    K = Cn * (xs4 - float(np.sum(1.0 / s2))) * np.exp(-xs / 2)
    return np.asfortranarray(K), tuple(-w for w in ws)


def multiLoG(img, sigmas, sigma_shape):
    """multiLoG (src/extrema.jl:87-98): -σ times the dense LoG filter with
    Pad(:reflect), stacked along a new first axis."""
    img = np.asfortranarray(np.asarray(img, dtype=np.float64))
    stack = np.zeros((len(sigmas),) + img.shape, order="F")
    for i, s in enumerate(sigmas):
        K, first = log_kernel([s * f for f in sigma_shape])
        stack[i] = imfilter_dense(img, K, first, "reflect") * (-s)
    return stack


def blob_LoG(img, sigmas, edges, sigma_shape, rthresh=0.001):
    """blob_LoG (src/extrema.jl:72-85): (location, σ tuple, amplitude) of the
    local maxima of the multiLoG stack above the threshold."""
    img = np.asarray(img, dtype=np.float64)
    N = img.ndim
    sig = sorted(float(s) for s in sigmas)
    stack = multiLoG(img, sig, sigma_shape)
    maxima = findlocalextrema(stack, (3,) * (N + 1), edges)
    out = []
    imgmax = float(np.max(np.abs(img))) if img.size else 0.0
    prod = float(np.prod(sigma_shape))
    for x in maxima:
        amp = stack[tuple(k - 1 for k in x)]
        if rthresh != 0 and not amp > rthresh / (sig[x[0] - 1] ** N * prod) * imgmax:
            continue
        out.append((x[1:], tuple(sig[x[0] - 1] * f for f in sigma_shape), amp))
    return out
