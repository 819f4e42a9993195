"""Known-answer cases of ImageFiltering.jl's own test suite, shared by the
oracle tests (CPU) and the GPU parity tests.

Each case cites the reference test it restates (paths relative to the
ImageFiltering.jl v0.7.12 tree).  Literal tables come from
tests/golden/reference_kats.json (extracted from the reference's test files by
tests/golden/extract_reference_kats.py); the structural cases (impulse
responses, edge coefficients, analytic targets) are rebuilt here with the same
construction as the reference test.

A backend is an object with the methods used below (see OracleBackend and, in
the GPU tests, GpuBackend).  Arrays are numpy arrays in Julia axis order
(index [i, j] is Julia's [i+1, j+1]).
"""
import json
import os

import numpy as np

GOLDEN = json.load(open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden",
                                     "reference_kats.json")))
BORDERS = ["replicate", "circular", "symmetric", "reflect", "fill"]


def F(a, dtype=np.float64):
    return np.asfortranarray(np.asarray(a, dtype=dtype))


# ------------------------------------------------------------------- backends
class OracleBackend:
    """The CPU oracle, FP64."""

    def __init__(self, O):
        self.O = O

    def padarray(self, A, style, lo, hi, fill=0.0):
        return self.O.padarray(A, style, lo, hi, fill)

    def cascade(self, img, factors, style, fill=0.0):
        return self.O.imfilter_cascade(img, factors, style, fill)

    def dense(self, img, K, kfirst, style, fill=0.0):
        return self.O.imfilter_dense(img, K, kfirst, style, fill)

    def laplacian(self, img, flags, style, fill=0.0, arith="f64"):
        return self.O.laplacian(img, flags, style, fill, arith)

    def median(self, img, wf, wl, style, fill=0.0):
        return self.O.mapwindow_median(img, wf, wl, style, fill)

    def extrema(self, img, wf, wl, style, fill=0.0):
        return self.O.mapwindow_extrema(img, wf, wl, style, fill)

    def extrema_lemire(self, img, w):
        return self.O.extrema_trunc(img, w)

    def localextrema(self, img, window=None, edges=True, minima=False):
        a = np.asarray(img)
        window = window or (3,) * a.ndim
        edges = (edges,) * a.ndim if isinstance(edges, bool) else edges
        return self.O.findlocalextrema(a, window, edges, minima)

    def blob_log(self, img, sigmas, edges=None, sigma_shape=None, rthresh=0.001):
        a = np.asarray(img, dtype=np.float64)
        N = a.ndim
        edges = (True,) + (False,) * N if edges is None else ((edges,) * (N + 1) if isinstance(edges, bool)
                                                               else edges)
        return self.O.blob_LoG(a, sigmas, tuple(edges), tuple(sigma_shape or (1.0,) * N), rthresh)

    def na_cascade(self, img, factors, na="isnan"):
        O = self.O
        filt = lambda a: O.imfilter_cascade(a, factors, "fill", 0.0)
        nd = np.asarray(img).ndim
        seps = [(f, w) for _, f, w in factors] if len(factors) == nd else None
        return O.imfilter_na(img, filt, seps, na)

    def na_dense(self, img, K, kfirst, na="isnan"):
        O = self.O
        K = np.asarray(K, np.float64)
        filt = lambda a: O.imfilter_dense(a, K, kfirst, "fill", 0.0)
        ext = [d for d in range(K.ndim) if K.shape[d] > 1]
        seps = None
        if np.asarray(img).ndim == 1 and len(ext) == 1:        # a 1-tuple kernel on a vector
            seps = [(kfirst[0], K.reshape(-1))]
        return O.imfilter_na(img, filt, seps, na)

    def fft(self, img, K, kfirst, style, fill=0.0):
        return self.O.imfilter_fft(img, K, kfirst, style, fill)

    def _iir_facs(self, sigmas):
        facs = []
        for ax, s in sigmas:
            a, b, B, M = self.O.iir_gaussian(s)
            if any(x != 0 for x in a) or B != 1:
                facs.append((ax, a, b, B, M))
        return facs

    def iir(self, img, sigmas, style, fill=0.0):
        """IIRGaussian factors (axis, σ) as a ReshapedOneD cascade."""
        return self.O.imfilter_iir(img, self._iir_facs(sigmas), "fill" if style == "fill" else "pad", fill)

    def iir_dim(self, img, sigma, dim, style):
        return self.iir(img, [(dim - 1, sigma)], style)

    def mixed(self, img, spec, style, fill=0.0):
        """spec: ("iir", axis, σ) | ("fir", K, first) | ("lap",) in cascade order."""
        nd = np.asarray(img).ndim
        stages = []
        for st in spec:
            if st[0] == "iir":
                stages.append(("iir", st[1], self.O.iir_gaussian(st[2])))
            elif st[0] == "lap":
                L = np.zeros((3,) * nd)
                for d in range(nd):
                    idx = [1] * nd
                    for e in (0, 2):
                        idx[d] = e
                        L[tuple(idx)] = 1
                L[(1,) * nd] = -2 * nd
                stages.append(("fir", L, (-1,) * nd))
            else:
                stages.append(("fir", np.asarray(st[1], np.float64), tuple(st[2])))
        return self.O.imfilter_mixed(img, stages, style, fill)

    def iir_na(self, img, sigmas, na="isnan"):
        O = self.O
        facs = self._iir_facs(sigmas)
        filt = lambda a: O.imfilter_iir(a, facs, "fill", 0.0)
        nd = np.asarray(img).ndim
        seps = None
        if len(sigmas) == nd and [ax for ax, _ in sigmas] == list(range(nd)):
            seps = [(lambda v, f=self._iir_facs([(0, s)]): O.imfilter_iir(v, f, "fill", 0.0)) for _, s in sigmas]
        return O.imfilter_na(img, filt, seps, na)

    def fft_cascade(self, img, factors, style, fill=0.0):
        nd = np.asarray(img).ndim
        K, first = cascade_kernel(factors, nd)
        return self.O.imfilter_fft(img, K, first, style, fill)

    def fft_nopad(self, img, K, kfirst):
        """imfilter!(CPU1(Algorithm.FFT()), out, img, kern, NoPad()): the
        circular correlation over the unpadded image."""
        a = np.asarray(img, np.float64)
        krn = np.zeros(a.shape)
        for idx in np.ndindex(*np.asarray(K).shape):
            krn[tuple((i + f) % n for i, f, n in zip(idx, kfirst, a.shape))] = K[idx]
        ax = list(range(a.ndim))
        R = np.fft.irfftn(np.fft.rfftn(a) * np.conj(np.fft.rfftn(krn)), s=a.shape, axes=ax)
        return R

    def inner_dense(self, img, K, kfirst):
        O = self.O
        K = np.asarray(K, np.float64)
        inds = O.interior(np.asarray(img).shape, kfirst, [f + n - 1 for f, n in zip(kfirst, K.shape)])
        full = O.imfilter_dense(img, K, kfirst, "replicate")
        return full[tuple(slice(a - 1, b) for a, b in inds)], tuple(a for a, _ in inds)

    def inner_cascade(self, img, factors):
        O = self.O
        nd = np.asarray(img).ndim
        lo, hi = [0] * nd, [0] * nd
        for ax, f, w in factors:
            lo[ax] += f
            hi[ax] += f + len(w) - 1
        inds = O.interior(np.asarray(img).shape, lo, hi)
        full = O.imfilter_cascade(img, factors, "replicate")
        return full[tuple(slice(a - 1, b) for a, b in inds)], tuple(a for a, _ in inds)


def cascade_kernel(factors, nd):
    """kernelconv of (axis, first, weights) factors: the dense composite and
    its first indices."""
    K = np.ones((1,) * nd)
    first = [0] * nd
    for ax, f, w in factors:
        shape = [1] * nd
        shape[ax] = len(w)
        b = np.asarray(w, np.float64).reshape(shape)
        out = np.zeros([sa + sb - 1 for sa, sb in zip(K.shape, b.shape)])
        for idx in np.ndindex(*b.shape):
            out[tuple(slice(i, i + s) for i, s in zip(idx, K.shape))] += K * b[idx]
        K = out
        first[ax] += f
    return K, tuple(first)


# ------------------------------------------------------------------- padarray
def padarray_cases():
    """test/border.jl:35-206 golden tables."""
    for k in GOLDEN["padarray"]:
        A = F(k["A"])
        b = k["border"]
        yield k["source"], A, b["style"], b["lo"], b["hi"], b.get("fill", 0), F(k["expected"])


def check_padarray(be, dtype=np.float64, unsigned=False):
    n = 0
    for src, A, style, lo, hi, fill, exp in padarray_cases():
        if unsigned and fill < 0:        # Fill(-1) has no UInt8 value
            continue
        got = be.padarray(F(A, dtype), style, lo, hi, fill)
        assert got.shape == exp.shape, src
        assert np.array_equal(np.asarray(got, np.float64), exp), "%s %s" % (src, style)
        n += 1
    assert n >= 19


def check_padindex_vs_numpy(be, O):
    """Border maps against numpy's np.pad on random sizes (test/border.jl:15-23
    checks BorderArray == padarray the same way)."""
    rng = np.random.default_rng(7)
    for _ in range(30):
        A = F(rng.standard_normal((int(rng.integers(2, 7)), int(rng.integers(2, 7)))))
        style = ["replicate", "circular", "symmetric", "reflect"][int(rng.integers(0, 4))]
        lo = [int(x) for x in rng.integers(0, 9, 2)]
        hi = [int(x) for x in rng.integers(0, 9, 2)]
        got = be.padarray(A, style, lo, hi)
        exp = O.np_padarray(A, style, lo, hi)
        assert np.array_equal(np.asarray(got), exp), (style, lo, hi, A.shape)


# ------------------------------------------------------------------- impulses
KERN = np.array([[0.1, 0.2], [0.4, 0.5]])          # test/2d.jl:55-56, axes (-1:0, 1:2)
KFIRST = (-1, 1)
FACTORS = [(0, -1, np.array([0.2, 0.8])), (1, 1, np.array([0.3, 0.6]))]   # test/2d.jl:83


def rot180(a):
    return a[::-1, ::-1]


def check_impulse_interior(be):
    """test/2d.jl:49-79 and 82-100: impulse away from the edges; every border
    gives target[3:4,2:3] = rot180(kern) (correlation, origin at K[0,0])."""
    img = np.zeros((5, 7))
    img[2, 3] = 1
    img = F(img)
    target = np.zeros((5, 7))
    target[2:4, 1:3] = rot180(KERN)
    kf = np.outer(FACTORS[0][2], FACTORS[1][2])
    targetf = np.zeros((5, 7))
    targetf[2:4, 1:3] = rot180(kf)
    for style in BORDERS:
        got = be.dense(img, KERN, KFIRST, style)
        np.testing.assert_allclose(got, target, atol=1e-12, err_msg=style)
        got = be.cascade(img, FACTORS, style)
        np.testing.assert_allclose(got, targetf, atol=1e-12, err_msg=style)


def target1(style, kern):
    """test/2d.jl:171-195: impulse at [1,2] where the border matters."""
    ret = np.zeros((5, 7))
    x = 1.0
    if style in ("replicate", "symmetric"):
        ret[0, 0] = (kern[0, 0] + kern[1, 0]) * x
        ret[1, 0] = kern[0, 0] * x
    elif style == "circular":
        r = rot180(kern) * x                      # a[0:1, -1:0] of an FFTView
        ret[0, 6], ret[0, 0] = r[0, 0], r[0, 1]
        ret[1, 6], ret[1, 0] = r[1, 0], r[1, 1]
    else:                                         # reflect, Fill(0)
        ret[0, 0] = kern[1, 0] * x
        ret[1, 0] = kern[0, 0] * x
    return ret


def check_impulse_edge(be):
    img = np.zeros((5, 7))
    img[0, 1] = 1
    img = F(img)
    kf = np.outer(FACTORS[0][2], FACTORS[1][2])
    for style in BORDERS:
        np.testing.assert_allclose(be.dense(img, KERN, KFIRST, style), target1(style, KERN),
                                   atol=1e-12, err_msg=style)
        np.testing.assert_allclose(be.cascade(img, FACTORS, style), target1(style, kf),
                                   atol=1e-12, err_msg=style)


# ------------------------------------------------------------------- 1-D cascades
K1 = (0, -1, np.array([0.25, 0.5, 0.25]))             # test/nd.jl:58
K2 = (0, 1, np.array([0.5, 0.5]))                      # OffsetArray([0.5,0.5], 1:2)
KC = (0, 0, np.array([1.0]))                           # centered([1]): a copy kernel


def _golden_cascade(name):
    for k in GOLDEN["cascade_1d"]:
        if k["name"] == name:
            return k
    raise KeyError(name)


def check_cascade_1d(be):
    """test/nd.jl:56-75: cascade trimming and copy kernels on 1:8."""
    img = F(np.arange(1, 9))
    A2 = _golden_cascade("A2")
    a2 = np.array(A2["expected"])                       # axes 0:9
    a3 = np.array([0.25 * a2[i - 1] + 0.5 * a2[i] + 0.25 * a2[i + 1] for i in range(1, 9)])
    casc = be.cascade(img, [K1, K2, K1], "replicate")
    np.testing.assert_allclose(casc, a3, rtol=1e-12)
    # A1/A2 are the successive Inner filterings of the padded array
    A0 = be.padarray(img, "replicate", [2], [4])         # axes -1:12
    a1 = np.array([sum(A0[i + 1 + j - 1] * K1[2][j] for j in range(3)) for i in range(0, 12)])
    np.testing.assert_allclose(a1, _golden_cascade("A1")["expected"], rtol=1e-12)
    a2c = np.array([sum(a1[i + 1 + j] * K2[2][j] for j in range(2)) for i in range(10)])
    np.testing.assert_allclose(a2c, a2, rtol=1e-12)
    exp = _golden_cascade("k1_on_1to8")["expected"]
    np.testing.assert_allclose(be.cascade(img, [K1], "replicate"), exp, rtol=1e-12)
    np.testing.assert_allclose(be.cascade(img, [KC, K1], "replicate"), exp, rtol=1e-12)
    np.testing.assert_allclose(be.cascade(img, [K1, KC], "replicate"), exp, rtol=1e-12)


def check_offset_axes_1d(be):
    """test/nd.jl:84-93: impulse in the middle, every border."""
    img = np.zeros(11)
    img[5] = 1
    img = F(img)
    for style in BORDERS:
        f = be.cascade(img, [K1], style)
        assert f[4] == f[6] == 0.25 and f[5] == 0.5
        assert np.all(f[:4] == 0) and np.all(f[7:] == 0)


def check_nonfinite(be):
    """test/nd.jl:95-109: NaN/Inf spread over the 31-tap window only."""
    rng = np.random.default_rng(11)
    for x in (np.nan, np.inf, -np.inf):
        v = F(rng.random(100))
        i = int(rng.integers(0, 100))
        w = v.copy()
        w[i] = x
        k = [(0, -15, np.ones(31))]
        vf = be.cascade(v, k, "replicate")
        wf = be.cascade(w, k, "replicate")
        around = np.abs(np.arange(100) - i) <= 15
        assert np.all(np.isnan(wf[around])) if np.isnan(x) else np.all(wf[around] == x)
        np.testing.assert_allclose(wf[~around], vf[~around], rtol=1e-10)


def check_3d_box(be):
    """test/nd.jl:128-157: 3-D box kernel on ones; Fill(0) gives (2/3)^k at
    faces, edges and corners; every Pad style gives ones."""
    img = F(np.ones((10, 10, 10)))
    K = np.full((3, 3, 3), 1 / 27)
    for style in ["replicate", "circular", "symmetric", "reflect"]:
        np.testing.assert_allclose(be.dense(img, K, (-1, -1, -1), style), img, rtol=1e-12)
    t = np.ones((10, 10, 10))
    for i in (0, 9):
        t[:, :, i] = t[:, i, :] = t[i, :, :] = 2 / 3
    for i in (0, 9):
        for j in (0, 9):
            t[:, i, j] = t[i, :, j] = t[i, j, :] = (2 / 3) ** 2
    for i in (0, 9):
        for j in (0, 9):
            for k in (0, 9):
                t[i, j, k] = (2 / 3) ** 3
    np.testing.assert_allclose(be.dense(img, K, (-1, -1, -1), "fill"), t, rtol=1e-12)


def check_cascade_equals_dense(be):
    """test/cascade.jl:4-39: a cascade equals the convolved dense kernel for
    every border."""
    rng = np.random.default_rng(5)
    a = F(rng.random(15))
    c = np.array([1.0, 2, 3, 2, 1])
    for style in BORDERS:
        afc = be.cascade(a, [(0, -1, np.ones(3)), (0, -1, np.ones(3))], style)
        af2 = be.dense(a, c, (-2,), style)
        np.testing.assert_allclose(afc, af2, rtol=1e-12)
    a = F(rng.random((15, 15)))
    kx, ky = (0, -1, np.ones(3)), (1, -1, np.ones(3))
    kern2 = np.outer(c, c)
    kern2x = np.outer(c, np.ones(3))
    kern2y = np.outer(np.ones(3), c)
    for style in BORDERS:
        np.testing.assert_allclose(be.cascade(a, [kx, ky, kx, ky], style),
                                   be.dense(a, kern2, (-2, -2), style), rtol=1e-12)
        np.testing.assert_allclose(be.cascade(a, [kx, kx, ky, ky], style),
                                   be.dense(a, kern2, (-2, -2), style), rtol=1e-12)
        np.testing.assert_allclose(be.cascade(a, [kx, kx, ky], style),
                                   be.dense(a, kern2x, (-2, -1), style), rtol=1e-12)
        np.testing.assert_allclose(be.cascade(a, [ky, kx, ky], style),
                                   be.dense(a, kern2y, (-1, -2), style), rtol=1e-12)


def check_fill_interior(be, gauss_factors):
    """test/2d.jl:241-268 (issue #85): Fill(0) and Fill(10) agree inside and
    differ at the corner."""
    A = F(np.ones((8, 8)))
    r1 = be.cascade(A, gauss_factors, "fill", 0.0)
    r2 = be.cascade(A, gauss_factors, "fill", 10.0)
    assert r1[3, 3] == r2[3, 3]
    assert r1[0, 0] != r2[0, 0]


def check_prewitt_band(be):
    """test/2d.jl:7-25: Prewitt factors on a UInt8 diagonal band."""
    m = np.zeros((20, 20))
    for i in range(-2, 3):
        idx = np.arange(max(0, -i), min(20, 20 - i))
        m[idx, idx + i] = 255
    m = F(m)
    target = np.zeros((20, 20))
    dv = [42.5, 85, 85, 42.5]
    for i in range(1, 5):
        idx = np.arange(0, 20 - i)
        target[idx, idx + i] = dv[i - 1]
        target[idx + i, idx] = -dv[i - 1]
    facs = [(0, -1, np.array([-1.0, 0.0, 1.0]) / 2), (1, -1, np.array([1.0, 1.0, 1.0]) / 3)]
    mf = be.cascade(m, facs, "replicate")
    np.testing.assert_allclose(mf[1:19, 1:19], target[1:19, 1:19], rtol=1e-12, atol=1e-9)


# ------------------------------------------------------------------- Laplacian
def check_laplacian(be, arith="f64"):
    """test/specialty.jl:6-156: impulse goldens and edge coefficients, exact."""
    def imp(shape, idx):
        a = np.zeros(shape)
        a[idx] = 1
        return F(a)
    a = imp((5,), 2)
    assert np.array_equal(be.laplacian(a, [1], "replicate", arith=arith), [0, 1, -2, 1, 0])
    a = imp((5,), 0)
    for style, c in (("replicate", -1), ("fill", -2)):
        assert np.array_equal(be.laplacian(a, [1], style, arith=arith), [c, 1, 0, 0, 0])
    a = imp((5, 5), (2, 2))
    exp = np.zeros((5, 5))
    exp[2, 2] = -4
    exp[1, 2] = exp[3, 2] = exp[2, 1] = exp[2, 3] = 1
    assert np.array_equal(be.laplacian(a, [1, 1], "replicate", arith=arith), exp)
    a = imp((5, 5), (2, 0))
    for style, c in (("replicate", -3), ("fill", -4)):
        exp = np.zeros((5, 5))
        exp[1, 0] = exp[3, 0] = exp[2, 1] = 1
        exp[2, 0] = c
        assert np.array_equal(be.laplacian(a, [1, 1], style, arith=arith), exp), style
    a = imp((5, 5), (4, 4))
    for style, c in (("replicate", -2), ("fill", -4)):
        exp = np.zeros((5, 5))
        exp[3, 4] = exp[4, 3] = 1
        exp[4, 4] = c
        assert np.array_equal(be.laplacian(a, [1, 1], style, arith=arith), exp), style
    # vertical only: Laplacian((true,false))
    a = imp((5, 5), (2, 2))
    exp = np.zeros((5, 5))
    exp[1, 2] = exp[3, 2] = 1
    exp[2, 2] = -2
    assert np.array_equal(be.laplacian(a, [1, 0], "replicate", arith=arith), exp)
    a = imp((5, 5), (2, 0))
    for style, c in (("replicate", -2), ("fill", -2)):
        exp = np.zeros((5, 5))
        exp[1, 0] = exp[3, 0] = 1
        exp[2, 0] = c
        assert np.array_equal(be.laplacian(a, [1, 0], style, arith=arith), exp), style
    a = imp((5, 5), (4, 4))
    for style, c in (("replicate", -1), ("fill", -2)):
        exp = np.zeros((5, 5))
        exp[3, 4] = 1
        exp[4, 4] = c
        assert np.array_equal(be.laplacian(a, [1, 0], style, arith=arith), exp), style


# ------------------------------------------------------------------- gradients
SOBEL = (np.array([-1.0, 0.0, 1.0]) / 2, np.array([1.0, 2.0, 1.0]) / 4)


def sobel_factors(nd, d, extended=None):
    ext = extended or [True] * nd
    fs = []
    for e in range(nd):
        if not ext[e]:
            continue
        fs.append((e, -1, SOBEL[0] if e == d else SOBEL[1]))
    return fs


def check_gradient_ramps(be):
    """test/gradient.jl:4-70: linear ramps have constant gradients inside
    (the reference checks with Inner(); here the interior of a replicate result)."""
    y = np.arange(1, 6)[:, None] * np.ones((1, 7))
    x = np.ones((5, 1)) * np.arange(1, 8)[None, :]
    for img, ey, ex in ((F(y), 1, 0), (F(x), 0, 1)):
        gy = be.cascade(img, sobel_factors(2, 0), "replicate")
        gx = be.cascade(img, sobel_factors(2, 1), "replicate")
        assert np.all(np.abs(gy[1:-1, 1:-1] - ey) < 1e-4)
        assert np.all(np.abs(gx[1:-1, 1:-1] - ex) < 1e-4)
    y3 = np.arange(1, 6)[:, None, None] * np.ones((5, 7, 6))
    x3 = np.arange(1, 8)[None, :, None] * np.ones((5, 7, 6))
    z3 = np.arange(1, 7)[None, None, :] * np.ones((5, 7, 6))
    for img, e in ((F(y3), (1, 0, 0)), (F(x3), (0, 1, 0)), (F(z3), (0, 0, 1))):
        for d in range(3):
            g = be.cascade(img, sobel_factors(3, d), "replicate")
            assert np.all(np.abs(g[1:-1, 1:-1, 1:-1] - e[d]) < 1e-4)


# ------------------------------------------------------------------- mapwindow
def check_extrema_lemire_golden(be):
    """test/mapwindow.jl:17-46: 1-D extrema, windows 1..7 (even included)."""
    n = 0
    for k in GOLDEN["extrema_lemire_1d"]:
        A = F(k["A"])
        mn, mx = be.extrema_lemire(A, [k["window"]])
        exp = np.array(k["expected"])
        assert np.array_equal(mn, exp[:, 0]) and np.array_equal(mx, exp[:, 1]), k["source"]
        n += 1
    assert n == 14


def groundtruth(f, A, window):
    """test/mapwindow.jl:5-14: reduce over clamped shifts."""
    Aex = A.copy()
    h = [w // 2 + 1 for w in window]
    for shift in np.ndindex(*window):
        for I in np.ndindex(*A.shape):
            J = tuple(min(max(I[d] + shift[d] + 1 - h[d], 0), A.shape[d] - 1) for d in range(A.ndim))
            Aex[I] = f(Aex[I], A[J])
    return Aex


def check_extrema_nd(be, seed=3):
    """test/mapwindow.jl:47-73: 2-D and 3-D extrema against the clamp ground truth."""
    rng = np.random.default_rng(seed)
    A = rng.random((5, 5)) / 10
    A[1, 1] = 0.8
    A[3, 3] = 0.6
    A = F(A)
    for w in ((2, 2), (2, 3), (3, 2), (3, 3), (2, 5)):
        mn, mx = be.extrema_lemire(A, list(w))
        assert np.array_equal(mx, groundtruth(max, A, w))
        assert np.array_equal(mn, groundtruth(min, A, w))
    A = rng.random((5, 5, 5)) / 10
    A[1, 1, 1] = 0.7
    A[3, 3, 1] = 0.4
    A[1, 1, 3] = 0.5
    A = F(A)
    for w in ((2, 2, 2), (2, 3, 2), (3, 2, 2), (2, 2, 3), (3, 3, 3), (2, 5, 3)):
        mn, mx = be.extrema_lemire(A, list(w))
        assert np.array_equal(mx, groundtruth(max, A, w))
        assert np.array_equal(mn, groundtruth(min, A, w))


def check_median_golden(be):
    """test/mapwindow.jl:105-124: median goldens (default border replicate)."""
    n = 0
    for k in GOLDEN["median"]:
        A = F(k["A"])
        got = be.median(A, k["window_first"], k["window_len"], "replicate")
        assert np.array_equal(got, np.array(k["expected"], dtype=np.float64)), k["source"]
        n += 1
    assert n == 6


# ------------------------------------------------------------------- NA() and Inner()
def check_na_vectors(be):
    """test/border.jl:272-284 (the NA testset), literal expectations."""
    # imfilter(1:10, centered([1,1,1].//3), NA()) == [3//2; 2:9; 19//2]
    got = be.na_dense(F(np.arange(1, 11)), np.full(3, 1 / 3), (-1,))
    exp = np.concatenate([[1.5], np.arange(2, 10), [9.5]])
    np.testing.assert_allclose(got, exp, rtol=1e-12)
    x = F([1, np.nan, np.inf, 0, -np.inf, np.inf, np.nan, np.nan, 1])
    k, kf = np.array([1.0, 1.0]), (0,)                # OffsetArray([1,1], 0:1)
    assert np.array_equal(be.na_dense(x, k, kf), [1, np.inf, np.inf, -np.inf, np.nan, np.inf, np.nan, 1, 1],
                          equal_nan=True)
    assert np.array_equal(be.na_dense(x, k, kf, "notfinite"), [1, np.nan, 0, 0, np.nan, np.nan, np.nan, 1, 1],
                          equal_nan=True)
    assert np.array_equal(be.na_dense(x, k, kf, "none"),
                          [np.nan, np.nan, np.inf, -np.inf, np.nan, np.nan, np.nan, np.nan, 1], equal_nan=True)
    # imfilter(1:5, centered([1]), NA()) == 1:5
    np.testing.assert_array_equal(be.na_dense(F(np.arange(1, 6)), np.array([1.0]), (0,)), np.arange(1, 6))


def target1_na(kern):
    """test/2d.jl:174-181: the NA target of the impulse at [1,2]."""
    ret = np.zeros((5, 7))
    ret[0, 0] = kern[1, 0] / (kern[1, 0] + kern[1, 1])
    ret[1, 0] = kern[0, 0] / kern.sum()
    ret[:, -1] = np.nan
    return ret


def check_na_impulse(be):
    """test/2d.jl:192-200 and 216-224: NA() on the edge impulse, dense and
    factored kernels; NaN outputs (kernel entirely in the padding) compared as
    zeros, as zerona! does."""
    img = np.zeros((5, 7))
    img[0, 1] = 1
    img = F(img)
    kf = np.outer(FACTORS[0][2], FACTORS[1][2])
    zero = lambda a: np.where(np.isnan(a), 0.0, a)
    t = target1_na(KERN)
    got = be.na_dense(img, KERN, KFIRST)
    np.testing.assert_allclose(zero(got), zero(t), atol=1e-12)
    assert np.array_equal(np.isnan(got), np.isnan(t))
    t = target1_na(kf)
    got = be.na_cascade(img, FACTORS)
    np.testing.assert_allclose(zero(got), zero(t), atol=1e-12)
    assert np.array_equal(np.isnan(got), np.isnan(t))


def check_inner_impulse(be):
    """test/2d.jl:78-80 and 106-108: Inner() keeps targetimg[2:end, 1:end-2]
    with axes (2:5, 1:5)."""
    img = np.zeros((5, 7))
    img[2, 3] = 1
    img = F(img)
    target = np.zeros((5, 7))
    target[2:4, 1:3] = rot180(KERN)
    got, first = be.inner_dense(img, KERN, KFIRST)
    assert tuple(first) == (2, 1) and got.shape == (4, 5)
    np.testing.assert_allclose(got, target[1:, :-2], atol=1e-12)
    kf = np.outer(FACTORS[0][2], FACTORS[1][2])
    target = np.zeros((5, 7))
    target[2:4, 1:3] = rot180(kf)
    got, first = be.inner_cascade(img, FACTORS)
    assert tuple(first) == (2, 1) and got.shape == (4, 5)
    np.testing.assert_allclose(got, target[1:, :-2], atol=1e-12)


# ------------------------------------------------------------------- blob_LoG and local extrema
def check_localextrema(be):
    """test/extrema.jl:2-12."""
    A = np.zeros((9, 9))
    A[[0, 1, 4], 4] = 1
    assert be.localextrema(A) == [(5, 5)]
    assert be.localextrema(A, window=(1, 3)) == [(1, 5), (2, 5), (5, 5)]
    assert be.localextrema(A, window=(1, 3), edges=False) == [(2, 5), (5, 5)]
    A = np.zeros((9, 9, 9))
    A[[0, 1, 4], 4, 4] = 1
    assert be.localextrema(A) == [(5, 5, 5)]
    assert be.localextrema(A, window=(1, 3, 1)) == [(1, 5, 5), (2, 5, 5), (5, 5, 5)]
    assert be.localextrema(A, window=(1, 3, 1), edges=False) == [(2, 5, 5), (5, 5, 5)]
    A = np.zeros((9, 9))
    A[[0, 1, 4], 4] = -1
    assert be.localextrema(A, minima=True) == [(5, 5)]


def check_blob_log(be):
    """test/extrema.jl:14-63 (blob_LoG) and the docstring example of blob_LoG
    (src/extrema.jl:44-52)."""
    A = np.zeros((9, 9))
    A[4, 4] = 1
    blobs = be.blob_log(A, 2.0 ** np.array([0.5, 0, 1]))
    assert len(blobs) == 1
    loc, sig, amp = blobs[0]
    assert abs(amp - 0.3183098861837907) < 1e-12
    assert tuple(sig) == (1.0, 1.0) and tuple(loc) == (5, 5)
    assert [tuple(b[0]) for b in be.blob_log(A, [1.0])] == [(5, 5)]
    assert [tuple(b[0]) for b in be.blob_log(A, [1.0], edges=(True, False, False))] == [(5, 5)]
    assert be.blob_log(A, [1.0], edges=False) == []
    A = np.zeros((9, 9))
    A[0, 4] = 1
    assert all(b[2] < 1e-16 for b in be.blob_log(A, 2.0 ** np.array([0.5, 0, 1])))
    blobs = [b for b in be.blob_log(A, 2.0 ** np.array([0.5, 0, 1]), edges=True) if b[2] > 0.1]
    assert len(blobs) == 1 and tuple(blobs[0][0]) == (1, 5)
    assert [tuple(b[0]) for b in be.blob_log(A, 2.0 ** np.array([0.5, 0, 1]), edges=(True, True, False))
            if b[2] > 0.1] == [(1, 5)]
    assert be.blob_log(A, 2.0 ** np.array([0, 1]), edges=(False, True, False)) == []
    assert all(b[2] < 1e-16 for b in be.blob_log(A, 2.0 ** np.array([0, 0.5, 1]), edges=(True, False, True)))
    A = np.zeros((9, 9, 9))
    A[4, 4, 4] = 1
    blobs = be.blob_log(A, 2.0 ** np.array([0.5, 0, 1]))
    assert len(blobs) == 1 and tuple(blobs[0][0]) == (5, 5, 5)
    A = np.zeros((9, 9, 9))
    A[4, 3:6, 4] = 1
    blobs = be.blob_log(A, 2.0 ** np.array([1.0, 0, 0.5]), sigma_shape=(1.0, 3.0, 1.0))
    assert len(blobs) == 1 and tuple(blobs[0][0]) == (5, 5, 5)
    A = np.zeros((9, 9, 9))
    A[0, 0, 3:6] = 1
    blobs = [b for b in be.blob_log(A, 2.0 ** np.array([0.5, 0, 1]), edges=True, sigma_shape=(1.0, 1.0, 3.0))
             if b[2] > 0.1]
    assert len(blobs) == 1 and tuple(blobs[0][0]) == (1, 1, 5)
    assert be.blob_log(A, 2.0 ** np.array([0, 1]), edges=(False, True, False, False),
                       sigma_shape=(1.0, 1.0, 3.0)) == []
    x = np.zeros(12)
    x[10] = 1.0
    assert len(be.blob_log(x, [4.0], edges=True, rthresh=0)) > len(be.blob_log(x, [4.0], edges=True))
    # docstring example
    x = np.zeros(100)
    x[19:30] = np.exp(-np.arange(-5, 6) ** 2 / (2 * 4.0 ** 2))
    x[49:80] = np.exp(-np.arange(-15, 16) ** 2 / (2 * 8.0 ** 2))
    blobs = be.blob_log(x, 2.0 ** np.arange(1, 7), edges=False)
    assert [(tuple(b[0]), tuple(b[1])) for b in blobs] == [((25,), (4.0,)), ((65,), (8.0,))]
    assert abs(blobs[0][2] - 0.10453155018303673) < 1e-12 and abs(blobs[1][2] - 0.046175719034527364) < 1e-12


# ------------------------------------------------------------------- Algorithm.FFT()
def check_fft_impulses(be):
    """test/2d.jl:49-79, 82-100, 104-140, 171-195 with Algorithm.FFT(): the
    impulse targets (interior and at the edge) for the dense kernel, the
    factored kernel and the rational 3x3 box, every border."""
    img = np.zeros((5, 7))
    img[2, 3] = 1
    img = F(img)
    target = np.zeros((5, 7))
    target[2:4, 1:3] = rot180(KERN)
    kf = np.outer(FACTORS[0][2], FACTORS[1][2])
    targetf = np.zeros((5, 7))
    targetf[2:4, 1:3] = rot180(kf)
    box = [(0, -1, np.full(3, 1 / 3)), (1, -1, np.full(3, 1 / 3))]
    targetb = np.zeros((5, 7))
    targetb[1:4, 2:5] = 1 / 9
    edge = np.zeros((5, 7))
    edge[0, 1] = 1
    edge = F(edge)
    for style in BORDERS:
        np.testing.assert_allclose(be.fft(img, KERN, KFIRST, style), target, atol=1e-12, err_msg=style)
        np.testing.assert_allclose(be.fft_cascade(img, FACTORS, style), targetf, atol=1e-12, err_msg=style)
        np.testing.assert_allclose(be.fft_cascade(img, box, style), targetb, atol=1e-12, err_msg=style)
        np.testing.assert_allclose(be.fft(edge, KERN, KFIRST, style), target1(style, KERN), atol=1e-12,
                                   err_msg=style)
        np.testing.assert_allclose(be.fft_cascade(edge, FACTORS, style), target1(style, kf), atol=1e-12,
                                   err_msg=style)


def check_fft_3d_box(be):
    """test/nd.jl:128-157 with Algorithm.FFT(): the 3-D box on ones, every
    Pad style gives ones, Fill(0) gives (2/3)^k at faces, edges and corners."""
    img = F(np.ones((10, 10, 10)))
    K = np.full((3, 3, 3), 1 / 27)
    for style in ["replicate", "circular", "symmetric", "reflect"]:
        np.testing.assert_allclose(be.fft(img, K, (-1, -1, -1), style), img, rtol=1e-12)
    t = np.ones((10, 10, 10))
    for i in (0, 9):
        t[:, :, i] = t[:, i, :] = t[i, :, :] = 2 / 3
    for i in (0, 9):
        for j in (0, 9):
            t[:, i, j] = t[i, :, j] = t[i, j, :] = (2 / 3) ** 2
    for i in (0, 9):
        for j in (0, 9):
            for k in (0, 9):
                t[i, j, k] = (2 / 3) ** 3
    np.testing.assert_allclose(be.fft(img, K, (-1, -1, -1), "fill"), t, rtol=1e-12)


def check_fft_nopad(be):
    """test/nd.jl:77-81: FFT without padding on 1:8 with zero ends equals the
    replicate FIR result of the 3-tap kernel."""
    img = np.arange(1, 9, dtype=np.float64)
    img[0] = img[7] = 0
    img = F(img)
    exp = be.cascade(img, [K1], "replicate")
    np.testing.assert_allclose(be.fft_nopad(img, K1[2], (K1[1],)), exp, rtol=1e-12, atol=1e-14)


def check_fft_equals_fir(be, O, tol=1e-12):
    """Algorithm.FFT() agrees with the direct filter (the reference's tests
    compare every algorithm to the same target): random off-centre kernels in
    1-3 dimensions, kernels longer than the image, every border."""
    rng = np.random.default_rng(17)
    for shape, ks, first in [((40,), (9,), (-4,)), ((37, 29), (9, 4), (-4, 1)), ((12, 11, 9), (3, 5, 2), (-1, -2, 0)),
                             ((7, 6), (11, 9), (-5, -4)), ((33, 30), (31, 31), (-15, -15))]:
        a = F(rng.random(shape))
        K = rng.standard_normal(ks)
        for style in BORDERS:
            ref = O.imfilter_dense(a, K, first, style, 0.3)
            got = be.fft(a, K, first, style, 0.3)
            d = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
            assert d <= tol, (shape, ks, style, d)


# ------------------------------------------------------------------- IIR (Triggs-Sdika)
def check_iir_1d(be):
    """test/triggs.jl:6-33: impulses at the ends and inside a 1000-vector,
    IIRGaussian(σ) with Fill(0) stays within 10% (normwise) of the sampled
    Gaussian; a 2-vector is a DimensionMismatch."""
    l = 1000
    xs = [1, 2, 3, 5, 10, 20, l >> 1, l - 19, l - 9, l - 4, l - 2, l - 1, l]
    for sigma in [3.1, 5, 10.0, 20, 50.0, 100.0]:
        for c in xs:
            a = np.zeros(l)
            a[c - 1] = 1
            af = np.exp(-((np.arange(1, l + 1)) - c) ** 2 / (2 * sigma ** 2)) / (sigma * np.sqrt(2 * np.pi))
            got = be.iir(F(a), [(0, sigma)], "fill", 0.0)
            assert np.linalg.norm(got - af) < 0.1 * np.linalg.norm(af), (sigma, c)
    try:
        be.iir(F([1.0, 2.0]), [(0, 2.0)], "replicate")
    except Exception as e:                         # DimensionMismatch on both backends
        assert "DimensionMismatch" in type(e).__name__ + str(e)
    else:
        raise AssertionError("a 2-vector must be a DimensionMismatch")


def check_iir_images(be):
    """test/triggs.jl:45-82: the impulse of a 5x7 image filtered with
    IIRGaussian((5,5)) and Fill(0) is within 20% (L2) of the sampled 2-D
    Gaussian; (σ,0) and (0,σ) change the image; one pass along dimension 2
    equals the (0,σ) cascade; with a NaN and NA() the result is the Fill(0)
    filter of the zeroed image over the filter of the valid mask."""
    sigma = 5
    img = np.zeros((5, 7))
    img[2, 3] = 1
    img = F(img)
    x = np.arange(-2, 3).reshape(-1, 1)
    y = np.arange(-3, 4).reshape(1, -1)
    cmp = np.exp(-(x ** 2 + y ** 2) / (2 * sigma ** 2)) / (sigma ** 2 * 2 * np.pi)
    got = be.iir(img, [(0, sigma), (1, sigma)], "fill", 0.0)
    assert np.sum((cmp - got) ** 2) < 0.2 ** 2 * np.sum(cmp ** 2)
    r1 = be.iir(img, [(0, sigma), (1, 0)], "replicate")
    r2 = be.iir(img, [(0, 0), (1, sigma)], "replicate")
    assert not np.array_equal(r1, img) and not np.array_equal(r2, img)
    np.testing.assert_array_equal(be.iir_dim(img, sigma, 2, "replicate"), r2)
    nan = img.copy()
    num = img.copy()
    nan[0, 0] = np.nan
    num[0, 0] = 0
    den = np.ones(img.shape)
    den[0, 0] = 0
    rnum = be.iir(F(num), [(0, sigma), (1, sigma)], "fill", 0.0)
    rden = be.iir(F(den), [(0, sigma), (1, sigma)], "fill", 0.0)
    ret = be.iir_na(F(nan), [(0, sigma), (1, sigma)])
    ret[0, 0] = rnum[0, 0] = 0
    np.testing.assert_allclose(ret, rnum / rden, rtol=1e-10, atol=1e-14)


def check_iir_na_ramp(be):
    """test/triggs.jl:84-96: NA() on the 100x100 ramp 1:10000 (no NA element:
    the separable normalisation) -- finite and close to the ramp itself away
    from the edges (a Gaussian of a linear ramp is the ramp)."""
    A = F(np.arange(1, 100 * 100 + 1, dtype=np.float64).reshape(100, 100, order="F"))
    B = be.iir_na(A, [(0, 5.0), (1, 5.0)])
    assert np.all(np.isfinite(B))
    np.testing.assert_allclose(B[30:70, 30:70], A[30:70, 30:70], rtol=1e-3)


def check_mixed(be):
    """test/triggs.jl:35-43: IIR and FIR factors commute on 1:8 (Pad(:replicate)
    and Fill(0)); test/specialty.jl:217-231: (IIRGaussian(σs)..., Laplacian())
    correlates with the dense LoG (> 0.8) and the (Laplacian(), IIRGaussian...)
    order trims its edges without reading unset values (no NaN)."""
    img = F(np.arange(1, 9))
    for style in ("replicate", "fill"):
        a = be.mixed(img, [("iir", 0, 2.0), ("fir", np.ones(3) / 3, (-1,))], style, 0.0)
        b = be.mixed(img, [("fir", np.ones(3) / 3, (-1,)), ("iir", 0, 2.0)], style, 0.0)
        np.testing.assert_allclose(a, b, rtol=1e-10)
    rng = np.random.default_rng(217)
    im = F(rng.random((20, 21)))
    K, first = LOG_2_5_3_2
    f1 = be.dense(im, K, first, "replicate")
    f2 = be.mixed(im, [("iir", 0, 2.5), ("iir", 1, 3.2), ("lap",)], "replicate")
    assert np.corrcoef(f1.ravel(), f2.ravel())[0, 1] > 0.8
    f3 = be.mixed(im, [("lap",), ("iir", 0, 2.5), ("iir", 1, 3.2)], "replicate")
    assert not np.any(np.isnan(f3))


def _log_kernel(sigmas):
    """Kernel.LoG(σs) (src/kernel.jl:325-339), dense FP64, with its first indices."""
    import math
    N = len(sigmas)
    ws = [int(math.ceil(8.5 * s)) >> 1 for s in sigmas]
    s2 = np.array([float(s) ** 2 for s in sigmas])
    Cn = 1.0 / (float(np.prod(sigmas)) * (2 * math.pi) ** (N / 2))
    grids = np.meshgrid(*[np.arange(-w, w + 1, dtype=np.float64) for w in ws], indexing="ij")
    xs = sum(g * g / s for g, s in zip(grids, s2))
    xs4 = sum(g * g / (s * s) for g, s in zip(grids, s2))
    return np.asfortranarray(Cn * (xs4 - float(np.sum(1.0 / s2))) * np.exp(-xs / 2)), tuple(-w for w in ws)


LOG_2_5_3_2 = _log_kernel((2.5, 3.2))
