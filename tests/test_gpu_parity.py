"""GB300 kernels against the CPU oracle on seeded random inputs.

Tolerances (stated by the FIR path's contract): linear filters within 1e-5
normwise relative error (max|gpu - oracle| / max|oracle|) when the image is
not Float64 (FP32 arithmetic on the GPU against the FP64 oracle), 1e-12 for
Float64 images (FP64 on the GPU); border maps, Laplacian, median and extrema
bit-exact.
"""
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STYLES = ["replicate", "circular", "symmetric", "reflect", "fill"]
RTOL = {"F32": 1e-5, "F64": 1e-12, "N0F8": 1e-5, "U8": 1e-5}


def normwise(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = np.max(np.abs(a - b)) if a.size else 0.0
    m = np.max(np.abs(b)) if b.size else 0.0
    return d / m if m > 0 else d


def make_img(rng, shape, kind):
    if kind == "F32":
        return np.asfortranarray(rng.random(shape, dtype=np.float32))
    if kind == "F64":
        return np.asfortranarray(rng.random(shape))
    codes = np.asfortranarray(rng.integers(0, 256, shape, dtype=np.uint8))
    return codes


def values(ifx, img, kind):
    """The numeric values the reference sees (N0f8: c/255)."""
    if kind == "N0F8":
        return img.astype(np.float64) / 255.0
    return img.astype(np.float64)


def wrap(ifx, img, kind):
    return ifx.n0f8(img) if kind == "N0F8" else img


def border_of(ifx, style, fill=0.7):
    return ifx.Fill(fill) if style == "fill" else ifx.Pad(style)


def fill_value(kind, fill=0.7):
    if kind == "U8":
        return 0.0
    if kind == "N0F8":
        return round(fill * 255) / 255.0
    if kind == "F32":
        return float(np.float32(fill))
    return fill


# --------------------------------------------------------------------- separable
@pytest.mark.parametrize("kind", ["F32", "F64", "N0F8", "U8"])
@pytest.mark.parametrize("style", STYLES)
def test_separable_2d_random(gpu_ifx, oracle, kind, style):
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32((kind + style).encode()))
    for shape in [(67, 45), (130, 7), (3, 200), (64, 64), (203, 301)]:   # 203: rows off the copy rules
        img = make_img(rng, shape, kind)
        for _ in range(3):
            lx, ly = int(rng.integers(1, 34)), int(rng.integers(1, 34))
            fx, fy = int(rng.integers(-lx, 2)), int(rng.integers(-ly, 2))
            wx, wy = rng.standard_normal(lx), rng.standard_normal(ly)
            order = [(0, fx, wx), (1, fy, wy)] if rng.random() < 0.5 else [(1, fy, wy), (0, fx, wx)]
            ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w, (f,)), 2, ax) for ax, f, w in order)
            fill = 0.7 if kind != "U8" else 3.0
            b = ifx.Fill(fill) if style == "fill" else ifx.Pad(style)
            got = ifx.imfilter(wrap(ifx, img, kind), ks, b)
            fv = fill_value(kind, fill) if kind != "U8" else 3.0
            ref = oracle.imfilter_cascade(values(ifx, img, kind), order, style, fv)
            assert got.dtype == np.float64
            assert normwise(got, ref) <= RTOL[kind], (shape, order, style)


@pytest.mark.parametrize("kind", ["F32", "N0F8", "U8"])
@pytest.mark.parametrize("style", STYLES)
def test_separable_2d_tma_tiles(gpu_ifx, oracle, kind, style):
    """Images whose rows meet the bulk-copy rules (width a multiple of 16), so
    that the persistent kernel copies every tile by TMA and gives the window
    cells outside the image their border values in shared memory (from the
    tile, or from the image where the window does not hold the source):
    random factor lengths/offsets, both factor orders (the FP32 kernels run
    the x pass first either way; the y-first pass order is pinned in
    test_gpu_tune.py), Float32 and Float64 outputs, images smaller than one
    tile, several tiles per CTA on the largest image."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("tma" + kind + style).encode()))
    for shape in [(32, 7), (48, 70), (256, 200), (1040, 333), (4096, 1100)]:
        img = make_img(rng, shape, kind)
        for _ in range(2 if shape[0] < 4096 else 1):
            lx, ly = int(rng.integers(1, 34)), int(rng.integers(1, 34))
            fx, fy = int(rng.integers(-lx, 2)), int(rng.integers(-ly, 2))
            wx, wy = rng.standard_normal(lx), rng.standard_normal(ly)
            order = [(0, fx, wx), (1, fy, wy)] if rng.random() < 0.5 else [(1, fy, wy), (0, fx, wx)]
            f32w = rng.random() < 0.5          # Float32 weights keep a Float32 output
            ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w.astype(np.float32) if f32w else w, (f,)), 2, ax)
                       for ax, f, w in order)
            fill = 0.7 if kind != "U8" else 3.0
            b = ifx.Fill(fill) if style == "fill" else ifx.Pad(style)
            got = ifx.imfilter(wrap(ifx, img, kind), ks, b)
            fv = fill_value(kind, fill) if kind != "U8" else 3.0
            ref_order = [(ax, f, w.astype(np.float32).astype(np.float64) if f32w else w) for ax, f, w in order]
            ref = oracle.imfilter_cascade(values(ifx, img, kind), ref_order, style, fv)
            assert got.dtype == (np.float32 if f32w else np.float64), got.dtype
            assert normwise(got, ref) <= RTOL[kind], (shape, order, style)


@pytest.mark.parametrize("kind", ["F32", "N0F8"])
def test_separable_2d_tma_tile_heights(gpu_ifx, oracle, kind):
    """Long factors lower the TMA kernel's tile height below 64 rows (to 56,
    48, 40: not all multiples of 16); both factor orders, every tile row of the
    image, including a partial last one."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("tma-heights" + kind).encode()))
    img = make_img(rng, (320, 203), kind)
    for taps in (17, 25, 33, 36):
        wx, wy = rng.standard_normal(taps), rng.standard_normal(taps)
        fx, fy = -(taps // 2), -(taps // 2) + 1
        for x_first in (True, False):
            order = [(0, fx, wx), (1, fy, wy)] if x_first else [(1, fy, wy), (0, fx, wx)]
            ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w, (f,)), 2, ax) for ax, f, w in order)
            got = ifx.imfilter(wrap(ifx, img, kind), ks, ifx.Pad("symmetric"))
            ref = oracle.imfilter_cascade(values(ifx, img, kind), order, "symmetric", 0.0)
            assert normwise(got, ref) <= RTOL[kind], (taps, x_first)


def test_float64_widening_exact(gpu_ifx):
    """Float64 outputs of FP32 arithmetic are widened exactly: zeros,
    subnormals, the extremes of the normal range, Inf and NaN."""
    ifx = gpu_ifx
    rng = np.random.default_rng(3)
    special = np.array([0.0, 1e-40, -1e-40, 1.17549435e-38, -1.17549435e-38, 3.4028235e38 / 2,
                        -3.4028235e38 / 2, 3.4028235e38, np.inf, -np.inf, np.nan, 1.0, -2.5,
                        1.4e-45, 123456.789], dtype=np.float32)
    img = rng.standard_normal((256, 64)).astype(np.float32) * np.float32(1e3)
    img.flat[: special.size * 37: 37] = special
    img = np.asfortranarray(img)
    k = (ifx.ReshapedOneD(ifx.OffsetKernel(np.array([2.0]), (0,)), 2, 0),)
    for shape_img in (img, np.asfortranarray(img[:, :63])):   # TMA path and plain path
        got = ifx.imfilter(shape_img, k, "replicate")
        exp = (shape_img * np.float32(2)).astype(np.float64)
        assert got.dtype == np.float64
        assert np.array_equal(got.view(np.uint64)[~np.isnan(exp)], exp.view(np.uint64)[~np.isnan(exp)])
        assert np.array_equal(np.isnan(got), np.isnan(exp))


@pytest.mark.parametrize("taps", [9, 17])
def test_config_512_gaussian_replicate(gpu_ifx, oracle, taps):
    """512x512 Float32 uniform[0,1) seed 1, KernelFactors.gaussian((2,2)) (9 taps)
    and gaussian((2,2),(17,17)), Pad(:replicate): Float64 output."""
    ifx = gpu_ifx
    img = np.asfortranarray(np.random.default_rng(1).random((512, 512), dtype=np.float32))
    k = ifx.KernelFactors.gaussian((2, 2), None if taps == 9 else (17, 17))
    got = ifx.imfilter(img, k, "replicate", ifx.Algorithm.GB300())
    facs = [(f.axis, f.data.first[0], np.asarray(f.data.data)) for f in k]
    ref = oracle.imfilter_cascade(img.astype(np.float64), facs, "replicate")
    assert got.dtype == np.float64
    assert normwise(got, ref) <= 1e-5


@pytest.mark.parametrize("style", STYLES)
def test_separable_nd_generic(gpu_ifx, oracle, style):
    """1-D, 3-D, 4-D and repeated-axis cascades (the generic box pipeline)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(99)
    cases = [((50,), [(0, -3, rng.standard_normal(7))]),
             ((12, 9, 10), [(0, -2, rng.standard_normal(5)), (1, -1, rng.standard_normal(3)),
                            (2, -4, rng.standard_normal(9))]),
             ((6, 5, 4, 7), [(3, -1, rng.standard_normal(3)), (0, 0, rng.standard_normal(2)),
                             (2, -1, rng.standard_normal(3))]),
             ((20, 17), [(0, -1, np.ones(3)), (1, -1, np.ones(3)), (0, -1, np.ones(3)),
                         (1, 0, rng.standard_normal(4))])]
    for shape, facs in cases:
        for kind in ("F32", "F64"):
            img = make_img(rng, shape, kind)
            ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w, (f,)), len(shape), ax) for ax, f, w in facs)
            got = ifx.imfilter(img, ks, border_of(ifx, style))
            ref = oracle.imfilter_cascade(img.astype(np.float64), facs, style,
                                          fill_value(kind))
            assert normwise(got, ref) <= RTOL[kind], (shape, style, kind)


def test_separable_3d_volume(gpu_ifx, oracle):
    """σ=(3,3,1.5) Gaussian (13/13/9 taps), Pad(:symmetric), on a 64^3 volume with
    1% impulse outliers (the 256^3 workload's shape of input, smaller)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(3)
    vol = rng.random((64, 64, 64), dtype=np.float32)
    m = rng.random(vol.shape) < 0.01
    vol[m] = 1.0
    vol = np.asfortranarray(vol)
    k = ifx.KernelFactors.gaussian((3, 3, 1.5))
    assert [len(f.data) for f in k] == [13, 13, 9]
    got = ifx.imfilter(vol, k, "symmetric")
    facs = [(f.axis, f.data.first[0], np.asarray(f.data.data)) for f in k]
    ref = oracle.imfilter_cascade(vol.astype(np.float64), facs, "symmetric")
    assert normwise(got, ref) <= 1e-5


@pytest.mark.parametrize("kind", ["F32", "N0F8", "U8"])
@pytest.mark.parametrize("style", STYLES)
def test_separable_3d_split(gpu_ifx, oracle, kind, style):
    """3-D cascades with one factor per axis take the z sweep into a padded
    FP32 volume (its halo cells the z filter of the columns the border maps
    them to; Fill: of fill values) and the x/y TMA sweep over its planes,
    for any width (37 included: the padded rows meet the bulk-copy rules).
    Random lengths and offsets (positive ones too), Float64 and Float32
    outputs."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("3dsplit" + kind + style).encode()))
    for shape in [(16, 9, 13), (64, 33, 40), (37, 20, 11)]:
        img = make_img(rng, shape, kind)
        lens = [int(rng.integers(1, 20)) for _ in range(3)]
        facs = [(ax, int(rng.integers(-lens[ax], 2)), rng.standard_normal(lens[ax])) for ax in range(3)]
        f32w = rng.random() < 0.5
        ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w.astype(np.float32) if f32w else w, (f,)), 3, ax)
                   for ax, f, w in facs)
        fill = 0.7 if kind != "U8" else 3.0
        b = ifx.Fill(fill) if style == "fill" else ifx.Pad(style)
        got = ifx.imfilter(wrap(ifx, img, kind), ks, b)
        fv = fill_value(kind, fill) if kind != "U8" else 3.0
        ref_facs = [(ax, f, w.astype(np.float32).astype(np.float64) if f32w else w) for ax, f, w in facs]
        ref = oracle.imfilter_cascade(values(ifx, img, kind), ref_facs, style, fv)
        assert got.dtype == (np.float32 if f32w else np.float64)
        assert normwise(got, ref) <= RTOL[kind], (shape, style, lens)


# --------------------------------------------------------------------- dense
@pytest.mark.parametrize("ksz,seed", [(5, 20), (15, 21), (31, 22)])
@pytest.mark.parametrize("style", ["reflect", "fill", "replicate", "circular", "symmetric"])
def test_dense_2d(gpu_ifx, oracle, ksz, seed, style):
    """N(0,1) kernels normalised to sum 1 (seeds 20-22, |sum| >= 0.1)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(seed)
    while True:
        K = rng.standard_normal((ksz, ksz))
        if abs(K.sum()) >= 0.1:
            break
    K = K / K.sum()
    img = np.asfortranarray(np.random.default_rng(2).random((301, 257), dtype=np.float32))
    kern = ifx.centered(K)
    fk = ifx.factorkernel(kern)
    assert len(fk) == 2 and ifx.iscopy(fk[0])       # full rank: stays dense
    b = ifx.Fill(0) if style == "fill" else ifx.Pad(style)
    got = ifx.imfilter(img, kern, b)
    ref = oracle.imfilter_dense(img.astype(np.float64), K, kern.first, style, 0.0)
    assert got.dtype == np.float64
    assert normwise(got, ref) <= 1e-5
    got64 = ifx.imfilter(img.astype(np.float64), kern, b)
    assert normwise(got64, ref) <= 1e-12


def test_dense_nd_and_offcenter(gpu_ifx, oracle):
    ifx = gpu_ifx
    rng = np.random.default_rng(4)
    img = np.asfortranarray(rng.random((17, 13, 11)))
    K = rng.standard_normal((3, 4, 2))
    for style in STYLES:
        got = ifx.imfilter(img, (ifx.OffsetKernel(K, (-1, 0, -2)),), border_of(ifx, style))
        ref = oracle.imfilter_dense(img, K, (-1, 0, -2), style, 0.7)
        assert normwise(got, ref) <= 1e-12, style
    img2 = np.asfortranarray(rng.random((40, 33), dtype=np.float32))
    K2 = rng.standard_normal((4, 6))
    got = ifx.imfilter(img2, (ifx.OffsetKernel(K2, (1, -7)),), "circular")
    ref = oracle.imfilter_dense(img2.astype(np.float64), K2, (1, -7), "circular")
    assert normwise(got, ref) <= 1e-5


# --------------------------------------------------------------------- Laplacian
@pytest.mark.parametrize("kind,arith", [("F32", "f32"), ("F64", "f64"), ("N0F8", "f32"),
                                        ("U8", "int")])
@pytest.mark.parametrize("style", STYLES)
def test_laplacian_exact(gpu_ifx, oracle, kind, arith, style):
    ifx = gpu_ifx
    rng = np.random.default_rng(8)
    for shape, flags in [((37, 29), (True, True)), ((37, 29), (False, True)), ((9, 8, 7), (True, True, True)),
                         ((40,), (True,))]:
        img = make_img(rng, shape, kind)
        fill = 0.0 if kind in ("U8",) else 0.5
        b = ifx.Fill(fill) if style == "fill" else ifx.Pad(style)
        got = ifx.imfilter(wrap(ifx, img, kind), ifx.Kernel.Laplacian(flags), b)
        if kind == "N0F8":
            vals = (img.astype(np.float32) / np.float32(255)).astype(np.float64)
            fv = float(np.float32(round(fill * 255) / np.float32(255)))
        else:
            vals = img.astype(np.float64)
            fv = fill if kind != "F32" else float(np.float32(fill))
        ref = oracle.laplacian(vals, [int(f) for f in flags], style, fv, arith)
        assert got.dtype == {"F32": np.float32, "F64": np.float64, "N0F8": np.float32,
                             "U8": np.int16}[kind]
        assert np.array_equal(np.asarray(got, np.float64), ref), (shape, flags, style)


# --------------------------------------------------------------------- gradients
@pytest.mark.parametrize("name", ["sobel", "prewitt", "scharr", "bickley", "ando3"])
@pytest.mark.parametrize("style", STYLES)
def test_imgradients(gpu_ifx, oracle, name, style):
    ifx = gpu_ifx
    rng = np.random.default_rng(12)
    fn = getattr(ifx.KernelFactors, name)
    k1, k2 = fn.gradient_pair
    for shape in [(33, 28), (16, 12, 10), (25, 1, 9)]:
        img = np.asfortranarray(rng.random(shape, dtype=np.float32))
        if style == "reflect" and 1 in shape:
            with pytest.raises(ifx.ErrorException):
                ifx.imgradients(img, fn, ifx.Pad(style))
            continue
        gs = ifx.imgradients(img, fn, border_of(ifx, style))
        assert len(gs) == len(shape)
        for d, g in enumerate(gs):
            facs = []
            for e in range(len(shape)):
                if shape[e] > 1:
                    facs.append((e, -1, k1 if e == d else k2))
            ref = oracle.imfilter_cascade(img.astype(np.float64), facs, style,
                                          float(np.float32(0.7)))
            assert g.dtype == np.float64
            assert normwise(g, ref) <= 1e-5 or np.max(np.abs(g - ref)) < 1e-6, (shape, d)


@pytest.mark.parametrize("kind", ["F64", "F32", "N0F8"])
@pytest.mark.parametrize("style", STYLES)
def test_imgradients_3d_fused(gpu_ifx, oracle, kind, style):
    """3-D volumes with a 3-tap pair on every axis take the fused sweep (all
    three gradients at once, z-marching, several z chunks): each gradient equals
    its own pad-then-cascade (FP64 for Float64 volumes)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("g3" + kind + style).encode()))
    for shape, name in [((37, 21, 70), "sobel"), ((64, 17, 9), "scharr")]:
        img = make_img(rng, shape, kind)
        fn = getattr(ifx.KernelFactors, name)
        k1, k2 = fn.gradient_pair
        gs = ifx.imgradients(wrap(ifx, img, kind), fn, border_of(ifx, style, 0.3))
        assert len(gs) == 3
        for d, g in enumerate(gs):
            facs = [(e, -1, k1 if e == d else k2) for e in range(3)]
            ref = oracle.imfilter_cascade(values(ifx, img, kind), facs, style, fill_value(kind, 0.3))
            assert g.dtype == np.float64
            tol = 1e-12 if kind == "F64" else 1e-5
            assert normwise(g, ref) <= tol or np.max(np.abs(g - ref)) < tol / 10, (shape, d, style)


def test_imgradients_ando4_dense_kernels(gpu_ifx, oracle):
    ifx = gpu_ifx
    img = np.asfortranarray(np.random.default_rng(5).random((30, 31)))
    gy, gx = ifx.imgradients(img, ifx.KernelFactors.ando4, "replicate")
    k1, k2 = ifx.KernelFactors.ando4.gradient_pair
    ref = oracle.imfilter_cascade(img, [(0, -1, k1), (1, -1, k2)], "replicate")
    assert normwise(gy, ref) <= 1e-12
    dy, dx = ifx.imgradients(img, ifx.Kernel.sobel, "reflect")
    s1, s2 = ifx.KernelFactors.sobel.gradient_pair
    ref = oracle.imfilter_cascade(img, [(0, -1, s2), (1, -1, s1)], "reflect")
    assert normwise(dx, ref) <= 1e-12


# --------------------------------------------------------------------- median
@pytest.mark.parametrize("kind", ["N0F8", "U8"])
@pytest.mark.parametrize("style", STYLES)
def test_median_u8_exact(gpu_ifx, oracle, kind, style):
    ifx = gpu_ifx
    rng = np.random.default_rng(21)
    for shape in [(130, 37), (9, 300), (5, 6)]:
        img = make_img(rng, shape, kind)
        salt = rng.random(shape) < 0.05
        img[salt] = np.where(rng.random(salt.sum()) < 0.5, 0, 255)
        for win in [(3, 3), (5, 5), (7, 7), (9, 9), (3, 5), (1, 7)]:
            fill = 0.2 if kind == "N0F8" else 51
            b = ifx.Fill(fill) if style == "fill" else ifx.Pad(style)
            if style == "reflect" and 1 in win:
                continue
            got = ifx.mapwindow(ifx.median, wrap(ifx, img, kind), win, border=b)
            code = round(fill * 255) if kind == "N0F8" else fill
            ref = oracle.mapwindow_median(img.astype(np.float64), [-(w // 2) for w in win],
                                          list(win), style, float(code))
            if kind == "N0F8":
                assert got.dtype == np.float32
                exp = (ref.astype(np.float32) / np.float32(255))
                assert np.array_equal(got, exp), (shape, win, style)
            else:
                assert got.dtype == np.float64
                assert np.array_equal(got, ref), (shape, win, style)


@pytest.mark.parametrize("kind", ["F32", "F64"])
def test_median_float_nd(gpu_ifx, oracle, kind):
    ifx = gpu_ifx
    rng = np.random.default_rng(22)
    for shape, win in [((31, 17), (3, 5)), ((9, 8, 7), (3, 3, 3)), ((50,), (7,)),
                       ((40, 23), (3, 3)), ((40, 23), (5, 5)), ((19, 33), (7, 7)), ((4, 6), (5, 5))]:
        img = make_img(rng, shape, kind)
        for style in STYLES:
            got = ifx.mapwindow(ifx.median, img, win, border=border_of(ifx, style, 0.25))
            ref = oracle.mapwindow_median(img.astype(np.float64), [-(w // 2) for w in win],
                                          list(win), style, fill_value(kind, 0.25))
            assert np.array_equal(np.asarray(got, np.float64), ref), (shape, style)


# --------------------------------------------------------------------- extrema
@pytest.mark.parametrize("kind", ["U8", "F32", "F64"])
def test_extrema_exact(gpu_ifx, oracle, kind):
    ifx = gpu_ifx
    rng = np.random.default_rng(31)
    for shape in [(70, 45), (11, 9, 13)]:
        img = make_img(rng, shape, kind)
        nd = len(shape)
        for w in ([7] * nd, [15] * nd, [4] * nd, [2, 5, 3][:nd]):
            mm = ifx.mapwindow(ifx.extrema, img, tuple(w))              # Lemire path
            mn, mx = oracle.extrema_trunc(img.astype(np.float64), w)
            assert np.array_equal(np.asarray(mm[0], np.float64), mn)
            assert np.array_equal(np.asarray(mm[1], np.float64), mx)
        for style in STYLES:
            w = [7] * nd
            fill = 77 if kind == "U8" else 0.5
            b = ifx.Fill(fill) if style == "fill" else ifx.Pad(style)
            mm = ifx.mapwindow(ifx.extrema, img, tuple(w), border=b)
            mn, mx = oracle.mapwindow_extrema(img.astype(np.float64), [-3] * nd, w, style,
                                              float(fill) if kind != "F32" else float(np.float32(fill)))
            assert np.array_equal(np.asarray(mm[0], np.float64), mn), style
            assert np.array_equal(np.asarray(mm[1], np.float64), mx), style
            lo = ifx.mapwindow(ifx.minimum, img, tuple(w), border=b)
            hi = ifx.mapwindow(ifx.maximum, img, tuple(w), border=b)
            assert np.array_equal(np.asarray(lo, np.float64), mn)
            assert np.array_equal(np.asarray(hi, np.float64), mx)


@pytest.mark.parametrize("w", [3, 5, 7, 9, 11, 13, 15, 17, 21, 25, 31, 33])
def test_extrema_2d_tile_kernel(gpu_ifx, oracle, w):
    """8-bit square windows take the one-launch 2-D tile kernel: against the
    oracle for images smaller than a window, odd widths and several tiles per
    axis, widths a multiple of 16 (interior tiles staged by 16-byte loads),
    every Pad style and Fill, and min, max or both."""
    ifx = gpu_ifx
    rng = np.random.default_rng(1000 + w)
    for shape in [(5, 3), (w + 2, 2 * w + 1), (301, 157), (512, 203)]:
        img = np.asfortranarray(rng.integers(0, 256, shape, dtype=np.uint8))
        mm = ifx.mapwindow(ifx.extrema, ifx.n0f8(img), (w, w))
        mn, mx = oracle.extrema_trunc(img.astype(np.float64), [w, w])
        assert np.array_equal(np.asarray(mm[0], np.float64), mn), shape       # N0f8 codes
        assert np.array_equal(np.asarray(mm[1], np.float64), mx), shape
        for style in STYLES:
            b = ifx.Fill(91) if style == "fill" else ifx.Pad(style)
            if style == "reflect" and min(shape) < 2:
                continue
            mn, mx = oracle.mapwindow_extrema(img.astype(np.float64), [-(w // 2)] * 2, [w, w], style, 91.0)
            mm = ifx.mapwindow(ifx.extrema, img, (w, w), border=b)
            assert np.array_equal(np.asarray(mm[0], np.float64), mn), (shape, style)
            assert np.array_equal(np.asarray(mm[1], np.float64), mx), (shape, style)
            lo = ifx.mapwindow(ifx.minimum, img, (w, w), border=b)
            hi = ifx.mapwindow(ifx.maximum, img, (w, w), border=b)
            assert np.array_equal(np.asarray(lo, np.float64), mn) and np.array_equal(np.asarray(hi, np.float64), mx)


def test_config_2048_rank_filters(gpu_ifx, oracle):
    """2048x2048 Gray{N0f8} with 5% salt-and-pepper, median 3x3/5x5 and extrema
    7x7/15x15, Pad(:symmetric): bit-exact on sampled rows and on all edges."""
    ifx = gpu_ifx
    rng = np.random.default_rng(4)
    img = rng.integers(0, 256, (2048, 2048), dtype=np.uint8)
    r = rng.random(img.shape)
    img[r < 0.025] = 0
    img[(r >= 0.025) & (r < 0.05)] = 255
    img = np.asfortranarray(img)
    for w in (3, 5):
        got = ifx.mapwindow(ifx.median, ifx.n0f8(img), (w, w), border="symmetric")
        codes = np.rint(got.astype(np.float64) * 255).astype(np.uint8)
        rows = [0, 1, 2, 1000, 2045, 2046, 2047]
        for y in rows:
            ref = oracle.median_u8_rows(img, [-(w // 2)] * 2, [w, w], "symmetric", 0.0, y, y + 1)
            assert np.array_equal(codes[:, y], ref[:, y])
        exp = got[:, 7]
        assert np.array_equal(exp, codes[:, 7].astype(np.float32) / np.float32(255))
    for w in (7, 15):
        mm = ifx.mapwindow(ifx.extrema, ifx.n0f8(img), (w, w), border="symmetric")
        sub = np.asfortranarray(img[:, :64])
        mn, mx = oracle.extrema_trunc(sub.astype(np.float64), [w, w])
        h = w // 2
        assert np.array_equal(mm[0][:, : 64 - h].astype(np.float64), mn[:, : 64 - h])
        assert np.array_equal(mm[1][:, : 64 - h].astype(np.float64), mx[:, : 64 - h])


# --------------------------------------------------------------------- full-size properties
def test_dense_4096_circular_shift_equivariance(gpu_ifx):
    """4096x4096, 31x31 dense, circular border: filtering commutes with a
    circular shift (exactly: the same products and sums in the same order)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(2)
    img = np.asfortranarray(rng.random((4096, 4096), dtype=np.float32))
    K = rng.standard_normal((31, 31))
    K /= K.sum()
    a = ifx.imfilter(img, ifx.centered(K), "circular")
    b = ifx.imfilter(np.asfortranarray(np.roll(img, (64, 32), axis=(0, 1))), ifx.centered(K), "circular")
    assert np.array_equal(np.roll(a, (64, 32), axis=(0, 1)), b)


def test_linearity_full_size(gpu_ifx):
    """256^3 volume, σ=(3,3,1.5), symmetric: filtering is linear."""
    ifx = gpu_ifx
    rng = np.random.default_rng(3)
    a = np.asfortranarray(rng.random((256, 256, 256), dtype=np.float32))
    b = np.asfortranarray(rng.random((256, 256, 256), dtype=np.float32))
    k = ifx.KernelFactors.gaussian((3, 3, 1.5))
    fa = ifx.imfilter(a, k, "symmetric")
    fb = ifx.imfilter(b, k, "symmetric")
    fab = ifx.imfilter(np.asfortranarray(a + b), k, "symmetric")
    assert normwise(fab, fa + fb) <= 1e-5
    c = np.asfortranarray(np.full((256, 256, 256), 0.25, dtype=np.float32))
    fc = ifx.imfilter(c, k, "symmetric")
    assert np.max(np.abs(fc - 0.25)) < 1e-6


# --------------------------------------------------------------------- device arrays
def test_device_resident_arrays(gpu_ifx, oracle):
    ifx = gpu_ifx
    import torch
    rng = np.random.default_rng(6)
    img = np.asfortranarray(rng.random((300, 200), dtype=np.float32))
    d = ifx.DeviceArray.from_host(img)
    k = ifx.KernelFactors.gaussian((2, 2))
    out = ifx.imfilter(d, k, "reflect")
    torch.cuda.synchronize()
    assert isinstance(out, ifx.DeviceArray)
    host = ifx.imfilter(img, k, "reflect")
    assert np.array_equal(out.numpy(), host)
    u = ifx.DeviceArray.from_host(ifx.n0f8(rng.integers(0, 256, (128, 96), dtype=np.uint8)))
    med = ifx.mapwindow(ifx.median, u, (5, 5), border="symmetric")
    torch.cuda.synchronize()
    assert np.array_equal(med.numpy(), ifx.mapwindow(ifx.median, u.numpy(), (5, 5), border="symmetric"))


def test_launch_counter_counts_kernels(gpu_ifx):
    ifx = gpu_ifx
    before = ifx.launch_count()
    ifx.imfilter(np.asfortranarray(np.ones((40, 40), np.float32)), ifx.KernelFactors.gaussian((1, 1)))
    assert ifx.launch_count() == before + 1          # one fused tile kernel


# --------------------------------------------------------------------- dense on tensor cores
@pytest.mark.parametrize("ksz,seed", [(11, 5), (15, 21), (31, 22)])
@pytest.mark.parametrize("style", ["reflect", "fill", "circular"])
def test_dense_tensor_cores(gpu_ifx, oracle, ksz, seed, style):
    """tcgen05 implicit GEMM (BF16 hi/lo split, three products, FP32 accumulation)
    within 1e-5 normwise of the FP64 oracle."""
    ifx = gpu_ifx
    rng = np.random.default_rng(seed)
    while True:
        K = rng.standard_normal((ksz, ksz))
        if abs(K.sum()) >= 0.1:
            break
    K = K / K.sum()
    img = np.asfortranarray(np.random.default_rng(2).random((301, 257), dtype=np.float32))
    kern = ifx.centered(K)
    b = ifx.Fill(0) if style == "fill" else ifx.Pad(style)
    got = ifx.imfilter(img, kern, b, ifx.Algorithm.GB300("tensor_cores"))
    ref = oracle.imfilter_dense(img.astype(np.float64), K, kern.first, style, 0.0)
    assert got.dtype == np.float64
    assert normwise(got, ref) <= 1e-5
    # the automatic method: these kernels have weights of both signs, so the
    # CUDA-core kernel (reference precision); a sign-definite kernel of the
    # same size takes the tensor cores
    auto = ifx.imfilter(img, kern, b, ifx.Algorithm.GB300())
    assert np.array_equal(auto, ifx.imfilter(img, kern, b, ifx.Algorithm.GB300("cuda_cores")))
    Kp = np.abs(K) / np.abs(K).sum()
    kp = ifx.centered(Kp)
    assert np.array_equal(ifx.imfilter(img, kp, b, ifx.Algorithm.GB300()),
                          ifx.imfilter(img, kp, b, ifx.Algorithm.GB300("tensor_cores")))


def test_dense_tensor_cores_shapes(gpu_ifx, oracle):
    """Rectangular and off-centre kernels, 8-bit input, image edges not multiples
    of the 128 x 32 tile."""
    ifx = gpu_ifx
    rng = np.random.default_rng(7)
    for (kw, kh, f), shape in [((13, 21, (-3, -17)), (517, 130)), ((33, 40, (-16, -20)), (129, 33)),
                               ((11, 11, (0, 0)), (31, 300))]:
        K = rng.standard_normal((kw, kh)) / (kw * kh)
        img = np.asfortranarray(rng.random(shape, dtype=np.float32))
        k = (ifx.OffsetKernel(K, f),)
        got = ifx.imfilter(img, k, "symmetric", ifx.Algorithm.GB300("tensor_cores"))
        ref = oracle.imfilter_dense(img.astype(np.float64), K, f, "symmetric")
        assert normwise(got, ref) <= 1e-5, (kw, kh, shape)
    codes = np.asfortranarray(rng.integers(0, 256, (200, 90), dtype=np.uint8))
    K = rng.standard_normal((15, 15))
    K /= K.sum()
    got = ifx.imfilter(ifx.n0f8(codes), ifx.centered(K), "replicate", ifx.Algorithm.GB300("tensor_cores"))
    ref = oracle.imfilter_dense(codes.astype(np.float64) / 255.0, K, (-7, -7), "replicate")
    assert normwise(got, ref) <= 1e-5


def test_dense_tensor_cores_many_tiles(gpu_ifx, oracle):
    """Images with several 128 x 32 tiles per CTA, so that the double-buffered
    pipeline (gather of tile k+1 and epilogue of tile k-1 around the MMAs of
    tile k) runs many rounds: against the oracle, and at 4096 x 2048 against
    the CUDA-core path."""
    ifx = gpu_ifx
    rng = np.random.default_rng(31)
    K = rng.standard_normal((15, 15))
    K /= K.sum()
    img = np.asfortranarray(rng.random((2049, 1031), dtype=np.float32))
    got = ifx.imfilter(img, ifx.centered(K), "reflect", ifx.Algorithm.GB300("tensor_cores"))
    ref = oracle.imfilter_dense(img.astype(np.float64), K, (-7, -7), "reflect")
    assert normwise(got, ref) <= 1e-5
    K = rng.standard_normal((31, 31))
    K /= K.sum()
    big = np.asfortranarray(rng.random((4096, 2048), dtype=np.float32))
    tc = ifx.imfilter(big, ifx.centered(K), "circular", ifx.Algorithm.GB300("tensor_cores"))
    cc = ifx.imfilter(big, ifx.centered(K), "circular", ifx.Algorithm.GB300("cuda_cores"))
    assert normwise(tc, cc) <= 1e-5


# --------------------------------------------------------------------- NA / Inner / NoPad
@pytest.mark.parametrize("kind", ["F32", "F64", "N0F8"])
@pytest.mark.parametrize("na", ["isnan", "notfinite", "none"])
def test_na_border(gpu_ifx, oracle, kind, na):
    """NA(): separable factors without NA elements (per-axis normalisation),
    with NaN/Inf elements (masked filters), and a dense kernel -- against the
    oracle's restatement of _imfilter_na!."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("na" + kind + na).encode()))
    for shape in [(67, 45), (256, 33)]:
        img = make_img(rng, shape, kind)
        vals = values(ifx, img, kind)
        if kind != "N0F8":
            bad = rng.random(shape) < 0.05
            img[bad] = rng.choice(np.array([np.nan, np.inf, -np.inf], dtype=img.dtype), bad.sum())
            vals = values(ifx, img, kind)
        fx = (0, -3, rng.random(7) + 0.1)
        fy = (1, -1, rng.random(4) + 0.1)
        ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w, (f,)), 2, ax) for ax, f, w in (fx, fy))
        got = ifx.imfilter(wrap(ifx, img, kind), ks, ifx.NA(na))
        filt = lambda a: oracle.imfilter_cascade(a, [fx, fy], "fill", 0.0)
        onan = na if kind != "N0F8" else "none"
        ref = oracle.imfilter_na(vals, filt, [(fx[1], fx[2]), (fy[1], fy[2])], onan)
        assert np.array_equal(np.isnan(got), np.isnan(ref)), (shape, na)
        fin = np.isfinite(ref)
        inf = np.isinf(ref)
        assert np.array_equal(np.asarray(got, np.float64)[inf], ref[inf]), (shape, na)
        tol = 1e-12 if kind == "F64" else 1e-5
        assert normwise(np.where(fin, got, 0), np.where(fin, ref, 0)) <= tol, (shape, na)
        K = rng.random((5, 3)) + 0.05
        got = ifx.imfilter(wrap(ifx, img, kind), ifx.OffsetKernel(K, (-2, -1)), ifx.NA(na))
        filt = lambda a: oracle.imfilter_dense(a, K, (-2, -1), "fill", 0.0)
        ref = oracle.imfilter_na(vals, filt, None, onan)
        assert np.array_equal(np.isnan(got), np.isnan(ref)), (shape, na, "dense")
        fin = np.isfinite(ref)
        assert normwise(np.where(fin, got, 0), np.where(fin, ref, 0)) <= tol, (shape, na, "dense")


@pytest.mark.parametrize("kind", ["F32", "N0F8"])
def test_inner_border(gpu_ifx, oracle, kind):
    """Inner() and Inner(lo, hi): the interior with its first indices;
    imgradients and mapwindow with Inner(); a window longer than the array
    is a DimensionMismatch."""
    ifx = gpu_ifx
    rng = np.random.default_rng(77)
    img = make_img(rng, (61, 40), kind)
    vals = values(ifx, img, kind)
    facs = [(0, -4, rng.standard_normal(9)), (1, -2, rng.standard_normal(5))]
    ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w, (f,)), 2, ax) for ax, f, w in facs)
    got = ifx.imfilter(wrap(ifx, img, kind), ks, ifx.Inner())
    assert got.first == (5, 3) and got.shape == (61 - 8, 40 - 4)
    ref = oracle.imfilter_cascade(vals, facs, "replicate")[4:-4, 2:-2]
    assert normwise(got, ref) <= 1e-5
    got = ifx.imfilter(wrap(ifx, img, kind), ks, ifx.Inner((6, 3), (7, 2)))
    assert got.first == (7, 4) and got.shape == (61 - 13, 40 - 5)
    ref = oracle.imfilter_cascade(vals, facs, "replicate")[6:-7, 3:-2]
    assert normwise(got, ref) <= 1e-5
    with pytest.raises(ifx.ArgumentError):                 # Inner(1, 1) leaves reads outside
        ifx.imfilter(wrap(ifx, img, kind), ks, ifx.Inner((1, 1), (1, 1)))
    gy, gx = ifx.imgradients(wrap(ifx, img, kind), ifx.KernelFactors.sobel, ifx.Inner())
    assert gy.first == (2, 2) and gy.shape == (59, 38)
    k1, k2 = ifx.KernelFactors.sobel.gradient_pair
    ref = oracle.imfilter_cascade(vals, [(0, -1, k1), (1, -1, k2)], "replicate")[1:-1, 1:-1]
    assert normwise(gy, ref) <= 1e-5
    med = ifx.mapwindow(ifx.median, wrap(ifx, img, kind), (5, 3), border=ifx.Inner())
    assert med.first == (3, 2) and med.shape == (57, 38)
    code = img if kind == "N0F8" else vals
    ref = oracle.mapwindow_median(np.asarray(code, np.float64), [-2, -1], [5, 3], "replicate")[2:-2, 1:-1]
    exp = (ref.astype(np.float32) / np.float32(255)) if kind == "N0F8" else ref
    assert np.array_equal(np.asarray(med, np.float64), np.asarray(exp, np.float64))
    with pytest.raises(ifx.DimensionMismatch):
        ifx.mapwindow(ifx.median, wrap(ifx, img[:4, :4], kind), (5, 3), border=ifx.Inner())


def test_nopad_subregion(gpu_ifx, oracle):
    """imfilter!(out, img, kernel, NoPad(), inds): only out[inds] is written,
    reads stay inside img; other borders with inds raise; reads outside raise."""
    ifx = gpu_ifx
    rng = np.random.default_rng(78)
    img = np.asfortranarray(rng.random((50, 37)))
    K = rng.standard_normal((3, 5))
    k = ifx.OffsetKernel(K, (-1, -2))
    out = np.asfortranarray(np.full((50, 37), -7.0))
    ifx.imfilter_(out, img, k, ifx.NoPad(), inds=[(3, 40), (4, 30)])
    ref = oracle.imfilter_dense(img, K, (-1, -2), "replicate")
    assert normwise(out[2:40, 3:30], ref[2:40, 3:30]) <= 1e-12
    mask = np.ones(out.shape, bool)
    mask[2:40, 3:30] = False
    assert np.all(out[mask] == -7.0)
    with pytest.raises(ifx.ErrorException):
        ifx.imfilter_(out, img, k, ifx.Pad("replicate"), inds=[(3, 40), (4, 30)])
    with pytest.raises(ifx.ArgumentError):
        ifx.imfilter_(out, img, k, ifx.NoPad(), inds=[(1, 40), (4, 30)])


# --------------------------------------------------------------------- blob_LoG
@pytest.mark.parametrize("kind", ["F64", "F32", "N0F8"])
def test_findlocalextrema_random(gpu_ifx, oracle, kind):
    """findlocalmaxima / findlocalminima on random 2-D to 4-D arrays with ties
    (8-bit values), windows 1..5 and edge flags: the same indices in the same
    order as the oracle's restatement."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("le" + kind).encode()))
    for shape, window, edges in [((31, 17), (3, 3), (True, True)), ((12, 9, 7), (3, 1, 5), (False, True, False)),
                                 ((6, 5, 4, 3), (3, 3, 3, 3), (True, False, True, True))]:
        img = make_img(rng, shape, kind)
        vals = values(ifx, img, kind)
        for minima in (False, True):
            f = ifx.findlocalminima if minima else ifx.findlocalmaxima
            got = f(wrap(ifx, img, kind), window=window, edges=edges)
            assert got == oracle.findlocalextrema(vals, window, edges, minima), (shape, minima)


@pytest.mark.parametrize("kind", ["F64", "F32"])
def test_multilog_and_blobs(gpu_ifx, oracle, kind):
    """multiLoG (LoG as a sum of separable terms) against the oracle's dense
    LoG with Pad(:reflect); blob_LoG on an image of Gaussian blobs of several
    sizes: same locations and scales, amplitudes within the tolerance."""
    ifx = gpu_ifx
    rng = np.random.default_rng(91)
    ny, nx = 96, 80
    yy, xx = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    img = np.zeros((ny, nx))
    for cy, cx, s in [(20, 18, 2.0), (60, 30, 4.0), (40, 62, 3.0), (80, 70, 1.5)]:
        img += np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * s * s))
    img += 0.01 * rng.random((ny, nx))
    img = np.asfortranarray(img.astype(np.float32 if kind == "F32" else np.float64))
    sig = [1.0, 1.5, 2.0, 3.0, 4.0]
    st = ifx.multiLoG(img, sig)
    ref = oracle.multiLoG(img.astype(np.float64), sig, (1.0, 1.0))
    assert st.shape == (5, ny, nx)
    tol = 1e-12 if kind == "F64" else 1e-5
    assert normwise(np.asarray(st, np.float64), ref) <= tol
    got = ifx.blob_LoG(img, sig)
    exp = oracle.blob_LoG(img.astype(np.float64), sig, (True, False, False), (1.0, 1.0))
    assert [(b.location, b.sigma) for b in got] == [(tuple(l), tuple(s)) for l, s, _ in exp]
    assert all(abs(b.amplitude - a) <= 1e-5 * max(1.0, abs(a)) for b, (_, _, a) in zip(got, exp))
    assert len(got) >= 4


# --------------------------------------------------------------------- Algorithm.FFT()
@pytest.mark.parametrize("kind", ["F32", "F64", "N0F8"])
@pytest.mark.parametrize("style", STYLES)
def test_fft_matches_fir_oracle(gpu_ifx, oracle, kind, style):
    """Algorithm.FFT() (cuFFT in the output's precision) against the FP64
    direct oracle: a 69x69 LoG (σ = 8), an off-centre random 7x5 kernel and a
    Gaussian cascade (kernelconv), within 1e-5 normwise (1e-12 for Float64)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("fft" + kind + style).encode()))
    img = make_img(rng, (301, 257), kind)
    vals = values(ifx, img, kind)
    fill = fill_value(kind)
    tol = 1e-12 if kind == "F64" else 1e-5
    K, first = oracle.log_kernel((8.0, 8.0))
    cases = [(K, first), (rng.standard_normal((7, 5)), (-3, 1))]
    for K, first in cases:
        got = ifx.imfilter(wrap(ifx, img, kind), (ifx.OffsetKernel(K, first),), border_of(ifx, style),
                           ifx.Algorithm.FFT())
        ref = oracle.imfilter_dense(vals, K, first, style, fill)
        assert normwise(got, ref) <= tol, (K.shape, style)
    g = ifx.KernelFactors.gaussian((3.0, 2.0))
    got = ifx.imfilter(wrap(ifx, img, kind), g, border_of(ifx, style), ifx.Algorithm.GB300("fft"))
    fir = ifx.imfilter(wrap(ifx, img, kind), g, border_of(ifx, style))
    assert normwise(got, fir) <= tol


def test_fft_volume_and_limits(gpu_ifx, oracle):
    ifx = gpu_ifx
    rng = np.random.default_rng(44)
    vol = np.asfortranarray(rng.random((40, 33, 21), dtype=np.float32))
    K = rng.standard_normal((5, 3, 7))
    got = ifx.imfilter(vol, (ifx.OffsetKernel(K, (-2, -1, -3)),), "symmetric", ifx.Algorithm.FFT())
    ref = oracle.imfilter_dense(vol.astype(np.float64), K, (-2, -1, -3), "symmetric")
    assert normwise(got, ref) <= 1e-5
    v = np.asfortranarray(rng.random(1000))
    k = rng.standard_normal(61)
    got = ifx.imfilter(v, (ifx.OffsetKernel(k, (-30,)),), "reflect", ifx.Algorithm.FFT())
    assert normwise(got, oracle.imfilter_dense(v, k, (-30,), "reflect")) <= 1e-12
    with pytest.raises(ifx.Unsupported):
        ifx.imfilter(np.zeros((4, 4, 4, 4)), (ifx.OffsetKernel(np.ones((3, 3, 3, 3)), (-1,) * 4),),
                     "replicate", ifx.Algorithm.FFT())
    with pytest.raises(ifx.Unsupported):
        ifx.imfilter(np.zeros((20, 20)), (ifx.OffsetKernel(np.ones((3, 3)), (-1, -1)),),
                     ifx.Pad("replicate", (1, 1), (1, 1)), ifx.Algorithm.FFT())


def test_dense_auto_takes_fft(gpu_ifx, oracle):
    """The automatic dense method takes the FFT for Float64 images with large
    kernels and for kernels over 3600 taps, and the direct kernels when an
    element is not finite (NaN spreads over the kernel's reach only, as in
    the reference's FIR fallback)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(55)
    img = np.asfortranarray(rng.random((300, 260)))
    K = rng.standard_normal((31, 31))
    k = (ifx.OffsetKernel(K, (-15, -15)),)
    ref = oracle.imfilter_dense(img, K, (-15, -15), "reflect")
    assert normwise(ifx.imfilter(img, k, "reflect"), ref) <= 1e-12
    K2 = rng.standard_normal((61, 61))
    img32 = np.asfortranarray(rng.random((200, 180), dtype=np.float32))
    got = ifx.imfilter(img32, (ifx.OffsetKernel(K2, (-30, -30)),), "replicate")
    assert normwise(got, oracle.imfilter_dense(img32.astype(np.float64), K2, (-30, -30), "replicate")) <= 1e-5
    bad = img.copy()
    bad[150, 100] = np.nan
    got = ifx.imfilter(bad, k, "reflect")
    refb = oracle.imfilter_dense(bad, K, (-15, -15), "reflect")
    assert np.array_equal(np.isnan(got), np.isnan(refb))
    fin = ~np.isnan(refb)
    assert np.isnan(refb).sum() == 31 * 31
    assert normwise(got[fin], refb[fin]) <= 1e-12


# --------------------------------------------------------------------- IIR (Triggs-Sdika)
def _iir_ref(oracle, vals, sigmas, style, fill, T=np.float64, arith="f64"):
    facs = []
    for ax, s in sigmas:
        a, b, B, M = oracle.iir_gaussian(s, T)
        facs.append((ax, a, b, B, M))
    return oracle.imfilter_iir(vals, facs, "fill" if style == "fill" else "pad", fill, arith,
                               T == np.float32)


@pytest.mark.parametrize("kind", ["F32", "F64", "N0F8"])
@pytest.mark.parametrize("style", ["replicate", "circular", "fill"])
def test_iir_matches_oracle_bitwise(gpu_ifx, oracle, kind, style):
    """IIRGaussian cascades (Float64 coefficients, Float64 results) on 1-D to
    3-D arrays, both the contiguous and the strided axes, small and large σ:
    the same bits as the oracle (same operation order, every product and sum
    rounded once, results kept in the output eltype between steps)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("iir" + kind + style).encode()))
    for shape, sig in [((1000,), (30.0,)), ((301, 257), (1.5, 4.0)), ((40, 33, 21), (2.0, 0.0, 3.5)),
                       ((5, 7), (5.0, 5.0)), ((64, 4), (9.0, 1.2))]:
        img = make_img(rng, shape, kind)
        vals = values(ifx, img, kind)
        kern = ifx.KernelFactors.IIRGaussian(sig) if len(sig) > 1 else \
            (ifx.ReshapedOneD(ifx.KernelFactors.IIRGaussian(sig[0]), 1, 0),)
        got = ifx.imfilter(wrap(ifx, img, kind), kern, border_of(ifx, style))
        assert got.dtype == np.float64
        ref = _iir_ref(oracle, vals, [(d, s) for d, s in enumerate(sig) if s != 0], style, 0.7)
        assert np.array_equal(got, ref), (shape, sig, np.max(np.abs(got - ref)))


def test_iir_float32_forms(gpu_ifx, oracle):
    """Float32 coefficients on a Float32 image (Float32 arithmetic and
    results) and Float64 coefficients into a Float32 output (Float64
    arithmetic, Float32 results): the same bits as the oracle's Float32 forms;
    bare TriggsSdika tuples take the axes in order and refuse other Pad styles;
    in place on a vector; one pass along a dimension."""
    ifx = gpu_ifx
    rng = np.random.default_rng(606)
    img = np.asfortranarray(rng.random((123, 77), dtype=np.float32))
    s32 = (np.float32(2.5), np.float32(6.0))
    got = ifx.imfilter(img, ifx.KernelFactors.IIRGaussian(s32), "replicate")
    assert got.dtype == np.float32
    ref = _iir_ref(oracle, img.astype(np.float64), [(0, s32[0]), (1, s32[1])], "replicate", 0.0,
                   np.float32, "f32")
    assert np.array_equal(got.astype(np.float64), ref)
    out = np.asfortranarray(np.zeros(img.shape, np.float32))
    ifx.imfilter_(out, img, ifx.KernelFactors.IIRGaussian((3.0, 7.0)), ifx.Fill(0.25))
    ref = _iir_ref(oracle, img.astype(np.float64), [(0, 3.0), (1, 7.0)], "fill", 0.25, np.float64, "f64/f32")
    assert np.array_equal(out.astype(np.float64), ref)
    ts = ifx.KernelFactors.IIRGaussian(4.0)
    bare = ifx.imfilter(img, (ts, ts), "replicate")
    assert np.array_equal(bare, ifx.imfilter(img, ifx.KernelFactors.IIRGaussian((4.0, 4.0)), "replicate"))
    with pytest.raises(ifx.ArgumentError):
        ifx.imfilter(img, (ts, ts), "circular")
    with pytest.raises(ifx.DimensionMismatch):
        ifx.imfilter(img, (ts, ts, ts), "replicate")
    v = np.asfortranarray(rng.random(500))
    exp = _iir_ref(oracle, v, [(0, 4.0)], "fill", 0.0)
    ifx.imfilter_(v, v, (ts,), ifx.Fill(0))
    assert np.array_equal(v, exp)
    o2 = np.asfortranarray(np.zeros(img.shape))
    ifx.imfilter_(o2, img, ts, 2, "replicate")
    assert np.array_equal(o2, _iir_ref(oracle, img.astype(np.float64), [(1, 4.0)], "replicate", 0.0))


def test_iir_full_size_bitwise(gpu_ifx, oracle):
    """A 2048x2048 Float32 image through IIRGaussian((3, 8)) with Fill(0):
    bit-exact with the oracle at full size."""
    ifx = gpu_ifx
    img = np.asfortranarray(np.random.default_rng(2048).random((2048, 2048), dtype=np.float32))
    got = ifx.imfilter(img, ifx.KernelFactors.IIRGaussian((3.0, 8.0)), ifx.Fill(0))
    ref = _iir_ref(oracle, img.astype(np.float64), [(0, 3.0), (1, 8.0)], "fill", 0.0)
    assert np.array_equal(got, ref)


def test_iir_na_and_errors(gpu_ifx, oracle):
    ifx = gpu_ifx
    rng = np.random.default_rng(707)
    img = np.asfortranarray(rng.random((60, 45)))
    img[10, 7] = np.nan
    img[33, 40] = np.nan
    kern = ifx.KernelFactors.IIRGaussian((2.0, 3.0))
    got = ifx.imfilter(img, kern, ifx.NA())
    a1, b1, B1, M1 = oracle.iir_gaussian(2.0)
    a2, b2, B2, M2 = oracle.iir_gaussian(3.0)
    facs = [(0, a1, b1, B1, M1), (1, a2, b2, B2, M2)]
    ref = oracle.imfilter_na(img, lambda a: oracle.imfilter_iir(a, facs, "fill", 0.0), None)
    assert normwise(got, ref) <= 1e-12
    with pytest.raises(ifx.DimensionMismatch):
        ifx.imfilter(np.zeros((3, 10)), kern, "replicate")
    with pytest.raises(ifx.ArgumentError):
        ifx.imfilter(np.zeros((30, 10)), kern, ifx.Inner())
    with pytest.raises(ifx.ArgumentError):
        ifx.imfilter(np.zeros((30, 10)), (kern[0], ifx.Kernel.Laplacian()), ifx.Inner())


@pytest.mark.parametrize("style", ["replicate", "reflect", "fill"])
def test_mixed_cascades_match_oracle(gpu_ifx, oracle, style):
    """Cascades of IIRGaussian factors with FIR filters (a Laplacian, a dense
    kernel, a Gaussian factor) in several orders on 2-D and 3-D arrays: the
    doubled padding, the shrinking stage ranges and the IIR boundary values at
    each range's edges as the oracle's restatement, within 1e-12 (Float64
    stages)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("mixed" + style).encode()))
    lap2 = np.array([[0, 1, 0], [1, -4, 1], [0, 1, 0]], dtype=np.float64)
    D = rng.standard_normal((3, 5))
    g = np.asarray(ifx.KernelFactors.gaussian(1.5).data, np.float64)
    for shape, kind in [((37, 29), "F64"), ((40, 33), "F32")]:
        img = make_img(rng, shape, kind)
        vals = values(ifx, img, kind)
        a1, a2 = (oracle.iir_gaussian(s) for s in (2.5, 3.2))
        I0 = ifx.ReshapedOneD(ifx.KernelFactors.IIRGaussian(2.5), 2, 0)
        I1 = ifx.ReshapedOneD(ifx.KernelFactors.IIRGaussian(3.2), 2, 1)
        G1 = ifx.ReshapedOneD(ifx.centered(g), 2, 1)
        cases = [((I0, I1, ifx.Kernel.Laplacian()), [("iir", 0, a1), ("iir", 1, a2), ("fir", lap2, (-1, -1))]),
                 ((ifx.Kernel.Laplacian(), I0, I1), [("fir", lap2, (-1, -1)), ("iir", 0, a1), ("iir", 1, a2)]),
                 ((I0, ifx.OffsetKernel(D, (-1, -3)), G1),
                  [("iir", 0, a1), ("fir", D, (-1, -3)), ("fir", g.reshape(1, -1), (0, -(g.size // 2)))])]
        for ks, stages in cases:
            got = ifx.imfilter(img, ks, border_of(ifx, style, 0.0))
            ref = oracle.imfilter_mixed(vals, stages, style, 0.0)
            assert not np.any(np.isnan(ref))
            assert normwise(got, ref) <= 1e-12, (shape, style, len(stages))


def test_fft_full_size_against_direct(gpu_ifx):
    """4096x4096 Float32 with a normalised N(0,1) 31x31 kernel and Pad(:reflect)
    (the dense configuration's largest kernel): the FFT path and the FP32
    CUDA-core direct path agree within 2e-5 normwise (each is within 1e-5 of
    the FP64 result at the sizes the oracle checks); Float64 within 1e-12."""
    ifx = gpu_ifx
    import torch
    rng = np.random.default_rng(22)
    while True:
        K = rng.standard_normal((31, 31))
        if abs(K.sum()) >= 0.1:
            break
    K = K / K.sum()
    ker = (ifx.OffsetKernel(K, (-15, -15)),)
    g = torch.Generator(device="cuda")
    g.manual_seed(2)
    for dt, kind, tol in [(torch.float32, "F32", 2e-5), (torch.float64, "F64", 1e-12)]:
        img = ifx.DeviceArray(torch.rand((4096, 4096), device="cuda", generator=g, dtype=dt).t(), kind)
        a = ifx.DeviceArray.empty((4096, 4096), kind)
        b = ifx.DeviceArray.empty((4096, 4096), kind)
        ifx.imfilter_(a, img, ker, "reflect", ifx.Algorithm.FFT())
        ifx.imfilter_(b, img, ker, "reflect", ifx.Algorithm.GB300("cuda_cores"))
        d = (a.tensor.double() - b.tensor.double()).abs().max() / b.tensor.double().abs().max()
        assert float(d) <= tol, (kind, float(d))


def test_dense_tensor_cores_31x31_twelve_seeds(gpu_ifx, oracle):
    """The tensor-core error at 31 x 31 over twelve kernel seeds, normwise,
    max_abs and max_rel against the FP64 oracle.  Kernels of both signs
    (N(0,1) normalised to sum 1, |sum| >= 0.1) stay within 1.5e-5 on the
    tensor cores -- above 1e-5 for some seeds, so the automatic method gives
    them the CUDA cores, within 1e-5 for every seed; sign-definite kernels
    (|N(0,1)| normalised) stay within 1e-5 on the tensor cores, which the
    automatic method takes for them."""
    ifx = gpu_ifx
    img = np.asfortranarray(np.random.default_rng(3).random((320, 288), dtype=np.float32))

    def err(got, ref):
        d = np.abs(np.asarray(got, np.float64) - ref)
        big = np.abs(ref) >= 1e-3 * np.max(np.abs(ref))
        return normwise(got, ref), float(d.max()), float(np.max(d[big] / np.abs(ref[big])))

    mixed, definite = [], []
    for seed in range(100, 112):
        rng = np.random.default_rng(seed)
        while True:
            K = rng.standard_normal((31, 31))
            if abs(K.sum()) >= 0.1:
                break
        for kind, Kk, out in (("mixed", K / K.sum(), mixed), ("definite", np.abs(K) / np.abs(K).sum(), definite)):
            kern = ifx.centered(Kk)
            ref = oracle.imfilter_dense(img.astype(np.float64), Kk, kern.first, "reflect", 0.0)
            tc = err(ifx.imfilter(img, kern, "reflect", ifx.Algorithm.GB300("tensor_cores")), ref)
            auto = err(ifx.imfilter(img, kern, "reflect", ifx.Algorithm.GB300()), ref)
            out.append((seed, tc, auto))
            print("seed %d %s: tensor cores normwise %.3g max_abs %.3g max_rel %.3g; automatic normwise %.3g"
                  % (seed, kind, tc[0], tc[1], tc[2], auto[0]))
    assert max(t[0] for _, t, _ in mixed) <= 1.5e-5
    assert max(a[0] for _, _, a in mixed + definite) <= 1e-5
    assert max(t[0] for _, t, _ in definite) <= 1e-5
