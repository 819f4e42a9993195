"""Eltypes beyond Float32/Float64/N0f8/UInt8, against the oracle:

* ifx_convert: every eltype to Float32/Float64 (N0f8 c/255 and N0f16 c/65535
  correctly rounded), Float64 to integers with Julia's InexactError;
* integer images (Int8 .. Int64, UInt16) with float kernels (Float64 / Float32
  results) and with integer kernels (integer results, exact; the reference's
  own impulse test filters an Int image, test/2d.jl:47), and the Laplacian's
  signed_type rule;
* Gray{N0f16} images (src/precompile.jl:8-9): linear filters, median, extrema;
* RGB images as channel planes (RGB{N0f8} impulse of test/2d.jl:49);
* mapwindow(...; indices=) == mapwindow(...)[indices...] (test/mapwindow.jl:131-150).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def normwise(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_convert_to_float(gpu_ifx):
    ifx = gpu_ifx
    rng = np.random.default_rng(1)
    codes16 = np.asfortranarray(np.arange(65536, dtype=np.uint16).reshape(256, 256, order="F"))
    codes8 = np.asfortranarray(np.arange(256, dtype=np.uint8).reshape(16, 16, order="F"))
    for src, vals in [(ifx.n0f16(codes16), codes16.astype(np.float64) / 65535.0),
                      (ifx.n0f8(codes8), codes8.astype(np.float64) / 255.0)]:
        for dt in (np.float32, np.float64):
            out = np.asfortranarray(np.zeros(src.shape, dt))
            ifx.convert_(out, src)
            assert np.array_equal(out, vals.astype(dt))       # correctly rounded quotients
    for dt in (np.int8, np.int16, np.uint16, np.int32, np.int64):
        info = np.iinfo(dt)
        a = np.asfortranarray(rng.integers(info.min, info.max, (33, 17), dtype=dt, endpoint=True))
        for ot in (np.float32, np.float64):
            out = np.asfortranarray(np.zeros(a.shape, ot))
            ifx.convert_(out, a)
            assert np.array_equal(out, a.astype(ot))


def test_convert_to_integer_and_inexact(gpu_ifx):
    ifx = gpu_ifx
    a = np.asfortranarray(np.array([[1.0, -3.0], [127.0, -128.0]]))
    out = np.asfortranarray(np.zeros((2, 2), np.int8))
    ifx.convert_(out, a)
    assert np.array_equal(out, a.astype(np.int8))
    with pytest.raises(ifx.InexactError):
        ifx.convert_(out, np.asfortranarray(np.array([[1.5, 0.0], [0.0, 0.0]])))
    with pytest.raises(ifx.InexactError):
        ifx.convert_(out, np.asfortranarray(np.array([[128.0, 0.0], [0.0, 0.0]])))
    # N0f8 / N0f16 values are integers at 0 and 1 only (convert(Int, N0f8(1)) == 1)
    for codes, src in [(np.array([[0, 255], [255, 0]], np.uint8), ifx.n0f8),
                       (np.array([[65535, 0], [0, 65535]], np.uint16), ifx.n0f16)]:
        ifx.convert_(out, src(np.asfortranarray(codes)))
        assert np.array_equal(out, (codes > 0).astype(np.int8))
        bad = codes.copy()
        bad[0, 0] = 128
        with pytest.raises(ifx.InexactError):
            ifx.convert_(out, src(np.asfortranarray(bad)))


@pytest.mark.parametrize("dt", [np.int8, np.int16, np.uint16, np.int32, np.int64])
def test_integer_images_float_kernels(gpu_ifx, oracle, dt):
    ifx = gpu_ifx
    rng = np.random.default_rng(7)
    hi = min(np.iinfo(dt).max, 1 << 20)
    img = np.asfortranarray(rng.integers(0 if dt == np.uint16 else -hi, hi, (61, 47)).astype(dt))
    vals = img.astype(np.float64)
    for sigma, kt, okind in [(2.0, np.float64, np.float64), (np.float32(1.5), np.float32, np.float32)]:
        k = ifx.KernelFactors.gaussian((sigma, sigma))
        assert ifx.filter_type({np.int8: "I8", np.int16: "I16", np.uint16: "U16", np.int32: "I32",
                                np.int64: "I64"}[dt], ifx.factorkernel(k)) == ("F64" if kt == np.float64 else "F32")
        for style in ("replicate", "reflect"):
            got = ifx.imfilter(img, k, style)
            assert got.dtype == okind
            facs = [(f.axis, f.data.first[0], np.asarray(f.data.data, np.float64)) for f in k]
            ref = oracle.imfilter_cascade(vals, facs, style)
            tol = 1e-12 if (dt in (np.int32, np.int64) and okind == np.float64) else 1e-5
            assert normwise(got, ref) <= tol, (dt, style, sigma)
    # the reference's impulse test (test/2d.jl:39-56) on an Int image
    imgi = np.asfortranarray(np.zeros((5, 7), dtype=dt))
    imgi[2, 3] = 1
    kern = ifx.OffsetKernel(np.array([[0.1, 0.2], [0.4, 0.5]]), (-1, 1))
    got = ifx.imfilter(imgi, kern)
    target = np.zeros((5, 7))
    target[2:4, 1:3] = np.rot90(np.array([[0.1, 0.2], [0.4, 0.5]]), 2)
    assert got.dtype == np.float64 and np.allclose(got, target, atol=1e-15)


def test_integer_kernels_on_integer_images(gpu_ifx, oracle):
    """Integer accumulation (accumfilter, src/utils.jl:124-129): exact, in the
    eltype Julia's promotion gives."""
    ifx = gpu_ifx
    rng = np.random.default_rng(8)
    img = np.asfortranarray(rng.integers(-200, 200, (40, 33)).astype(np.int16))
    K = np.array([[1, 2, 0], [0, 1, -1], [3, 0, 1]], dtype=np.int64)      # full rank: stays dense
    got = ifx.imfilter(img, ifx.centered(K), "symmetric")
    assert got.dtype == np.int64                    # promote_type(Int16, Int64)
    ref = oracle.imfilter_dense(img.astype(np.float64), K.astype(np.float64), (-1, -1), "symmetric")
    assert np.array_equal(got, ref.astype(np.int64))
    # a separable integer kernel factors through the SVD into Float64 factors
    # (src/imfilter.jl:1167-1184), so the result is Float64, as in the reference
    sob = ifx.imfilter(img, ifx.centered(np.array([[1, 2, 1], [0, 0, 0], [-1, -2, -1]], dtype=np.int64)))
    assert sob.dtype == np.float64
    # Int8 image, Int8 kernel: the result is Int8, and values that do not fit raise
    K8 = np.array([[1, 1, 1], [1, 2, 1], [1, 1, 1]], dtype=np.int8)
    img8 = np.asfortranarray(np.full((6, 6), 100, dtype=np.int8))
    with pytest.raises(ifx.InexactError):
        ifx.imfilter(img8, ifx.centered(K8), "replicate")
    small = np.asfortranarray(rng.integers(-3, 4, (6, 6)).astype(np.int8))
    r8 = ifx.imfilter(small, ifx.centered(K8), "replicate")
    assert r8.dtype == np.int8
    ref = oracle.imfilter_dense(small.astype(np.float64), K8.astype(np.float64), (-1, -1), "replicate")
    assert np.array_equal(r8, ref.astype(np.int8))
    # Laplacian: UInt16 -> Int32 (signed_type), Int32 -> Int32
    u16 = np.asfortranarray(rng.integers(0, 65536, (30, 20)).astype(np.uint16))
    lap = ifx.imfilter(u16, ifx.Kernel.Laplacian(), "replicate")
    assert lap.dtype == np.int32
    ref = oracle.laplacian(u16.astype(np.float64), [1, 1], "replicate", 0.0, "int")
    assert np.array_equal(lap, ref.astype(np.int32))


def test_n0f16_images(gpu_ifx, oracle):
    ifx = gpu_ifx
    rng = np.random.default_rng(9)
    codes = np.asfortranarray(rng.integers(0, 65536, (70, 45)).astype(np.uint16))
    img = ifx.n0f16(codes)
    vals = codes.astype(np.float64) / 65535.0
    k = ifx.KernelFactors.gaussian((2, 2))
    got = ifx.imfilter(img, k, "circular")
    assert got.dtype == np.float64
    facs = [(f.axis, f.data.first[0], np.asarray(f.data.data, np.float64)) for f in k]
    assert normwise(got, oracle.imfilter_cascade(vals, facs, "circular")) <= 1e-5
    med = ifx.mapwindow(ifx.median, img, (3, 3), border="symmetric")
    assert med.dtype == np.float32
    mref = oracle.mapwindow_median(codes.astype(np.float64), [-1, -1], [3, 3], "symmetric")
    assert np.array_equal(med, (mref / 65535.0).astype(np.float32))
    mm = ifx.mapwindow(ifx.extrema, img, (5, 5))
    mn, mx = oracle.extrema_trunc(codes.astype(np.float64), [5, 5])
    assert isinstance(mm, ifx.N0f16Array)
    assert np.array_equal(np.asarray(mm[0]).view(np.uint16), mn) and np.array_equal(np.asarray(mm[1]).view(np.uint16), mx)


@pytest.mark.parametrize("dt", [np.int16, np.int32, np.uint16])
def test_integer_rank_filters(gpu_ifx, oracle, dt):
    ifx = gpu_ifx
    rng = np.random.default_rng(10)
    img = np.asfortranarray(rng.integers(0, 30000, (37, 29)).astype(dt))
    med = ifx.mapwindow(ifx.median, img, (5, 5), border="reflect")
    assert med.dtype == np.float64
    assert np.array_equal(med, oracle.mapwindow_median(img.astype(np.float64), [-2, -2], [5, 5], "reflect"))
    lo = ifx.mapwindow(ifx.minimum, img, (3, 3), border="replicate")
    assert lo.dtype == dt
    mn, _ = oracle.mapwindow_extrema(img.astype(np.float64), [-1, -1], [3, 3], "replicate")
    assert np.array_equal(lo, mn.astype(dt))


def test_rgb_images(gpu_ifx, oracle):
    """RGB{N0f8} impulse (test/2d.jl:39-56): the red channel holds rot180(kern),
    the others stay zero; random RGB images against the oracle per channel."""
    ifx = gpu_ifx
    planes = np.zeros((3, 5, 7), dtype=np.uint8)
    planes[0, 2, 3] = 255                            # RGB(1, 0, 0) at [3, 4]
    img = ifx.rgb(ifx.n0f8(np.asfortranarray(planes)))
    kern = ifx.OffsetKernel(np.array([[0.1, 0.2], [0.4, 0.5]]), (-1, 1))
    got = ifx.imfilter(img, kern)
    assert isinstance(got, ifx.RGB) and got.data.dtype == np.float64
    target = np.zeros((5, 7))
    target[2:4, 1:3] = np.rot90(np.array([[0.1, 0.2], [0.4, 0.5]]), 2)
    assert np.allclose(got.data[0], target, atol=1e-7) and not np.any(got.data[1:])
    rng = np.random.default_rng(11)
    data = np.asfortranarray(rng.random((3, 50, 41), dtype=np.float32))
    k = ifx.KernelFactors.gaussian((1.5, 1.5))
    for kernel in (k, ifx.Kernel.Laplacian()):
        res = ifx.imfilter(ifx.rgb(data), kernel, "symmetric")
        for c in range(3):
            one = ifx.imfilter(np.asfortranarray(data[c]), kernel, "symmetric")
            assert normwise(res.data[c], one) <= 1e-6


def test_mapwindow_indices(gpu_ifx, oracle):
    ifx = gpu_ifx
    import torch
    rng = np.random.default_rng(12)
    img = np.asfortranarray(rng.random((10, 5)))
    for f, w, inds in [(ifx.median, (3, 1), (range(1, 9, 2), range(1, 4))),
                       (ifx.median, (3, 3), (range(1, 3), range(1, 4))),
                       (ifx.extrema, (3, 3), (range(2, 11, 3), range(1, 6, 2)))]:
        full = ifx.mapwindow(f, img, w)
        got = ifx.mapwindow(f, img, w, indices=inds)
        sel = tuple(np.asarray(list(r)) - 1 for r in inds)
        exp = full[np.ix_(*sel)] if f is not ifx.extrema else full[(slice(None),) + np.ix_(*sel)]
        assert np.array_equal(np.asarray(got), exp)
        d = ifx.mapwindow(f, ifx.DeviceArray.from_host(img), w, indices=inds)
        torch.cuda.synchronize()
        assert np.array_equal(d.numpy(), exp)
