"""Full-size parity against the oracle on the benchmark workloads themselves.

* The mixed serving stream (seed 5): a wave of stream requests run as one
  validated batch plan (the launch the throughput figure times), with images
  up to 4096 wide, 33-tap Gaussians, both median windows, both eltypes and
  every Pad style, each output compared with the oracle.
* Dense 4096^2 with a 31x31 N(0,1) kernel on the tensor cores, reflect and
  Fill(0): interior crops, an image corner and an image edge against the
  oracle run on the crop plus its halo.
* One 256^3 volume with 1% impulse outliers: Gaussian sigma=(3,3,1.5),
  Pad(:symmetric), then imgradients with KernelFactors.sobel on all three axes.

Tolerances are those of the FIR path: FP32 arithmetic within 1e-5 normwise
(max|gpu - oracle| / max|oracle|) of the FP64 oracle, Float64 arithmetic within
1e-12, Laplacian and median bit-exact.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def normwise(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def stream_wave(S):
    """About 30 requests of the seed-5 stream, taken in stream order: the first
    request with a side >= 2048 for six (op, eltype) pairs (33-tap Gaussians),
    the first 33-tap Gaussian of each eltype up to 1024 wide, then the first
    request (side <= 1024) of every (op, eltype, style) and (median window,
    eltype) combination not yet held."""
    rs = S.stream_requests(10000, seed=5)
    picked, seen = [], set()

    def take(r):
        if r.idx not in seen:
            seen.add(r.idx)
            picked.append(r)

    big = [("gaussian", "F32"), ("gaussian", "N0F8"), ("median", "N0F8"), ("median", "F32"),
           ("sobel", "F32"), ("laplacian", "N0F8")]
    for op, kind in big:
        take(next(r for r in rs if r.op == op and r.kind == kind and max(r.h, r.w) >= 2048
                  and (op != "gaussian" or r.taps() == 33)))
    for kind in ("F32", "N0F8"):
        take(next(r for r in rs if r.op == "gaussian" and r.kind == kind and r.taps() == 33
                  and max(r.h, r.w) <= 1024))
    have = {(r.op, r.kind, r.style) for r in picked} | {("median", r.kind, r.win) for r in picked
                                                        if r.op == "median"}
    for r in rs:
        if max(r.h, r.w) > 1024:
            continue
        keys = [(r.op, r.kind, r.style)] + ([("median", r.kind, r.win)] if r.op == "median" else [])
        if any(k not in have for k in keys):
            take(r)
            have.update(keys)
    return picked


def oracle_outputs(ifx, oracle, r, img):
    """The reference's results for stream request r on host image img (codes
    for N0f8), as float64 arrays, and whether they must match bit for bit."""
    if r.kind == "N0F8":
        vals = img.astype(np.float64) / 255.0
    else:
        vals = img.astype(np.float64)
    if r.op == "gaussian":
        g = np.asarray(ifx.KernelFactors.gaussian(r.sigma).data, np.float64)
        f = -(g.size // 2)
        return [oracle.imfilter_cascade(vals, [(0, f, g), (1, f, g)], r.style)], False
    if r.op == "sobel":
        d, s = ifx.KernelFactors.sobel.gradient_pair
        return [oracle.imfilter_cascade(vals, [(0, -1, d), (1, -1, s)], r.style),
                oracle.imfilter_cascade(vals, [(0, -1, s), (1, -1, d)], r.style)], False
    if r.op == "laplacian":
        if r.kind == "N0F8":       # the N0f8 values as Float32, the Laplacian in Float32
            vals = (img.astype(np.float32) / np.float32(255)).astype(np.float64)
        return [oracle.laplacian(vals, [1, 1], r.style, 0.0, "f32")], True
    med = oracle.mapwindow_median(img.astype(np.float64), [-(r.win // 2)] * 2, [r.win] * 2, r.style)
    if r.kind == "N0F8":           # the median code as N0f8 -> Float32
        med = (med.astype(np.float32) / np.float32(255)).astype(np.float64)
    return [med], True


def test_stream_wave_against_oracle(gpu_ifx, oracle):
    """A wave of the mixed stream through one batch plan launch (the launch the
    headline throughput times), every output against the oracle."""
    ifx = gpu_ifx
    import torch
    from imagefiltering_gb300 import batch as B
    from imagefiltering_gb300 import synthetic as S
    wave = stream_wave(S)
    assert len(wave) >= 30
    assert sum(max(r.h, r.w) >= 2048 for r in wave) >= 4
    assert {r.style for r in wave} == {"replicate", "circular", "symmetric", "reflect"}
    assert {(r.kind, r.win) for r in wave if r.op == "median"} >= {("F32", 3), ("F32", 5),
                                                                   ("N0F8", 3), ("N0F8", 5)}
    assert {r.kind for r in wave if r.op == "gaussian" and r.taps() == 33} == {"F32", "N0F8"}
    bt = B.Batch()
    imgs, outs = [], []
    for r in wave:
        img = S.image_for(r)
        d = ifx.DeviceArray.from_host(ifx.n0f8(img) if r.kind == "N0F8" else img)
        op = {"gaussian": ("gaussian", r.sigma), "sobel": ("sobel",), "laplacian": ("laplacian",),
              "median": ("median", r.win)}[r.op]
        o = B.outputs_for(op, d)
        bt.add(op, d, o, r.style)
        imgs.append(img)
        outs.append(o)
    torch.cuda.synchronize()
    plan = B.Plan(bt)
    plan.launch()
    torch.cuda.synchronize()
    oracle.set_threads(16)
    worst = {}
    try:
        for r, img, o in zip(wave, imgs, outs):
            refs, exact = oracle_outputs(ifx, oracle, r, img)
            assert len(refs) == len(o)
            for got, ref in zip(o, refs):
                g = np.asarray(got.numpy(), np.float64)
                if exact:
                    assert np.array_equal(g, ref), (r, "bit-exact")
                else:
                    e = normwise(g, ref)
                    worst[r.op] = max(worst.get(r.op, 0.0), e)
                    assert e <= 1e-5, (r, e)
    finally:
        oracle.set_threads(1)
        plan.close()
    print("stream wave: %d requests, worst normwise %s" % (len(wave), worst))


def dense_kernel(seed, ksz):
    rng = np.random.default_rng(seed)
    while True:
        K = rng.standard_normal((ksz, ksz))
        if abs(K.sum()) >= 0.1:
            return K / K.sum()


@pytest.mark.parametrize("style", ["reflect", "fill"])
def test_dense_4096_tensor_cores_crops(gpu_ifx, oracle, style):
    """4096^2 Float32 uniform[0,1), 31x31 N(0,1) kernel normalised to sum 1 on the
    tensor cores (BF16 hi/lo, three products, FP32 accumulation): three interior
    512^2 crops, the first corner and a stretch of the last column edge against
    the oracle on the crop plus its 15-pixel halo (taken from the image, or
    the image's own border where the crop touches it)."""
    ifx = gpu_ifx
    img = np.asfortranarray(np.random.default_rng(2).random((4096, 4096), dtype=np.float32))
    K = dense_kernel(22, 31)
    kern = ifx.centered(K)
    b = ifx.Fill(0) if style == "fill" else ifx.Pad(style)
    got = ifx.imfilter(img, kern, b, ifx.Algorithm.GB300("tensor_cores"))
    assert got.dtype == np.float64
    h, n = 15, 512
    worst = 0.0
    for (y0, x0) in [(1024, 1536), (2048, 640), (3000, 3100), (0, 0), (1700, 4096 - n)]:
        ya, xa = max(y0 - h, 0), max(x0 - h, 0)
        yb, xb = min(y0 + n + h, 4096), min(x0 + n + h, 4096)
        sub = img[ya:yb, xa:xb].astype(np.float64)
        ref = oracle.imfilter_dense(sub, K, (-h, -h), style, 0.0)[y0 - ya:y0 - ya + n, x0 - xa:x0 - xa + n]
        e = normwise(got[y0:y0 + n, x0:x0 + n], ref)
        worst = max(worst, e)
        assert e <= 1e-5, ((y0, x0), e)
    print("dense 4096^2 31x31 %s on tensor cores: worst normwise %.3g" % (style, worst))


def test_volume_256_gaussian_then_sobel(gpu_ifx, oracle):
    """One 256^3 Float32 volume, uniform[0,1) with 1% impulse outliers set to
    1.0: Gaussian sigma=(3,3,1.5) with Pad(:symmetric) (Float64 result, FP32
    arithmetic, within 1e-5 of the oracle over the whole volume), then
    imgradients(KernelFactors.sobel, "symmetric") of that Float64 result (FP64
    arithmetic, within 1e-12 of the oracle's gradients of the same input)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(3)
    vol = rng.random((256, 256, 256), dtype=np.float32)
    vol[rng.random(vol.shape) < 0.01] = 1.0
    vol = np.asfortranarray(vol)
    k = ifx.KernelFactors.gaussian((3, 3, 1.5))
    smooth = ifx.imfilter(vol, k, "symmetric")
    assert smooth.dtype == np.float64
    oracle.set_threads(16)
    try:
        facs = [(f.axis, f.data.first[0], np.asarray(f.data.data)) for f in k]
        ref = oracle.imfilter_cascade(vol.astype(np.float64), facs, "symmetric")
        e_smooth = normwise(smooth, ref)
        assert e_smooth <= 1e-5
        del ref
        grads = ifx.imgradients(smooth, ifx.KernelFactors.sobel, "symmetric")
        assert len(grads) == 3
        d, s = ifx.KernelFactors.sobel.gradient_pair
        planes = [0, 1, 77, 128, 254, 255]
        e_grad = 0.0
        for ax, g in enumerate(grads):
            facs = [(a, -1, d if a == ax else s) for a in range(3)]
            ref = oracle.imfilter_cascade(smooth, facs, "symmetric")
            e = normwise(g, ref)
            e_grad = max(e_grad, e)
            assert e <= 1e-12, (ax, e)
            # sampled planes along every axis, max-abs against the plane's own scale
            for p in planes:
                for sl in (np.s_[p, :, :], np.s_[:, p, :], np.s_[:, :, p]):
                    assert np.max(np.abs(g[sl] - ref[sl])) <= 1e-12 * np.max(np.abs(ref))
    finally:
        oracle.set_threads(1)
    print("volume 256^3: Gaussian normwise %.3g, gradients normwise %.3g" % (e_smooth, e_grad))
