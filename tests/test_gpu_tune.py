"""The autotuner of the separable paths: it times the candidates on the
first device-array call per key, keeps the fastest, caches the choice in a
file, and the tuned call stays within the FP32 tolerance of the oracle; every
value of every tuned parameter, pinned, stays within it too."""
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def normwise(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_autotune_separable(gpu_ifx, oracle, tmp_path):
    ifx = gpu_ifx
    cache = tmp_path / "tune.txt"
    rng = np.random.default_rng(303)
    host = np.asfortranarray(rng.random((1000, 777), dtype=np.float32))
    img = ifx.DeviceArray.from_host(host)
    k = ifx.KernelFactors.gaussian((2.5, 1.5))
    facs = [(f.axis, f.data.first[0], np.asarray(f.data.data, np.float64)) for f in k]
    kx, ky = (len(f.data) for f in k)
    try:
        ifx.autotune_clear()
        ifx.autotune(True, cache)
        for style, border, okind in [("replicate", "replicate", "F32"), ("fill", ifx.Fill(0.25), "F64")]:
            assert ifx.autotune_choice("F32", okind, kx, ky, style == "fill", host.shape) is None
            out = ifx.DeviceArray.empty(host.shape, okind)
            ifx.imfilter_(out, img, k, border)
            first = out.numpy().copy()
            choice = ifx.autotune_choice("F32", okind, kx, ky, style == "fill", host.shape)
            assert choice is not None and choice[0] in (0, 1) and choice[1] in (1, 2) and choice[2] > 0
            ref = oracle.imfilter_cascade(host.astype(np.float64), facs, style, float(np.float32(0.25)))
            assert normwise(first, ref) <= 1e-5
            ifx.imfilter_(out, img, k, border)               # cached: same candidate, same bits
            assert np.array_equal(out.numpy(), first)
        lines = cache.read_text().strip().splitlines()
        assert len(lines) == 2 and all(line.split()[0] == "t2" and len(line.split()) == 16 for line in lines)
        # host arrays are not tuned
        h = np.asfortranarray(rng.random((300, 200), dtype=np.float32))
        ifx.imfilter(h, ifx.KernelFactors.gaussian((1.0, 1.0)), "reflect")
        assert ifx.autotune_choice("F32", "F64", 5, 5, False, h.shape) is None
        # a fresh load of the file restores the choices
        ifx.autotune(True, cache)
        assert ifx.autotune_choice("F32", "F32", kx, ky, False, host.shape) is not None
    finally:
        ifx.autotune(False, None)
        ifx.autotune_clear()


# ---------------------------------------------------------------- every tuned parameter
STYLES = ["replicate", "circular", "symmetric", "reflect", "fill"]


def _img(rng, shape, kind):
    if kind == "F32":
        return np.asfortranarray(rng.random(shape, dtype=np.float32))
    if kind == "F64":
        return np.asfortranarray(rng.random(shape))
    return np.asfortranarray(rng.integers(0, 256, shape, dtype=np.uint8))


def _values(img, kind):
    return img.astype(np.float64) / 255.0 if kind == "N0F8" else img.astype(np.float64)


# (variant, tile widths, tile heights) per compute type: the TMA kernel takes
# 64 / 128 wide tiles, the gather kernel 64 / 128 (FP32) or 32 / 64 (FP64)
TILES_2D = {"tma": (1, (64, 128), (8, 16, 24, 48, 96, 128)),
            "gather32": (2, (64, 128), (8, 16, 40, 64, 128)),
            "gather64": (2, (32, 64), (8, 24, 32, 64))}


@pytest.mark.parametrize("kind", ["F32", "N0F8", "F64"])
@pytest.mark.parametrize("style", STYLES)
def test_pinned_2d_choices(gpu_ifx, oracle, kind, style):
    """Every value of every tuned 2-D parameter -- kernel, pass order, tile
    width, tile height -- pinned in turn, on images with partial edge tiles:
    each result within the tolerance of the oracle, and the tile shape does
    not change a single output's arithmetic (the same bits for every shape of
    one kernel and pass order)."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("pin2d" + kind + style).encode()))
    shape = (336, 203)                         # rows meet the 16-byte rule: the TMA kernel applies
    img = _img(rng, shape, kind)
    src = ifx.n0f8(img) if kind == "N0F8" else img
    kx, ky = 13, 21
    wx, wy = rng.standard_normal(kx), rng.standard_normal(ky)
    facs = [(0, -6, wx), (1, -11, wy)]
    ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w, (f,)), 2, ax) for ax, f, w in facs)
    border = ifx.Fill(0.7) if style == "fill" else ifx.Pad(style)
    fv = {"F32": float(np.float32(0.7)), "F64": 0.7, "N0F8": round(0.7 * 255) / 255.0}[kind]
    ref = oracle.imfilter_cascade(_values(img, kind), facs, style, fv)
    tol = 1e-12 if kind == "F64" else 1e-5
    groups = ["gather64"] if kind == "F64" else ["tma", "gather32"]
    try:
        for g in groups:
            variant, widths, heights = TILES_2D[g]
            for x_first in (1, 0):
                first = None
                for tw in widths:
                    for th in heights:
                        ifx.autotune_pin(kind, "F64", (kx, ky), style == "fill", shape, variant=variant,
                                         x_first=x_first, tile_w=tw, tile_h=th)
                        got = ifx.imfilter(src, ks, border)
                        assert got.dtype == np.float64
                        assert normwise(got, ref) <= tol, (g, x_first, tw, th)
                        if first is None:
                            first = got
                        else:
                            assert np.array_equal(got, first), (g, x_first, tw, th)
    finally:
        ifx.autotune_clear()


@pytest.mark.parametrize("kind", ["F32", "N0F8"])
@pytest.mark.parametrize("style", ["symmetric", "fill", "circular"])
def test_pinned_3d_choices(gpu_ifx, oracle, kind, style):
    """3-D: the split sweeps with every x/y tile shape, and the fused
    z-marching kernel with every z chunk depth (chunks shorter than, equal
    to and longer than the z factor's halo), pinned in turn."""
    ifx = gpu_ifx
    rng = np.random.default_rng(zlib.crc32(("pin3d" + kind + style).encode()))
    shape = (68, 45, 37)
    img = _img(rng, shape, kind)
    src = ifx.n0f8(img) if kind == "N0F8" else img
    taps = (9, 7, 11)
    facs = [(ax, -(taps[ax] // 2), rng.standard_normal(taps[ax])) for ax in range(3)]
    ks = tuple(ifx.ReshapedOneD(ifx.OffsetKernel(w, (f,)), 3, ax) for ax, f, w in facs)
    border = ifx.Fill(0.7) if style == "fill" else ifx.Pad(style)
    fv = {"F32": float(np.float32(0.7)), "N0F8": round(0.7 * 255) / 255.0}[kind]
    ref = oracle.imfilter_cascade(_values(img, kind), facs, style, fv)
    try:
        split = [dict(variant=1, tile_w=tw, tile_h=th) for tw, th in [(0, 0), (64, 16), (64, 64), (128, 32),
                                                                      (128, 96)]]
        fused = [dict(variant=2, depth=d) for d in (4, 5, 8, 16, 37, 64)]
        for ch in split + fused:
            ifx.autotune_pin(kind, "F64", taps, style == "fill", shape, **ch)
            got = ifx.imfilter(src, ks, border)
            assert normwise(got, ref) <= 1e-5, ch
    finally:
        ifx.autotune_clear()


def test_autotune_widened(gpu_ifx, oracle, tmp_path):
    """The tuner picks a tile shape for the 2-D path and a z strategy (with a
    tile shape or a chunk depth) for the 3-D path, stores them in the cache
    file, and a fresh load restores them."""
    ifx = gpu_ifx
    cache = tmp_path / "tune2.txt"
    rng = np.random.default_rng(404)
    try:
        ifx.autotune_clear()
        ifx.autotune(True, cache)
        h2 = np.asfortranarray(rng.random((1024, 600), dtype=np.float32))
        k2 = ifx.KernelFactors.gaussian((2.0, 3.0))
        taps2 = tuple(len(f.data) for f in k2)
        out2 = ifx.DeviceArray.empty(h2.shape, "F64")
        ifx.imfilter_(out2, ifx.DeviceArray.from_host(h2), k2, "reflect")
        c2 = ifx.autotune_lookup("F32", "F64", taps2, False, h2.shape)
        assert c2 is not None and c2["variant"] in (1, 2) and c2["tile_w"] in (64, 128) and c2["tile_h"] >= 8
        facs2 = [(f.axis, f.data.first[0], np.asarray(f.data.data, np.float64)) for f in k2]
        assert normwise(out2.numpy(), oracle.imfilter_cascade(h2.astype(np.float64), facs2, "reflect")) <= 1e-5

        h3 = np.asfortranarray(rng.random((96, 80, 64), dtype=np.float32))
        k3 = ifx.KernelFactors.gaussian((1.5, 1.5, 1.0))
        taps3 = tuple(len(f.data) for f in k3)
        out3 = ifx.DeviceArray.empty(h3.shape, "F64")
        ifx.imfilter_(out3, ifx.DeviceArray.from_host(h3), k3, "symmetric")
        c3 = ifx.autotune_lookup("F32", "F64", taps3, False, h3.shape)
        assert c3 is not None and c3["variant"] in (1, 2)
        assert (c3["variant"] == 2 and c3["depth"] >= 4) or c3["variant"] == 1
        facs3 = [(f.axis, f.data.first[0], np.asarray(f.data.data, np.float64)) for f in k3]
        assert normwise(out3.numpy(), oracle.imfilter_cascade(h3.astype(np.float64), facs3, "symmetric")) <= 1e-5

        lines = [ln.split() for ln in cache.read_text().strip().splitlines()]
        assert len(lines) == 2 and all(ln[0] == "t2" and len(ln) == 16 for ln in lines)
        ifx.autotune_clear()
        assert ifx.autotune_lookup("F32", "F64", taps2, False, h2.shape) is None
        ifx.autotune(True, cache)
        for taps, shape, c in ((taps2, h2.shape, c2), (taps3, h3.shape, c3)):
            got = ifx.autotune_lookup("F32", "F64", taps, False, shape)
            assert got is not None and abs(got.pop("ms") - c.pop("ms")) < 1e-5 and got == c   # ms: 6 decimals
    finally:
        ifx.autotune(False, None)
        ifx.autotune_clear()


# ---------------------------------------------------------------- the batched engine's tiles
def _batch_items(ifx, rng, op, kind, n=10):
    items = []
    for i in range(n):
        h, w = int(rng.integers(1, 420)), int(rng.integers(2, 700))
        style = STYLES[int(rng.integers(0, 5))]
        if style == "reflect" and (h == 1 or w == 1):
            style = "symmetric"
        fill = {"F32": 0.3, "N0F8": 0.6, "U8": 17}[kind]
        border = ifx.Fill(fill) if style == "fill" else ifx.Pad(style)
        img = _img(rng, (h, w), kind)
        items.append((ifx.n0f8(img) if kind == "N0F8" else img, op, border))
    return items


def _batch_oracle(ifx, oracle, img, op, border):
    kind = "N0F8" if isinstance(img, ifx.N0f8Array) else ("U8" if img.dtype == np.uint8 else "F32")
    vals = img.astype(np.float64) / 255.0 if kind == "N0F8" else img.astype(np.float64)
    style = "fill" if isinstance(border, ifx.Fill) else border.style
    fv = {"F32": float(np.float32(0.3)), "N0F8": round(0.6 * 255) / 255.0, "U8": 17.0}[kind] if style == "fill" \
        else 0.0
    if op[0] == "gaussian":
        k = np.asarray(ifx.KernelFactors.gaussian(op[1]).data)
        return [oracle.imfilter_cascade(vals, [(0, -(k.size // 2), k), (1, -(k.size // 2), k)], style, fv)]
    if op[0] == "sobel":
        d, s = ifx.KernelFactors.sobel.gradient_pair
        return [oracle.imfilter_cascade(vals, [(0, -1, d if ax == 0 else s), (1, -1, s if ax == 0 else d)], style,
                                        fv) for ax in range(2)]
    vals32 = (img.astype(np.float32) / np.float32(255)).astype(np.float64) if kind == "N0F8" else vals
    fv32 = float(np.float32(round(0.6 * 255)) / np.float32(255)) if kind == "N0F8" else float(np.float32(fv))
    return [oracle.laplacian(vals32, [1, 1], style, fv32 if style == "fill" else 0.0, "f32")]


@pytest.mark.parametrize("op,kind,tiles", [
    (("gaussian", 2.0), "N0F8", [(64, 56), (64, 24), (128, 56), (128, 24), (256, 56), (256, 24)]),
    (("gaussian", 7.5), "U8", [(64, 32), (128, 16), (256, 32)]),
    (("gaussian", 1.2), "F32", [(64, 56), (64, 24)]),
    (("sobel",), "N0F8", [(88, 56), (176, 56), (352, 56)]),
    (("laplacian",), "N0F8", [(88, 56), (176, 56), (352, 56)]),
])
def test_batch_pinned_tiles(gpu_ifx, oracle, op, kind, tiles):
    """Every tile the batched engine's tuner may pick, pinned in turn: the
    batch's results against the oracle (Laplacian exact), and the same bits
    for every tile (the tile does not change an output's arithmetic)."""
    ifx = gpu_ifx
    import torch
    from imagefiltering_gb300 import batch as B
    rng = np.random.default_rng(zlib.crc32(repr((op, kind)).encode()))
    items = _batch_items(ifx, rng, op, kind)
    name = {"gaussian": "factored", "sobel": "gradients", "laplacian": "laplacian"}[op[0]]
    taps = len(ifx.KernelFactors.gaussian(op[1]).data) if op[0] == "gaussian" else 3
    refs = [_batch_oracle(ifx, oracle, img, o, b) for img, o, b in items]
    first = None
    try:
        for tw, th in tiles:
            B.autotune_pin(name, kind, B.out_kinds(op)[0] if op[0] != "laplacian" else "F32", tw, th, taps, taps)
            bt = B.Batch()
            outs = []
            for img, o, border in items:
                d = ifx.DeviceArray.from_host(img)
                oo = B.outputs_for(o, d)
                bt.add(o, d, oo, border)
                outs.append(oo)
            bt.run()
            torch.cuda.synchronize()
            got = [[x.numpy() for x in oo] for oo in outs]
            for g, r, (img, _, border) in zip(got, refs, items):
                for a, b in zip(g, r):
                    if op[0] == "laplacian":
                        assert np.array_equal(np.asarray(a, np.float64), b), (tw, th, img.shape, border)
                    else:
                        assert normwise(a, b) <= 1e-5 or np.max(np.abs(a - b)) < 1e-6, (tw, th, img.shape)
            if first is None:
                first = got
            else:
                for u, v in zip(first, got):
                    for a, b in zip(u, v):
                        assert np.array_equal(a, b), (tw, th)
    finally:
        ifx.autotune_clear()


def test_batch_plan_tuned_on_first_launch(gpu_ifx, oracle):
    """With the tuner enabled, a plan's first launch times the candidate tiles
    of its keys, caches the fastest, and its results match the untuned run."""
    ifx = gpu_ifx
    import torch
    from imagefiltering_gb300 import batch as B
    rng = np.random.default_rng(77)
    items = _batch_items(ifx, rng, ("gaussian", 3.0), "N0F8", n=12) + \
        _batch_items(ifx, rng, ("laplacian",), "N0F8", n=6)
    bt = B.Batch()
    outs = []
    for img, o, border in items:
        d = ifx.DeviceArray.from_host(img)
        oo = B.outputs_for(o, d)
        bt.add(o, d, oo, border)
        outs.append(oo)
    try:
        ifx.autotune_clear()
        bt.run()
        torch.cuda.synchronize()
        base = [[x.numpy() for x in oo] for oo in outs]
        plan = B.Plan(bt)
        ifx.autotune(True, None)
        plan.launch()
        torch.cuda.synchronize()
        taps = len(ifx.KernelFactors.gaussian(3.0).data)
        cf = B.autotune_lookup("factored", "N0F8", "F64", taps, taps)
        cl = B.autotune_lookup("laplacian", "N0F8", "F32")
        assert cf is not None and cf["tile_w"] in (64, 128, 256) and cf["ms"] > 0
        assert cl is not None and cl["tile_w"] in (88, 176, 352)
        again = [[x.numpy() for x in oo] for oo in outs]
        for u, v in zip(base, again):
            for a, b in zip(u, v):
                assert np.array_equal(a, b)
        plan.close()
    finally:
        ifx.autotune(False, None)
        ifx.autotune_clear()
