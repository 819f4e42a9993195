"""The batched engine (one persistent launch over a tile work-queue) against
the oracle, and each request's result alone versus inside a mixed batch."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STYLES = ["replicate", "circular", "symmetric", "reflect", "fill"]


def normwise(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def rand_img(ifx, rng, h, w, kind):
    if kind == "F32":
        a = np.asfortranarray(rng.random((h, w), dtype=np.float32))
    else:
        a = np.asfortranarray(rng.integers(0, 256, (h, w), dtype=np.uint8))
        if kind == "N0F8":
            a = ifx.n0f8(a)
    return a


def mixed_requests(ifx, seed=0, n=60):
    rng = np.random.default_rng(seed)
    ops = [("gaussian", 0.7), ("gaussian", 3.3), ("gaussian", 8.0), ("sobel",), ("prewitt",),
           ("laplacian",), ("median", 3), ("median", 5)]
    out = []
    for i in range(n):
        h = int(rng.integers(1, 300)) if i % 7 else int(rng.integers(64, 700))
        w = int(rng.integers(2, 300))
        kind = ["F32", "N0F8", "U8"][i % 3]
        op = ops[int(rng.integers(0, len(ops)))]
        style = STYLES[int(rng.integers(0, 5))]
        if style == "reflect" and (h == 1 or w == 1):
            style = "symmetric"
        if op[0] == "laplacian" and kind == "U8":
            kind = "N0F8"
        fill = {"F32": 0.3, "N0F8": 0.6, "U8": 17}[kind]
        border = ifx.Fill(fill) if style == "fill" else ifx.Pad(style)
        out.append((rand_img(ifx, rng, h, w, kind), op, border))
    return out


def reference_call(ifx, img, op, border):
    """The same request through the single-request API (host arrays)."""
    name = op[0]
    if name == "gaussian":
        return [ifx.imfilter(img, ifx.KernelFactors.gaussian((op[1], op[1])), border)]
    if name in ("sobel", "prewitt"):
        return list(ifx.imgradients(img, getattr(ifx.KernelFactors, name), border))
    if name == "laplacian":
        return [ifx.imfilter(img, ifx.Kernel.Laplacian(), border)]
    return [ifx.mapwindow(ifx.median, img, (op[1], op[1]), border=border)]


def run_batch(ifx, items):
    from imagefiltering_gb300 import batch as B
    import torch
    bt = B.Batch()
    outs = []
    for img, op, border in items:
        d = ifx.DeviceArray.from_host(img)
        o = B.outputs_for(op, d)
        bt.add(op, d, o, border)
        outs.append(o)
    tiles = bt.run()
    torch.cuda.synchronize()
    return [[x.numpy() for x in o] for o in outs], tiles


def test_batch_matches_single_calls(gpu_ifx):
    ifx = gpu_ifx
    items = mixed_requests(ifx)
    got, tiles = run_batch(ifx, items)
    assert tiles > len(items)
    for (img, op, border), outs in zip(items, got):
        ref = reference_call(ifx, img, op, border)
        assert len(ref) == len(outs)
        for g, r in zip(outs, ref):
            assert g.dtype == np.asarray(r).dtype, op
            if op[0] in ("laplacian", "median"):
                assert np.array_equal(g, r), (op, img.shape, border)
            else:
                assert normwise(g, r) <= 1e-6, (op, img.shape, border)


def test_batch_against_oracle(gpu_ifx, oracle):
    ifx = gpu_ifx
    items = mixed_requests(ifx, seed=1, n=40)
    got, _ = run_batch(ifx, items)
    for (img, op, border), outs in zip(items, got):
        kind = "N0F8" if isinstance(img, ifx.N0f8Array) else ("U8" if img.dtype == np.uint8 else "F32")
        vals = img.astype(np.float64) / 255.0 if kind == "N0F8" else img.astype(np.float64)
        style = "fill" if isinstance(border, ifx.Fill) else border.style
        fv = 0.0
        if style == "fill":
            fv = {"F32": float(np.float32(0.3)), "N0F8": round(0.6 * 255) / 255.0, "U8": 17.0}[kind]
        if op[0] == "gaussian":
            k = np.asarray(ifx.KernelFactors.gaussian(op[1]).data)
            ref = oracle.imfilter_cascade(vals, [(0, -(k.size // 2), k), (1, -(k.size // 2), k)], style, fv)
            assert normwise(outs[0], ref) <= 1e-5
        elif op[0] in ("sobel", "prewitt"):
            d, s = getattr(ifx.KernelFactors, op[0]).gradient_pair
            for ax, g in enumerate(outs):
                facs = [(0, -1, d if ax == 0 else s), (1, -1, s if ax == 0 else d)]
                ref = oracle.imfilter_cascade(vals, facs, style, fv)
                assert normwise(g, ref) <= 1e-5 or np.max(np.abs(g - ref)) < 1e-6
        elif op[0] == "median":
            codes = img.astype(np.float64)
            ref = oracle.mapwindow_median(codes, [-(op[1] // 2)] * 2, [op[1]] * 2, style,
                                          {"F32": fv, "N0F8": round(0.6 * 255), "U8": 17.0}[kind]
                                          if style == "fill" else 0.0)
            if kind == "N0F8":
                ref = ref.astype(np.float32) / np.float32(255)
            assert np.array_equal(np.asarray(outs[0], np.float64), np.asarray(ref, np.float64)), (img.shape, style)


def test_same_alone_and_in_the_mix(gpu_ifx):
    """Each request gives bit-identical results alone and inside a mixed batch."""
    ifx = gpu_ifx
    items = mixed_requests(ifx, seed=2, n=24)
    mixed, _ = run_batch(ifx, items)
    for item, outs in zip(items, mixed):
        alone, _ = run_batch(ifx, [item])
        for a, b in zip(alone[0], outs):
            assert np.array_equal(a, b)


def test_batch_rejects_host_memory(gpu_ifx):
    ifx = gpu_ifx
    from imagefiltering_gb300 import batch as B
    bt = B.Batch()
    img = np.asfortranarray(np.zeros((8, 8), np.float32))
    out = np.asfortranarray(np.zeros((8, 8), np.float32))
    bt.add(("laplacian",), img, [out])
    with pytest.raises(ifx.ArgumentError, match="device memory"):
        bt.run()


def test_plan_replays_match_batch_run(gpu_ifx):
    """A validated plan launched twice gives the batch results both times."""
    ifx = gpu_ifx
    import torch
    from imagefiltering_gb300 import batch as B
    items = mixed_requests(ifx, seed=5, n=20)
    bt = B.Batch()
    outs = []
    for img, op, border in items:
        d = ifx.DeviceArray.from_host(img)
        o = B.outputs_for(op, d)
        bt.add(op, d, o, border)
        outs.append(o)
    torch.cuda.synchronize()
    bt.run()
    torch.cuda.synchronize()
    first = [[x.numpy() for x in o] for o in outs]
    plan = B.Plan(bt)
    for _ in range(2):
        for o in outs:
            for x in o:
                x.tensor.zero_()
        plan.launch()
        torch.cuda.synchronize()
        again = [[x.numpy() for x in o] for o in outs]
        for a, b in zip(first, again):
            for u, v in zip(a, b):
                assert np.array_equal(u, v)
    plan.close()
