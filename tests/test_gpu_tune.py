"""The autotuner of the fused 2-D separable path: it times the candidates on
the first device-array call per key, keeps the fastest, caches the choice in
a file, and the tuned call stays within the FP32 tolerance of the oracle."""
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
        assert len(lines) == 2 and all(len(line.split()) == 10 for line in lines)
        # host arrays are not tuned
        h = np.asfortranarray(rng.random((300, 200), dtype=np.float32))
        ifx.imfilter(h, ifx.KernelFactors.gaussian((1.0, 1.0)), "reflect")
        assert ifx.autotune_choice("F32", "F64", 5, 5, False, h.shape) is None
        # a fresh load of the file restores the choices
        ifx.autotune(True, cache)
        assert ifx.autotune_choice("F32", "F32", kx, ky, False, host.shape) is not None
    finally:
        ifx.autotune(False, None)
