"""ifx_imfilter_factored_noalloc -- the separable cascade for callers that
cannot allocate device memory while they filter (a real-time frame loop that
must not stall on cudaMalloc/cudaFree, an application that reserves its whole
device-memory budget at start-up).  Its scratch is a fixed device array
compiled into the library instead of buffers the library allocates.

Checked through the C ABI against the allocating entry point
(ifx_imfilter_factored) on two calls in a row that reuse the shared scratch,
and against the oracle, within the tolerance of the other parity tests: 1e-5
normwise for Float32 images (FP32 arithmetic), 1e-12 for Float64 images.  This file is collected
last (tests/conftest.py runs test_zz_* files after the others) and also
passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dev(ifx, a):
    import torch
    d = ifx.DeviceArray.from_host(a)
    torch.cuda.synchronize()
    return d


def _desc(ifx, d):
    A = ifx._abi
    return A.describe(d.ptr(), d.kind, d.shape, d.strides())


def _factors(ifx, facs):
    A = ifx._abi
    arr = (A.IfxFactor * len(facs))()
    keep = []
    for i, (ax, first, w) in enumerate(facs):
        w = np.ascontiguousarray(w, dtype=np.float64)
        keep.append(w)
        arr[i].axis, arr[i].length, arr[i].first, arr[i].weights = ax, w.size, first, A.dptr(w)
    return arr, keep


def _run_both(ifx, img, facs, style, out_kind):
    """(no-alloc result, allocating result) for one image."""
    import torch
    A = ifx._abi
    ctx = A.context()
    d_in = _dev(ifx, img)
    d_a = ifx.DeviceArray.empty(img.shape, out_kind)
    d_b = ifx.DeviceArray.empty(img.shape, out_kind)
    arr, keep = _factors(ifx, facs)
    b = A.border_struct(style, None, None, 0.25 if style == "fill" else 0.0)
    stream = ifx.arrays.torch_stream()
    A.check(ctx.lib.ifx_imfilter_factored_noalloc(_desc(ifx, d_a), _desc(ifx, d_in), len(facs), arr,
                                                  C.byref(b), stream))
    A.check(ctx.lib.ifx_imfilter_factored(ctx.handle, _desc(ifx, d_b), _desc(ifx, d_in), len(facs), arr,
                                          C.byref(b), stream))
    torch.cuda.synchronize()
    return d_a.numpy(), d_b.numpy()


def _normwise(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_noalloc_matches_allocating_entry_point(gpu_ifx, oracle):
    ifx = gpu_ifx
    rng = np.random.default_rng(17)
    g13 = np.asarray(ifx.KernelFactors.gaussian(3.0).data)
    g9 = np.asarray(ifx.KernelFactors.gaussian(1.5).data)
    # call 1: a 3-D Float32 volume, three factors (two intermediate buffers)
    vol = np.asfortranarray(rng.random((96, 80, 40), dtype=np.float32))
    facs3 = [(0, -6, g13), (1, -6, g13), (2, -4, g9)]
    a1, b1 = _run_both(ifx, vol, facs3, "symmetric", "F64")
    # call 2, right after, reusing the same scratch: a 2-D Float64 image with a
    # repeated axis and a Fill border
    img = np.asfortranarray(rng.random((300, 211)))
    facs2 = [(0, -1, np.ones(3) / 3), (1, -6, g13), (0, -2, rng.standard_normal(5))]
    a2, b2 = _run_both(ifx, img, facs2, "fill", "F64")
    assert _normwise(a1, b1) <= 1e-5
    assert _normwise(a2, b2) <= 1e-12
    # both against the oracle (pad-then-cascade in FP64)
    assert _normwise(a1, oracle.imfilter_cascade(vol.astype(np.float64), facs3, "symmetric")) <= 1e-5
    assert _normwise(a2, oracle.imfilter_cascade(img, facs2, "fill", 0.25)) <= 1e-12
    # and the first result again, after the scratch was overwritten by call 2
    a3, _ = _run_both(ifx, vol, facs3, "symmetric", "F64")
    assert np.array_equal(a3, a1)


def test_noalloc_rejects_oversize_and_host_arrays(gpu_ifx):
    ifx = gpu_ifx
    A = ifx._abi
    lib = A.context().lib
    cap = int(lib.ifx_noalloc_scratch_bytes())
    assert cap == 32 << 20
    # a volume whose padded box alone exceeds the fixed scratch: rejected before any launch
    n = 256
    big = ifx.DeviceArray.empty((n, n, n), "F32")
    out = ifx.DeviceArray.empty((n, n, n), "F32")
    g = np.asarray(ifx.KernelFactors.gaussian(1.0).data)
    arr, keep = _factors(ifx, [(0, -2, g), (1, -2, g), (2, -2, g)])
    b = A.border_struct("replicate")
    rc = lib.ifx_imfilter_factored_noalloc(_desc(ifx, out), _desc(ifx, big), 3, arr, C.byref(b), None)
    assert rc == 5 and "fixed scratch" in lib.ifx_last_error().decode()
    # host arrays need staging buffers, which this entry point does not allocate
    h = np.asfortranarray(np.zeros((16, 16), np.float32))
    ho = np.asfortranarray(np.zeros((16, 16), np.float32))
    hi = A.describe(h.ctypes.data, "F32", h.shape)
    hout = A.describe(ho.ctypes.data, "F32", ho.shape)
    arr1, keep1 = _factors(ifx, [(0, -2, g)])
    rc = lib.ifx_imfilter_factored_noalloc(hout, hi, 1, arr1, C.byref(b), None)
    assert rc == 1 and "device arrays only" in lib.ifx_last_error().decode()


def test_noalloc_copy_factors_and_long_factors(gpu_ifx):
    """Factors that are all identity copies take the conversion-only branch (no
    scratch): the output is the input in the output eltype.  Factors longer
    than 129 taps are refused before any launch."""
    ifx = gpu_ifx
    A = ifx._abi
    lib = A.context().lib
    rng = np.random.default_rng(3)
    img = np.asfortranarray(rng.random((70, 33), dtype=np.float32))
    a, b = _run_both(ifx, img, [(0, 0, np.ones(1)), (1, 0, np.ones(1))], "replicate", "F64")
    assert np.array_equal(a, img.astype(np.float64)) and np.array_equal(a, b)
    d_in = _dev(ifx, img)
    d_out = ifx.DeviceArray.empty(img.shape, "F64")
    arr, keep = _factors(ifx, [(0, -65, np.ones(131) / 131)])
    bd = A.border_struct("replicate")
    rc = lib.ifx_imfilter_factored_noalloc(_desc(ifx, d_out), _desc(ifx, d_in), 1, arr, C.byref(bd), None)
    assert rc == 7 and "129 taps" in lib.ifx_last_error().decode()


def test_noalloc_rejects_arrays_of_another_device(gpu_ifx):
    """The scratch used is the current device's: arrays on another GPU are
    refused before any launch (needs two GPUs)."""
    import torch
    if torch.cuda.device_count() < 2:
        pytest.skip("one GPU visible")
    ifx = gpu_ifx
    A = ifx._abi
    lib = A.context().lib
    other = torch.zeros((16, 16), dtype=torch.float32, device="cuda:1")
    out = torch.zeros((16, 16), dtype=torch.float32, device="cuda:1")
    g = np.asarray(ifx.KernelFactors.gaussian(1.0).data)
    arr, keep = _factors(ifx, [(0, -2, g)])
    bd = A.border_struct("replicate")
    with torch.cuda.device(0):
        rc = lib.ifx_imfilter_factored_noalloc(A.describe(out.data_ptr(), "F32", (16, 16)),
                                               A.describe(other.data_ptr(), "F32", (16, 16)), 1, arr,
                                               C.byref(bd), None)
    assert rc == 1 and "device 1" in lib.ifx_last_error().decode()
