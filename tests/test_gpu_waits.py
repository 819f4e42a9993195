"""The device-side bounded waits, run out on purpose without any GPU fault.

The copy-fed kernels (the TMA-fed separable kernel and the batched engine)
wait for each tile's copies on an mbarrier with a bounded number of polls.
ifx_debug_force_wait_timeout sets the budget of those first waits to zero:
every such wait gives up at once, the kernel sets its error word, waits --
with its full bound -- for the copies it still has in flight, and returns.
The test checks that ifx_synchronize then reports IFX_ERR_TIMEOUT, and that
with the default budget restored the next calls are correct again.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = 6


def _force(ifx, on):
    ctx = ifx._abi.context()
    ifx._abi.check(ctx.lib.ifx_debug_force_wait_timeout(ctx.handle, 1 if on else 0))


def test_tma_separable_wait_runs_out(gpu_ifx, oracle):
    ifx = gpu_ifx
    import torch
    A = ifx._abi
    ctx = A.context()
    rng = np.random.default_rng(8)
    img = np.asfortranarray(rng.random((256, 192), dtype=np.float32))    # rows meet the copy rules
    k = ifx.KernelFactors.gaussian((2.0, 2.0))
    d = ifx.DeviceArray.from_host(img)
    torch.cuda.synchronize()
    assert ctx.lib.ifx_synchronize(ctx.handle, None) == 0
    _force(ifx, True)
    try:
        before = ifx.launch_count()
        ifx.imfilter(d, k, "replicate")
        torch.cuda.synchronize()
        assert ifx.launch_count() > before
        rc = ctx.lib.ifx_synchronize(ctx.handle, None)
        assert rc == TIMEOUT and "bounded wait" in ctx.lib.ifx_last_error().decode()
    finally:
        _force(ifx, False)
    # the timeout was reported once; the context works again
    assert ctx.lib.ifx_synchronize(ctx.handle, None) == 0
    out = ifx.imfilter(d, k, "replicate")
    torch.cuda.synchronize()
    facs = [(f.axis, f.data.first[0], np.asarray(f.data.data, np.float64)) for f in k]
    ref = oracle.imfilter_cascade(img.astype(np.float64), facs, "replicate")
    got = out.numpy()
    assert np.max(np.abs(got - ref)) / np.max(np.abs(ref)) <= 1e-5


def test_batch_wait_runs_out(gpu_ifx):
    ifx = gpu_ifx
    import torch
    from imagefiltering_gb300 import batch as B
    A = ifx._abi
    ctx = A.context()
    rng = np.random.default_rng(9)
    img = np.asfortranarray(rng.random((600, 400), dtype=np.float32))    # interior tiles arrive by copies
    d = ifx.DeviceArray.from_host(img)
    bt = B.Batch()
    outs = []
    for op in (("gaussian", 2.0), ("laplacian",), ("median", 5)):
        o = B.outputs_for(op, d)
        bt.add(op, d, o, "reflect")
        outs.append(o)
    torch.cuda.synchronize()
    plan = B.Plan(bt)
    try:
        plan.launch()
        torch.cuda.synchronize()
        good = [[x.numpy().copy() for x in o] for o in outs]
        assert ctx.lib.ifx_synchronize(ctx.handle, None) == 0
        _force(ifx, True)
        try:
            for o in outs:
                for x in o:
                    x.tensor.zero_()
            plan.launch()
            torch.cuda.synchronize()
            rc = ctx.lib.ifx_synchronize(ctx.handle, None)
            assert rc == TIMEOUT
        finally:
            _force(ifx, False)
        assert ctx.lib.ifx_synchronize(ctx.handle, None) == 0
        plan.launch()
        torch.cuda.synchronize()
        again = [[x.numpy() for x in o] for o in outs]
        for a, b in zip(good, again):
            for u, v in zip(a, b):
                assert np.array_equal(u, v)
    finally:
        plan.close()
