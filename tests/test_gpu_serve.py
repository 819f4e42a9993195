"""The serving loop: continuous batching under an HBM cap, host and device
arrays, results equal to the single-request API, latency metrics, bounded
waits (a wait that runs out returns a timeout status, nothing hangs)."""
import time

import numpy as np
import pytest

from test_gpu_batch import mixed_requests, reference_call

pytestmark = pytest.mark.gpu


def host_outputs(ifx, img, op):
    from imagefiltering_gb300 import batch as B
    kinds = B.out_kinds(op)
    if op[0] == "median":
        kind = "N0F8" if isinstance(img, ifx.N0f8Array) else ("U8" if img.dtype == np.uint8 else "F32")
        kinds = [B.MEDIAN_OUT[kind]]
    return [np.empty(img.shape, dtype=np.float64 if k == "F64" else np.float32, order="F") for k in kinds]


def check_outputs(ifx, items, outs):
    for (img, op, border), got in zip(items, outs):
        ref = reference_call(ifx, img, op, border)
        for g, r in zip(got, ref):
            if op[0] in ("laplacian", "median"):
                assert np.array_equal(g, r), (op, img.shape)
            else:
                d = np.max(np.abs(g - r)) / max(np.max(np.abs(r)), 1e-300)
                assert d <= 1e-6, (op, img.shape)


def test_server_host_arrays_match_single_calls(gpu_ifx):
    ifx = gpu_ifx
    from imagefiltering_gb300.serve import Server
    items = mixed_requests(ifx, seed=3, n=50)
    with Server(hbm_cap_bytes=1 << 30, max_batch=16) as srv:
        outs, tickets = [], []
        for img, op, border in items:
            o = host_outputs(ifx, img, op)
            outs.append(o)
            tickets.append(srv.submit(op, img, o, border))
        for t in tickets:
            srv.wait(t, timeout=60)
        m = srv.metrics()
    assert m["completed"] == len(items) and m["failed"] == 0
    assert m["batches"] >= 4                      # max_batch 16 -> several launches
    assert 0 < m["p50_latency_s"] <= m["p99_latency_s"]
    check_outputs(ifx, items, outs)


def test_server_admission_under_a_small_cap(gpu_ifx):
    """Total device footprint far above the cap: everything completes and the
    server never holds more than the cap."""
    ifx = gpu_ifx
    from imagefiltering_gb300.serve import Server
    rng = np.random.default_rng(9)
    cap = 24 << 20
    items = []
    for i in range(40):
        img = np.asfortranarray(rng.random((512, 512), dtype=np.float32))   # 1 MiB in, 2-4 MiB out
        items.append((img, ("gaussian", 1.5) if i % 2 else ("median", 5), ifx.Pad("reflect")))
    with Server(hbm_cap_bytes=cap, max_batch=8) as srv:
        outs = [host_outputs(ifx, img, op) for img, op, b in items]
        ts = [srv.submit(op, img, o, b) for (img, op, b), o in zip(items, outs)]
        srv.drain(timeout=120)
        m = srv.metrics()
        for t in ts:
            srv.wait(t, timeout=1)
    assert m["completed"] == 40
    assert m["hbm_peak"] <= cap
    check_outputs(ifx, items[:6], outs[:6])


def test_server_device_arrays_and_arrivals(gpu_ifx):
    """Device-resident requests arriving while earlier ones run."""
    ifx = gpu_ifx
    import torch
    from imagefiltering_gb300 import batch as B
    from imagefiltering_gb300.serve import Server
    items = mixed_requests(ifx, seed=4, n=30)
    with Server(hbm_cap_bytes=1 << 30, max_batch=4) as srv:
        douts, ts = [], []
        for img, op, border in items:
            d = ifx.DeviceArray.from_host(img)
            torch.cuda.synchronize()
            o = B.outputs_for(op, d)
            douts.append(o)
            ts.append(srv.submit(op, d, o, border))
            time.sleep(0.0005)
        for t in ts:
            srv.wait(t, timeout=60)
    check_outputs(ifx, items, [[x.numpy() for x in o] for o in douts])


def test_server_bounded_wait_and_oversize(gpu_ifx):
    ifx = gpu_ifx
    from imagefiltering_gb300.serve import Server
    img = np.asfortranarray(np.ones((2048, 2048), np.float32))
    out = [np.empty((2048, 2048), np.float64, order="F")]
    with Server(hbm_cap_bytes=8 << 20, max_batch=4) as srv:
        with pytest.raises(ifx.OutOfMemory):
            srv.submit(("gaussian", 2.0), img, out)          # needs 48 MiB > cap
        small = np.asfortranarray(np.ones((64, 64), np.float32))
        so = [np.empty((64, 64), np.float32, order="F")]
        t = srv.submit(("median", 3), small, so)
        try:
            srv.wait(t, timeout=0.0)                          # may or may not be done yet
        except TimeoutError:
            srv.wait(t, timeout=30)
        assert np.all(so[0] == 1.0)


def test_server_concurrent_submitters(gpu_ifx):
    """Four host threads submit and wait at once (the C calls release the
    GIL): every result equals the single-request API, the ramp of batch sizes
    after idle periods included."""
    import threading
    ifx = gpu_ifx
    from imagefiltering_gb300.serve import Server
    items = mixed_requests(ifx, seed=11, n=64)
    outs = [host_outputs(ifx, img, op) for img, op, _ in items]
    errors = []
    with Server(hbm_cap_bytes=1 << 30, max_batch=8, max_inflight=3) as srv:
        def worker(k):
            try:
                for i in range(k, len(items), 4):
                    img, op, border = items[i]
                    t = srv.submit(op, img, outs[i], border)
                    srv.wait(t, timeout=60.0)
            except Exception as e:            # reported on the main thread
                errors.append(e)
        threads = [threading.Thread(target=worker, args=(k,)) for k in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        m = srv.metrics()
    assert not errors, errors
    assert m["completed"] >= len(items)
    check_outputs(ifx, items, outs)


def test_server_cancel_before_launch(gpu_ifx):
    """Requests cancelled while queued or admitted complete as Cancelled and
    give their device memory back; the others complete correctly."""
    ifx = gpu_ifx
    from imagefiltering_gb300.serve import Server
    items = mixed_requests(ifx, seed=21, n=40)
    outs = [host_outputs(ifx, img, op) for img, op, _ in items]
    with Server(hbm_cap_bytes=1 << 30, max_batch=4, max_inflight=1) as srv:
        srv.pause(True)                          # requests are admitted but wait for launch
        tickets = [srv.submit(op, img, o, border) for (img, op, border), o in zip(items, outs)]
        cancelled = set()
        for i in range(30, 40):
            srv.cancel(tickets[i])
            cancelled.add(i)
        srv.pause(False)
        img0, op0, border0 = items[0]
        done = srv.submit(op0, img0, host_outputs(ifx, img0, op0), border0)
        srv.wait(done, timeout=60)
        with pytest.raises(ifx.ArgumentError):  # waited for: unknown to the server now
            srv.cancel(done)
        for i, t in enumerate(tickets):
            if i in cancelled:
                with pytest.raises(ifx.Cancelled):
                    srv.wait(t, timeout=60)
            else:
                srv.wait(t, timeout=60)
        srv.drain()
        m = srv.metrics()
    assert len(cancelled) == 10
    assert m["completed"] == len(items) + 1 - len(cancelled) and m["failed"] == len(cancelled)
    assert m["hbm_in_use"] == 0
    keep = [i for i in range(len(items)) if i not in cancelled]
    check_outputs(ifx, [items[i] for i in keep], [outs[i] for i in keep])


def test_server_injected_launch_failure(gpu_ifx):
    """A batched launch reported failed (injected on the host, no GPU fault):
    its requests fail with CudaError, their memory is released, and the
    server goes on serving correct results."""
    ifx = gpu_ifx
    from imagefiltering_gb300.serve import Server
    items = mixed_requests(ifx, seed=22, n=16)
    outs = [host_outputs(ifx, img, op) for img, op, _ in items]
    with Server(hbm_cap_bytes=1 << 30, max_batch=8, max_inflight=1) as srv:
        srv.pause(True)                          # all eight join the one failing launch
        srv.inject_launch_error(1)
        first = [srv.submit(op, img, o, border) for (img, op, border), o in zip(items[:8], outs[:8])]
        srv.pause(False)
        for t in first:
            with pytest.raises(ifx.CudaError):
                srv.wait(t, timeout=60)
        second = [srv.submit(op, img, o, border) for (img, op, border), o in zip(items[8:], outs[8:])]
        for t in second:
            srv.wait(t, timeout=60)
        srv.drain()
        m = srv.metrics()
    assert m["failed"] == 8 and m["completed"] == 8 and m["hbm_in_use"] == 0
    check_outputs(ifx, items[8:], outs[8:])


def test_server_admission_by_free_device_memory(gpu_ifx):
    """A cap far above what the device has free (another user holds most of
    it): admission follows the device's free memory, so requests wait instead
    of failing their allocations, and all complete with correct results."""
    ifx = gpu_ifx
    import torch
    from imagefiltering_gb300.serve import Server
    torch.cuda.synchronize()
    free, _ = torch.cuda.mem_get_info()
    keep = 640 << 20                                   # what the other user leaves free
    hog = torch.empty(max(free - keep, 0), dtype=torch.uint8, device="cuda")
    try:
        rng = np.random.default_rng(12)
        items = []
        for i in range(12):                            # 4096^2 Float32 -> Float64: 192 MiB each on the device
            img = np.asfortranarray(rng.random((4096, 4096), dtype=np.float32))
            items.append((img, ("gaussian", 1.0 + (i % 3)), ifx.Pad("reflect")))
        with Server(hbm_cap_bytes=100 << 30, max_batch=2, max_inflight=2) as srv:
            outs, tickets = [], []
            # paused: admission goes on but no batch launches, so the admitted
            # requests hold their memory until every request is queued (else
            # a fast device finishes each one before the next arrives)
            srv.pause(True)
            for img, op, border in items:
                o = host_outputs(ifx, img, op)
                outs.append(o)
                tickets.append(srv.submit(op, img, o, border))
            srv.pause(False)
            for t in tickets:
                srv.wait(t, timeout=120)
            m = srv.metrics()
        assert m["completed"] == len(items) and m["failed"] == 0, m
        assert m["deferred_free"] > 0, m               # admissions waited for memory
        assert m["hbm_peak"] <= keep, m
    finally:
        del hog
        torch.cuda.empty_cache()
    check_outputs(ifx, items[:3], outs[:3])
