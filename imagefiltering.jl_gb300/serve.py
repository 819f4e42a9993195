"""The serving loop from Python: ``Server`` wraps ifx_server_* (continuous
batching with HBM-capped admission, native engine thread).

    srv = Server(hbm_cap_bytes=150 << 30)
    t = srv.submit(("gaussian", 2.0), img, outs, "reflect")   # host or device arrays
    srv.wait(t)
    srv.metrics()   # completed, pixels, p50/p99 latency, hbm peak, ...

Host arrays must stay alive (and unmodified) until their request is done;
pinned host memory makes the copies asynchronous.
"""
import ctypes as C

from . import _abi
from .batch import Batch


class Server:
    def __init__(self, hbm_cap_bytes=150 << 30, max_batch=512, max_inflight=2):
        self.ctx = _abi.context()
        cfg = _abi.IfxServerConfig(int(hbm_cap_bytes), int(max_batch), int(max_inflight))
        h = C.c_void_p()
        _abi.check(self.ctx.lib.ifx_server_create(self.ctx.handle, C.byref(cfg), C.byref(h)))
        self.handle = h
        self._pending = {}

    def submit(self, op, img, outs, border="replicate"):
        """Queue one request (same forms as batch.Batch.add); returns a ticket."""
        b = Batch()
        q = b.add(op, img, outs, border)
        t = C.c_uint64()
        _abi.check(self.ctx.lib.ifx_server_submit(self.handle, C.byref(q), C.byref(t)))
        self._pending[t.value] = (img, outs)
        return t.value

    def submit_struct(self, q, keep=None):
        t = C.c_uint64()
        _abi.check(self.ctx.lib.ifx_server_submit(self.handle, C.byref(q), C.byref(t)))
        if keep is not None:
            self._pending[t.value] = keep
        return t.value

    def wait(self, ticket, timeout=60.0):
        st = C.c_int32()
        rc = self.ctx.lib.ifx_server_wait(self.handle, C.c_uint64(ticket), float(timeout), C.byref(st))
        if rc == 6:
            raise TimeoutError("request %d not done within %.3f s" % (ticket, timeout))
        _abi.check(rc)
        self._pending.pop(ticket, None)
        if st.value:
            raise _abi._EXC.get(st.value, RuntimeError)("request %d failed (status %d)" % (ticket, st.value))

    def cancel(self, ticket):
        """Cancel a request that has not joined a launched batch (its wait then
        raises Cancelled); ArgumentError when it is done or already running."""
        _abi.check(self.ctx.lib.ifx_server_cancel(self.handle, C.c_uint64(ticket)))
        self._pending.pop(ticket, None)

    def pause(self, paused=True):
        """Stop launching new batches (admission and uploads go on) or resume."""
        _abi.check(self.ctx.lib.ifx_server_pause(self.handle, int(bool(paused))))

    def inject_launch_error(self, count=1):
        """Failure injection on the host, for tests: the next `count` batched
        launches are reported as failed without running; their requests fail
        with CudaError and the server keeps serving."""
        _abi.check(self.ctx.lib.ifx_server_inject_launch_error(self.handle, int(count)))

    def drain(self, timeout=600.0):
        rc = self.ctx.lib.ifx_server_drain(self.handle, float(timeout))
        if rc == 6:
            raise TimeoutError("server not drained within %.1f s" % timeout)
        _abi.check(rc)
        self._pending.clear()

    def metrics(self):
        m = _abi.IfxServerMetrics()
        _abi.check(self.ctx.lib.ifx_server_metrics(self.handle, C.byref(m)))
        return {k: getattr(m, k) for k, _ in m._fields_}

    def reset_metrics(self):
        _abi.check(self.ctx.lib.ifx_server_reset_metrics(self.handle))

    def close(self):
        if self.handle:
            self.ctx.lib.ifx_server_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
