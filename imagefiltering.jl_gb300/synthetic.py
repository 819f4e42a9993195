"""Seeded synthetic inputs for benchmarking and serving tests.

No public dataset is involved: every workload is generated from a fixed
numpy PCG64 seed with the shapes, eltypes and value distributions of the
benchmark configurations:

  * ``stream_requests``: the mixed serving stream -- 2-D images, one side
    log-uniform in [64, 4096], aspect log-uniform in [1/4, 4] (the other side
    clipped to [64, 4096]); eltype Float32 or N0f8 with probability 1/2; op
    uniform over {Gaussian σ ~ U[0.5, 8], Sobel gradient, Laplacian 3x3,
    median 3x3 / 5x5}; border uniform over the four Pad styles; Poisson
    arrivals.
"""
import math

import numpy as np

OPS = ("gaussian", "sobel", "laplacian", "median")
PAD_STYLES = ("replicate", "circular", "symmetric", "reflect")


class Request:
    __slots__ = ("idx", "h", "w", "kind", "op", "sigma", "win", "style", "arrival")

    def __init__(self, **kw):
        for k, v in kw.items():
            setattr(self, k, v)

    @property
    def pixels(self):
        return self.h * self.w

    def in_bytes(self):
        return self.pixels * (4 if self.kind == "F32" else 1)

    def out_kinds(self):
        """Output eltypes the reference returns (filter_type / median eltype)."""
        if self.op == "gaussian":
            return ["F64"]                   # Float64 weights promote (src/imfilter.jl:1133)
        if self.op == "sobel":
            return ["F64", "F64"]            # imgradients: one Float64 array per axis
        return ["F32"]                       # Laplacian of F32/N0f8 and the median of both

    def out_bytes(self):
        return self.pixels * sum(8 if k == "F64" else 4 for k in self.out_kinds())

    def taps(self):
        return 4 * int(math.ceil(self.sigma)) + 1 if self.op == "gaussian" else 0

    def __repr__(self):
        return "Request(%d: %dx%d %s %s %s)" % (self.idx, self.h, self.w, self.kind, self.op,
                                               self.style)


def stream_requests(n=10000, seed=5, rate=None):
    """The mixed stream; `rate` (requests/s) sets Poisson arrival times
    (None: all arrive at t=0)."""
    rng = np.random.default_rng(seed)
    out = []
    t = 0.0
    for i in range(n):
        h = int(round(math.exp(rng.uniform(math.log(64), math.log(4096)))))
        a = math.exp(rng.uniform(math.log(0.25), math.log(4.0)))
        w = int(min(4096, max(64, round(h * a))))
        kind = "F32" if rng.random() < 0.5 else "N0F8"
        op = OPS[int(rng.integers(0, 4))]
        sigma = float(rng.uniform(0.5, 8.0))
        win = 3 if rng.random() < 0.5 else 5
        style = PAD_STYLES[int(rng.integers(0, 4))]
        if rate:
            t += float(rng.exponential(1.0 / rate))
        out.append(Request(idx=i, h=h, w=w, kind=kind, op=op, sigma=sigma, win=win, style=style,
                           arrival=t if rate else 0.0))
    return out


def image_for(req, seed=5):
    """Host image of a request: uniform values (F32 in [0,1), N0f8 codes 0..255)."""
    rng = np.random.default_rng((seed, req.idx))
    if req.kind == "F32":
        return np.asfortranarray(rng.random((req.h, req.w), dtype=np.float32))
    return np.asfortranarray(rng.integers(0, 256, (req.h, req.w), dtype=np.uint8))
