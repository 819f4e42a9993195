"""CPU restatements of two exact-arithmetic devices of the GPU kernels.

* Float32 -> Float64 widening in integer operations (`f32_to_f64` in
  csrc/ifx_common.cuh): for a normal number the sign and mantissa move up 29
  bits and the exponent is rebiased by 1023 - 127; one unsigned compare selects
  the normal range.  Checked bit for bit against the IEEE conversion.
* Sobel-structured gradient sums (`k_grad3d` with `sob_d` / `sob_s` in
  csrc/ifx_fir.cu): derivative (-h, 0, h) and smoothing (q, 2q, q), h and q
  powers of two, summed unscaled as c - a and (a + c) + 2b and scaled once by
  h q^2.  Checked against the reference's per-pass order (sum of tap products,
  src/imfilter.jl:671-739) within the Float64 tolerance.
"""
import numpy as np


def widen_bits(b):
    """The integer widening of float32 bit patterns b (uint32) for the normal
    range; returns (float64 bit patterns, mask of the normal inputs)."""
    b = b.astype(np.uint32)
    a = b & np.uint32(0x7FFFFFFF)
    normal = (a - np.uint32(0x00800000)).astype(np.uint32) < np.uint32(0x7F000000)
    hi = ((b & np.uint32(0x80000000)) | ((a >> np.uint32(3)) + np.uint32(896 << 20))).astype(np.uint64)
    lo = (b.astype(np.uint64) << np.uint64(29)) & np.uint64(0xFFFFFFFF)
    return (hi << np.uint64(32)) | lo, normal


def test_integer_widening_is_the_ieee_conversion():
    rng = np.random.default_rng(0)
    edges = np.array([0x00800000, 0x80800000, 0x7F7FFFFF, 0xFF7FFFFF, 0x3F800000, 0x00000001,
                      0x807FFFFF, 0x7F800000, 0x7FC00000, 0x00000000, 0x80000000], dtype=np.uint64)
    b = np.concatenate([rng.integers(0, 2 ** 32, 1_000_000, dtype=np.uint64), edges]).astype(np.uint32)
    bits, normal = widen_bits(b)
    e = (b >> np.uint32(23)) & np.uint32(0xFF)
    assert np.array_equal(normal, (e > 0) & (e < 255))      # one compare classifies
    ref = b.view(np.float32)[normal].astype(np.float64).view(np.uint64)
    assert np.array_equal(bits[normal], ref)


def _pass(v, w, axis):
    """One 3-tap pass, reference order: w0*v[i-1] + w1*v[i] + w2*v[i+1]
    (replicate border), each product rounded, summed left to right."""
    p = np.pad(v, [(1, 1) if d == axis else (0, 0) for d in range(v.ndim)], mode="edge")
    sl = lambda k: tuple(slice(k, k + v.shape[d]) if d == axis else slice(None) for d in range(v.ndim))
    return (w[0] * p[sl(0)] + w[1] * p[sl(1)]) + w[2] * p[sl(2)]


def _sob(v, kind, axis):
    p = np.pad(v, [(1, 1) if d == axis else (0, 0) for d in range(v.ndim)], mode="edge")
    sl = lambda k: tuple(slice(k, k + v.shape[d]) if d == axis else slice(None) for d in range(v.ndim))
    a, b, c = p[sl(0)], p[sl(1)], p[sl(2)]
    return c - a if kind == "d" else (a + c) + 2.0 * b


def test_sobel_structured_sums_within_float64_tolerance():
    rng = np.random.default_rng(1)
    vol = rng.random((24, 20, 18))
    vol[rng.random(vol.shape) < 0.01] = 1.0
    d, s = np.array([-0.5, 0.0, 0.5]), np.array([0.25, 0.5, 0.25])
    scale = 0.5 * 0.25 * 0.25                           # h q^2, a power of two
    for g in range(3):
        ref = vol
        fast = vol
        for ax in range(3):
            ref = _pass(ref, d if ax == g else s, ax)
            fast = _sob(fast, "d" if ax == g else "s", ax)
        fast = fast * scale                            # exact: scaling by a power of two
        err = np.max(np.abs(fast - ref)) / np.max(np.abs(ref))
        assert err <= 1e-12, (g, err)
