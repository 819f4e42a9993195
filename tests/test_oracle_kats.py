"""The CPU oracle against ImageFiltering.jl's own known answers (CPU only).

Pins the oracle before it is trusted as the checker of the GPU path: every
literal table in tests/golden/reference_kats.json and every structural case
of the reference's tests (tests/kat_cases.py) must hold for it.
"""
import numpy as np
import pytest

import kat_cases as K


@pytest.fixture(scope="module")
def be(oracle):
    return K.OracleBackend(oracle)


def test_padarray_golden_tables(be):
    K.check_padarray(be)


def test_border_maps_match_numpy(be, oracle):
    K.check_padindex_vs_numpy(be, oracle)


def test_padindex_divide_error(oracle):
    # reflect on a length-1 axis has period 0 (src/border.jl:581-586): DivideError
    with pytest.raises(RuntimeError):
        oracle.padindex("reflect", 1, 1, 1)
    assert list(oracle.padindex("reflect", 0, 2, 0)) == [0, 1]


def test_impulse_interior(be):
    K.check_impulse_interior(be)


def test_impulse_edge(be):
    K.check_impulse_edge(be)


def test_cascade_1d_goldens(be):
    K.check_cascade_1d(be)


def test_offset_axes_1d(be):
    K.check_offset_axes_1d(be)


def test_nonfinite(be):
    K.check_nonfinite(be)


def test_3d_box(be):
    K.check_3d_box(be)


def test_cascade_equals_dense(be):
    K.check_cascade_equals_dense(be)


def test_fill_interior(be):
    g = np.exp(-np.arange(-1, 2) ** 2 / 2.0)
    g /= g.sum()
    K.check_fill_interior(be, [(0, -1, g), (1, -1, g)])


def test_prewitt_band(be):
    K.check_prewitt_band(be)


@pytest.mark.parametrize("arith", ["f64", "f32", "int"])
def test_laplacian(be, arith):
    K.check_laplacian(be, arith)


def test_gradient_ramps(be):
    K.check_gradient_ramps(be)


def test_extrema_lemire_golden(be):
    K.check_extrema_lemire_golden(be)


def test_extrema_nd_groundtruth(be):
    K.check_extrema_nd(be)


def test_median_golden(be):
    K.check_median_golden(be)


def test_window_pad_relative_to_intersection(oracle):
    """copy_win! pads relative to window-intersect-image (src/mapwindow.jl:
    311-314): for circular the wrap stays inside the truncated window, so
    circular min/max equal the truncated window's."""
    rng = np.random.default_rng(2)
    A = np.asfortranarray(rng.random((9, 8)))
    mn_t, mx_t = oracle.extrema_trunc(A, [5, 5])
    for style in ("replicate", "circular", "symmetric", "reflect"):
        mn, mx = oracle.mapwindow_extrema(A, [-2, -2], [5, 5], style)
        assert np.array_equal(mn, mn_t) and np.array_equal(mx, mx_t), style
    # median: circular wraps inside window-intersect-image, not the whole axis.
    # A = 1..9, window -2:2 at index 1: inner = 1..3 -> window (2,3,1,2,3) -> 2,
    # whereas whole-axis wrapping would give (8,9,1,2,3) -> 3.
    a = np.asfortranarray(np.arange(1.0, 10.0))
    assert oracle.mapwindow_median(a, [-2], [5], "circular")[0] == 2.0
    assert oracle.mapwindow_median(a, [-2], [5], "replicate")[0] == 1.0


def test_fill_cascade_scales_halo(oracle):
    """Pad-then-cascade with Fill(v): pass 2 sees v*sum(k1) in the halo
    (src/imfilter.jl:331-341, 385-446)."""
    A = np.asfortranarray(np.zeros((6, 6)))
    k1 = (0, -1, np.array([1.0, 2.0, 3.0]))
    k2 = (1, -1, np.array([1.0, 1.0, 1.0]))
    out = oracle.imfilter_cascade(A, [k1, k2], "fill", 1.0)
    # corner: pass-1 column values 6 (halo col) / 5 (image col 0, rows -1..1 -> 1*1+0+0..)
    P = oracle.padarray(A, "fill", [1, 1], [1, 1], 1.0)
    T = np.zeros((6, 8))
    for i in range(6):
        for j in range(8):
            T[i, j] = sum(P[i + t, j] * k1[2][t] for t in range(3))
    exp = np.array([[sum(T[i, j + t] for t in range(3)) for j in range(6)] for i in range(6)])
    np.testing.assert_allclose(out, exp, rtol=0, atol=0)


def test_na_vectors(be):
    K.check_na_vectors(be)


def test_na_impulse(be):
    K.check_na_impulse(be)


def test_inner_impulse(be):
    K.check_inner_impulse(be)


def test_localextrema(be):
    K.check_localextrema(be)


def test_blob_log(be):
    K.check_blob_log(be)


def test_fft_impulses(be):
    K.check_fft_impulses(be)


def test_fft_3d_box(be):
    K.check_fft_3d_box(be)


def test_fft_nopad(be):
    K.check_fft_nopad(be)


def test_fft_equals_fir(be, oracle):
    K.check_fft_equals_fir(be, oracle)


def test_iir_1d(be):
    K.check_iir_1d(be)


def test_iir_images(be):
    K.check_iir_images(be)


def test_iir_na_ramp(be):
    K.check_iir_na_ramp(be)


def test_mixed_cascades(be):
    K.check_mixed(be)
