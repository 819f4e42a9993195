"""The reference's known answers through the GB300 kernels (C ABI), in FP64
and, for the exact cases, in the other eltypes.  Same cases as the oracle's
tests (tests/kat_cases.py)."""
import numpy as np
import pytest

import kat_cases as K
from gpu_backend import GpuBackend

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def be(gpu_ifx):
    return GpuBackend(gpu_ifx, np.float64)


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.uint8])
def test_padarray_golden_tables(gpu_ifx, dtype):
    K.check_padarray(GpuBackend(gpu_ifx, dtype), unsigned=dtype == np.uint8)


def test_border_maps_match_numpy(be, oracle):
    K.check_padindex_vs_numpy(be, oracle)


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
