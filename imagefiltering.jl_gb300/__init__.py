"""GB300 (sm_103a) backend for ImageFiltering.jl's FIR and rank-filter path.

Python mirror of the reference API over the C ABI in include/ifx_gb300.h:

    imfilter, imfilter_ (imfilter!), imgradients, mapwindow, mapwindow_
    (mapwindow!), padarray, Pad, Fill, Kernel, KernelFactors, centered,
    Algorithm (with the new tag Algorithm.GB300), KernelFactors.IIRGaussian /
    TriggsSdika (recursive filters), NA/Inner/NoPad borders, blob_LoG

Arrays use Julia's memory order (Fortran-ordered numpy arrays on the host,
``DeviceArray`` for device-resident data).  Every result is computed by the
CUDA kernels of ``_build/libifx_gb300.so``; there is no CPU fallback, and the
functions raise if the library is missing.
"""
from . import _abi
from ._abi import (ArgumentError, Cancelled, DimensionMismatch, ErrorException, CudaError, InexactError,
                   OutOfMemory, Unsupported, launch_count)
from .arrays import RGB, DeviceArray, N0f8Array, N0f16Array, n0f8, n0f16, rgb
from .blobs import BlobLoG, blob_LoG, findlocalmaxima, findlocalminima, multiLoG
from .borders import Fill, Inner, NA, NoPad, Pad, borderinstance, padarray
from .filtering import (Algorithm, autotune, autotune_choice, autotune_clear, autotune_lookup, autotune_pin,
                        convert_, factorkernel, filter_type, imfilter, imfilter_, imgradients, maxabs)
from .kernels import (Kernel, KernelFactors, LaplacianKernel, OffsetKernel, ReshapedOneD, TriggsSdika,
                      centered, iscopy, kernelfactors)
from .rank import extrema, mapwindow, mapwindow_, maximum, median, median_, minimum

OffsetArray = OffsetKernel


def library_path() -> str:
    return _abi.LIB_PATH


__all__ = [
    "imfilter", "imfilter_", "imgradients", "mapwindow", "mapwindow_", "padarray", "Pad", "Fill",
    "Inner", "NA", "NoPad", "BlobLoG", "blob_LoG", "multiLoG", "findlocalmaxima", "findlocalminima", "Kernel", "KernelFactors", "centered", "kernelfactors", "Algorithm",
    "OffsetArray", "OffsetKernel", "ReshapedOneD", "LaplacianKernel", "TriggsSdika", "DeviceArray", "N0f8Array",
    "n0f8", "N0f16Array", "n0f16", "RGB", "rgb", "convert_", "maxabs", "InexactError", "median", "median_", "extrema", "minimum", "maximum", "filter_type", "factorkernel",
    "iscopy", "borderinstance", "autotune", "autotune_choice", "autotune_lookup", "autotune_pin", "autotune_clear", "ArgumentError", "DimensionMismatch", "ErrorException",
    "CudaError", "OutOfMemory", "Unsupported", "Cancelled", "launch_count", "library_path",
]
