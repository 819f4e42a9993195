"""Array handling for the host layer: element kinds, Julia memory order and
device arrays.

Images use Julia's memory order: axis 0 is Julia's axis 1 and is contiguous
(numpy arrays in Fortran order).  8-bit images come in two flavours that the
reference distinguishes by eltype: ``N0f8`` (code c means c/255; also
``Gray{N0f8}``), marked by the ``N0f8Array`` subclass, and plain ``UInt8``
(code c means c), a plain uint8 array.

Device-resident arrays are ``DeviceArray`` objects wrapping a torch CUDA tensor
with column-major strides; the library detects device memory and then only
enqueues work.  torch is used for device allocation only.
"""
import numpy as np


class N0f8Array(np.ndarray):
    """uint8 codes interpreted as N0f8 (c/255)."""


class N0f16Array(np.ndarray):
    """uint16 codes interpreted as N0f16 (c/65535), the Gray{N0f16} of the reference."""


def n0f8(a) -> "N0f8Array":
    return np.asfortranarray(np.asarray(a, dtype=np.uint8)).view(N0f8Array)


def n0f16(a) -> "N0f16Array":
    return np.asfortranarray(np.asarray(a, dtype=np.uint16)).view(N0f16Array)


_NP_KIND = {np.dtype(np.float32): "F32", np.dtype(np.float64): "F64", np.dtype(np.uint8): "U8",
            np.dtype(np.int16): "I16", np.dtype(np.int8): "I8", np.dtype(np.uint16): "U16",
            np.dtype(np.int32): "I32", np.dtype(np.int64): "I64"}
_KIND_NP = {"F32": np.float32, "F64": np.float64, "U8": np.uint8, "N0F8": np.uint8,
            "I16": np.int16, "I8": np.int8, "U16": np.uint16, "N0F16": np.uint16, "I32": np.int32,
            "I64": np.int64}
# kinds the filters take directly; the others go through ifx_convert
NATIVE_KINDS = ("F32", "F64", "N0F8", "U8")
INT_KINDS = ("U8", "I8", "I16", "U16", "I32", "I64")


def _torch_dtype(kind):
    import torch
    # 16-bit unsigned kinds are stored as int16 (the same bits)
    return {"F32": torch.float32, "F64": torch.float64, "U8": torch.uint8, "N0F8": torch.uint8,
            "I16": torch.int16, "I8": torch.int8, "U16": torch.int16, "N0F16": torch.int16,
            "I32": torch.int32, "I64": torch.int64}[kind]


class RGB:
    """An RGB image (Array{RGB{T}}) as its channel planes in Julia's memory
    order: ``data`` has shape (3,) + image shape and axis 0 is the channel --
    reinterpret(T, img) of the reference's array, T N0f8, Float32 or Float64
    (host array or DeviceArray).  Linear filters act on the image axes of each
    channel; filter_type gives RGB of the promoted eltype
    (src/imfilter.jl:1133)."""

    def __init__(self, data):
        if data.shape[0] != 3:
            raise ValueError("RGB data needs the channel axis (length 3) first")
        self.data = data

    @property
    def shape(self):
        return tuple(self.data.shape[1:])

    @property
    def ndim(self):
        return len(self.data.shape) - 1

    def channel(self, i):
        return self.data[i] if not isinstance(self.data, DeviceArray) else DeviceArray(self.data.tensor[i], self.data.kind)


def rgb(data):
    return RGB(data)


class DeviceArray:
    """A torch CUDA tensor in Julia memory order plus its element kind."""

    def __init__(self, tensor, kind=None, first=None):
        import torch
        self.tensor = tensor
        if kind is None:
            kind = {torch.float32: "F32", torch.float64: "F64", torch.uint8: "U8",
                    torch.int16: "I16", torch.int8: "I8", torch.int32: "I32", torch.int64: "I64"}[tensor.dtype]
        self.kind = kind
        self.first = first

    @property
    def shape(self):
        return tuple(self.tensor.shape)

    @property
    def ndim(self):
        return self.tensor.dim()

    def ptr(self):
        return self.tensor.data_ptr()

    def strides(self):
        return tuple(self.tensor.stride())

    def numpy(self):
        a = self.tensor.detach().cpu().numpy()
        a = np.asfortranarray(a)
        if self.kind in ("U16", "N0F16"):
            a = a.view(np.uint16)
        if self.kind == "N0F16":
            return a.view(N0f16Array)
        return a.view(N0f8Array) if self.kind == "N0F8" else a

    @staticmethod
    def empty(shape, kind, device="cuda"):
        """A column-major tensor of Julia shape `shape`."""
        import torch
        dt = _torch_dtype(kind)
        rev = tuple(reversed(shape))
        t = torch.empty(rev, dtype=dt, device=device)
        t = t.permute(*reversed(range(len(shape)))) if len(shape) > 1 else t
        return DeviceArray(t, kind)

    @staticmethod
    def from_host(a, device="cuda"):
        import torch
        k = kind_of(a)
        a = np.asfortranarray(a)
        d = DeviceArray.empty(a.shape, k, device)
        host = a.view(np.ndarray)
        if k in ("U16", "N0F16"):
            host = host.view(np.int16)
        src = torch.from_numpy(np.ascontiguousarray(host.T))
        d.tensor.copy_(src.permute(*reversed(range(a.ndim))) if a.ndim > 1 else src)
        return d


def kind_of(a) -> str:
    if isinstance(a, DeviceArray):
        return a.kind
    if isinstance(a, N0f8Array):
        return "N0F8"
    if isinstance(a, N0f16Array):
        return "N0F16"
    dt = np.asarray(a).dtype
    if dt not in _NP_KIND:
        raise NotImplementedError("eltype %s is not supported by the GB300 path" % dt)
    return _NP_KIND[dt]


def host_view(a, kind=None):
    """Fortran-ordered numpy array (keeps the N0f8 marker)."""
    if kind == "N0F8" or isinstance(a, N0f8Array):
        return n0f8(a)
    if kind == "N0F16" or isinstance(a, N0f16Array):
        return n0f16(a)
    return np.asfortranarray(a)


def alloc_like(img, shape, kind):
    """Output allocation on the same side (host/device) as `img`."""
    if isinstance(img, DeviceArray):
        return DeviceArray.empty(shape, kind, img.tensor.device)
    out = np.empty(shape, dtype=_KIND_NP[kind], order="F")
    if kind == "N0F16":
        return out.view(N0f16Array)
    return out.view(N0f8Array) if kind == "N0F8" else out


def ptr_strides(a, values_per_elem=1):
    if isinstance(a, DeviceArray):
        st = a.strides()
        return a.ptr(), tuple(s // values_per_elem for s in st)
    arr = a.view(np.ndarray)
    if not arr.flags.f_contiguous:
        raise ValueError("host arrays must be in Fortran (Julia) order")
    return arr.ctypes.data, tuple(s // (arr.itemsize * values_per_elem) for s in arr.strides)


def stream_for(*arrays):
    """torch's current stream when any array is device-resident (so the library
    orders its kernels after the producer of the input and before its
    consumers), else None (the library's own stream, synchronous call)."""
    for a in arrays:
        if isinstance(a, DeviceArray):
            return torch_stream(a.tensor.device)
    return None


def torch_stream(device=None):
    """torch's current stream as a handle for the C ABI.  torch reports the
    legacy default stream as 0, which the ABI would read as "the context's
    own stream" (not ordered with torch's work), so it becomes cudaStreamLegacy."""
    import torch
    h = torch.cuda.current_stream(device).cuda_stream
    return h if h else 1          # 1 == cudaStreamLegacy
