// ifx_common.cuh -- shared device helpers: border index maps, element
// conversion, launch accounting.  Included by every .cu file of the library.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "../../include/ifx_gb300.h"

#define IFX_MAXD IFX_MAX_DIMS

namespace ifx {

// Count of this library's kernel launches (read through ifx_launch_count).
void note_launch(int n = 1);

// ---------------------------------------------------------------------------
// Border index map along one axis of length n (src/border.jl:564-596 with
// the mod-based tables; src/borderarray.jl:114-144 gives the same values for
// pads smaller than the axis).  Returns the source index in [0,n), or -1 for
// a Fill position outside the axis.  The caller guarantees n >= 1 and, for
// reflect, n >= 2 (the host reports the reference's DivideError otherwise).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int map_index(int x, int n, int style)
{
    if ((unsigned)x < (unsigned)n) return x;
    switch (style) {
    case IFX_REPLICATE:
        return x < 0 ? 0 : n - 1;
    case IFX_CIRCULAR: {
        int r = x % n;
        return r < 0 ? r + n : r;
    }
    case IFX_SYMMETRIC: {
        int p = 2 * n;
        int r = x % p;
        if (r < 0) r += p;
        return r < n ? r : p - 1 - r;
    }
    case IFX_REFLECT: {
        int p = 2 * n - 2;
        int r = x % p;
        if (r < 0) r += p;
        return r < n ? r : p - r;
    }
    default:
        return -1;
    }
}

// Same map relative to the sub-range [lo, lo+len) of an axis: mapwindow's
// copy_win! pads relative to window-intersect-image (src/mapwindow.jl:311-314).
__device__ __forceinline__ int map_index_in(int x, int lo, int len, int style)
{
    int r = map_index(x - lo, len, style);
    return r < 0 ? -1 : r + lo;
}

// ---------------------------------------------------------------------------
// Element conversion.  8-bit inputs carry a flag: N0f8 code c is c/255 (the
// correctly rounded quotient, as the FixedPointNumbers conversion), UInt8 is c.
// ---------------------------------------------------------------------------
template <class Tc> __device__ __forceinline__ Tc to_c(float v, bool) { return (Tc)v; }
template <class Tc> __device__ __forceinline__ Tc to_c(double v, bool) { return (Tc)v; }
template <class Tc> __device__ __forceinline__ Tc to_c(uint8_t v, bool norm)
{
    return norm ? (Tc)v / (Tc)255 : (Tc)v;
}

template <class To> __device__ __forceinline__ To from_c(float v) { return (To)v; }
template <class To> __device__ __forceinline__ To from_c(double v) { return (To)v; }

// Dense N-d box of an index space (lo .. lo+size-1 per axis), column-major.
struct Box {
    int nd;
    int lo[IFX_MAXD];
    int size[IFX_MAXD];
    long long stride[IFX_MAXD];
    long long count;
};

inline Box make_box(int nd, const int *lo, const int *size)
{
    Box b;
    b.nd = nd;
    long long s = 1;
    for (int d = 0; d < IFX_MAXD; ++d) {
        b.lo[d] = d < nd ? lo[d] : 0;
        b.size[d] = d < nd ? size[d] : 1;
        b.stride[d] = s;
        s *= b.size[d];
    }
    b.count = s;
    return b;
}

} // namespace ifx
