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

// N0f8 code c as Float32, c/255 correctly rounded, without a table or a
// division: c is made exact from the mantissa bits of 2^23 + c, q = c * r
// with r = fl(1/255), and one correction step q + (c - 255 q) r (Markstein's
// correction of a quotient from a reciprocal; the residual c - 255 q is exact
// in one fused multiply-add).  Checked against the correctly rounded quotient
// for all 256 codes.
__device__ __forceinline__ float u8_to_f32(uint32_t c)
{
    return __fsub_rn(__uint_as_float(0x4B000000u | c), 8388608.0f);     // (2^23 + c) - 2^23
}
__device__ __forceinline__ float n0f8_to_f32(uint32_t c)
{
    const float f = u8_to_f32(c);
    const float r = 1.0f / 255.0f;
    const float q = __fmul_rn(f, r);
    return __fmaf_rn(__fmaf_rn(-q, 255.0f, f), r, q);
}

template <class To> __device__ __forceinline__ To from_c(float v) { return (To)v; }
template <class To> __device__ __forceinline__ To from_c(double v) { return (To)v; }

// Float32 -> Float64 widening, exact, in integer operations (the FP64 pipe of
// this part is narrow, and every Float64 output of an FP32 computation passes
// through here).  From the IEEE-754 binary32/binary64 formats: a normal
// number keeps sign and mantissa (shifted up 29 bits) and its exponent is
// rebiased by 1023 - 127 = 896; zeros keep their sign; subnormals, Inf and
// NaN take the hardware conversion.
__device__ __forceinline__ double f32_to_f64(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t a = b & 0x7FFFFFFFu;
    // one unsigned compare: the magnitude lies in [2^-126, 2^128), exponent 1..254
    if (a - 0x00800000u < 0x7F000000u)
        return __hiloint2double((int)((b & 0x80000000u) | ((a >> 3) + (896u << 20))), (int)(b << 29));
    if (a == 0u) return __hiloint2double((int)(b & 0x80000000u), 0);
    return (double)f;
}

// Output store conversion from an FP32 result.
template <class To> __device__ __forceinline__ To out_cvt(float v) { return (To)v; }
template <> __device__ __forceinline__ double out_cvt<double>(float v) { return f32_to_f64(v); }
template <class To> __device__ __forceinline__ To out_cvt(double v) { return (To)v; }

// The same, alternating (by an unrolled index) between the conversion
// instruction on the narrow FP64 pipe and the integer widening on the ALU
// pipe for Float64, so that a run of stores loads neither pipe alone.
template <class To> __device__ __forceinline__ To out_cvt_alt(float v, int i)
{
    if constexpr (sizeof(To) == 8) return (i & 1) ? f32_to_f64(v) : (double)v;
    else return out_cvt<To>(v);
}
template <class To> __device__ __forceinline__ To out_cvt_alt(double v, int) { return (To)v; }

__host__ __device__ __forceinline__ int up4(int k) { return (k + 3) & ~3; }

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

// =========================================================================
// Register-blocked 1-D correlation on shared memory:
//   acc[i] = sum_{t < k} w[t] * p[(i+t)*step],  i < NB
// The window of NB(+4) values slides through registers so each loaded value
// feeds up to NB multiply-adds.  Taps go four at a time and the last k mod 4
// one at a time, so no padded weight ever multiplies data (0*Inf would be NaN).
// Reads p[0 .. NB+k-2] only.
// =========================================================================
template <class Tc, int NB>
__device__ __forceinline__ void corr_run(const Tc *p, int step, const Tc *w, int k, Tc *acc)
{
    Tc v[NB + 4];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        v[i] = p[i * step];
        acc[i] = 0;
    }
    v[NB + 3] = 0;
    int t0 = 0;
    for (; t0 + 4 <= k; t0 += 4) {
#pragma unroll
        for (int j = 0; j < 3; ++j) v[NB + j] = p[(NB + t0 + j) * step];
        // v[NB+3] first serves the next chunk: not loaded after the last one
        if (t0 + 4 < k) v[NB + 3] = p[(NB + t0 + 3) * step];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const Tc wt = w[t0 + j];
#pragma unroll
            for (int i = 0; i < NB; ++i) acc[i] = fma(wt, v[i + j], acc[i]);
        }
#pragma unroll
        for (int i = 0; i < NB; ++i) v[i] = v[i + 4];
    }
    for (; t0 < k; ++t0) {
        const Tc wt = w[t0];
#pragma unroll
        for (int i = 0; i < NB; ++i) acc[i] = fma(wt, v[i], acc[i]);
        if (t0 + 1 < k) {
#pragma unroll
            for (int i = 0; i < NB - 1; ++i) v[i] = v[i + 1];
            v[NB - 1] = p[(NB + t0) * step];
        }
    }
}

// Unrolled forms of corr_run for k <= kCorrKmax taps: the tap loop is
// unrolled at compile time and left when t reaches k, so every window value
// has a fixed register and nothing is shifted.
constexpr int kCorrKmax = 36;

// Column form: acc[i] = sum_{t<k} w[t] p[(i+t)*step], i < NB; reads
// p[0 .. NB+k-2] only.
template <int NB>
__device__ __forceinline__ void corr_col(const float *p, int step, const float *w, int k, float *acc)
{
    float v[NB + kCorrKmax - 1];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        v[i] = p[i * step];
        acc[i] = 0.0f;
    }
#pragma unroll
    for (int t = 0; t < kCorrKmax; ++t) {
        if (t >= k) break;
        if (t > 0) v[NB - 1 + t] = p[(NB - 1 + t) * step];
        const float wt = w[t];
#pragma unroll
        for (int i = 0; i < NB; ++i) acc[i] = fmaf(wt, v[i + t], acc[i]);
    }
}

// Row form on a 16-byte aligned window, loaded four values at a time:
// acc[i] = sum_{t<k} w[t] p[i+t], i < NB (NB a multiple of 4); reads
// p[0 .. 4*ceil((NB+k-1)/4) - 1], up to 3 values past the window.
template <int NB>
__device__ __forceinline__ void corr_row4(const float *p, const float *w, int k, float *acc)
{
    float v[NB + kCorrKmax + 3];
    const float4 *q = reinterpret_cast<const float4 *>(p);
#pragma unroll
    for (int c = 0; c < NB / 4; ++c) {
        const float4 f = q[c];
        v[4 * c] = f.x;
        v[4 * c + 1] = f.y;
        v[4 * c + 2] = f.z;
        v[4 * c + 3] = f.w;
    }
#pragma unroll
    for (int i = 0; i < NB; ++i) acc[i] = 0.0f;
#pragma unroll
    for (int t = 0; t < kCorrKmax; ++t) {
        if (t >= k) break;
        if (t > 0 && ((NB - 1 + t) & 3) == 0) {
            const float4 f = q[(NB - 1 + t) >> 2];
            v[NB - 1 + t] = f.x;
            v[NB + t] = f.y;
            v[NB + 1 + t] = f.z;
            v[NB + 2 + t] = f.w;
        }
        const float wt = w[t];
#pragma unroll
        for (int i = 0; i < NB; ++i) acc[i] = fmaf(wt, v[i + t], acc[i]);
    }
}

// Packed form on the FP32x2 pipe (__ffma2_rn: two lanes of one FMA
// instruction, each rounded as fmaf).  Per output the taps accumulate in the
// order of corr_col, so the results are bit-identical to it.  Weights come as
// (w, w) pairs.
// Column-pair form: acc[i] = (out(i, 0), out(i, 1)) with
// out(i, j) = sum_{t<k} w[t] p[(i+t)*step + j], i < NB; p and step*4 bytes
// 8-byte aligned.  Reads rows 0 .. NB+k-2 of the two columns.
template <int NB>
__device__ __forceinline__ void corr_col_x2(const float *p, int step, const float2 *w2, int k, float2 *acc)
{
    float2 v[NB + kCorrKmax - 1];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        v[i] = *reinterpret_cast<const float2 *>(p + i * step);
        acc[i] = make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int t = 0; t < kCorrKmax; ++t) {
        if (t >= k) break;
        if (t > 0) v[NB - 1 + t] = *reinterpret_cast<const float2 *>(p + (NB - 1 + t) * step);
        const float2 w = w2[t];
#pragma unroll
        for (int i = 0; i < NB; ++i) acc[i] = __ffma2_rn(w, v[i + t], acc[i]);
    }
}

// Tile gather with U independent loads in flight per thread: load(idx)
// returns element idx of the tile (row-major in shared memory).  All U
// loads of a round are issued before any shared-memory store, so a CTA keeps
// U*blockDim.x global loads outstanding instead of one per thread.
template <int U, class T, class F>
__device__ __forceinline__ void gather_tile(T *dst, int total, F load)
{
    const int nth = blockDim.x;
    for (int base = threadIdx.x; base < total; base += nth * U) {
        T v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int idx = base + u * nth;
            v[u] = idx < total ? load(idx) : T(0);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int idx = base + u * nth;
            if (idx < total) dst[idx] = v[u];
        }
    }
}

} // namespace ifx
