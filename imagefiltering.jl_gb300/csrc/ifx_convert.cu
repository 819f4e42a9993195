// ifx_convert.cu -- element conversion between the eltypes of the ABI
// (out .= convert.(eltype(out), img)): the conversions around the reference's
// filters (its padded copy in the filter type, src/border.jl:324-331, and the
// store of each result into the output's eltype, src/imfilter.jl:660-666),
// which let integer, N0f16 and other images use the Float32/Float64 filters.
//
// To Float32: integers rounded to nearest (exact below 2^24), N0f8 c/255 and
// N0f16 c/65535 correctly rounded (q = c * fl(1/d) with one correction step,
// checked for every code); to Float64: integers rounded to nearest (exact
// below 2^53), codes divided correctly rounded.  To an integer type: the
// value must be an integer inside the type's range, as Julia's convert
// demands (InexactError; N0f8/N0f16 values are integers at 0 and 1 only);
// offending elements set *bad and are written as 0.
#include "ifx_internal.h"

namespace ifx {

__device__ __forceinline__ bool conv_is_int(int t)
{
    return t == IFX_U8 || t == IFX_I16 || t == IFX_I8 || t == IFX_U16 || t == IFX_I32 || t == IFX_I64;
}

// Element i of a source array as an exact integer (integer sources).
__device__ __forceinline__ long long conv_load_int(const void *p, int t, long long i)
{
    switch (t) {
    case IFX_U8: return ((const uint8_t *)p)[i];
    case IFX_I8: return ((const int8_t *)p)[i];
    case IFX_I16: return ((const int16_t *)p)[i];
    case IFX_U16: return ((const uint16_t *)p)[i];
    case IFX_I32: return ((const int32_t *)p)[i];
    default: return ((const long long *)p)[i];
    }
}

__device__ __forceinline__ float conv_code_f32(uint32_t c, float d, float r)
{
    const float f = (float)c;                     // exact: c < 2^24
    const float q = __fmul_rn(f, r);
    return __fmaf_rn(__fmaf_rn(-q, d, f), r, q);
}

__global__ void k_convert(const void *__restrict__ src, int st, void *__restrict__ dst, int dt, long long n,
                          int *bad)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        if (dt == IFX_F32 || dt == IFX_F64) {
            float f;
            double d;
            if (st == IFX_N0F8 || st == IFX_N0F16) {
                const uint32_t c = st == IFX_N0F8 ? ((const uint8_t *)src)[i] : ((const uint16_t *)src)[i];
                const float den = st == IFX_N0F8 ? 255.0f : 65535.0f;
                f = conv_code_f32(c, den, 1.0f / den);
                d = __ddiv_rn((double)c, (double)den);
            } else if (st == IFX_F32) {
                f = ((const float *)src)[i];
                d = (double)f;
            } else if (st == IFX_F64) {
                d = ((const double *)src)[i];
                f = __double2float_rn(d);
            } else {
                const long long v = conv_load_int(src, st, i);
                f = __ll2float_rn(v);
                d = __ll2double_rn(v);
            }
            if (dt == IFX_F32) ((float *)dst)[i] = f;
            else ((double *)dst)[i] = d;
            continue;
        }
        // integer target: an integer value inside the target's range
        long long v = 0;
        bool ok = true;
        if (conv_is_int(st)) {
            v = conv_load_int(src, st, i);
        } else if (st == IFX_F32 || st == IFX_F64) {
            const double x = st == IFX_F32 ? (double)((const float *)src)[i] : ((const double *)src)[i];
            // |x| < 2^63 and integral (NaN fails both tests)
            ok = fabs(x) < 9.2233720368547758e18 && trunc(x) == x;
            v = ok ? (long long)x : 0;
        } else {
            // N0f8 / N0f16: the value c/255 (c/65535) is an integer only at 0 and 1
            const uint32_t c = st == IFX_N0F8 ? ((const uint8_t *)src)[i] : ((const uint16_t *)src)[i];
            const uint32_t one = st == IFX_N0F8 ? 255u : 65535u;
            ok = c == 0 || c == one;
            v = c == one ? 1 : 0;
        }
        long long lo, hi;
        switch (dt) {
        case IFX_U8: lo = 0; hi = 255; break;
        case IFX_I8: lo = -128; hi = 127; break;
        case IFX_I16: lo = -32768; hi = 32767; break;
        case IFX_U16: lo = 0; hi = 65535; break;
        case IFX_I32: lo = -2147483648LL; hi = 2147483647LL; break;
        default: lo = -9223372036854775807LL - 1; hi = 9223372036854775807LL; break;
        }
        if (!ok || v < lo || v > hi) {
            atomicExch(bad, 1);
            v = 0;
        }
        switch (dt) {
        case IFX_U8: ((uint8_t *)dst)[i] = (uint8_t)v; break;
        case IFX_I8: ((int8_t *)dst)[i] = (int8_t)v; break;
        case IFX_I16: ((int16_t *)dst)[i] = (int16_t)v; break;
        case IFX_U16: ((uint16_t *)dst)[i] = (uint16_t)v; break;
        case IFX_I32: ((int32_t *)dst)[i] = (int32_t)v; break;
        default: ((long long *)dst)[i] = v; break;
        }
    }
}

cudaError_t launch_convert(const void *src, int st, void *dst, int dt, long long n, int *bad, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    long long g = (n + 255) / 256;
    if (g > 152LL * 32) g = 152LL * 32;
    k_convert<<<(int)g, 256, 0, s>>>(src, st, dst, dt, n, bad);
    note_launch();
    return cudaGetLastError();
}

} // namespace ifx
