// ifx_na.cu -- the pieces of NA() filtering (src/imfilter.jl:280-318,
// 1094-1130, 1234-1250) that are not a filter:
//   * ifx_na_prepare: the NA flags of an image (isnan, !isfinite or none), the
//     image with NA elements set to zero in the output eltype (`imgtmp`), the
//     valid-pixel mask (`validpixels`) and whether any element is NA;
//   * ifx_na_divide: out ./= den, elementwise (imfilter_na_inseparable!);
//   * ifx_na_normalize_separable: out[I] = (((out[I] / f1[i1]) / f2[i2]) ...)
//     with per-axis 1-D sums (normalize_dims!), the division in Float64.
// The filters themselves (Fill(0) cascades of the image and of the mask) are
// the library's ordinary entry points.
#include "ifx_internal.h"
#include <cstring>

namespace ifx {

static inline bool is8(int t) { return t == IFX_N0F8 || t == IFX_U8; }

template <class T> __device__ __forceinline__ bool na_test(T v, int na)
{
    if (na == IFX_NA_ISNAN) return isnan(v);
    if (na == IFX_NA_NOTFINITE) return !isfinite(v);
    return false;
}

template <class Tin, class Tz, class Tv>
__global__ void k_na_prepare(const Tin *__restrict__ img, Tz *__restrict__ zeroed, Tv *__restrict__ valid,
                             long long n, int na, bool norm, int *flag)
{
    bool any = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const Tin v = img[i];
        bool isna = false;
        if constexpr (sizeof(Tin) > 1) isna = na_test(v, na);
        Tz z;
        if constexpr (sizeof(Tin) == 1)
            z = norm ? (Tz)v / (Tz)255 : (Tz)v;
        else
            z = (Tz)v;
        zeroed[i] = isna ? (Tz)0 : z;
        valid[i] = isna ? (Tv)0 : (Tv)1;
        any |= isna;
    }
    if (__any_sync(0xffffffffu, any) && (threadIdx.x & 31) == 0) atomicExch(flag, 1);
}

template <class T, class Td>
__global__ void k_na_divide(T *__restrict__ out, const Td *__restrict__ den, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        out[i] = (T)((double)out[i] / (double)den[i]);
}

struct NaFactors {
    const double *f[IFX_MAXD];
    long long n[IFX_MAXD];
    int nd;
};

template <class T>
__global__ void k_na_normalize(T *__restrict__ out, long long total, NaFactors F)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        long long rem = i;
        double tmp = (double)out[i];
        for (int d = 0; d < F.nd; ++d) {
            const long long c = rem % F.n[d];
            rem /= F.n[d];
            tmp /= F.f[d][c];
        }
        out[i] = (T)tmp;
    }
}

static int grid_for(long long n)
{
    long long g = (n + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152LL * 32) g = 152LL * 32;
    return (int)g;
}

template <class Tin, class Tz, class Tv>
static cudaError_t na_prepare_t(const void *img, void *z, void *v, long long n, int na, bool norm, int *flag,
                                cudaStream_t s)
{
    k_na_prepare<Tin, Tz, Tv><<<grid_for(n), 256, 0, s>>>((const Tin *)img, (Tz *)z, (Tv *)v, n, na, norm, flag);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_na_prepare(const void *img, int it, void *z, int zt, void *v, int vt, long long n, int na,
                              int *flag, cudaStream_t s)
{
    const bool norm = it == IFX_N0F8;
    if (n == 0) return cudaSuccess;
#define IFX_NA_V(TIN, TZ)                                                                            \
    do {                                                                                             \
        if (vt == IFX_F32) return na_prepare_t<TIN, TZ, float>(img, z, v, n, na, norm, flag, s);     \
        if (vt == IFX_F64) return na_prepare_t<TIN, TZ, double>(img, z, v, n, na, norm, flag, s);    \
    } while (0)
    if (it == IFX_F32 && zt == IFX_F32) IFX_NA_V(float, float);
    if (it == IFX_F32 && zt == IFX_F64) IFX_NA_V(float, double);
    if (it == IFX_F64 && zt == IFX_F64) IFX_NA_V(double, double);
    if (it == IFX_F64 && zt == IFX_F32) IFX_NA_V(double, float);
    if (is8(it) && zt == IFX_F32) IFX_NA_V(uint8_t, float);
    if (is8(it) && zt == IFX_F64) IFX_NA_V(uint8_t, double);
#undef IFX_NA_V
    return cudaErrorInvalidValue;
}

cudaError_t launch_na_divide(void *out, int ot, const void *den, int dt, long long n, cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    const int g = grid_for(n);
    if (ot == IFX_F32 && dt == IFX_F32) k_na_divide<float, float><<<g, 256, 0, s>>>((float *)out, (const float *)den, n);
    else if (ot == IFX_F32 && dt == IFX_F64) k_na_divide<float, double><<<g, 256, 0, s>>>((float *)out, (const double *)den, n);
    else if (ot == IFX_F64 && dt == IFX_F64) k_na_divide<double, double><<<g, 256, 0, s>>>((double *)out, (const double *)den, n);
    else if (ot == IFX_F64 && dt == IFX_F32) k_na_divide<double, float><<<g, 256, 0, s>>>((double *)out, (const float *)den, n);
    else return cudaErrorInvalidValue;
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_na_normalize(void *out, int ot, long long total, const double *const *f, const long long *n,
                                int nd, cudaStream_t s)
{
    if (total == 0) return cudaSuccess;
    NaFactors F;
    memset(&F, 0, sizeof F);
    F.nd = nd;
    for (int d = 0; d < nd; ++d) {
        F.f[d] = f[d];
        F.n[d] = n[d];
    }
    const int g = grid_for(total);
    if (ot == IFX_F32) k_na_normalize<float><<<g, 256, 0, s>>>((float *)out, total, F);
    else if (ot == IFX_F64) k_na_normalize<double><<<g, 256, 0, s>>>((double *)out, total, F);
    else return cudaErrorInvalidValue;
    note_launch();
    return cudaGetLastError();
}

} // namespace ifx
