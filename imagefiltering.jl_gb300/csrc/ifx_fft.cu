// ifx_fft.cu -- Algorithm.FFT() (src/imfilter.jl:776-884) with cuFFT.
//
// The reference pads each axis of length l, for a kernel of length lk on
// offsets kfirst..kfirst+lk-1, to P = nextprod([2,3], l + lk) elements with the
// border style (padfft, src/border.jl:239-248; Fill 551-555), then takes the
// circular cross-correlation of the padded image with the kernel through real
// FFTs (filtfft: rfft(A) .* conj(rfft(krn)), irfft) and keeps the image's
// indices.  With the padded image A0 covering image indices kfirst+1 ..
// kfirst+P and the kernel placed at 0..lk-1 of a zero array krn0,
//     R0[p] = sum_q A0[p+q] krn0[q] = sum_j img_padded[p+1+j] K[j]  = out[p+1],
// and P >= l + lk keeps p + q < P for every p < l: no wrap reaches the
// outputs.  Transforms run in the output's precision.
//
// cuFFT is loaded at run time (dlopen), so the library has no link-time
// dependency on it; without it this entry point reports IFX_ERR_UNSUPPORTED.
#include "ifx_internal.h"
#include <cufft.h>
#include <dlfcn.h>
#include <algorithm>
#include <mutex>
#include <vector>

namespace ifx {

struct CufftApi {
    decltype(&cufftPlanMany) plan_many = nullptr;
    decltype(&cufftExecR2C) r2c = nullptr;
    decltype(&cufftExecC2R) c2r = nullptr;
    decltype(&cufftExecD2Z) d2z = nullptr;
    decltype(&cufftExecZ2D) z2d = nullptr;
    decltype(&cufftSetStream) set_stream = nullptr;
    decltype(&cufftDestroy) destroy = nullptr;
    bool ok = false;
};

static const CufftApi &cufft_api()
{
    static CufftApi api;
    static std::once_flag once;
    std::call_once(once, [] {
        void *h = nullptr;
        for (const char *name : {"libcufft.so.12", "libcufft.so.13", "libcufft.so"})
            if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL))) break;
        if (!h) return;
        api.plan_many = (decltype(api.plan_many))dlsym(h, "cufftPlanMany");
        api.r2c = (decltype(api.r2c))dlsym(h, "cufftExecR2C");
        api.c2r = (decltype(api.c2r))dlsym(h, "cufftExecC2R");
        api.d2z = (decltype(api.d2z))dlsym(h, "cufftExecD2Z");
        api.z2d = (decltype(api.z2d))dlsym(h, "cufftExecZ2D");
        api.set_stream = (decltype(api.set_stream))dlsym(h, "cufftSetStream");
        api.destroy = (decltype(api.destroy))dlsym(h, "cufftDestroy");
        api.ok = api.plan_many && api.r2c && api.c2r && api.d2z && api.z2d && api.set_stream && api.destroy;
    });
    return api;
}

bool fft_available() { return cufft_api().ok; }

long long fft_size(long long l, long long lk)
{
    const long long need = l + lk;
    long long best = -1;
    for (long long p2 = 1; p2 <= 2 * need; p2 *= 2)
        for (long long p = p2; p <= 2 * need; p *= 3)
            if (p >= need && (best < 0 || p < best)) best = p;
    return best;
}

// kernel K (column-major, ksize) into the zeroed padded array at 0..lk-1
template <class T>
__global__ void k_fft_place(T *krn, const double *K, int nd, int4 P, int4 ks, long long kn)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < kn;
         i += (long long)gridDim.x * blockDim.x) {
        const int ksa[4] = {ks.x, ks.y, ks.z, ks.w}, Pa[4] = {P.x, P.y, P.z, P.w};
        long long rem = i, o = 0, st = 1;
        for (int d = 0; d < 4; ++d) {
            const long long c = rem % ksa[d];
            rem /= ksa[d];
            o += c * st;
            st *= Pa[d];
        }
        krn[o] = (T)K[i];
    }
}

template <class C>
__global__ void k_fft_mulconj(C *a, const C *b, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const C x = a[i], y = b[i];
        a[i].x = x.x * y.x + x.y * y.y;             // x * conj(y)
        a[i].y = x.y * y.x - x.x * y.y;
    }
}

// out[i] = R0[i] * scale for the image's indices (R0 has the padded sizes):
// one output row (axis 0) per block row, the row index split once per row
template <class Tc, class Tout>
__global__ void k_fft_crop(const Tc *R, Tout *out, int4 n, int4 P, long long rows, Tc scale)
{
    for (long long row = blockIdx.y * (long long)blockDim.y + threadIdx.y; row < rows;
         row += (long long)gridDim.y * blockDim.y) {
        const long long y = row % n.y, zw = row / n.y, z = zw % n.z, w = zw / n.z;
        const Tc *src = R + ((w * P.z + z) * P.y + y) * (long long)P.x;
        Tout *dst = out + row * (long long)n.x;
        for (int x = blockIdx.x * blockDim.x + threadIdx.x; x < n.x; x += gridDim.x * blockDim.x)
            dst[x] = out_cvt<Tout>(src[x] * scale);
    }
}

static int grid_of(long long n)
{
    long long g = (n + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152LL * 32) g = 152LL * 32;
    return (int)g;
}

// Plans are kept between calls (creating one allocates its work area): keyed
// by rank, sizes, transform type and stream, so that two streams never share a
// work area.  A short list, oldest out first.
struct PlanEntry {
    int nd, dims[3];
    cufftType type;
    cudaStream_t stream;
    cufftHandle h;
};
static std::mutex g_plan_mu;
static std::vector<PlanEntry> g_plans;
constexpr size_t kMaxPlans = 16;

static int plan_get(int nd, const int *dims, cufftType type, cudaStream_t s, cufftHandle *out)
{
    for (const PlanEntry &e : g_plans)
        if (e.nd == nd && e.type == type && e.stream == s && std::equal(dims, dims + nd, e.dims)) {
            *out = e.h;
            return 0;
        }
    const CufftApi &api = cufft_api();
    PlanEntry e{};
    e.nd = nd;
    std::copy(dims, dims + nd, e.dims);
    e.type = type;
    e.stream = s;
    if (api.plan_many(&e.h, nd, e.dims, nullptr, 1, 0, nullptr, 1, 0, type, 1) != CUFFT_SUCCESS) return -1;
    if (api.set_stream(e.h, s) != CUFFT_SUCCESS) {
        api.destroy(e.h);
        return -1;
    }
    if (g_plans.size() >= kMaxPlans) {
        // the oldest plan's work may still be queued (its stream may be gone)
        cudaDeviceSynchronize();
        api.destroy(g_plans.front().h);
        g_plans.erase(g_plans.begin());
    }
    g_plans.push_back(e);
    *out = e.h;
    return 0;
}

// padded: the padded image in the compute type (P elements, column-major);
// buffers: krn (real, P), spectra A and K (complex, Pc each), result R (real, P).
template <class Tc, class Tout>
static int fft_run_t(const FftArgs &f, cudaStream_t s)
{
    using Cx = typename std::conditional<sizeof(Tc) == 8, cufftDoubleComplex, cufftComplex>::type;
    const CufftApi &api = cufft_api();
    int dims[3];                                       // slowest first for cuFFT
    for (int d = 0; d < f.nd; ++d) dims[d] = (int)f.P[f.nd - 1 - d];
    const cufftType tf = sizeof(Tc) == 8 ? CUFFT_D2Z : CUFFT_R2C, ti = sizeof(Tc) == 8 ? CUFFT_Z2D : CUFFT_C2R;
    std::lock_guard<std::mutex> lk(g_plan_mu);
    cufftHandle fwd, inv;
    if (plan_get(f.nd, dims, tf, s, &fwd) || plan_get(f.nd, dims, ti, s, &inv)) return -1;
    Tc *krn = (Tc *)f.krn;
    Cx *A = (Cx *)f.specA, *K = (Cx *)f.specK;
    if (cudaMemsetAsync(krn, 0, sizeof(Tc) * f.Ptotal, s) != cudaSuccess) return -2;
    int4 P4 = make_int4((int)f.P[0], (int)f.P[1], (int)f.P[2], (int)f.P[3]);
    int4 k4 = make_int4(f.ksize[0], f.ksize[1], f.ksize[2], f.ksize[3]);
    k_fft_place<Tc><<<grid_of(f.kn), 256, 0, s>>>(krn, f.Kdev, f.nd, P4, k4, f.kn);
    cufftResult r;
    if constexpr (sizeof(Tc) == 8) {
        r = api.d2z(fwd, (cufftDoubleReal *)f.padded, (cufftDoubleComplex *)A);
        if (r == CUFFT_SUCCESS) r = api.d2z(fwd, (cufftDoubleReal *)krn, (cufftDoubleComplex *)K);
    } else {
        r = api.r2c(fwd, (cufftReal *)f.padded, (cufftComplex *)A);
        if (r == CUFFT_SUCCESS) r = api.r2c(fwd, (cufftReal *)krn, (cufftComplex *)K);
    }
    if (r != CUFFT_SUCCESS) return -1;
    k_fft_mulconj<Cx><<<grid_of(f.Pc), 256, 0, s>>>(A, K, f.Pc);
    Tc *R = krn;                                       // the kernel's real buffer is free again
    if constexpr (sizeof(Tc) == 8) r = api.z2d(inv, (cufftDoubleComplex *)A, (cufftDoubleReal *)R);
    else r = api.c2r(inv, (cufftComplex *)A, (cufftReal *)R);
    if (r != CUFFT_SUCCESS) return -1;
    int4 n4 = make_int4((int)f.n[0], (int)f.n[1], (int)f.n[2], (int)f.n[3]);
    {
        const long long rows = f.total / f.n[0];
        const dim3 blk(128, 2);
        const unsigned gx = (unsigned)((f.n[0] + 127) / 128);
        const long long gy = (rows + 1) / 2 < 65535 ? (rows + 1) / 2 : 65535;
        k_fft_crop<Tc, Tout><<<dim3(gx, (unsigned)gy), blk, 0, s>>>(R, (Tout *)f.out, n4, P4, rows,
                                                                    (Tc)(1.0 / (double)f.Ptotal));
    }
    note_launch(4);
    return cudaGetLastError() == cudaSuccess ? 0 : -2;
}

int launch_fft(const FftArgs &f, cudaStream_t s)
{
    if (!fft_available()) return -3;
    if (f.compute_f64) {
        if (f.out_type == IFX_F64) return fft_run_t<double, double>(f, s);
        if (f.out_type == IFX_F32) return fft_run_t<double, float>(f, s);
    } else {
        if (f.out_type == IFX_F32) return fft_run_t<float, float>(f, s);
        if (f.out_type == IFX_F64) return fft_run_t<float, double>(f, s);
    }
    return -4;
}

} // namespace ifx
