// ifx_blob.cu -- the callers of the filter path used by blob_LoG
// (src/extrema.jl:72-164):
//   * ifx_findlocalextrema: findlocalmaxima / findlocalminima
//     (findlocalextrema, src/extrema.jl:125-159) on an N-d array (N <= 4):
//     element i is kept when img[i] > img[i+j] (or <) for every j != 0 of the
//     window that lies in the array, over the indices that the `edges` flags
//     leave in; the kept linear indices come back in column-major order (the
//     order of CartesianIndices), with their values.
//   * ifx_maxabs: maximum(abs, img).
// Compaction keeps the order: per block of kLeChunk elements a count, one
// scan of the counts, then each block writes its indices at its offset in
// element order (warp ballots).
#include "ifx_internal.h"
#include <cstring>
#include <vector>

namespace ifx {

constexpr int kLeChunk = 2048;      // elements per block
constexpr int kLeThreads = 256;

template <class T>
__device__ __forceinline__ double le_val(const T *p, long long i, bool norm)
{
    if constexpr (sizeof(T) == 1) return norm ? (double)p[i] / 255.0 : (double)p[i];
    else return (double)p[i];
}

// Is element e a strict local extremum?
template <class T>
__device__ bool le_test(const LeArgs &a, long long e)
{
    const T *p = (const T *)a.img;
    const bool norm = a.eltype == IFX_N0F8;
    long long c[IFX_MAXD] = {0, 0, 0, 0};
    long long rem = e;
    for (int d = 0; d < a.nd; ++d) {
        c[d] = rem % a.n[d];
        rem /= a.n[d];
        if (c[d] < a.lo[d] || c[d] > a.hi[d]) return false;
    }
    const double v = le_val<T>(p, e, norm);
    if (v != v) return false;                        // NaN: no comparison holds
    long long st[IFX_MAXD];
    long long s = 1;
    for (int d = 0; d < IFX_MAXD; ++d) {
        st[d] = s;
        s *= d < a.nd ? a.n[d] : 1;
    }
    const int h0 = a.half[0], h1 = a.nd > 1 ? a.half[1] : 0, h2 = a.nd > 2 ? a.half[2] : 0,
              h3 = a.nd > 3 ? a.half[3] : 0;
    for (int j3 = -h3; j3 <= h3; ++j3) {
        if (c[3] + j3 < 0 || (a.nd > 3 && c[3] + j3 >= a.n[3])) continue;
        for (int j2 = -h2; j2 <= h2; ++j2) {
            if (c[2] + j2 < 0 || (a.nd > 2 && c[2] + j2 >= a.n[2])) continue;
            for (int j1 = -h1; j1 <= h1; ++j1) {
                if (c[1] + j1 < 0 || (a.nd > 1 && c[1] + j1 >= a.n[1])) continue;
                for (int j0 = -h0; j0 <= h0; ++j0) {
                    if (c[0] + j0 < 0 || c[0] + j0 >= a.n[0]) continue;
                    if (j0 == 0 && j1 == 0 && j2 == 0 && j3 == 0) continue;
                    const double w = le_val<T>(p, e + j0 * st[0] + j1 * st[1] + j2 * st[2] + j3 * st[3], norm);
                    if (a.minima ? !(v < w) : !(v > w)) return false;
                }
            }
        }
    }
    return true;
}

template <class T>
__global__ void __launch_bounds__(kLeThreads) k_le_count(LeArgs a, unsigned long long *counts)
{
    const long long base = (long long)blockIdx.x * kLeChunk;
    int cnt = 0;
    for (int k = threadIdx.x; k < kLeChunk; k += kLeThreads) {
        const long long e = base + k;
        if (e < a.total && le_test<T>(a, e)) ++cnt;
    }
    cnt = __reduce_add_sync(0xffffffffu, cnt);
    __shared__ int s_w[kLeThreads / 32];
    if ((threadIdx.x & 31) == 0) s_w[threadIdx.x >> 5] = cnt;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < kLeThreads / 32; ++w) t += s_w[w];
        counts[blockIdx.x] = t;
    }
}

// exclusive scan of the block counts: one block of 1024 threads, each owning a
// contiguous segment of the counts
__global__ void __launch_bounds__(1024) k_le_scan(unsigned long long *counts, long long nblocks,
                                                  unsigned long long *total)
{
    __shared__ unsigned long long s_seg[1024];
    const int t = threadIdx.x;
    const long long per = (nblocks + 1023) / 1024;
    const long long b0 = (long long)t * per, b1 = b0 + per < nblocks ? b0 + per : nblocks;
    unsigned long long sum = 0;
    for (long long b = b0; b < b1; ++b) sum += counts[b];
    s_seg[t] = sum;
    __syncthreads();
    if (t == 0) {
        unsigned long long run = 0;
        for (int k = 0; k < 1024; ++k) {
            const unsigned long long c = s_seg[k];
            s_seg[k] = run;
            run += c;
        }
        *total = run;
    }
    __syncthreads();
    unsigned long long run = s_seg[t];
    for (long long b = b0; b < b1; ++b) {
        const unsigned long long c = counts[b];
        counts[b] = run;
        run += c;
    }
}

template <class T>
__global__ void __launch_bounds__(kLeThreads)
k_le_scatter(LeArgs a, const unsigned long long *offsets, long long *idx, double *val, long long capacity)
{
    const long long base = (long long)blockIdx.x * kLeChunk;
    __shared__ unsigned long long s_run;
    __shared__ int s_w[kLeThreads / 32];
    if (threadIdx.x == 0) s_run = offsets[blockIdx.x];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool norm = a.eltype == IFX_N0F8;
    for (int k0 = 0; k0 < kLeChunk; k0 += kLeThreads) {
        const long long e = base + k0 + threadIdx.x;
        const bool keep = e < a.total && le_test<T>(a, e);
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) s_w[warp] = __popc(m);
        __syncthreads();
        unsigned long long off = s_run;
        for (int w = 0; w < warp; ++w) off += s_w[w];
        off += __popc(m & ((1u << lane) - 1));
        if (keep && off < (unsigned long long)capacity) {
            idx[off] = e;
            val[off] = le_val<T>((const T *)a.img, e, norm);
        }
        __syncthreads();
        if (threadIdx.x == 0)
            for (int w = 0; w < kLeThreads / 32; ++w) s_run += s_w[w];
        __syncthreads();
    }
}

template <class T>
static cudaError_t le_run(const LeArgs &a, long long nblocks, unsigned long long *counts, unsigned long long *total,
                          long long *idx, double *val, long long capacity, cudaStream_t s)
{
    k_le_count<T><<<(unsigned)nblocks, kLeThreads, 0, s>>>(a, counts);
    k_le_scan<<<1, 1024, 0, s>>>(counts, nblocks, total);
    k_le_scatter<T><<<(unsigned)nblocks, kLeThreads, 0, s>>>(a, counts, idx, val, capacity);
    note_launch(3);
    return cudaGetLastError();
}

cudaError_t launch_localextrema(const LeArgs &a, unsigned long long *counts, unsigned long long *total,
                                long long *idx, double *val, long long capacity, cudaStream_t s)
{
    const long long nblocks = (a.total + kLeChunk - 1) / kLeChunk;
    if (a.eltype == IFX_F32) return le_run<float>(a, nblocks, counts, total, idx, val, capacity, s);
    if (a.eltype == IFX_F64) return le_run<double>(a, nblocks, counts, total, idx, val, capacity, s);
    if (a.eltype == IFX_N0F8 || a.eltype == IFX_U8) return le_run<uint8_t>(a, nblocks, counts, total, idx, val, capacity, s);
    return cudaErrorInvalidValue;
}

long long localextrema_blocks(long long total) { return (total + kLeChunk - 1) / kLeChunk; }

// ---------------------------------------------------------------- term sums
// out = (out + term) * scale (scale applied with the last term), in the
// output eltype: the separable terms of a kernel written as a sum.
template <class T>
__global__ void k_sum_scale(T *__restrict__ out, const T *__restrict__ term, long long n, double scale, int last)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        T v = out[i] + term[i];
        if (last) v = (T)(v * (T)scale);
        out[i] = v;
    }
}

cudaError_t launch_sum_scale(void *out, const void *term, int eltype, long long n, double scale, int last,
                             cudaStream_t s)
{
    if (n == 0) return cudaSuccess;
    long long g = (n + 255) / 256;
    if (g > 152LL * 32) g = 152LL * 32;
    if (eltype == IFX_F32) k_sum_scale<float><<<(int)g, 256, 0, s>>>((float *)out, (const float *)term, n, scale, last);
    else if (eltype == IFX_F64) k_sum_scale<double><<<(int)g, 256, 0, s>>>((double *)out, (const double *)term, n, scale, last);
    else return cudaErrorInvalidValue;
    note_launch();
    return cudaGetLastError();
}

// ---------------------------------------------------------------- max |x|
// out[0]: bits of the largest |x| that is not NaN (non-negative doubles order
// like their bit patterns); out[1]: 1 when some element is NaN.
template <class T>
__global__ void k_maxabs(const T *__restrict__ p, long long n, bool norm, unsigned long long *out)
{
    double m = 0.0;
    bool nan = false;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const double v = fabs(le_val<T>(p, i, norm));
        if (v != v) nan = true;
        else if (v > m) m = v;
    }
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    nan = __any_sync(0xffffffffu, nan);
    if ((threadIdx.x & 31) == 0) {
        atomicMax(out, (unsigned long long)__double_as_longlong(m));
        if (nan) atomicExch(out + 1, 1ull);
    }
}

cudaError_t launch_maxabs(const void *img, int eltype, long long n, unsigned long long *out, cudaStream_t s)
{
    long long g = (n + 255) / 256;
    if (g < 1) g = 1;
    if (g > 152LL * 16) g = 152LL * 16;
    const bool norm = eltype == IFX_N0F8;
    if (eltype == IFX_F32) k_maxabs<float><<<(int)g, 256, 0, s>>>((const float *)img, n, norm, out);
    else if (eltype == IFX_F64) k_maxabs<double><<<(int)g, 256, 0, s>>>((const double *)img, n, norm, out);
    else if (eltype == IFX_N0F8 || eltype == IFX_U8) k_maxabs<uint8_t><<<(int)g, 256, 0, s>>>((const uint8_t *)img, n, norm, out);
    else return cudaErrorInvalidValue;
    note_launch();
    return cudaGetLastError();
}

} // namespace ifx
