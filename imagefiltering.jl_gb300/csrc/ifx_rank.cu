// ifx_rank.cu -- rank filters for sm_103a: median (mapwindow(median!, ...))
// and running min/max (mapwindow(extrema / minimum / maximum, ...)).
// Both are bit-exact: they select or compare input values, never compute new
// ones.
//
// Median (src/mapwindow.jl:123-131): the ((1+m) div 2)-th smallest of the m
// window values.  8-bit images take a packed-SIMD path: each thread owns four
// horizontally adjacent outputs in one 32-bit word and finds the median bit by
// bit from the most significant: the answer is the largest v with
// #{window values < v} < rank, and every candidate test is one byte-wise
// compare (__vcmpltu4) and one byte-wise count update (__vsub4) per window
// element, for all four pixels at once.
//
// Windows at the border follow copy_win! (src/mapwindow.jl:310-333): a Pad
// style pads relative to window-intersect-image.  For replicate, symmetric and
// reflect that is the same as mapping through the whole image (the truncated
// window never needs a second reflection), so the 2-D tile kernels gather a
// padded tile.  Circular wraps inside the truncated window: the tile kernels
// read the windows that leave the image straight from the image through the
// window-relative map (win_index2); N-d images and other window shapes use the
// per-pixel kernel, which applies the window-relative map literally.
#include "ifx_internal.h"
#include "ifx_select.cuh"
#include <cstring>
#include <type_traits>
#include <utility>

namespace ifx {

static inline int grid1(long long n, int block)
{
    long long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 152LL * 64) g = 152LL * 64;
    return (int)g;
}

template <class T> __device__ __forceinline__ void store_sel(void *out, int out_type, long long i,
                                                             T v, bool norm);
template <> __device__ __forceinline__ void store_sel<uint8_t>(void *out, int out_type, long long i,
                                                               uint8_t v, bool norm)
{
    if (out_type == IFX_F32)
        ((float *)out)[i] = norm ? n0f8_to_f32(v) : (float)v;
    else if (out_type == IFX_F64)
        ((double *)out)[i] = norm ? __ddiv_rn((double)v, 255.0) : (double)v;
    else
        ((uint8_t *)out)[i] = v;
}
template <> __device__ __forceinline__ void store_sel<float>(void *out, int out_type, long long i,
                                                             float v, bool)
{
    if (out_type == IFX_F64) ((double *)out)[i] = (double)v;
    else ((float *)out)[i] = v;
}
template <> __device__ __forceinline__ void store_sel<double>(void *out, int out_type, long long i,
                                                              double v, bool)
{
    if (out_type == IFX_F32) ((float *)out)[i] = (float)v;
    else ((double *)out)[i] = v;
}

// Julia's isless order for floats (NaN after everything); plain < for codes.
template <class T> __device__ __forceinline__ bool lt(T a, T b) { return a < b; }
template <> __device__ __forceinline__ bool lt<float>(float a, float b)
{
    return isnan(b) ? !isnan(a) : a < b;
}
template <> __device__ __forceinline__ bool lt<double>(double a, double b)
{
    return isnan(b) ? !isnan(a) : a < b;
}

// Offset in a 2-D image of window element (i, j) of output (x, y) under the
// window-relative map of copy_win! (window first offsets f0/f1, lengths
// w0/w1): the Pad style is applied relative to window-intersect-image.
__device__ __forceinline__ long long win_index2(int x, int y, int i, int j, int f0, int f1, int w0,
                                                int w1, int nx, int ny, int style)
{
    const int ofx = x + f0, olx = ofx + w0 - 1, ofy = y + f1, oly = ofy + w1 - 1;
    const int ax = ofx > 0 ? ofx : 0, bx = olx < nx - 1 ? olx : nx - 1;
    const int ay = ofy > 0 ? ofy : 0, by = oly < ny - 1 ? oly : ny - 1;
    const int mx = map_index_in(ofx + i, ax, bx - ax + 1, style);
    const int my = map_index_in(ofy + j, ay, by - ay + 1, style);
    return (long long)my * nx + mx;
}

// Does the window of output (x, y) leave the image?
__device__ __forceinline__ bool win_leaves(int x, int y, int f0, int f1, int w0, int w1, int nx, int ny)
{
    return x + f0 < 0 || x + f0 + w0 > nx || y + f1 < 0 || y + f1 + w1 > ny;
}

// 8-bit median of the window of output (x, y) read from the image through
// the window-relative map: the largest code v with #{window codes < v} < rank,
// found bit by bit from the most significant.
__device__ __forceinline__ uint32_t median_u8_direct(const uint8_t *img, int x, int y, int f0, int f1, int w0,
                                                     int w1, int nx, int ny, int style)
{
    const int rank = (w0 * w1 + 1) / 2;
    uint32_t res = 0;
    for (int b = 7; b >= 0; --b) {
        const uint32_t trial = res | (1u << b);
        int cnt = 0;
        for (int j = 0; j < w1; ++j)
            for (int i = 0; i < w0; ++i) cnt += img[win_index2(x, y, i, j, f0, f1, w0, w1, nx, ny, style)] < trial;
        if (cnt < rank) res = trial;
    }
    return res;
}

// Circular images: after a tile's outputs are stored, the outputs whose
// windows leave the image (they wrap inside window-intersect-image, which the
// tile gathered through the whole-image map does not hold) are recomputed,
// shared evenly by the CTA's threads.  The condition is uniform in the CTA.
template <class F>
__device__ __forceinline__ void circular_edges(int style, int tx0, int ty0, int tw, int th, int nx, int ny, int f0,
                                               int f1, int w0, int w1, F one)
{
    if (style != IFX_CIRCULAR) return;
    const EdgeRects E(tx0, ty0, tw, th, nx, ny, -f0, f0 + w0 - 1, -f1, f1 + w1 - 1);
    if (E.count == 0) return;
    __syncthreads();
    for (int e = threadIdx.x; e < E.count; e += blockDim.x) {
        int x, y;
        E.at(e, x, y);
        one(x, y);
    }
}

// =========================================================================
// Per-pixel median, any eltype, N-d, window up to kMaxWin values.
// =========================================================================
constexpr int kMaxWin = 256;

template <class T>
__global__ void k_median_px(const T *__restrict__ img, void *out, int out_type, int nd, int4 n4,
                            int4 wf4, int4 wl4, int style, T fill, bool norm)
{
    const int n[4] = {n4.x, n4.y, n4.z, n4.w};
    const int wf[4] = {wf4.x, wf4.y, wf4.z, wf4.w};
    const int wl[4] = {wl4.x, wl4.y, wl4.z, wl4.w};
    const long long total = (long long)n[0] * n[1] * n[2] * n[3];
    const int m = wl[0] * wl[1] * wl[2] * wl[3];
    const int rank = (m + 1) / 2;             // 1-based
    T buf[kMaxWin];
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        int c[4], ilo[4], ilen[4];
        long long rem = p;
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            c[d] = (int)(rem % n[d]);
            rem /= n[d];
            int of = c[d] + wf[d], ol = of + wl[d] - 1;
            int a = of > 0 ? of : 0, b = ol < n[d] - 1 ? ol : n[d] - 1;
            ilo[d] = a;
            ilen[d] = b - a + 1;
        }
        // gather (copy_win!: Pad styles relative to window-intersect-image)
        int t = 0;
        for (int l = 0; l < wl[3]; ++l)
            for (int k = 0; k < wl[2]; ++k)
                for (int j = 0; j < wl[1]; ++j)
                    for (int i = 0; i < wl[0]; ++i, ++t) {
                        const int q[4] = {c[0] + wf[0] + i, c[1] + wf[1] + j, c[2] + wf[2] + k,
                                          c[3] + wf[3] + l};
                        long long off = 0, st = 1;
                        bool outside = false;
#pragma unroll
                        for (int d = 0; d < 4; ++d) {
                            int mm = style == IFX_FILL
                                         ? (((unsigned)q[d] < (unsigned)n[d]) ? q[d] : -1)
                                         : map_index_in(q[d], ilo[d], ilen[d], style);
                            outside |= mm < 0;
                            off += (long long)mm * st;
                            st *= n[d];
                        }
                        buf[t] = outside ? fill : img[off];
                    }
        // selection: the value with #less < rank <= #less + #equal
        T med = buf[0];
        for (int a = 0; a < m; ++a) {
            int less = 0, eq = 0;
            for (int b = 0; b < m; ++b) {
                less += lt(buf[b], buf[a]);
                eq += !lt(buf[b], buf[a]) && !lt(buf[a], buf[b]);
            }
            if (less < rank && rank <= less + eq) {
                med = buf[a];
                break;
            }
        }
        store_sel<T>(out, out_type, p, med, norm);
    }
}

// =========================================================================
// Packed 8-bit median, 2-D.  CTA tile: TX = 128 outputs wide (32 threads x 4
// pixels), TY = 8 rows; the padded input tile is gathered into shared memory
// through the whole-image border map.  W0/W1 > 0 fixes the window at compile
// time (the words stay in registers); W0 == 0 reads them from shared memory
// every round.
// =========================================================================
constexpr int kMedTX = 128, kMedTY = 8;

template <int W0, int W1>
__global__ void __launch_bounds__(256)
k_median_u8(const uint8_t *__restrict__ img, void *out, int out_type, int nx, int ny, int f0,
            int f1, int w0rt, int w1rt, int style, uint8_t fill, bool norm)
{
    const int w0 = W0 > 0 ? W0 : w0rt, w1 = W1 > 0 ? W1 : w1rt;
    extern __shared__ __align__(16) uint8_t tile[];
    const int CT = ((kMedTX + w0 - 1 + 3) & ~3) + 4;
    const int RT = kMedTY + w1 - 1;
    const int tx0 = blockIdx.x * kMedTX, ty0 = blockIdx.y * kMedTY;
    gather_tile<8>(tile, RT * CT, [&](int idx) -> uint8_t {
        const int r = idx / CT, c = idx - r * CT;
        if (c >= kMedTX + w0 - 1) return 0;
        const int mx = map_index(tx0 + f0 + c, nx, style);
        const int my = map_index(ty0 + f1 + r, ny, style);
        return (mx < 0 || my < 0) ? fill : img[(long long)my * nx + mx];
    });
    __syncthreads();
    const int lx = (threadIdx.x & 31) * 4, ly = threadIdx.x >> 5;
    const int m = w0 * w1;
    const uint32_t rank4 = 0x01010101u * (uint32_t)((m + 1) / 2);
    auto word = [&](int j, int i) -> uint32_t { return load_word(tile + (size_t)(ly + j) * CT, lx + i); };
    uint32_t res = 0;
    if constexpr (W0 == 3 && W1 == 3) {               // shared column sorts
        uint32_t A[W0], B[W0];
#pragma unroll
        for (int j = 0; j < W0; ++j) {
            A[j] = word(j, 0);
            B[j] = word(j, 4);
        }
        res = median3x3_u8x4(A, B);
    } else if constexpr (W0 > 0 && W1 > 0) {
        // fixed window: byte-wise selection network (four windows per word)
        uint32_t w[W0 * W1];
#pragma unroll
        for (int j = 0; j < W1; ++j)
#pragma unroll
            for (int i = 0; i < W0; ++i) w[j * W0 + i] = word(j, i);
        res = median_u8x4<W0 * W1>(w);
    } else {
        for (int b = 7; b >= 0; --b) {
            const uint32_t trial = res | (0x01010101u << b);
            uint32_t cnt = 0;
            for (int j = 0; j < w1; ++j)
                for (int i = 0; i < w0; ++i) cnt = count_lt(cnt, word(j, i), trial);
            const uint32_t below = __vcmpltu4(cnt, rank4);
            res = (trial & below) | (res & ~below);
        }
    }
    const int y = ty0 + ly;
    if (y < ny) {
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const int x = tx0 + lx + q;
            if (x < nx) store_sel<uint8_t>(out, out_type, (long long)y * nx + x,
                                           (uint8_t)(res >> (8 * q)), norm);
        }
    }
    circular_edges(style, tx0, ty0, kMedTX, kMedTY, nx, ny, f0, f1, w0, w1, [&](int xe, int ye) {
        store_sel<uint8_t>(out, out_type, (long long)ye * nx + xe,
                           (uint8_t)median_u8_direct(img, xe, ye, f0, f1, w0, w1, nx, ny, style), norm);
    });
}

constexpr int kFmTX = 32, kFmTY = 8;

template <class T, int W0, int W1>
__global__ void __launch_bounds__(256)
k_median_float(const T *__restrict__ img, void *out, int out_type, int nx, int ny, int f0, int f1,
               int style, T fill)
{
    using SK = SortKey<T>;
    using K = typename SK::K;
    constexpr int CT = kFmTX + W0 - 1, RT = kFmTY + W1 - 1, N = W0 * W1;
    __shared__ K tile[RT * CT];                 // order-preserving keys of the window values
    const int tx0 = blockIdx.x * kFmTX, ty0 = blockIdx.y * kFmTY;
    gather_tile<8>(tile, RT * CT, [&](int idx) -> K {
        const int r = idx / CT, c = idx - r * CT;
        const int mx = map_index(tx0 + f0 + c, nx, style);
        const int my = map_index(ty0 + f1 + r, ny, style);
        return SK::key((mx < 0 || my < 0) ? fill : img[(long long)my * nx + mx]);
    });
    __syncthreads();
    const int lx = threadIdx.x % kFmTX, ly = threadIdx.x / kFmTX;
    const int x = tx0 + lx, y = ty0 + ly;
    K v[N];
#pragma unroll
    for (int j = 0; j < W1; ++j)
#pragma unroll
        for (int i = 0; i < W0; ++i) v[j * W0 + i] = tile[(ly + j) * CT + lx + i];
    net_sort<N, K>(v);
    if (x < nx && y < ny) store_sel<T>(out, out_type, (long long)y * nx + x, SK::val(v[(N - 1) / 2]), false);
    circular_edges(style, tx0, ty0, kFmTX, kFmTY, nx, ny, f0, f1, W0, W1, [&](int xe, int ye) {
        K u[N];
#pragma unroll
        for (int j = 0; j < W1; ++j)
#pragma unroll
            for (int i = 0; i < W0; ++i) u[j * W0 + i] = SK::key(img[win_index2(xe, ye, i, j, f0, f1, W0, W1, nx, ny, style)]);
        net_sort<N, K>(u);
        store_sel<T>(out, out_type, (long long)ye * nx + xe, SK::val(u[(N - 1) / 2]), false);
    });
}

// =========================================================================
// Square 3 x 3 and 5 x 5 medians, 2-D, through the generated block networks
// (ifx_median_nets.cuh): each thread computes a block of 4 x BH adjacent
// outputs from their shared footprint, sharing the column sorts and merges
// between the block's windows.  Floats run on order-preserving integer keys
// (Julia's isless order), 8-bit codes in the two 16-bit lanes of a word (two
// blocks per thread).  Circular windows that leave the image are recomputed
// afterwards through the window-relative map (circular_edges).
// =========================================================================
constexpr int kMbTX = 64, kMbTY = 32, kMbThreads = 128;

template <class T, int W>
__global__ void __launch_bounds__(kMbThreads)
k_median_block(const T *__restrict__ img, void *out, int out_type, int nx, int ny, int f0, int f1, int style,
               T fill)
{
    using SK = SortKey<T>;
    using K = typename SK::K;
    using CX = std::conditional_t<sizeof(K) == 4, CxKey32, CxKey64>;
    constexpr int BH = MedBlock<W>::BH, CT = kMbTX + W - 1, RT = kMbTY + W - 1, N = W * W;
    __shared__ K tile[RT * CT];
    const int tx0 = blockIdx.x * kMbTX, ty0 = blockIdx.y * kMbTY;
    gather_tile<8>(tile, RT * CT, [&](int idx) -> K {
        const int r = idx / CT, c = idx - r * CT;
        const int mx = map_index(tx0 + f0 + c, nx, style);
        const int my = map_index(ty0 + f1 + r, ny, style);
        return SK::key((mx < 0 || my < 0) ? fill : img[(long long)my * nx + mx]);
    });
    __syncthreads();
    constexpr int BX = kMbTX / 4, NBLK = BX * (kMbTY / BH);
    for (int b = threadIdx.x; b < NBLK; b += kMbThreads) {
        const int lx = (b % BX) * 4, ly = (b / BX) * BH;
        const int x0 = tx0 + lx, y = ty0 + ly;
        if (x0 >= nx || y >= ny) continue;
        K in[BH + W - 1][W + 3], res[BH][4];
#pragma unroll
        for (int r = 0; r < BH + W - 1; ++r)
#pragma unroll
            for (int c = 0; c < W + 3; ++c) in[r][c] = tile[(ly + r) * CT + lx + c];
        median_block4<W, CX>(in, res);
#pragma unroll
        for (int j = 0; j < BH; ++j)
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (x0 + q < nx && y + j < ny)
                    store_sel<T>(out, out_type, (long long)(y + j) * nx + x0 + q, SK::val(res[j][q]), false);
    }
    circular_edges(style, tx0, ty0, kMbTX, kMbTY, nx, ny, f0, f1, W, W, [&](int x, int ye) {
        K v[N];
#pragma unroll
        for (int jj = 0; jj < W; ++jj)
#pragma unroll
            for (int ii = 0; ii < W; ++ii) v[jj * W + ii] = SK::key(img[win_index2(x, ye, ii, jj, f0, f1, W, W, nx, ny, style)]);
        net_sort<N, K>(v);
        store_sel<T>(out, out_type, (long long)ye * nx + x, SK::val(v[(N - 1) / 2]), false);
    });
}

template <class T, int W>
static cudaError_t median_block_t(const MedianArgs &a, cudaStream_t s)
{
    const int nx = a.n[0], ny = a.nd > 1 ? a.n[1] : 1;
    dim3 grid((nx + kMbTX - 1) / kMbTX, (ny + kMbTY - 1) / kMbTY);
    k_median_block<T, W><<<grid, kMbThreads, 0, s>>>((const T *)a.img, a.out, a.out_type, nx, ny, a.wfirst[0],
                                                     a.nd > 1 ? a.wfirst[1] : 0, a.style, (T)a.fill);
    note_launch();
    return cudaGetLastError();
}

// 8-bit 5 x 5: a CTA tile of 128 x 16 outputs, each thread two 4 x 1 blocks
// side by side (outputs x0 .. x0+7 of one row), one per 16-bit lane.
constexpr int kM5TX = 128, kM5TY = 16, kM5CT = kM5TX + 8, kM5RT = kM5TY + 4;

__global__ void __launch_bounds__(256)
k_median_u8_5x5(const uint8_t *__restrict__ img, void *out, int out_type, int nx, int ny, int f0, int f1,
                int style, uint8_t fill, bool norm)
{
    __shared__ __align__(16) uint8_t tile[kM5RT * kM5CT];
    const int tx0 = blockIdx.x * kM5TX, ty0 = blockIdx.y * kM5TY;
    gather_tile<8>(tile, kM5RT * kM5CT, [&](int idx) -> uint8_t {
        const int r = idx / kM5CT, c = idx - r * kM5CT;
        if (c >= kM5TX + 4) return 0;
        const int mx = map_index(tx0 + f0 + c, nx, style);
        const int my = map_index(ty0 + f1 + r, ny, style);
        return (mx < 0 || my < 0) ? fill : img[(long long)my * nx + mx];
    });
    __syncthreads();
    const int lx = (threadIdx.x % (kM5TX / 8)) * 8, ly = threadIdx.x / (kM5TX / 8);
    const int x0 = tx0 + lx, y = ty0 + ly;
    if (x0 < nx && y < ny) {
        uint32_t in[5][8], o[1][4];
#pragma unroll
        for (int r = 0; r < 5; ++r) {
            const uint32_t *w = reinterpret_cast<const uint32_t *>(tile + (ly + r) * kM5CT + lx);
            const uint32_t bytes[3] = {w[0], w[1], w[2]};
#pragma unroll
            for (int c = 0; c < 8; ++c) in[r][c] = lanes_c_c4(bytes, c);
        }
        median_block4<5, CxU16x2>(in, o);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const uint32_t code = q < 4 ? (o[0][q] & 0xFFFFu) : (o[0][q - 4] >> 16);
            if (x0 + q < nx) store_sel<uint8_t>(out, out_type, (long long)y * nx + x0 + q, (uint8_t)code, norm);
        }
    }
    circular_edges(style, tx0, ty0, kM5TX, kM5TY, nx, ny, f0, f1, 5, 5, [&](int x, int yy) {
        store_sel<uint8_t>(out, out_type, (long long)yy * nx + x,
                           (uint8_t)median_u8_direct(img, x, yy, f0, f1, 5, 5, nx, ny, style), norm);
    });
}

static cudaError_t median_u8_5x5_t(const MedianArgs &a, cudaStream_t s)
{
    const int nx = a.n[0], ny = a.nd > 1 ? a.n[1] : 1;
    dim3 grid((nx + kM5TX - 1) / kM5TX, (ny + kM5TY - 1) / kM5TY);
    k_median_u8_5x5<<<grid, 256, 0, s>>>((const uint8_t *)a.img, a.out, a.out_type, nx, ny, a.wfirst[0],
                                         a.nd > 1 ? a.wfirst[1] : 0, a.style, (uint8_t)a.fill,
                                         a.in_type == IFX_N0F8);
    note_launch();
    return cudaGetLastError();
}

template <class T, int W0, int W1>
static cudaError_t median_float_t(const MedianArgs &a, cudaStream_t s)
{
    const int nx = a.n[0], ny = a.nd > 1 ? a.n[1] : 1;
    dim3 grid((nx + kFmTX - 1) / kFmTX, (ny + kFmTY - 1) / kFmTY);
    k_median_float<T, W0, W1><<<grid, kFmTX * kFmTY, 0, s>>>(
        (const T *)a.img, a.out, a.out_type, nx, ny, a.wfirst[0], a.nd > 1 ? a.wfirst[1] : 0,
        a.style, (T)a.fill);
    note_launch();
    return cudaGetLastError();
}

template <class T>
static cudaError_t median_px_t(const MedianArgs &a, cudaStream_t s)
{
    int4 n = make_int4(a.n[0], a.nd > 1 ? a.n[1] : 1, a.nd > 2 ? a.n[2] : 1, a.nd > 3 ? a.n[3] : 1);
    int4 wf = make_int4(a.wfirst[0], a.nd > 1 ? a.wfirst[1] : 0, a.nd > 2 ? a.wfirst[2] : 0,
                        a.nd > 3 ? a.wfirst[3] : 0);
    int4 wl = make_int4(a.wlen[0], a.nd > 1 ? a.wlen[1] : 1, a.nd > 2 ? a.wlen[2] : 1,
                        a.nd > 3 ? a.wlen[3] : 1);
    long long total = (long long)n.x * n.y * n.z * n.w;
    k_median_px<T><<<grid1(total, 128), 128, 0, s>>>((const T *)a.img, a.out, a.out_type, a.nd, n,
                                                      wf, wl, a.style, (T)a.fill,
                                                      a.in_type == IFX_N0F8);
    note_launch();
    return cudaGetLastError();
}

template <int W0, int W1>
static cudaError_t median_u8_t(const MedianArgs &a, cudaStream_t s)
{
    const int nx = a.n[0], ny = a.nd > 1 ? a.n[1] : 1;
    const int w0 = a.wlen[0], w1 = a.nd > 1 ? a.wlen[1] : 1;
    const int CT = ((kMedTX + w0 - 1 + 3) & ~3) + 4;
    const size_t smem = (size_t)(kMedTY + w1 - 1) * CT;
    auto kern = k_median_u8<W0, W1>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((nx + kMedTX - 1) / kMedTX, (ny + kMedTY - 1) / kMedTY);
    kern<<<grid, 256, smem, s>>>((const uint8_t *)a.img, a.out, a.out_type, nx, ny, a.wfirst[0],
                                 a.nd > 1 ? a.wfirst[1] : 0, w0, w1, a.style, (uint8_t)a.fill,
                                 a.in_type == IFX_N0F8);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_median(const MedianArgs &a, cudaStream_t s)
{
    long long total = 1;
    for (int d = 0; d < a.nd; ++d) total *= a.n[d];
    if (total == 0) return cudaSuccess;
    const bool u8 = a.in_type == IFX_N0F8 || a.in_type == IFX_U8;
    const int m = a.wlen[0] * (a.nd > 1 ? a.wlen[1] : 1);
    if (u8 && a.nd <= 2 && m <= 255) {
        const int w0 = a.wlen[0], w1 = a.nd > 1 ? a.wlen[1] : 1;
        if (w0 == 3 && w1 == 3) return median_u8_t<3, 3>(a, s);
        if (w0 == 5 && w1 == 5) return median_u8_5x5_t(a, s);
        if (w0 == 7 && w1 == 7) return median_u8_t<7, 7>(a, s);
        return median_u8_t<0, 0>(a, s);
    }
    if (u8) return median_px_t<uint8_t>(a, s);
    const bool fast2d = a.nd <= 2;
    if (fast2d && (a.in_type == IFX_F32 || a.in_type == IFX_F64)) {
        const int w0 = a.wlen[0], w1 = a.nd > 1 ? a.wlen[1] : 1;
        const bool f32 = a.in_type == IFX_F32;
        if (w0 == 3 && w1 == 3) return f32 ? median_block_t<float, 3>(a, s) : median_block_t<double, 3>(a, s);
        if (w0 == 5 && w1 == 5) return f32 ? median_block_t<float, 5>(a, s) : median_block_t<double, 5>(a, s);
        if (w0 == 7 && w1 == 7) return f32 ? median_float_t<float, 7, 7>(a, s) : median_float_t<double, 7, 7>(a, s);
    }
    if (a.in_type == IFX_F32) return median_px_t<float>(a, s);
    if (a.in_type == IFX_F64) return median_px_t<double>(a, s);
    return cudaErrorInvalidValue;
}

// =========================================================================
// Separable running min/max.  The min (max) of a box is the min (max) of
// per-axis mins (maxes), and truncating a box at the image edges is truncating
// each axis interval, so one pass per axis is exact.  For a Fill border the
// fill value joins every window that leaves the image along some axis, which
// the per-axis passes reproduce by adding it in the pass of that axis.
// One thread per output element; loads coalesce along axis 0.
// =========================================================================
template <class T>
__global__ void k_extrema_pass(const T *__restrict__ smin, const T *__restrict__ smax,
                               T *__restrict__ dmin, T *__restrict__ dmax, int4 n4, int axis,
                               int a0, int a1, int use_fill, T fill, int interleaved,
                               int want_min, int want_max)
{
    const int n[4] = {n4.x, n4.y, n4.z, n4.w};
    const long long total = (long long)n[0] * n[1] * n[2] * n[3];
    long long st = 1;
    for (int d = 0; d < axis; ++d) st *= n[d];
    const int na = n[axis];
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        const int c = (int)((p / st) % na);
        int lo = c + a0, hi = c + a1;
        const bool leaves = lo < 0 || hi > na - 1;
        lo = lo < 0 ? 0 : lo;
        hi = hi > na - 1 ? na - 1 : hi;
        const long long base = p - (long long)c * st;
        T mn = fill, mx = fill;
        bool have = use_fill && leaves;
        for (int q = lo; q <= hi; ++q) {
            const long long o = base + (long long)q * st;
            if (want_min) {
                const T v = smin[o];
                mn = (!have || v < mn) ? v : mn;
            }
            if (want_max) {
                const T v = smax[o];
                mx = (!have || v > mx) ? v : mx;
            }
            have = true;
        }
        if (interleaved) {
            dmin[2 * p] = mn;
            dmin[2 * p + 1] = mx;
        } else {
            if (want_min) dmin[p] = mn;
            if (want_max) dmax[p] = mx;
        }
    }
}

// =========================================================================
// The same pass for 8-bit codes by van Herk / Gil-Werman: the line is cut
// into segments of the window length w, aligned so that the lowest index lo
// of a window lies in segment k = floor(lo / w); the window [lo, lo+w-1] is
// then the suffix of segment k from lo joined with the prefix of segment k+1
// up to lo+w-1.  One thread per (line, segment): a backward sweep over
// segment k leaves the suffix minima/maxima in shared memory (per-thread
// columns, conflict-free), a forward sweep over segment k+1 keeps the running
// prefix and writes the w outputs whose windows start in segment k -- two
// loads per output and source whatever w.  Positions outside the line are the
// identity (255 for min, 0 for max), which is the truncation; the window
// always holds its centre (a0 <= 0 <= a1), so it is never empty.  8-bit codes
// order totally, so the result equals the direct scan's exactly.
// =========================================================================
constexpr int kVhgwThreads = 128;

__global__ void __launch_bounds__(kVhgwThreads)
k_extrema_vhgw_u8(const uint8_t *__restrict__ smin, const uint8_t *__restrict__ smax,
                  uint8_t *__restrict__ dmin, uint8_t *__restrict__ dmax, int4 n4, int axis, int a0, int w,
                  int use_fill, uint8_t fill, int interleaved, int want_min, int want_max, long long kmin,
                  long long nseg, long long nlines)
{
    extern __shared__ uint8_t vh[];                     // [w][threads] suffix min, then suffix max
    const int n[4] = {n4.x, n4.y, n4.z, n4.w};
    long long st = 1;
    for (int d = 0; d < axis; ++d) st *= n[d];
    const long long na = n[axis];
    const int a1 = a0 + w - 1;
    const int tid = threadIdx.x, bt = blockDim.x;
    uint8_t *hmn = vh, *hmx = vh + (size_t)w * bt;
    const bool same = smin == smax;
    const long long items = nseg * nlines;
    for (long long it = blockIdx.x * (long long)bt + tid; it < items; it += (long long)gridDim.x * bt) {
        // axis 0: neighbouring threads take neighbouring segments of a line (their
        // ranges are contiguous); other axes: neighbouring lines (coalesced)
        long long line, sg;
        if (axis == 0) {
            line = it / nseg;
            sg = it - line * nseg;
        } else {
            sg = it / nlines;
            line = it - sg * nlines;
        }
        const long long o = line / st, p = line - o * st;
        const long long base = o * st * na + p;
        const long long seg_lo = (kmin + sg) * w;
        uint8_t vmn = 255, vmx = 0;
        for (int j = w - 1; j >= 0; --j) {             // suffix of segment k
            const long long pos = seg_lo + j;
            if (pos >= 0 && pos < na) {
                const long long off = base + pos * st;
                const uint8_t x = smin[off];
                const uint8_t y = same ? x : smax[off];
                vmn = x < vmn ? x : vmn;
                vmx = y > vmx ? y : vmx;
            }
            hmn[j * bt + tid] = vmn;
            hmx[j * bt + tid] = vmx;
        }
        uint8_t gmn = 255, gmx = 0;                     // running prefix of segment k+1
        for (int j = 0; j < w; ++j) {
            if (j > 0) {
                const long long pos = seg_lo + w + j - 1;
                if (pos >= 0 && pos < na) {
                    const long long off = base + pos * st;
                    const uint8_t x = smin[off];
                    const uint8_t y = same ? x : smax[off];
                    gmn = x < gmn ? x : gmn;
                    gmx = y > gmx ? y : gmx;
                }
            }
            const long long c = seg_lo + j - a0;        // the output whose window starts here
            if (c < 0 || c >= na) continue;
            uint8_t mn = hmn[j * bt + tid], mx = hmx[j * bt + tid];
            mn = gmn < mn ? gmn : mn;
            mx = gmx > mx ? gmx : mx;
            if (use_fill && (c + a0 < 0 || c + a1 > na - 1)) {
                mn = fill < mn ? fill : mn;
                mx = fill > mx ? fill : mx;
            }
            const long long q = base + c * st;
            if (interleaved) {
                dmin[2 * q] = mn;
                dmin[2 * q + 1] = mx;
            } else {
                if (want_min) dmin[q] = mn;
                if (want_max) dmax[q] = mx;
            }
        }
    }
}

static bool extrema_vhgw_u8(const ExtremaPassArgs &a, cudaStream_t s, cudaError_t *e)
{
    const int w = a.a1 - a.a0 + 1;
    if (a.a0 > 0 || a.a1 < 0 || w < 2 || 2 * (size_t)w * kVhgwThreads > 48 * 1024) return false;
    int4 n = make_int4(a.n[0], a.nd > 1 ? a.n[1] : 1, a.nd > 2 ? a.n[2] : 1, a.nd > 3 ? a.n[3] : 1);
    const int nn[4] = {n.x, n.y, n.z, n.w};
    const long long total = (long long)n.x * n.y * n.z * n.w, na = nn[a.axis];
    const long long nlines = total / na;
    // segments holding the lowest window index of some output: lo = c + a0, c in [0, na)
    const long long kmin = (a.a0 - (w - 1)) / w;        // floor(a0 / w) for a0 in (-w, 0]
    const long long kmax = (na - 1 + a.a0) / w;
    const long long nseg = kmax - kmin + 1;
    const long long items = nseg * nlines;
    k_extrema_vhgw_u8<<<grid1(items, kVhgwThreads), kVhgwThreads, 2 * (size_t)w * kVhgwThreads, s>>>(
        (const uint8_t *)a.src_min, (const uint8_t *)a.src_max, (uint8_t *)a.dst_min, (uint8_t *)a.dst_max, n,
        a.axis, a.a0, w, a.use_fill, (uint8_t)a.fill, a.dst_interleaved, a.want_min, a.want_max, kmin, nseg,
        nlines);
    note_launch();
    *e = cudaGetLastError();
    return true;
}

// =========================================================================
// 8-bit running min and max of square W x W windows, 2-D, both axes in one
// launch.  A CTA stages its tile plus halo in shared memory with coordinates
// clamped to the image: a window truncated at an edge holds the edge value
// whenever it would reach past it (windows contain their output), so
// clamping gives exactly the truncated-window extrema (and with them every
// Pad style, see the pass kernel above).  The x pass runs van Herk /
// Gil-Werman on runs of W outputs (one segment: suffix extrema of the run's
// W inputs, prefix extrema of the next W-1, one combine per output) with two
// rows in the 16-bit lanes of a word; the y pass does the same down column
// pairs.  The x pass writes its results by row pairs (a 32-bit word holds two
// rows of two columns), so that its stores and the y pass's loads move four
// bytes each: byte-wise stores and 16-bit loads made the shared-memory queue
// the kernel's first stall.  A Fill value joins the outputs whose window
// leaves the image along the pass's axis.  Outputs: interleaved (min, max)
// codes, or one of them.
// =========================================================================
template <int W> struct ExTile {
    // runs per row: a multiple of 4, so that the tile width is (the y pass
    // takes four columns per word, and their stores align)
    static constexpr int NRX = ((128 + W - 1) / W + 1) & ~1;
    // runs per column: tiles about 32 tall (2048^2, 15 x 15: 18.4 us with
    // 60-row tiles, 16.8-17.3 with 30-row ones, whose 966 CTAs spread more
    // evenly over the SMs than 490 do; 80-row tiles were slower still)
    static constexpr int NRY = (32 + W / 2) / W;
    static constexpr int TX = W * NRX, TY = W * NRY;
    static constexpr int R = TY + W - 1, C = TX + W - 1;
    static constexpr int RP = (R + 1) & ~1;                    // rows staged (even: row pairs)
    static constexpr int CP = (C + 3) & ~3;
    static constexpr int NV = (C + 30) / 16;                   // 16-byte vectors of a row's aligned superset
    static constexpr int CV = 16 * NV;                         // bytes staged per row
    // staged row pitch: an odd number of 16-byte vectors, so that the rows of
    // the four row pairs one warp reads in the x pass fall in different banks
    static constexpr int XP = 16 * (NV | 1);
    // the pair layout's 32-bit accesses are 4-byte aligned when a pair row is
    static_assert(TX % 2 == 0, "tile width must be even");
    // the y pass's last run loads pairs up to (r0 >> 1) + W - 1; RP / 2 + 1 pairs are allocated
    static_assert(((NRY - 1) * W) / 2 + W - 1 < RP / 2 + 1, "y runs stay inside the pair rows");
    // staging and both pair arrays are static shared memory (48 KB at most)
    static_assert(RP * XP + 2 * (RP + 2) * TX <= 48 * 1024, "tile exceeds static shared memory");
};

// Van Herk / Gil-Werman over a run: out[i] = op over v[i .. i+W-1], i < W,
// from v[0 .. 2W-2] (two independent 16-bit lanes per word).
template <int W, bool MAX>
__device__ __forceinline__ void vhgw_run(const uint32_t (&v)[2 * W - 1], uint32_t (&out)[W])
{
    auto op = [](uint32_t a, uint32_t b) { return MAX ? __vmaxu2(a, b) : __vminu2(a, b); };
    out[W - 1] = v[W - 1];
#pragma unroll
    for (int j = W - 2; j >= 0; --j) out[j] = op(v[j], out[j + 1]);   // suffix extrema of the run
    uint32_t g = v[W];
#pragma unroll
    for (int i = 1; i < W; ++i) {                                       // prefix extrema of the next W-1
        out[i] = op(out[i], g);
        if (i + 1 < W) g = op(g, v[W + i]);
    }
}

// Stores W x-pass results of a row pair (row 2p in byte 0, row 2p + 1 in byte
// 2 of each word) at columns c0 .. c0 + W - 1 of the pair layout: two columns
// per 32-bit store on even columns, the odd one out (the last column for an
// even c0, the first for an odd one) as 16 bits.  Neighbouring lanes hold
// runs of both parities, so the words of both cases are formed and selected
// rather than branched on (`odd`: c0 is odd).
template <int W>
__device__ __forceinline__ void ex_put_pairs(uint8_t *p, const uint32_t (&v)[W], int odd)
{
#pragma unroll
    for (int i = 0; i + 1 < W; i += 2) {
        const uint32_t even_w = __byte_perm(v[i], v[i + 1], 0x6420);
        const uint32_t odd_w = __byte_perm(v[i + 1], v[i + 2], 0x6420);
        *reinterpret_cast<uint32_t *>(p + 2 * (i + odd)) = odd ? odd_w : even_w;
    }
    const uint32_t lone = odd ? v[0] : v[W - 1];
    *reinterpret_cast<uint16_t *>(p + (odd ? 0 : 2 * (W - 1))) = (uint16_t)__byte_perm(lone, 0u, 0x0020);
}

// Rows r0 .. r0 + 2W - 2 of columns (c, c + 1) from the pair layout, column c
// in the low 16-bit lane: W word loads, each giving two rows (S = r0 & 1;
// `p` addresses pair r0 / 2 at column c, PITCH bytes per pair).
template <int W, int S, int PITCH>
__device__ __forceinline__ void ex_get_column(const uint8_t *p, uint32_t (&v)[2 * W - 1])
{
    uint32_t w[W];
#pragma unroll
    for (int k = 0; k < W; ++k) w[k] = *reinterpret_cast<const uint32_t *>(p + k * PITCH);
#pragma unroll
    for (int j = 0; j < 2 * W - 1; ++j)
        v[j] = __byte_perm(w[(j + S) >> 1], 0u, ((j + S) & 1) ? 0x4341 : 0x4240);
}

// Four CTAs per SM up to W = 17 (64 registers: at five CTAs and 48 registers
// the small windows spilled and ran slower); W > 17 needs more registers for
// its runs.
template <int W>
__global__ void __launch_bounds__(256, W <= 17 ? 4 : 2)
k_extrema2d_u8(const uint8_t *__restrict__ img, uint8_t *__restrict__ out, int nx, int ny, int a0, int use_fill,
               uint32_t fill, int which)
{
    using G = ExTile<W>;
    __shared__ __align__(16) uint8_t xin[G::RP * G::XP];
    // x-pass results by row pairs: byte 2c + h of pair p is column c of row
    // 2p + h, so one 32-bit word holds two rows of two columns (one pair row
    // beyond the staged rows: a y run may load the word of its last row's pair)
    __shared__ __align__(16) uint8_t xmn[(G::RP + 2) * G::TX];
    __shared__ __align__(16) uint8_t xmx[(G::RP + 2) * G::TX];
    const int tx0 = blockIdx.x * G::TX, ty0 = blockIdx.y * G::TY;
    // The staged window: rows ty0 + a0 .. + RP - 1, columns from tx0 + a0,
    // coordinates clamped to the image (equal to the truncated windows).  A
    // window inside the image, in an image whose rows start on 16-byte
    // boundaries, is staged by 16-byte loads of each row's aligned superset
    // (its first `lead` bytes precede the window); others byte by byte
    // through the clamp (lead 0).
    const int gx0 = tx0 + a0, gy0 = ty0 + a0, ax = gx0 & ~15;
    const bool vec = ((uintptr_t)img & 15) == 0 && (nx & 15) == 0 && gx0 >= 0 && gy0 >= 0 &&
                     gy0 + G::RP <= ny && ax + G::CV <= nx;
    const int lead = vec ? gx0 - ax : 0;
    if (vec) {
        // (row, vector) items, four loads in flight per thread before the stores
        constexpr int TOT = G::RP * G::NV;
        const uint4 *src = reinterpret_cast<const uint4 *>(img + (long long)gy0 * nx + ax);
        const int rowv = nx >> 4;
        for (int base = threadIdx.x; base < TOT; base += 4 * blockDim.x) {
            uint4 v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int it = base + q * blockDim.x;
                if (it < TOT) {
                    const int r = it / G::NV, k = it - r * G::NV;
                    v[q] = __ldg(src + (long long)r * rowv + k);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int it = base + q * blockDim.x;
                if (it < TOT) {
                    const int r = it / G::NV, k = it - r * G::NV;
                    *reinterpret_cast<uint4 *>(xin + r * G::XP + 16 * k) = v[q];
                }
            }
        }
    } else {   // a warp per staged row, four columns per lane (one 32-bit shared store);
        // a warp's loads for up to four rows are in flight before it stores
        constexpr int kChunks = (G::CP + 127) / 128;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
        for (int r0 = warp; r0 < G::RP; r0 += 4 * nw) {
            uint32_t word[4][kChunks];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int r = r0 + q * nw;
                const uint8_t *row = img + (long long)min(max(ty0 + a0 + r, 0), ny - 1) * nx;
#pragma unroll
                for (int k = 0; k < kChunks; ++k) {
                    const int c = 4 * lane + 128 * k, x = tx0 + a0 + c;
                    uint32_t wv = 0;
                    if (r < G::RP && c < G::CP) {
#pragma unroll
                        for (int j = 0; j < 4; ++j) wv |= (uint32_t)__ldg(row + min(max(x + j, 0), nx - 1)) << (8 * j);
                    }
                    word[q][k] = wv;
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int k = 0; k < kChunks; ++k) {
                    const int r = r0 + q * nw, c = 4 * lane + 128 * k;
                    if (r < G::RP && c < G::CP) *reinterpret_cast<uint32_t *>(xin + r * G::XP + c) = word[q][k];
                }
        }
    }
    __syncthreads();
    const uint32_t fill2 = fill * 0x00010001u;
    // x pass: row pairs (r, r+1) x runs of W outputs
    for (int it = threadIdx.x; it < (G::RP / 2) * G::NRX; it += blockDim.x) {
        const int rp = it / G::NRX, run = it - rp * G::NRX, r = 2 * rp, c0 = run * W;
        // bytes c0 .. c0+2W-2 of the window's rows r and r+1, read as aligned words
        constexpr int NWD = (2 * W - 1 + 3) / 4 + 1;
        const int a = (lead + c0) & ~3, sh = (lead + c0) & 3;
        uint32_t ra[NWD], rb[NWD];
#pragma unroll
        for (int q = 0; q < NWD; ++q) {
            ra[q] = a + 4 * q < G::CV ? *reinterpret_cast<const uint32_t *>(xin + r * G::XP + a + 4 * q) : 0u;
            rb[q] = a + 4 * q < G::CV ? *reinterpret_cast<const uint32_t *>(xin + (r + 1) * G::XP + a + 4 * q) : 0u;
        }
        // realigned so that byte j is byte j % 4 of word j / 4 (compile-time indices)
        uint32_t al[NWD - 1], bl[NWD - 1];
#pragma unroll
        for (int q = 0; q < NWD - 1; ++q) {
            al[q] = __funnelshift_r(ra[q], ra[q + 1], 8 * sh);
            bl[q] = __funnelshift_r(rb[q], rb[q + 1], 8 * sh);
        }
        uint32_t v[2 * W - 1];
#pragma unroll
        for (int j = 0; j < 2 * W - 1; ++j)
            v[j] = __byte_perm(al[j >> 2], bl[j >> 2], (uint32_t)((j & 3) | (4 + (j & 3)) << 8)) & 0x00FF00FFu;
        uint32_t mn[W], mx[W];
        vhgw_run<W, false>(v, mn);
        vhgw_run<W, true>(v, mx);
        if (use_fill) {
#pragma unroll
            for (int i = 0; i < W; ++i) {
                const int x = tx0 + c0 + i;
                if (x + a0 < 0 || x + a0 + W - 1 > nx - 1) {
                    mn[i] = __vminu2(mn[i], fill2);
                    mx[i] = __vmaxu2(mx[i], fill2);
                }
            }
        }
        const int at = rp * 2 * G::TX + 2 * c0;          // column c0 of the pair (even: TX is)
        ex_put_pairs<W>(xmn + at, mn, c0 & 1);
        ex_put_pairs<W>(xmx + at, mx, c0 & 1);
    }
    __syncthreads();
    // y pass: column pairs (c, c+1) x runs of W outputs down
    for (int it = threadIdx.x; it < (G::TX / 2) * G::NRY; it += blockDim.x) {
        const int run = it / (G::TX / 2), c = 2 * (it - run * (G::TX / 2)), r0 = run * W;
        const int x = tx0 + c;
        if (x >= nx || ty0 + r0 >= ny) continue;
        uint32_t v[2 * W - 1], mn[W], mx[W];
        const int at = (r0 >> 1) * 2 * G::TX + 2 * c;       // 4-byte aligned: c is even
        if (r0 & 1) ex_get_column<W, 1, 2 * G::TX>(xmn + at, v);
        else ex_get_column<W, 0, 2 * G::TX>(xmn + at, v);
        vhgw_run<W, false>(v, mn);
        if (r0 & 1) ex_get_column<W, 1, 2 * G::TX>(xmx + at, v);
        else ex_get_column<W, 0, 2 * G::TX>(xmx + at, v);
        vhgw_run<W, true>(v, mx);
        const bool two = x + 1 < nx;
#pragma unroll
        for (int i = 0; i < W; ++i) {
            const int y = ty0 + r0 + i;
            if (y >= ny) break;
            uint32_t m = mn[i], M = mx[i];
            if (use_fill && (y + a0 < 0 || y + a0 + W - 1 > ny - 1)) {
                m = __vminu2(m, fill2);
                M = __vmaxu2(M, fill2);
            }
            const long long p = (long long)y * nx + x;
            if (which == 0) {
                // (min, max) of x, then of x+1
                const uint32_t word = __byte_perm(m, M, 0x6240);
                uint8_t *q = out + 2 * p;
                if (two && ((uintptr_t)q & 3) == 0) {
                    *reinterpret_cast<uint32_t *>(q) = word;
                } else {
                    *reinterpret_cast<uint16_t *>(q) = (uint16_t)word;
                    if (two) *reinterpret_cast<uint16_t *>(q + 2) = (uint16_t)(word >> 16);
                }
            } else {
                const uint32_t sel = which == 1 ? m : M;
                out[p] = (uint8_t)sel;
                if (two) out[p + 1] = (uint8_t)(sel >> 16);
            }
        }
    }
}

template <int W>
static cudaError_t extrema2d_u8_t(const uint8_t *img, uint8_t *out, int nx, int ny, int a0, int use_fill, int fill,
                                  int which, cudaStream_t s)
{
    using G = ExTile<W>;
    dim3 grid((nx + G::TX - 1) / G::TX, (ny + G::TY - 1) / G::TY);
    k_extrema2d_u8<W><<<grid, 256, 0, s>>>(img, out, nx, ny, a0, use_fill, (uint32_t)fill & 0xFFu, which);
    note_launch();
    return cudaGetLastError();
}

bool launch_extrema2d_u8(const void *img, void *out, int nx, int ny, int w, int a0, int use_fill, double fill,
                         int which, cudaStream_t s, cudaError_t *e)
{
    const uint8_t *i = (const uint8_t *)img;
    uint8_t *o = (uint8_t *)out;
    const int f = (int)fill;
    switch (w) {
    case 3: *e = extrema2d_u8_t<3>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 5: *e = extrema2d_u8_t<5>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 7: *e = extrema2d_u8_t<7>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 9: *e = extrema2d_u8_t<9>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 11: *e = extrema2d_u8_t<11>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 13: *e = extrema2d_u8_t<13>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 15: *e = extrema2d_u8_t<15>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 17: *e = extrema2d_u8_t<17>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 21: *e = extrema2d_u8_t<21>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 25: *e = extrema2d_u8_t<25>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 31: *e = extrema2d_u8_t<31>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    case 33: *e = extrema2d_u8_t<33>(i, o, nx, ny, a0, use_fill, f, which, s); return true;
    default: return false;
    }
}

template <class T>
static cudaError_t extrema_t(const ExtremaPassArgs &a, cudaStream_t s)
{
    int4 n = make_int4(a.n[0], a.nd > 1 ? a.n[1] : 1, a.nd > 2 ? a.n[2] : 1, a.nd > 3 ? a.n[3] : 1);
    long long total = (long long)n.x * n.y * n.z * n.w;
    k_extrema_pass<T><<<grid1(total, 256), 256, 0, s>>>(
        (const T *)a.src_min, (const T *)a.src_max, (T *)a.dst_min, (T *)a.dst_max, n, a.axis,
        a.a0, a.a1, a.use_fill, (T)a.fill, a.dst_interleaved, a.want_min, a.want_max);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_extrema_pass(const ExtremaPassArgs &a, cudaStream_t s)
{
    long long total = 1;
    for (int d = 0; d < a.nd; ++d) total *= a.n[d];
    if (total == 0) return cudaSuccess;
    if (a.type == IFX_F32) return extrema_t<float>(a, s);
    if (a.type == IFX_F64) return extrema_t<double>(a, s);
    if (a.type == IFX_N0F8 || a.type == IFX_U8) {
        cudaError_t e;
        if (extrema_vhgw_u8(a, s, &e)) return e;
        return extrema_t<uint8_t>(a, s);
    }
    return cudaErrorInvalidValue;
}

} // namespace ifx
