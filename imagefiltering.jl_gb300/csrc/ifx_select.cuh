// ifx_select.cuh -- exact selection primitives shared by the median kernels
// and the batched engine: packed 8-bit rank counting and a compile-time
// sorting network on order-preserving keys.
#pragma once
#include <cstdint>
#include <utility>
#include "ifx_common.cuh"
#include "ifx_median_nets.cuh"

namespace ifx {

// Compare-exchange halves for the generated block networks: order-preserving
// 32/64-bit keys, and 8-bit codes zero-extended into the two 16-bit lanes of a
// word (two independent blocks per word, one lane-wise min or max each).
struct CxKey32 {
    using T = uint32_t;
    static __device__ __forceinline__ T lo(T a, T b) { return min(a, b); }
    static __device__ __forceinline__ T hi(T a, T b) { return max(a, b); }
};
struct CxKey64 {
    using T = unsigned long long;
    static __device__ __forceinline__ T lo(T a, T b) { return min(a, b); }
    static __device__ __forceinline__ T hi(T a, T b) { return max(a, b); }
};
struct CxU16x2 {
    using T = uint32_t;
    static __device__ __forceinline__ T lo(T a, T b) { return __vminu2(a, b); }
    static __device__ __forceinline__ T hi(T a, T b) { return __vmaxu2(a, b); }
};

// Rows of a 4-wide block of W x W medians: two for 3 x 3 windows, one for
// 5 x 5 (whose two-row block needs more registers than the kernels that use
// it can hold).
template <int W> struct MedBlock {
    static constexpr int BH = W == 3 ? 2 : 1;
};

// The W x W medians of a 4 x BH block of outputs from its (BH+W-1) x (W+3) footprint.
template <int W, class CX>
__device__ __forceinline__ void median_block4(const typename CX::T (&in)[MedBlock<W>::BH + W - 1][W + 3],
                                              typename CX::T (&out)[MedBlock<W>::BH][4])
{
    static_assert(W == 3 || W == 5, "generated blocks: 3 x 3 and 5 x 5 windows");
    if constexpr (W == 3) median3_block4x2<CX>(in, out);
    else median5_block4x1<CX>(in, out);
}

// Outputs of a tile whose windows leave the image -- the tile's part of the
// image minus the interior [hx0, nx-hx1) x [hy0, ny-hy1) -- as up to four
// rectangles (rows above and below the interior, then columns left and right
// of it), enumerated by one index so that the threads of a CTA share them
// evenly.  Median windows that leave a circular image wrap inside
// window-intersect-image (copy_win!), which a tile gathered through the
// whole-image map does not hold: the tile kernels compute every output from
// their tile and then recompute these few, one per thread.
struct EdgeRects {
    int x0[4], x1[4], y0[4], y1[4];
    int count;

    __device__ __forceinline__ EdgeRects(int tx0, int ty0, int tw, int th, int nx, int ny, int hx0, int hx1,
                                         int hy0, int hy1)
    {
        const int X1 = min(tx0 + tw, nx), Y1 = min(ty0 + th, ny);
        const int ym0 = max(ty0, hy0), ym1 = min(Y1, ny - hy1);
        set(0, tx0, X1, ty0, min(Y1, hy0));                       // above
        set(1, tx0, X1, max(max(ty0, ny - hy1), hy0), Y1);        // below
        set(2, tx0, min(X1, hx0), ym0, ym1);                      // left
        set(3, max(max(tx0, nx - hx1), hx0), X1, ym0, ym1);       // right
        count = 0;
        for (int k = 0; k < 4; ++k) count += (x1[k] - x0[k]) * (y1[k] - y0[k]);
    }
    __device__ __forceinline__ void set(int k, int a, int b, int c, int d)
    {
        const bool e = b <= a || d <= c;
        x0[k] = a;
        x1[k] = e ? a : b;
        y0[k] = c;
        y1[k] = e ? c : d;
    }
    // output e of the set (e < count)
    __device__ __forceinline__ void at(int e, int &x, int &y) const
    {
        int k = 0;
        for (; k < 3; ++k) {
            const int n = (x1[k] - x0[k]) * (y1[k] - y0[k]);
            if (e < n) break;
            e -= n;
        }
        const int w = x1[k] - x0[k];
        y = y0[k] + e / w;
        x = x0[k] + e - (e / w) * w;
    }
};

// Bytes c and c+4 of the 12 bytes b[0..2] as the two 16-bit lanes of a word.
__device__ __forceinline__ uint32_t lanes_c_c4(const uint32_t (&b)[3], int c)
{
    const uint32_t lo = c < 4 ? b[0] : b[1], hi = c < 4 ? b[1] : b[2];
    const int q = c & 3;
    return __byte_perm(lo, hi, (uint32_t)(q | ((4 + q) << 8))) & 0x00FF00FFu;
}

__device__ __forceinline__ uint32_t load_word(const uint8_t *row, int col)
{
    const int a = col & ~3, sh = col & 3;
    const uint32_t lo = *reinterpret_cast<const uint32_t *>(row + a);
    const uint32_t hi = *reinterpret_cast<const uint32_t *>(row + a + 4);
    return __byte_perm(lo, hi, 0x3210 + 0x1111 * sh);
}

__device__ __forceinline__ uint32_t count_lt(uint32_t cnt, uint32_t w, uint32_t trial)
{
    return __vsub4(cnt, __vcmpltu4(w, trial));
}

// =========================================================================
// Float median, 2-D, fixed window: a sorting network on order-preserving
// integer keys.  The network is Batcher's odd-even merge sort for arbitrary n
// (the iterative formulation: for p = 1,2,4..; k = p,p/2..1; j = k mod p,
// step 2k; i < min(k, n-j-k); compare (i+j, i+j+k) when both lie in the same
// 2p block), built at compile time; only the comparators the middle output
// depends on survive dead-code elimination.  Keys map floats so that unsigned
// order is Julia's isless order (-0.0 < 0.0, NaN after +Inf), which is what
// partialsort! uses (src/mapwindow.jl:123-128).
// =========================================================================
template <int N> struct Net {
    int n = 0;
    short a[640] = {};
    short b[640] = {};
};

template <int N> constexpr Net<N> make_net()
{
    Net<N> r{};
    for (int p = 1; p < N; p <<= 1)
        for (int k = p; k >= 1; k >>= 1)
            for (int j = k % p; j + k < N; j += 2 * k)
                for (int i = 0; i < k && i < N - j - k; ++i)
                    if ((i + j) / (2 * p) == (i + j + k) / (2 * p)) {
                        r.a[r.n] = (short)(i + j);
                        r.b[r.n] = (short)(i + j + k);
                        ++r.n;
                    }
    return r;
}

template <int N> struct NetOf { static constexpr Net<N> net = make_net<N>(); };

template <class T> struct SortKey;
template <> struct SortKey<float> {
    using K = uint32_t;
    static __device__ __forceinline__ K key(float x)
    {
        uint32_t b = isnan(x) ? 0x7fffffffu : __float_as_uint(x);
        return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
    }
    static __device__ __forceinline__ float val(K k)
    {
        return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
    }
};
template <> struct SortKey<double> {
    using K = unsigned long long;
    static __device__ __forceinline__ K key(double x)
    {
        unsigned long long b = isnan(x) ? 0x7fffffffffffffffull : (unsigned long long)__double_as_longlong(x);
        return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
    }
    static __device__ __forceinline__ double val(K k)
    {
        return __longlong_as_double((long long)((k & 0x8000000000000000ull) ? (k & 0x7fffffffffffffffull) : ~k));
    }
};

template <int N, int I, class K> __device__ __forceinline__ void net_cx(K (&v)[N])
{
    constexpr int x = NetOf<N>::net.a[I];
    constexpr int y = NetOf<N>::net.b[I];
    const K lo = min(v[x], v[y]);
    const K hi = max(v[x], v[y]);
    v[x] = lo;
    v[y] = hi;
}

template <int N, class K, size_t... I>
__device__ __forceinline__ void net_apply(K (&v)[N], std::index_sequence<I...>)
{
    (net_cx<N, (int)I, K>(v), ...);
}

template <int N, class K> __device__ __forceinline__ void net_sort(K (&v)[N])
{
    net_apply<N, K>(v, std::make_index_sequence<NetOf<N>::net.n>{});
}

// The same network on packed codes: each word holds two 8-bit codes
// zero-extended to 16-bit lanes, and each compare-exchange is a lane-wise min
// and max (__vminu2 / __vmaxu2, single instructions here, where the 8-bit
// four-lane forms are emulated).  When only the middle word is used
// afterwards, the compiler keeps just the comparators (and the min or max
// halves) it depends on.
template <int N, int I> __device__ __forceinline__ void net_cx_u16x2(uint32_t (&v)[N])
{
    constexpr int x = NetOf<N>::net.a[I];
    constexpr int y = NetOf<N>::net.b[I];
    const uint32_t lo = __vminu2(v[x], v[y]);
    const uint32_t hi = __vmaxu2(v[x], v[y]);
    v[x] = lo;
    v[y] = hi;
}

template <int N, size_t... I>
__device__ __forceinline__ void net_apply_u16x2(uint32_t (&v)[N], std::index_sequence<I...>)
{
    (net_cx_u16x2<N, (int)I>(v), ...);
}

// Medians of the four byte lanes of w[0..N) (four horizontally adjacent
// windows), returned packed like the input.
template <int N> __device__ __forceinline__ uint32_t median_u8x4(const uint32_t (&w)[N])
{
    uint32_t a[N], b[N];
#pragma unroll
    for (int k = 0; k < N; ++k) {
        a[k] = __byte_perm(w[k], 0u, 0x4140);      // bytes 0, 1 -> 16-bit lanes
        b[k] = __byte_perm(w[k], 0u, 0x4342);      // bytes 2, 3
    }
    net_apply_u16x2<N>(a, std::make_index_sequence<NetOf<N>::net.n>{});
    net_apply_u16x2<N>(b, std::make_index_sequence<NetOf<N>::net.n>{});
    return __byte_perm(a[(N - 1) / 2], b[(N - 1) / 2], 0x6420);
}

// 3 x 3 medians of four horizontally adjacent windows, sharing the sorting of
// their columns.  A[j] holds columns 0..3 of window row j, the low two bytes
// of B[j] columns 4 and 5; output q's window is columns q..q+2.  Each column
// of three is sorted once (in 16-bit lanes, two columns per word) and the
// median of the nine is med3(max of the column minima, med3 of the column
// middles, min of the column maxima) -- a min/max identity that holds for
// all 0-1 inputs, hence for all inputs.  Columns 0..5 serve the four windows:
// 3 x 3 compare-exchanges for the six columns plus 12 lane operations per
// pair of outputs, against 24 compare-exchanges per pair in the pruned
// nine-input network.
__device__ __forceinline__ void cs_u16x2(uint32_t &a, uint32_t &b)
{
    const uint32_t lo = __vminu2(a, b);
    b = __vmaxu2(a, b);
    a = lo;
}
__device__ __forceinline__ uint32_t med3_u16x2(uint32_t a, uint32_t b, uint32_t c)
{
    return __vmaxu2(__vminu2(a, b), __vminu2(__vmaxu2(a, b), c));
}
__device__ __forceinline__ uint32_t median3x3_u8x4(const uint32_t (&A)[3], const uint32_t (&B)[3])
{
    uint32_t p[3][3];                            // [column pair 01, 23, 45][sorted rank]
#pragma unroll
    for (int j = 0; j < 3; ++j) {
        p[0][j] = __byte_perm(A[j], 0u, 0x4140);
        p[1][j] = __byte_perm(A[j], 0u, 0x4342);
        p[2][j] = __byte_perm(B[j], 0u, 0x4140);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        cs_u16x2(p[k][0], p[k][1]);
        cs_u16x2(p[k][1], p[k][2]);
        cs_u16x2(p[k][0], p[k][1]);
    }
    // columns (c+1, c+2) from the pairs (c, c+1) and (c+2, c+3)
    auto mid = [](uint32_t x, uint32_t y) { return __byte_perm(x, y, 0x5432); };
    uint32_t r[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {                // outputs (0, 1), then (2, 3)
        const uint32_t lo = __vmaxu2(__vmaxu2(p[h][0], mid(p[h][0], p[h + 1][0])), p[h + 1][0]);
        const uint32_t hi = __vminu2(__vminu2(p[h][2], mid(p[h][2], p[h + 1][2])), p[h + 1][2]);
        const uint32_t md = med3_u16x2(p[h][1], mid(p[h][1], p[h + 1][1]), p[h + 1][1]);
        r[h] = med3_u16x2(lo, md, hi);
    }
    return __byte_perm(r[0], r[1], 0x6420);
}

} // namespace ifx
