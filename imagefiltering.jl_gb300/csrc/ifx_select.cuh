// ifx_select.cuh -- exact selection primitives shared by the median kernels
// and the batched engine: packed 8-bit rank counting and a compile-time
// sorting network on order-preserving keys.
#pragma once
#include <cstdint>
#include <utility>
#include "ifx_common.cuh"

namespace ifx {

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

// 5 x 5 medians of four horizontally adjacent windows.  A[j] / B[j] hold
// columns 0..3 / 4..7 of window row j; output q's window is columns q..q+4.
// Every column's five values are sorted once (Batcher's network for five, in
// 16-bit lanes, shared by the windows that contain the column); the median of
// a window is then selected from its five sorted columns by a 63-comparator
// network.  That network was derived offline for this purpose: sorting the
// ranks across the columns and taking the median of the 13 elements of a
// rows-and-columns-sorted 5 x 5 array that can hold rank 13 (those with
// (c+1)(r+1) <= 13 and (5-c)(5-r) <= 13) is exact, and greedy removal of
// comparators from that composite, checked after each removal against all
// 6^5 column-sorted 0-1 inputs (0-1 principle), left these 63 (102 live
// min/max operations against 202 for the pruned 25-input Batcher network).
// Wire c*5 + r is column c, rank r (0 = smallest); the median is wire 12.
struct Med25 {
    static constexpr int n = 63;
    static constexpr unsigned char a[63] = {0, 10, 0, 5, 5, 10, 15, 1, 1, 6, 1, 11, 6, 16, 2, 12, 2, 7, 7, 2, 12, 7, 17, 3, 13, 3, 8, 8, 3, 13, 8, 4, 14, 4, 9, 14, 9, 9, 15, 17, 3, 4, 9, 11, 4, 11, 4, 7, 8, 7, 8, 8, 11, 16, 20, 4, 8, 9, 11, 12, 8, 12, 11};
    static constexpr unsigned char b[63] = {5, 15, 10, 15, 10, 20, 20, 6, 11, 16, 21, 21, 11, 21, 7, 17, 12, 17, 12, 22, 22, 12, 22, 8, 18, 13, 18, 13, 23, 23, 13, 9, 19, 14, 19, 24, 14, 11, 16, 20, 7, 8, 12, 13, 7, 12, 11, 12, 13, 9, 11, 9, 12, 17, 21, 16, 20, 15, 16, 17, 11, 15, 12};
};

template <int I> __device__ __forceinline__ void med25_cx(uint32_t (&v)[25])
{
    constexpr int x = Med25::a[I];
    constexpr int y = Med25::b[I];
    const uint32_t lo = __vminu2(v[x], v[y]);
    const uint32_t hi = __vmaxu2(v[x], v[y]);
    v[x] = lo;
    v[y] = hi;
}

template <size_t... I> __device__ __forceinline__ void med25_apply(uint32_t (&v)[25], std::index_sequence<I...>)
{
    (med25_cx<(int)I>(v), ...);
}

__device__ __forceinline__ uint32_t median5x5_u8x4(const uint32_t (&A)[5], const uint32_t (&B)[5])
{
    uint32_t p[4][5];                            // [column pair 01, 23, 45, 67][sorted rank]
#pragma unroll
    for (int j = 0; j < 5; ++j) {
        p[0][j] = __byte_perm(A[j], 0u, 0x4140);
        p[1][j] = __byte_perm(A[j], 0u, 0x4342);
        p[2][j] = __byte_perm(B[j], 0u, 0x4140);
        p[3][j] = __byte_perm(B[j], 0u, 0x4342);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k) net_apply_u16x2<5>(p[k], std::make_index_sequence<NetOf<5>::net.n>{});
    auto mid = [](uint32_t x, uint32_t y) { return __byte_perm(x, y, 0x5432); };
    uint32_t r[2];
#pragma unroll
    for (int h = 0; h < 2; ++h) {                // outputs (0, 1), then (2, 3)
        uint32_t v[25];
#pragma unroll
        for (int i = 0; i < 5; ++i)              // window column slot i: columns (2h+i, 2h+i+1)
#pragma unroll
            for (int k = 0; k < 5; ++k)
                v[i * 5 + k] = (i & 1) ? mid(p[h + (i - 1) / 2][k], p[h + (i + 1) / 2][k]) : p[h + i / 2][k];
        med25_apply(v, std::make_index_sequence<Med25::n>{});
        r[h] = v[12];
    }
    return __byte_perm(r[0], r[1], 0x6420);
}

} // namespace ifx
