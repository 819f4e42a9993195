// ifx_iir.cu -- Triggs-Sdika recursive (IIR) filtering, one pass per axis:
// _imfilter_dim! (src/imfilter.jl:961-1030) with its border initialisation,
// _leftborder! (1033-1045), _rightborder! (1057-1084) and rightΔu (1087-1092).
//
// A pass runs an order-3 causal recursion over a line, then the right-edge
// initialisation of Triggs & Sdika (2006, Eqs. 14-15), an order-3 anticausal
// recursion and the final scaling.  Each line is sequential; lines run in
// parallel, one thread per line.
//
// The arithmetic keeps the reference's operation order and its roundings:
// every recursion step is ((x + a1*y1) + a2*y2) + a3*y3 with separately
// rounded products and sums in the compute type C = promote(eltype(out),
// coefficient type), the intermediate results are stored -- and rounded -- in
// the output eltype S, as the reference keeps them in `out`, and the scaling is
// a separate multiply.  With C = Float64 the result is the reference's to the
// last bit on the same inputs.
//
// Two layouts:
//   * k_iir_strided(_async): the filtered axis is not the contiguous one;
//     adjacent threads take adjacent lines, so every step is one coalesced
//     load/store per warp.
//   * k_iir_rows(_async): the filtered axis is the contiguous one; a warp takes
//     32 lines and moves them through shared memory in 32-element chunks
//     (coalesced loads and stores, a 33-element pitch so that every lane reads
//     its own bank while it recurses along its line).
// 4- and 8-byte elements are staged with cp.async, many steps ahead (the
// _async kernels); 8-bit first-stage inputs are loaded a few steps ahead in
// registers.
// The uniform forms of the recursions: the left border of _leftborder! is the
// causal recursion started from three copies of u- = i-/(1 - sum(a)); the
// right border of _rightborder! is the anticausal recursion started from
// (round_S(v1), v2, v3), v = M * Δu + v+.
#include "ifx_internal.h"

namespace ifx {

template <class C> __device__ __forceinline__ C radd(C x, C y);
template <class C> __device__ __forceinline__ C rsub(C x, C y);
template <class C> __device__ __forceinline__ C rmul(C x, C y);
template <class C> __device__ __forceinline__ C rdiv(C x, C y);
template <> __device__ __forceinline__ float radd(float x, float y) { return __fadd_rn(x, y); }
template <> __device__ __forceinline__ float rsub(float x, float y) { return __fsub_rn(x, y); }
template <> __device__ __forceinline__ float rmul(float x, float y) { return __fmul_rn(x, y); }
template <> __device__ __forceinline__ float rdiv(float x, float y) { return __fdiv_rn(x, y); }
template <> __device__ __forceinline__ double radd(double x, double y) { return __dadd_rn(x, y); }
template <> __device__ __forceinline__ double rsub(double x, double y) { return __dsub_rn(x, y); }
template <> __device__ __forceinline__ double rmul(double x, double y) { return __dmul_rn(x, y); }
template <> __device__ __forceinline__ double rdiv(double x, double y) { return __ddiv_rn(x, y); }

template <class C> struct IirCoef {
    C a1, a2, a3, b1, b2, b3, scale, om_a, om_b, M[9];
};

template <class C> __device__ __forceinline__ IirCoef<C> iir_coef(const IirArgs &A)
{
    IirCoef<C> k;
    k.a1 = (C)A.a[0];
    k.a2 = (C)A.a[1];
    k.a3 = (C)A.a[2];
    k.b1 = (C)A.b[0];
    k.b2 = (C)A.b[1];
    k.b3 = (C)A.b[2];
    k.scale = (C)A.scale;
    k.om_a = (C)A.om_a;
    k.om_b = (C)A.om_b;
#pragma unroll
    for (int r = 0; r < 9; ++r) k.M[r] = (C)A.M[r];
    return k;
}

// the stage input element as the reference sees it: converted to S (padarray
// to the output eltype), then widened to C
template <class Tin, class S, class C> __device__ __forceinline__ C iir_in(Tin v, bool norm)
{
    return (C)to_c<S>(v, norm);
}

template <class S, class C> __device__ __forceinline__ C round_s(C v) { return (C)(S)v; }

// causal step: ((x + a1*y1) + a2*y2) + a3*y3, rounded to S
template <class S, class C>
__device__ __forceinline__ C iir_fwd_step(const IirCoef<C> &k, C x, C y1, C y2, C y3)
{
    C t = radd(x, rmul(k.a1, y1));
    t = radd(t, rmul(k.a2, y2));
    t = radd(t, rmul(k.a3, y3));
    return round_s<S>(t);
}

template <class S, class C>
__device__ __forceinline__ C iir_bwd_step(const IirCoef<C> &k, C y, C p1, C p2, C p3)
{
    C t = radd(y, rmul(k.b1, p1));
    t = radd(t, rmul(k.b2, p2));
    t = radd(t, rmul(k.b3, p3));
    return round_s<S>(t);
}

// the right-edge state (Triggs & Sdika Eqs. 14-15) from the last three causal
// outputs o1 = y[L-1], o2 = y[L-2], o3 = y[L-3] and the right boundary input
template <class S, class C>
__device__ __forceinline__ void iir_right(const IirCoef<C> &k, C iplus, C o1, C o2, C o3, C &p1, C &p2, C &p3)
{
    const C uplus = rdiv(iplus, k.om_a);
    const C vplus = rdiv(uplus, k.om_b);
    const C d0 = rsub(o1, uplus), d1 = rsub(o2, uplus), d2 = rsub(o3, uplus);
    C v[3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
        v[r] = radd(radd(radd(rmul(k.M[3 * r], d0), rmul(k.M[3 * r + 1], d1)), rmul(k.M[3 * r + 2], d2)), vplus);
    p1 = round_s<S>(v[0]);
    p2 = v[1];
    p3 = v[2];
}

constexpr int kIirAhead = 8;

template <class Tin, class S, class C>
__global__ void __launch_bounds__(128) k_iir_strided(IirArgs A)
{
    const long long line = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (line >= A.lines) return;
    const long long o = line / A.inner, p = line - o * A.inner;
    const long long base = o * A.inner * A.L + p, st = A.inner, L = A.L;
    const Tin *src = (const Tin *)A.src;
    S *dst = (S *)A.dst;
    const bool norm = A.src_type == IFX_N0F8;
    const IirCoef<C> k = iir_coef<C>(A);
    // both boundary inputs before anything is written (in-place passes)
    const C xm = iir_in<Tin, S, C>(src[base], norm), xp = iir_in<Tin, S, C>(src[base + (L - 1) * st], norm);
    const C fillv = (C)(S)A.fill;
    const C uminus = rdiv(A.edge ? fillv : xm, k.om_a);
    C y1 = uminus, y2 = uminus, y3 = uminus;
    C buf[kIirAhead];
#pragma unroll
    for (int u = 0; u < kIirAhead; ++u) buf[u] = u < L ? iir_in<Tin, S, C>(src[base + u * st], norm) : (C)0;
    for (long long i0 = 0; i0 < L; i0 += kIirAhead) {
#pragma unroll
        for (int u = 0; u < kIirAhead; ++u) {
            const long long i = i0 + u;
            if (i < L) {
                const C x = buf[u];
                if (i + kIirAhead < L) buf[u] = iir_in<Tin, S, C>(src[base + (i + kIirAhead) * st], norm);
                const C y = iir_fwd_step<S>(k, x, y1, y2, y3);
                dst[base + i * st] = (S)y;
                y3 = y2;
                y2 = y1;
                y1 = y;
            }
        }
    }
    C p1, p2, p3;
    iir_right<S>(k, A.edge ? fillv : xp, y1, y2, y3, p1, p2, p3);
    dst[base + (L - 1) * st] = (S)rmul(p1, k.scale);
    // anticausal pass over i = L-2 .. 0 (step j = L-2-i), reading the causal outputs
    const long long n = L - 1;
#pragma unroll
    for (int u = 0; u < kIirAhead; ++u) buf[u] = u < n ? (C)dst[base + (n - 1 - u) * st] : (C)0;
    for (long long j0 = 0; j0 < n; j0 += kIirAhead) {
#pragma unroll
        for (int u = 0; u < kIirAhead; ++u) {
            const long long j = j0 + u;
            if (j < n) {
                const long long i = n - 1 - j;
                const C yv = buf[u];
                if (j + kIirAhead < n) buf[u] = (C)dst[base + (i - kIirAhead) * st];
                const C y = iir_bwd_step<S>(k, yv, p1, p2, p3);
                dst[base + i * st] = (S)rmul(y, k.scale);
                p3 = p2;
                p2 = p1;
                p1 = y;
            }
        }
    }
}

template <class Tin, class S, class C>
__global__ void __launch_bounds__(128) k_iir_rows(IirArgs A)
{
    __shared__ C sm[4][32][33];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long l0 = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * 32;
    if (l0 >= A.lines) return;                            // uniform over the warp
    C(*T)[33] = sm[warp];
    const long long L = A.L, me = l0 + lane;
    const bool act = me < A.lines;
    const Tin *src = (const Tin *)A.src;
    S *dst = (S *)A.dst;
    const bool norm = A.src_type == IFX_N0F8;
    const IirCoef<C> k = iir_coef<C>(A);
    const C fillv = (C)(S)A.fill;
    C xm = 0, xp = 0;
    if (act) {
        xm = iir_in<Tin, S, C>(src[me * L], norm);
        xp = iir_in<Tin, S, C>(src[me * L + L - 1], norm);
    }
    __syncwarp();                                         // boundary reads before any write
    const C uminus = rdiv(A.edge ? fillv : xm, k.om_a);
    C y1 = uminus, y2 = uminus, y3 = uminus;
    const long long nch = (L + 31) / 32;
    for (long long c = 0; c < nch; ++c) {
        const long long idx = c * 32 + lane;
#pragma unroll 4
        for (int r = 0; r < 32; ++r) {
            const long long ln = l0 + r;
            T[r][lane] = (ln < A.lines && idx < L) ? iir_in<Tin, S, C>(src[ln * L + idx], norm) : (C)0;
        }
        __syncwarp();
        if (act) {
            const int tn = (int)(L - c * 32 < 32 ? L - c * 32 : 32);
            for (int t = 0; t < tn; ++t) {
                const C y = iir_fwd_step<S>(k, T[lane][t], y1, y2, y3);
                T[lane][t] = y;
                y3 = y2;
                y2 = y1;
                y1 = y;
            }
        }
        __syncwarp();
#pragma unroll 4
        for (int r = 0; r < 32; ++r) {
            const long long ln = l0 + r;
            if (ln < A.lines && idx < L) dst[ln * L + idx] = (S)T[r][lane];
        }
        __syncwarp();
    }
    C p1 = 0, p2 = 0, p3 = 0;
    if (act) iir_right<S>(k, A.edge ? fillv : xp, y1, y2, y3, p1, p2, p3);
    for (long long c = nch - 1; c >= 0; --c) {
        const long long idx = c * 32 + lane;
#pragma unroll 4
        for (int r = 0; r < 32; ++r) {
            const long long ln = l0 + r;
            T[r][lane] = (ln < A.lines && idx < L) ? (C)dst[ln * L + idx] : (C)0;
        }
        __syncwarp();
        if (act) {
            const int tn = (int)(L - c * 32 < 32 ? L - c * 32 : 32);
            for (int t = tn - 1; t >= 0; --t) {
                if (c * 32 + t == L - 1) {
                    T[lane][t] = rmul(p1, k.scale);
                    continue;
                }
                const C y = iir_bwd_step<S>(k, T[lane][t], p1, p2, p3);
                T[lane][t] = rmul(y, k.scale);
                p3 = p2;
                p2 = p1;
                p1 = y;
            }
        }
        __syncwarp();
#pragma unroll 4
        for (int r = 0; r < 32; ++r) {
            const long long ln = l0 + r;
            if (ln < A.lines && idx < L) dst[ln * L + idx] = (S)T[r][lane];
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Asynchronous staging for 4- and 8-byte elements.  A line is sequential, so a
// thread has one element per step to wait for; what hides the memory latency
// is the number of steps in flight.  Both kernels below keep kIirDepth steps
// (strided) or kIirChunks chunks of 32 steps (rows) of every line in flight
// with cp.async copies into shared memory, one commit group per step (chunk):
// `cp.async.wait_group depth-1` then releases the oldest.  The anticausal pass
// reads the causal results back from global memory after a block-scope fence.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t iir_saddr(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

template <class E> __device__ __forceinline__ void iir_cp_async(E *sdst, const E *gsrc)
{
    static_assert(sizeof(E) == 4 || sizeof(E) == 8, "cp.async element size");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(iir_saddr(sdst)), "l"(gsrc), "n"(sizeof(E))
                 : "memory");
}
__device__ __forceinline__ void iir_cp_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void iir_cp_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

constexpr int kIirDepth = 32;      // steps in flight per line (strided layout)
constexpr int kIirChunks = 4;      // 32-step chunks in flight per warp (row layout)

template <class Tin, class S, class C>
__global__ void __launch_bounds__(128) k_iir_strided_async(IirArgs A)
{
    extern __shared__ __align__(16) unsigned char iir_dyn[];
    const int tid = threadIdx.x, bd = blockDim.x;
    const long long line = (long long)blockIdx.x * bd + tid;
    if (line >= A.lines) return;                          // no block-wide barrier below
    const long long o = line / A.inner, p = line - o * A.inner;
    const long long base = o * A.inner * A.L + p, st = A.inner, L = A.L;
    const Tin *src = (const Tin *)A.src;
    S *dst = (S *)A.dst;
    const IirCoef<C> k = iir_coef<C>(A);
    const C xm = (C)(S)src[base], xp = (C)(S)src[base + (L - 1) * st];
    const C fillv = (C)(S)A.fill;
    const C uminus = rdiv(A.edge ? fillv : xm, k.om_a);
    C y1 = uminus, y2 = uminus, y3 = uminus;
    {
        Tin *ring = (Tin *)iir_dyn;
#pragma unroll 1
        for (int u = 0; u < kIirDepth; ++u) {
            if (u < L) iir_cp_async(&ring[u * bd + tid], src + base + u * st);
            iir_cp_commit();
        }
        int slot = 0;
#pragma unroll 1
        for (long long i = 0; i < L; ++i) {
            iir_cp_wait<kIirDepth - 1>();
            const C x = (C)(S)ring[slot * bd + tid];
            if (i + kIirDepth < L) iir_cp_async(&ring[slot * bd + tid], src + base + (i + kIirDepth) * st);
            iir_cp_commit();
            slot = slot == kIirDepth - 1 ? 0 : slot + 1;
            const C y = iir_fwd_step<S>(k, x, y1, y2, y3);
            dst[base + i * st] = (S)y;
            y3 = y2;
            y2 = y1;
            y1 = y;
        }
    }
    iir_cp_wait<0>();
    C p1, p2, p3;
    iir_right<S>(k, A.edge ? fillv : xp, y1, y2, y3, p1, p2, p3);
    dst[base + (L - 1) * st] = (S)rmul(p1, k.scale);
    __threadfence_block();                                // the causal results before they are re-read
    const long long n = L - 1;
    S *ring = (S *)iir_dyn;
#pragma unroll 1
    for (int u = 0; u < kIirDepth; ++u) {
        if (u < n) iir_cp_async(&ring[u * bd + tid], dst + base + (n - 1 - u) * st);
        iir_cp_commit();
    }
    int slot = 0;
#pragma unroll 1
    for (long long j = 0; j < n; ++j) {
        const long long i = n - 1 - j;
        iir_cp_wait<kIirDepth - 1>();
        const C yv = (C)ring[slot * bd + tid];
        if (j + kIirDepth < n) iir_cp_async(&ring[slot * bd + tid], dst + base + (i - kIirDepth) * st);
        iir_cp_commit();
        slot = slot == kIirDepth - 1 ? 0 : slot + 1;
        const C y = iir_bwd_step<S>(k, yv, p1, p2, p3);
        dst[base + i * st] = (S)rmul(y, k.scale);
        p3 = p2;
        p2 = p1;
        p1 = y;
    }
    iir_cp_wait<0>();
}

// rows: a warp, 32 lines, chunks of 32 steps through shared memory; chunk c
// lives in stage c % kIirChunks ([32 lines][33] raw elements); results go
// through a [32][33] output tile for coalesced stores.
template <class E, class S> struct IirRowSmem {
    E stage[kIirChunks][32][33];
    S outt[32][33];
};

template <class Tin, class S, class C>
__global__ void __launch_bounds__(128) k_iir_rows_async(IirArgs A)
{
    extern __shared__ __align__(16) unsigned char iir_dyn[];
    constexpr int kEsz = sizeof(Tin) > sizeof(S) ? sizeof(Tin) : sizeof(S);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    unsigned char *mine = iir_dyn + (size_t)warp * (kIirChunks * 32 * 33 * kEsz + 32 * 33 * sizeof(S));
    const long long l0 = ((long long)blockIdx.x * (blockDim.x >> 5) + warp) * 32;
    if (l0 >= A.lines) return;                            // uniform over the warp; no block barrier
    const long long L = A.L, me = l0 + lane;
    const bool act = me < A.lines;
    const Tin *src = (const Tin *)A.src;
    S *dst = (S *)A.dst;
    const IirCoef<C> k = iir_coef<C>(A);
    const C fillv = (C)(S)A.fill;
    S(*outt)[33] = (S(*)[33])(mine + kIirChunks * 32 * 33 * kEsz);
    C xm = 0, xp = 0;
    if (act) {
        xm = (C)(S)src[me * L];
        xp = (C)(S)src[me * L + L - 1];
    }
    __syncwarp();
    const long long nch = (L + 31) / 32;
    // chunk loader: the 32 rows' elements c*32 + lane
    auto load_chunk = [&](auto *base_ptr, auto *stage, long long c) {
        const long long idx = c * 32 + lane;
        if (idx < L)
#pragma unroll 4
            for (int r = 0; r < 32; ++r) {
                const long long ln = l0 + r;
                if (ln < A.lines) iir_cp_async(&stage[r * 33 + lane], base_ptr + ln * L + idx);
            }
    };
    const C uminus = rdiv(A.edge ? fillv : xm, k.om_a);
    C y1 = uminus, y2 = uminus, y3 = uminus;
    {
        Tin *stg = (Tin *)mine;
        for (int u = 0; u < kIirChunks; ++u) {
            if (u < nch) load_chunk(src, stg + u * 32 * 33, u);
            iir_cp_commit();
        }
        for (long long c = 0; c < nch; ++c) {
            iir_cp_wait<kIirChunks - 1>();
            __syncwarp();
            const int sidx = (int)(c % kIirChunks);
            const Tin *T = stg + sidx * 32 * 33 + lane * 33;
            const int tn = (int)(L - c * 32 < 32 ? L - c * 32 : 32);
            if (act) {
                if (tn == 32) {
#pragma unroll
                    for (int t = 0; t < 32; ++t) {
                        const C y = iir_fwd_step<S>(k, (C)(S)T[t], y1, y2, y3);
                        outt[lane][t] = (S)y;
                        y3 = y2;
                        y2 = y1;
                        y1 = y;
                    }
                } else {
                    for (int t = 0; t < tn; ++t) {
                        const C y = iir_fwd_step<S>(k, (C)(S)T[t], y1, y2, y3);
                        outt[lane][t] = (S)y;
                        y3 = y2;
                        y2 = y1;
                        y1 = y;
                    }
                }
            }
            __syncwarp();                                 // stage and output tile read / written
            if (c + kIirChunks < nch) load_chunk(src, stg + sidx * 32 * 33, c + kIirChunks);
            iir_cp_commit();
            const long long idx = c * 32 + lane;
            if (idx < L)
#pragma unroll 4
                for (int r = 0; r < 32; ++r) {
                    const long long ln = l0 + r;
                    if (ln < A.lines) dst[ln * L + idx] = outt[r][lane];
                }
            __syncwarp();
        }
    }
    iir_cp_wait<0>();
    C p1 = 0, p2 = 0, p3 = 0;
    if (act) iir_right<S>(k, A.edge ? fillv : xp, y1, y2, y3, p1, p2, p3);
    __threadfence_block();                                // the causal results before they are re-read
    __syncwarp();
    S *stg = (S *)mine;
    for (int u = 0; u < kIirChunks; ++u) {
        if (u < nch) load_chunk(dst, stg + u * 32 * 33, nch - 1 - u);
        iir_cp_commit();
    }
    for (long long cc = 0; cc < nch; ++cc) {
        const long long c = nch - 1 - cc;
        iir_cp_wait<kIirChunks - 1>();
        __syncwarp();
        const int sidx = (int)(cc % kIirChunks);
        const S *T = stg + sidx * 32 * 33 + lane * 33;
        const int tn = (int)(L - c * 32 < 32 ? L - c * 32 : 32);
        if (act) {
            if (tn == 32 && c * 32 + 31 < L - 1) {
#pragma unroll
                for (int t = 31; t >= 0; --t) {
                    const C y = iir_bwd_step<S>(k, (C)T[t], p1, p2, p3);
                    outt[lane][t] = (S)rmul(y, k.scale);
                    p3 = p2;
                    p2 = p1;
                    p1 = y;
                }
            } else {
                for (int t = tn - 1; t >= 0; --t) {
                    if (c * 32 + t == L - 1) {
                        outt[lane][t] = (S)rmul(p1, k.scale);
                        continue;
                    }
                    const C y = iir_bwd_step<S>(k, (C)T[t], p1, p2, p3);
                    outt[lane][t] = (S)rmul(y, k.scale);
                    p3 = p2;
                    p2 = p1;
                    p1 = y;
                }
            }
        }
        __syncwarp();
        if (cc + kIirChunks < nch) load_chunk(dst, stg + sidx * 32 * 33, c - kIirChunks);
        iir_cp_commit();
        const long long idx = c * 32 + lane;
        if (idx < L)
#pragma unroll 4
            for (int r = 0; r < 32; ++r) {
                const long long ln = l0 + r;
                if (ln < A.lines) dst[ln * L + idx] = outt[r][lane];
            }
        __syncwarp();
    }
    iir_cp_wait<0>();
}

template <class Tin, class S> constexpr size_t iir_row_smem_per_warp()
{
    return (size_t)kIirChunks * 32 * 33 * (sizeof(Tin) > sizeof(S) ? sizeof(Tin) : sizeof(S)) +
           32 * 33 * sizeof(S);
}

template <class Tin, class S, class C> static cudaError_t iir_run(const IirArgs &a, cudaStream_t s)
{
    // few lines: small blocks, so that they spread over every SM
    if constexpr (sizeof(Tin) >= 4) {
        if (a.inner == 1) {
            const long long warps = (a.lines + 31) / 32;
            const int wpb = warps < 4LL * 152 ? 1 : 2;
            const size_t smem = wpb * iir_row_smem_per_warp<Tin, S>();
            // the opt-in above 48 KB, once per instantiation (thread-safe static initialisation)
            static const cudaError_t attr = cudaFuncSetAttribute(
                k_iir_rows_async<Tin, S, C>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                (int)(2 * iir_row_smem_per_warp<Tin, S>()));
            if (attr != cudaSuccess) return attr;
            k_iir_rows_async<Tin, S, C><<<(unsigned)((warps + wpb - 1) / wpb), 32 * wpb, smem, s>>>(a);
        } else {
            const int tpb = a.lines < 128LL * 152 ? 32 : 128;
            // one ring for the causal pass (Tin) and then the anticausal pass (S)
            const size_t esz = sizeof(Tin) > sizeof(S) ? sizeof(Tin) : sizeof(S);
            k_iir_strided_async<Tin, S, C><<<(unsigned)((a.lines + tpb - 1) / tpb), tpb,
                                             (size_t)kIirDepth * tpb * esz, s>>>(a);
        }
    } else {
        if (a.inner == 1) {
            const long long warps = (a.lines + 31) / 32;
            const int wpb = warps < 4LL * 152 ? 1 : 4;
            k_iir_rows<Tin, S, C><<<(unsigned)((warps + wpb - 1) / wpb), 32 * wpb, 0, s>>>(a);
        } else {
            const int tpb = a.lines < 128LL * 152 ? 32 : 128;
            k_iir_strided<Tin, S, C><<<(unsigned)((a.lines + tpb - 1) / tpb), tpb, 0, s>>>(a);
        }
    }
    note_launch();
    return cudaGetLastError();
}

template <class S, class C> static cudaError_t iir_in_type(const IirArgs &a, cudaStream_t s)
{
    switch (a.src_type) {
    case IFX_F32: return iir_run<float, S, C>(a, s);
    case IFX_F64: return iir_run<double, S, C>(a, s);
    case IFX_U8:
    case IFX_N0F8: return iir_run<uint8_t, S, C>(a, s);
    default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_iir(const IirArgs &a, cudaStream_t s)
{
    if (a.lines == 0) return cudaSuccess;
    if (a.L < 4 || a.L > (1LL << 30)) return cudaErrorInvalidValue;
    if (a.dst_type == IFX_F64) return iir_in_type<double, double>(a, s);
    if (a.dst_type == IFX_F32) return a.compute_f64 ? iir_in_type<float, double>(a, s) : iir_in_type<float, float>(a, s);
    return cudaErrorInvalidValue;
}

} // namespace ifx
