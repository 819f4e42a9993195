// ifx_dense_tc.cu -- dense 2-D correlation on the tcgen05 tensor cores
// (kernels of 11x11 and larger), as an implicit GEMM with BF16 hi/lo operands
// and FP32 accumulation in tensor memory.
//
// Correlation (src/imfilter.jl:624-669):  out[x,y] = sum_{i,j} P[x+fx+j, y+fy+i] K[j,i].
// One CTA computes an output tile of M = 128 rows (y) by N = 32 columns (x).
// With the tile's input patch Pt[r][c] = P[x0+fx+c, y0+fy+r] and v = u + j,
//   out[x0+u, y0+m] = sum_i sum_v Pt[m+i][v] * K[v-u, i]
// is, for each kernel row i, a GEMM  A_i (128 x V) * B_i (V x 32)  with
//   A_i[m][v] = Pt[m+i][v]        -- the patch shifted down by i rows
//   B_i[v][u] = K[v-u, i]         -- a banded (Toeplitz) matrix, zero off band
// and V = N + kw - 1 rounded up to 16.  The K index is enumerated in reverse
// (v' = V-1-v) for both operands; then B_i's 8x8 core matrix (row group g,
// column group q') depends only on d = q'+g, so each kernel row needs just
// Q+3 core matrices (Q = V/8) and the whole B for a 31x31 kernel (hi and lo)
// fits in shared memory.  A_i is the same patch for every i: stored as K-major
// core-matrix planes with 16-byte rows, shifting it by i rows is adding 16*i
// bytes to the descriptor's start address.
//
// Each product is split: a = a_hi + a_lo, k = k_hi + k_lo with BF16 parts and
// the three MMAs a_hi*k_hi + a_hi*k_lo + a_lo*k_hi accumulate in FP32 (about
// 2^-17 relative error per term; within 1e-5 normwise of the FP64 oracle).
//
// Waits are bounded: an mbarrier that never completes sets *err, the CTA frees
// its tensor memory and returns.
#include "ifx_internal.h"
#include "ifx_tma.cuh"
#include <cuda_bf16.h>
#include <cstring>

namespace ifx {

constexpr int kTcM = 128, kTcN = 32;
constexpr int kTcMaxKw = 33, kTcMaxKh = 40;
constexpr int kTcThreads = 256, kTcWarps = kTcThreads / 32;

struct TcWeights { float w[kTcMaxKw * kTcMaxKh]; };

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// Shared-memory matrix descriptor, no swizzle, K-major: start address, LBO =
// byte stride between core matrices along K, SBO = along M/N; bits 46-48 hold
// the fixed value 0b001.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr >> 4) & 0x3FFF) | ((uint64_t)((lbo >> 4) & 0x3FFF) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFF) << 32) | (1ull << 46);
}

__device__ __forceinline__ void tc_mma(uint32_t dtmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                 :: "r"(dtmem), "l"(a), "l"(b), "r"(idesc), "r"(acc) : "memory");
}

// Same MMA with the descriptors given as (low, high) 32-bit words: the issue
// loop advances only the low words (the start-address field, which never
// carries into the next field for shared-memory addresses of this kernel).
__device__ __forceinline__ void tc_mma_w(uint32_t dtmem, uint32_t a_lo, uint32_t a_hi, uint32_t b_lo,
                                         uint32_t b_hi, uint32_t idesc, uint32_t acc)
{
    asm volatile("{\n\t.reg .pred p;\n\t.reg .b64 da, db;\n\t"
                 "setp.ne.b32 p, %6, 0;\n\t"
                 "mov.b64 da, {%1, %2};\n\tmov.b64 db, {%3, %4};\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, db, %5, p;\n\t}\n"
                 :: "r"(dtmem), "r"(a_lo), "r"(a_hi), "r"(b_lo), "r"(b_hi), "r"(idesc), "r"(acc)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t mbar, uint32_t parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}\n"
                 : "=r"(ok) : "r"(mbar), "r"(parity) : "memory");
    return ok != 0;
}

struct TcArgs {
    const void *img;
    void *out;
    int in_type, out_type;
    int nx, ny, fx, fy, kw, kh, style;
    float fill;
    int V, Q, R;                // K extent, planes, patch rows
    int tiles_x, tiles;
    int *err;
};

// Shared memory: B hi | B lo | A buffer 0 (hi planes, lo planes) | A buffer 1
// | epilogue staging (8 warps x 32 rows x 17 floats).
struct TcLayout {
    size_t b_bytes;             // one of B hi / B lo
    size_t plane;               // one A plane: R rows x 16 bytes
    size_t a_off[2];            // A buffers
    size_t stage_off;
    size_t total;
};

__host__ __device__ inline TcLayout tc_layout(int kh, int Q, int R)
{
    TcLayout L;
    L.b_bytes = (size_t)kh * (Q + 3) * 128;
    L.plane = (size_t)R * 16;
    L.a_off[0] = 2 * L.b_bytes;
    L.a_off[1] = L.a_off[0] + 2 * (size_t)Q * L.plane;
    L.stage_off = L.a_off[1] + 2 * (size_t)Q * L.plane;
    L.total = L.stage_off + (size_t)kTcWarps * 32 * 17 * sizeof(float) + 128;
    return L;
}

template <class Tin>
__device__ __forceinline__ float tc_in(Tin raw, bool norm)
{
    if constexpr (sizeof(Tin) == 1)
        return norm ? __fdiv_rn((float)raw, 255.0f) : (float)raw;
    else
        return (float)raw;
}

__device__ __forceinline__ uint32_t bf2(float lo_elem, float hi_elem)
{
    __nv_bfloat162 p = __floats2bfloat162_rn(lo_elem, hi_elem);
    return *reinterpret_cast<uint32_t *>(&p);
}

// Split 8 patch values (x order) into BF16 hi and lo rows of one core-matrix
// plane; the K index runs in reverse, so row element t holds v[7 - t].
__device__ __forceinline__ void tc_store_chunk(uint16_t *hi_row, uint16_t *lo_row, const float v[8])
{
    float h[8], l[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
        h[e] = __bfloat162float(__float2bfloat16_rn(v[e]));
        l[e] = v[e] - h[e];
    }
    uint4 H, Lw;
    H.x = bf2(h[7], h[6]);
    H.y = bf2(h[5], h[4]);
    H.z = bf2(h[3], h[2]);
    H.w = bf2(h[1], h[0]);
    Lw.x = bf2(l[7], l[6]);
    Lw.y = bf2(l[5], l[4]);
    Lw.z = bf2(l[3], l[2]);
    Lw.w = bf2(l[1], l[0]);
    *reinterpret_cast<uint4 *>(hi_row) = H;
    *reinterpret_cast<uint4 *>(lo_row) = Lw;
}

// Gather the patch of tile (x0, y0) into A buffer (hi at `Ah`, lo at `Al`):
// chunk (r, m) is patch row r, columns 8m..8m+7, stored in plane Q-1-m.
// Columns at or past valid_c stay zero (written once at start-up).
template <class Tin>
__device__ __forceinline__ void tc_gather(const TcArgs &a, int x0, int y0, uint16_t *Ah, uint16_t *Al,
                                          size_t plane_el)
{
    const int valid_c = kTcN + a.kw - 1, Mv = (valid_c + 7) >> 3;
    const int R = a.R, Q = a.Q;
    const bool norm = a.in_type == IFX_N0F8;
    const Tin *img = (const Tin *)a.img;
    const int px0 = x0 + a.fx, py0 = y0 + a.fy;
    const bool interior = px0 >= 0 && px0 + valid_c <= a.nx && py0 >= 0 && py0 + R <= a.ny;
    const int nch = R * Mv;
    for (int base = threadIdx.x; base < nch; base += 2 * kTcThreads) {
        float v[2][8];
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int ch = base + u * kTcThreads;
            const int r = ch / Mv, m = ch - r * Mv;
#pragma unroll
            for (int e = 0; e < 8; ++e) v[u][e] = 0.0f;
            if (ch < nch) {
                const int c0 = 8 * m;
                if (interior) {
                    const Tin *rowp = img + (long long)(py0 + r) * a.nx + px0 + c0;
#pragma unroll
                    for (int e = 0; e < 8; ++e)
                        if (c0 + e < valid_c) v[u][e] = tc_in<Tin>(rowp[e], norm);
                } else {
                    const int my = map_index(py0 + r, a.ny, a.style);
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        if (c0 + e >= valid_c) continue;
                        const int mx = map_index(px0 + c0 + e, a.nx, a.style);
                        v[u][e] = (mx < 0 || my < 0) ? a.fill
                                                     : tc_in<Tin>(img[(long long)my * a.nx + mx], norm);
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int ch = base + u * kTcThreads;
            if (ch >= nch) continue;
            const int r = ch / Mv, m = ch - r * Mv;
            const size_t o = (size_t)(Q - 1 - m) * plane_el + (size_t)r * 8;
            tc_store_chunk(Ah + o, Al + o, v[u]);
        }
    }
}

__device__ __forceinline__ void tc_fence_sync()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

template <class Tin, class Tout>
__global__ void __launch_bounds__(kTcThreads, 1)
k_dense_tc(TcArgs a, const __grid_constant__ TcWeights W)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar[2];
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int kw = a.kw, kh = a.kh, V = a.V, Q = a.Q, R = a.R;
    const int ncm = Q + 3;
    const TcLayout L = tc_layout(kh, Q, R);
    const size_t plane_el = L.plane / 2;
    uint16_t *Bhi = reinterpret_cast<uint16_t *>(sm);
    uint16_t *Blo = Bhi + L.b_bytes / 2;
    // A buffer b: hi planes at Ahi(b), lo planes right after them
    const size_t a_step = L.a_off[1] - L.a_off[0];
    auto Ahi = [&](int b) { return reinterpret_cast<uint16_t *>(sm + L.a_off[0] + b * a_step); };
    auto Alo = [&](int b) { return Ahi(b) + (size_t)Q * plane_el; };
    float *stage = reinterpret_cast<float *>(sm + L.stage_off) + (size_t)warp * 32 * 17;

    // tensor memory: two accumulators of 32 columns (128 lanes x 32 FP32)
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_slot)), "r"(64) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        for (int b = 0; b < 2; ++b)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&mbar[b])) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        s_abort = 0;
    }
    // B: core matrix (i, d), row r, column t holds K[V-1-8d-t-r, i] (zero off band)
    for (int e = tid; e < kh * ncm * 64; e += blockDim.x) {
        const int t = e & 7, r = (e >> 3) & 7, cm = e >> 6;
        const int d = cm % ncm, i = cm / ncm;
        const int j = V - 1 - 8 * d - t - r;
        const float k = (j >= 0 && j < kw) ? W.w[j + kw * i] : 0.0f;
        const __nv_bfloat16 hi = __float2bfloat16_rn(k);
        const __nv_bfloat16 lo = __float2bfloat16_rn(k - __bfloat162float(hi));
        Bhi[e] = __bfloat16_as_ushort(hi);
        Blo[e] = __bfloat16_as_ushort(lo);
    }
    // both A buffers start zero: the columns past the patch are never rewritten
    {
        uint4 *z = reinterpret_cast<uint4 *>(sm + L.a_off[0]);
        const size_t n16 = (L.stage_off - L.a_off[0]) / 16;
        for (size_t e = tid; e < n16; e += blockDim.x) z[e] = make_uint4(0, 0, 0, 0);
    }
    __syncthreads();
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                           ((uint32_t)(kTcM >> 4) << 24);
    const uint32_t bhi_s = smem_u32(Bhi), blo_s = smem_u32(Blo);
    const uint32_t ps = (uint32_t)L.plane;
    uint32_t phase = 0;                 // bit b: parity awaited on mbar[b]

    int tile = blockIdx.x;
    if (tile < a.tiles) {
        const int ty = tile / a.tiles_x, tx = tile - ty * a.tiles_x;
        tc_gather<Tin>(a, tx * kTcN, ty * kTcM, Ahi(0), Alo(0), plane_el);
    }
    tc_fence_sync();
    int prev = -1;                      // tile whose accumulator awaits its epilogue
    for (int k = 0;; ++k, tile += gridDim.x) {
        const int b = k & 1;
        const bool have = tile < a.tiles;
        // 1. issue the MMAs of this tile into accumulator b
        if (have && tid == 0) {
            // descriptors: the high words are fixed, the low words advance by
            // byte offsets >> 4 (i rows: +i for A; core matrices: +8 for B)
            const uint64_t dAh = tc_desc(smem_u32(Ahi(b)), ps, 128), dAl = tc_desc(smem_u32(Alo(b)), ps, 128);
            const uint64_t dBh = tc_desc(bhi_s, 128, 128), dBl = tc_desc(blo_s, 128, 128);
            const uint32_t hAh = (uint32_t)(dAh >> 32), hAl = (uint32_t)(dAl >> 32);
            const uint32_t hBh = (uint32_t)(dBh >> 32), hBl = (uint32_t)(dBl >> 32);
            uint32_t ah = (uint32_t)dAh, al = (uint32_t)dAl, bh = (uint32_t)dBh, bl = (uint32_t)dBl;
            const uint32_t dt = tmem + 32u * (uint32_t)b;
            const uint32_t a_ks = (2u * ps) >> 4;          // next 16 K values: two planes
            const uint32_t b_row = (uint32_t)ncm * 8u;     // next kernel row of B
            const int ksteps = V / 16;
            uint32_t acc = 0;
            for (int i = 0; i < kh; ++i) {
                uint32_t a1 = ah, a2 = al, b1 = bh, b2 = bl;
                for (int s = 0; s < ksteps; ++s) {
                    tc_mma_w(dt, a1, hAh, b1, hBh, idesc, acc);
                    acc = 1;
                    tc_mma_w(dt, a1, hAh, b2, hBl, idesc, 1);
                    tc_mma_w(dt, a2, hAl, b1, hBh, idesc, 1);
                    a1 += a_ks;
                    a2 += a_ks;
                    b1 += 16u;
                    b2 += 16u;
                }
                ah += 1u;
                al += 1u;
                bh += b_row;
                bl += b_row;
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(smem_u32(&mbar[b])) : "memory");
        }
        // 2. epilogue of the previous tile (accumulator b^1), overlapping this tile's MMAs
        if (prev >= 0) {
            const int pb = b ^ 1;
            bool done = false;
            for (uint32_t it = 0; it < (1u << 22); ++it)
                if (mbar_try_wait(smem_u32(&mbar[pb]), (phase >> pb) & 1)) {
                    done = true;
                    break;
                }
            phase ^= 1u << pb;
            done = __all_sync(0xffffffffu, done);
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            if (!done) {
                if (lane == 0) atomicExch(a.err, 1);
                s_abort = 1;
            } else {
                const int q4 = warp & 3, half = warp >> 2;
                uint32_t r[16];
                const uint32_t taddr = tmem + ((uint32_t)(32 * q4) << 16) + 32u * (uint32_t)pb +
                                       16u * (uint32_t)half;
                asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                             "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                             : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]),
                               "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]),
                               "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                               "=r"(r[15])
                             : "r"(taddr) : "memory");
                asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                for (int u = 0; u < 16; ++u) stage[lane * 17 + u] = __uint_as_float(r[u]);
                __syncwarp();
                const int pty = prev / a.tiles_x, ptx = prev - pty * a.tiles_x;
                const int xo = ptx * kTcN + 16 * half + (lane & 15);
                const int yb = pty * kTcM + 32 * q4;
#pragma unroll 4
                for (int rr = 0; rr < 32; rr += 2) {
                    const int row = rr + (lane >> 4), y = yb + row;
                    if (y < a.ny && xo < a.nx)
                        ((Tout *)a.out)[(long long)y * a.nx + xo] = (Tout)stage[row * 17 + (lane & 15)];
                }
            }
        }
        // 3. gather the next tile into the other A buffer (its MMAs, two tiles
        //    back, completed before the epilogue above)
        const int next = tile + gridDim.x;
        if (have && next < a.tiles) {
            const int ty = next / a.tiles_x, tx = next - ty * a.tiles_x;
            tc_gather<Tin>(a, tx * kTcN, ty * kTcM, Ahi(b ^ 1), Alo(b ^ 1), plane_el);
        }
        tc_fence_sync();
        if (s_abort) {
            // let this tile's MMAs (if any) drain before the accumulator is freed
            if (have)
                for (uint32_t it = 0; it < (1u << 22); ++it)
                    if (mbar_try_wait(smem_u32(&mbar[b]), (phase >> b) & 1)) break;
            break;
        }
        if (!have) break;
        prev = tile;
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(64) : "memory");
}

bool dense_tc_supported(int in_type, int kw, int kh)
{
    if (!((in_type == IFX_F32 || in_type == IFX_N0F8 || in_type == IFX_U8) && kw >= 1 &&
          kw <= kTcMaxKw && kh >= 1 && kh <= kTcMaxKh))
        return false;
    const int V = (kTcN + kw - 1 + 15) / 16 * 16;
    return tc_layout(kh, V / 8, kTcM + kh - 1).total <= 225 * 1024;   // + static shared
}

template <class Tin, class Tout>
static cudaError_t dense_tc_t(const Dense2dArgs &d, cudaStream_t s, int device)
{
    TcArgs a;
    memset(&a, 0, sizeof a);
    a.img = d.img;
    a.out = d.out;
    a.in_type = d.in_type;
    a.out_type = d.out_type;
    a.nx = d.nx;
    a.ny = d.ny;
    a.fx = d.fx;
    a.fy = d.fy;
    a.kw = d.kw;
    a.kh = d.kh;
    a.style = d.style;
    a.fill = (float)d.fill;
    a.V = (kTcN + d.kw - 1 + 15) / 16 * 16;
    a.Q = a.V / 8;
    a.R = kTcM + d.kh - 1;
    a.tiles_x = (d.nx + kTcN - 1) / kTcN;
    a.tiles = a.tiles_x * ((d.ny + kTcM - 1) / kTcM);
    a.err = tma_error_word(device);
    if (!a.err) return cudaErrorMemoryAllocation;
    static thread_local TcWeights W;
    for (int t = 0; t < d.kw * d.kh; ++t) W.w[t] = (float)d.K[t];
    const size_t smem = tc_layout(d.kh, a.Q, a.R).total;
    auto kern = k_dense_tc<Tin, Tout>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int sms = 0, per_sm = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kTcThreads, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    if (per_sm > 4) per_sm = 4;               // 4 x 64 TMEM columns at most
    const long long slots = (long long)sms * per_sm;
    const int grid = a.tiles < slots ? a.tiles : (int)slots;
    kern<<<grid, kTcThreads, smem, s>>>(a, W);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_dense_tc(const Dense2dArgs &d, cudaStream_t s, int device)
{
    if (d.nx == 0 || d.ny == 0) return cudaSuccess;
    const bool u8 = d.in_type == IFX_N0F8 || d.in_type == IFX_U8;
    if (d.in_type == IFX_F32 && d.out_type == IFX_F32) return dense_tc_t<float, float>(d, s, device);
    if (d.in_type == IFX_F32 && d.out_type == IFX_F64) return dense_tc_t<float, double>(d, s, device);
    if (u8 && d.out_type == IFX_F32) return dense_tc_t<uint8_t, float>(d, s, device);
    if (u8 && d.out_type == IFX_F64) return dense_tc_t<uint8_t, double>(d, s, device);
    return cudaErrorInvalidValue;
}

} // namespace ifx
