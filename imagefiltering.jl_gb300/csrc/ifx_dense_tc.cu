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
#include <cuda_bf16.h>
#include <cstring>

namespace ifx {

constexpr int kTcM = 128, kTcN = 32;
constexpr int kTcMaxKw = 33, kTcMaxKh = 40;
constexpr int kTcThreads = 128;

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

__host__ __device__ inline size_t tc_smem_layout(int kh, int Q, int R, size_t *b_off, size_t *a_off,
                                                 size_t *plane)
{
    const size_t ncm = (size_t)Q + 3;
    const size_t bbytes = (size_t)kh * ncm * 128;          // one of hi / lo
    *plane = (size_t)R * 16;
    *b_off = 0;
    *a_off = 2 * bbytes;
    // A hi, A lo, then 16 planes of slack so that no descriptor of this kernel
    // can address past the allocation
    return *a_off + (2 * (size_t)Q + 16) * *plane + 64;
}

template <class Tin, class Tout>
__global__ void __launch_bounds__(kTcThreads, 1)
k_dense_tc(TcArgs a, const __grid_constant__ TcWeights W)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmem_slot;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int kw = a.kw, kh = a.kh, V = a.V, Q = a.Q, R = a.R;
    const int ncm = Q + 3;
    size_t b_off, a_off, plane;
    tc_smem_layout(kh, Q, R, &b_off, &a_off, &plane);
    uint16_t *Bhi = reinterpret_cast<uint16_t *>(sm + b_off);
    uint16_t *Blo = Bhi + (size_t)kh * ncm * 64;
    uint16_t *Ahi = reinterpret_cast<uint16_t *>(sm + a_off);
    uint16_t *Alo = Ahi + (size_t)Q * plane / 2;

    // tensor memory: 32 columns hold the 128 x 32 FP32 accumulator
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_slot)), "r"(32) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&mbar)) : "memory");
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
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kTcN >> 3) << 17) |
                           ((uint32_t)(kTcM >> 4) << 24);
    const uint32_t ahi_s = smem_u32(Ahi), alo_s = smem_u32(Alo);
    const uint32_t bhi_s = smem_u32(Bhi), blo_s = smem_u32(Blo);
    const uint32_t mb = smem_u32(&mbar);
    const int valid_c = kTcN + kw - 1;
    uint32_t phase = 0;

    for (int tile = blockIdx.x; tile < a.tiles; tile += gridDim.x) {
        const int ty = tile / a.tiles_x, tx = tile - ty * a.tiles_x;
        const int x0 = tx * kTcN, y0 = ty * kTcM;
        // A: plane q' row r column t = Pt[r][V-1-(8q'+t)], split into BF16 hi/lo
        for (int e = tid; e < R * V; e += blockDim.x) {
            const int r = e / V, c = e - r * V;          // c: patch column (x order)
            float v = 0.0f;
            if (c < valid_c) {
                const int mx = map_index(x0 + a.fx + c, a.nx, a.style);
                const int my = map_index(y0 + a.fy + r, a.ny, a.style);
                if (mx < 0 || my < 0) v = a.fill;
                else {
                    const Tin raw = ((const Tin *)a.img)[(long long)my * a.nx + mx];
                    if constexpr (sizeof(Tin) == 1)
                        v = a.in_type == IFX_N0F8 ? __fdiv_rn((float)raw, 255.0f) : (float)raw;
                    else
                        v = (float)raw;
                }
            }
            const int vr = V - 1 - c, q = vr >> 3, t = vr & 7;
            const size_t o = (size_t)q * (plane / 2) + (size_t)r * 8 + t;
            const __nv_bfloat16 hi = __float2bfloat16_rn(v);
            const __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
            Ahi[o] = __bfloat16_as_ushort(hi);
            Alo[o] = __bfloat16_as_ushort(lo);
        }
        // generic-proxy stores -> visible to the tensor core's async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        if (tid == 0) {
            const uint32_t ps = (uint32_t)plane;
            uint32_t acc = 0;
            for (int i = 0; i < kh; ++i) {
                for (int s = 0; s < V / 16; ++s) {
                    const uint32_t aoff = (uint32_t)(2 * s) * ps + 16u * (uint32_t)i;
                    const uint32_t boff = (uint32_t)((i * ncm + 2 * s) * 128);
                    const uint64_t da_hi = tc_desc(ahi_s + aoff, ps, 128);
                    const uint64_t da_lo = tc_desc(alo_s + aoff, ps, 128);
                    const uint64_t db_hi = tc_desc(bhi_s + boff, 128, 128);
                    const uint64_t db_lo = tc_desc(blo_s + boff, 128, 128);
                    tc_mma(tmem, da_hi, db_hi, idesc, acc);
                    acc = 1;
                    tc_mma(tmem, da_hi, db_lo, idesc, 1);
                    tc_mma(tmem, da_lo, db_hi, idesc, 1);
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                         :: "r"(mb) : "memory");
        }
        // bounded wait for the MMAs of this tile
        bool done = false;
        for (uint32_t it = 0; it < (1u << 22); ++it) {
            if (mbar_try_wait(mb, phase)) {
                done = true;
                break;
            }
        }
        phase ^= 1;
        if (!done) {
            if (lane == 0) atomicExch(a.err, 1);
            s_abort = 1;
        }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        __syncthreads();
        if (s_abort) break;
        // epilogue: warp w reads lanes 32w..32w+31 (rows m), 32 columns (u)
        uint32_t r[32];
        const uint32_t taddr = tmem + ((uint32_t)(32 * warp) << 16);
        asm volatile("tcgen05.ld.sync.aligned.32x32b.x32.b32 "
                     "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
                     "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
                     : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]),
                       "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]),
                       "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]),
                       "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
                       "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]),
                       "=r"(r[30]), "=r"(r[31])
                     : "r"(taddr) : "memory");
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        const int y = y0 + 32 * warp + lane;
        if (y < a.ny) {
            Tout *orow = (Tout *)a.out + (long long)y * a.nx;
#pragma unroll
            for (int u = 0; u < kTcN; ++u) {
                const int x = x0 + u;
                if (x < a.nx) orow[x] = (Tout)__uint_as_float(r[u]);
            }
        }
        // the next tile's MMAs overwrite the accumulator and the A planes
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    }
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(32) : "memory");
}

static int *g_tc_err[64];

bool dense_tc_supported(int in_type, int kw, int kh)
{
    return (in_type == IFX_F32 || in_type == IFX_N0F8 || in_type == IFX_U8) && kw >= 1 &&
           kw <= kTcMaxKw && kh >= 1 && kh <= kTcMaxKh;
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
    if (!g_tc_err[device]) {
        cudaError_t e = cudaMalloc(&g_tc_err[device], sizeof(int));
        if (e != cudaSuccess) return e;
        cudaMemset(g_tc_err[device], 0, sizeof(int));
    }
    a.err = g_tc_err[device];
    static thread_local TcWeights W;
    for (int t = 0; t < d.kw * d.kh; ++t) W.w[t] = (float)d.K[t];
    size_t b_off, a_off, plane;
    const size_t smem = tc_smem_layout(d.kh, a.Q, a.R, &b_off, &a_off, &plane);
    auto kern = k_dense_tc<Tin, Tout>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int grid = a.tiles < sms ? a.tiles : sms;
    kern<<<grid, kTcThreads, smem, s>>>(a, W);
    note_launch();
    return cudaGetLastError();
}

size_t dense_tc_smem_bytes(int kw, int kh)
{
    const int V = (kTcN + kw - 1 + 15) / 16 * 16;
    size_t b, a, p;
    return tc_smem_layout(kh, V / 8, kTcM + kh - 1, &b, &a, &p);
}

// Reads (and clears) the timeout flag of the tensor-core kernel on `device`.
int dense_tc_check_error(int device)
{
    if (device < 0 || device >= 64 || !g_tc_err[device]) return 0;
    int h = 0;
    cudaMemcpy(&h, g_tc_err[device], sizeof(int), cudaMemcpyDeviceToHost);
    if (h) cudaMemset(g_tc_err[device], 0, sizeof(int));
    return h;
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
