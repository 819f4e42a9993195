// ifx_fir.cu -- FIR kernels for sm_103a: border-mapped padding, separable
// passes (generic N-d box pass and the fused 2-D tile kernel), dense direct
// correlation and the Laplacian stencil.
//
// Reference semantics (ImageFiltering.jl v0.7.12):
//  * the image is padded once with the accumulated padding of every factor
//    (src/imfilter.jl:331-341), and each pass of a cascade is evaluated over
//    the index range that the later passes still need (src/imfilter.jl:
//    385-457).  Here the padding is never materialised for the fused kernel:
//    each tile gathers its input through the border index map
//    (src/border.jl:564-596), and pass 1 runs over the tile's halo rows too,
//    which reproduces pad-then-cascade exactly, Fill borders included.
//  * a pass is the correlation out[i] = sum_j A[i+j] k[j] (src/imfilter.jl:
//    671-739); dense kernels sum over all taps (src/imfilter.jl:624-669).
#include "ifx_internal.h"
#include "ifx_tma.cuh"
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

namespace ifx {

// ------------------------------------------------------------------ helpers
template <class To, class Ti> __device__ __forceinline__ To cvt(Ti v, bool norm);
template <> __device__ __forceinline__ float cvt<float, float>(float v, bool) { return v; }
template <> __device__ __forceinline__ float cvt<float, double>(double v, bool) { return (float)v; }
template <> __device__ __forceinline__ double cvt<double, float>(float v, bool) { return (double)v; }
template <> __device__ __forceinline__ double cvt<double, double>(double v, bool) { return v; }
template <> __device__ __forceinline__ float cvt<float, uint8_t>(uint8_t v, bool norm)
{
    return norm ? __fdiv_rn((float)v, 255.0f) : (float)v;
}
template <> __device__ __forceinline__ double cvt<double, uint8_t>(uint8_t v, bool norm)
{
    return norm ? __ddiv_rn((double)v, 255.0) : (double)v;
}
template <> __device__ __forceinline__ uint8_t cvt<uint8_t, uint8_t>(uint8_t v, bool) { return v; }
template <> __device__ __forceinline__ int16_t cvt<int16_t, uint8_t>(uint8_t v, bool) { return (int16_t)v; }
template <> __device__ __forceinline__ int cvt<int, uint8_t>(uint8_t v, bool) { return (int)v; }

static inline int grid_for(long long n, int block)
{
    long long g = (n + block - 1) / block;
    if (g < 1) g = 1;
    if (g > 152LL * 64) g = 152LL * 64;    // grid-stride beyond 64 blocks per SM
    return (int)g;
}

static inline bool is8(int t) { return t == IFX_N0F8 || t == IFX_U8; }

// =========================================================================
// Padded box: dst[p] = img[map(coords)] (or the fill value) for every p of a
// box of the image index space.  Serves padarray (a1) and the generic
// pipeline's first stage.
// =========================================================================
template <class Tin, class Tout>
__global__ void k_pad_box(const Tin *__restrict__ img, Tout *__restrict__ dst, Box B,
                          int nd, int4 n, int style, Tout fill, bool norm)
{
    const int nn[4] = {n.x, n.y, n.z, n.w};
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < B.count;
         p += (long long)gridDim.x * blockDim.x) {
        long long rem = p, src = 0, sstride = 1;
        bool outside = false;
#pragma unroll
        for (int d = 0; d < IFX_MAXD; ++d) {
            if (d < nd) {
                int c = B.lo[d] + (int)(rem % B.size[d]);
                rem /= B.size[d];
                int m = map_index(c, nn[d], style);
                outside |= (m < 0);
                src += (long long)m * sstride;
                sstride *= nn[d];
            }
        }
        dst[p] = outside ? fill : cvt<Tout, Tin>(img[src], norm);
    }
}

template <class Tin, class Tout>
static cudaError_t pad_box_t(const PadBoxArgs &a, cudaStream_t s)
{
    int4 n = make_int4(a.n[0], a.nd > 1 ? a.n[1] : 1, a.nd > 2 ? a.n[2] : 1, a.nd > 3 ? a.n[3] : 1);
    Tout fill = (Tout)a.fill;
    k_pad_box<Tin, Tout><<<grid_for(a.box.count, 256), 256, 0, s>>>(
        (const Tin *)a.img, (Tout *)a.dst, a.box, a.nd, n, a.style, fill, a.in_type == IFX_N0F8);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_pad_box(const PadBoxArgs &a, cudaStream_t s)
{
    if (a.box.count == 0) return cudaSuccess;
    const int it = a.in_type, ot = a.out_type;
    if (it == IFX_F32 && ot == IFX_F32) return pad_box_t<float, float>(a, s);
    if (it == IFX_F32 && ot == IFX_F64) return pad_box_t<float, double>(a, s);
    if (it == IFX_F64 && ot == IFX_F64) return pad_box_t<double, double>(a, s);
    if (it == IFX_F64 && ot == IFX_F32) return pad_box_t<double, float>(a, s);
    if (is8(it) && ot == IFX_F32) return pad_box_t<uint8_t, float>(a, s);
    if (is8(it) && ot == IFX_F64) return pad_box_t<uint8_t, double>(a, s);
    if (is8(it) && is8(ot)) return pad_box_t<uint8_t, uint8_t>(a, s);
    return cudaErrorInvalidValue;
}

// =========================================================================
// Generic pass over boxes: for each c in obox,
//   dst[c] = sum_t w[t] * src[c + (kfirst+t) e_axis]
// src/dst are laid out on their own boxes.  One thread per output; loads are
// coalesced along axis 0 for every axis choice.
// =========================================================================
template <class Tc, class Tout>
__global__ void k_pass_box(const Tc *__restrict__ src, Box S, Tout *__restrict__ dst, Box D,
                           Box O, int axis, int kfirst, int klen,
                           const __grid_constant__ Weights<Tc, IFX_MAX_TAPS> W, const Tc *__restrict__ gw)
{
    const Tc *w = gw ? gw : W.w;          // factors longer than IFX_MAX_TAPS: weights in device memory
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < O.count;
         p += (long long)gridDim.x * blockDim.x) {
        long long rem = p, so = 0, dof = 0;
#pragma unroll
        for (int d = 0; d < IFX_MAXD; ++d) {
            if (d < O.nd) {
                int c = O.lo[d] + (int)(rem % O.size[d]);
                rem /= O.size[d];
                so += (long long)(c - S.lo[d]) * S.stride[d];
                dof += (long long)(c - D.lo[d]) * D.stride[d];
            }
        }
        const long long st = S.stride[axis];
        const Tc *a = src + so + (long long)kfirst * st;
        Tc acc = 0;
        for (int t = 0; t < klen; ++t) acc = fma(a[t * st], w[t], acc);
        dst[dof] = (Tout)acc;
    }
}

template <class Tc, class Tout>
static cudaError_t pass_box_t(const PassBoxArgs &a, cudaStream_t s)
{
    Weights<Tc, IFX_MAX_TAPS> W;
    memset(&W, 0, sizeof W);
    Tc *gw = nullptr;
    if (a.klen <= IFX_MAX_TAPS) {
        for (int t = 0; t < a.klen; ++t) W.w[t] = (Tc)a.w[t];
    } else {                                  // stream-ordered weight buffer, freed after the pass
        std::vector<Tc> h(a.klen);
        for (int t = 0; t < a.klen; ++t) h[t] = (Tc)a.w[t];
        cudaError_t e = cudaMallocAsync(&gw, sizeof(Tc) * a.klen, s);
        if (e != cudaSuccess) return e;
        if ((e = cudaMemcpyAsync(gw, h.data(), sizeof(Tc) * a.klen, cudaMemcpyHostToDevice, s)) != cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return e;   // h is pageable host memory
    }
    k_pass_box<Tc, Tout><<<grid_for(a.obox.count, 256), 256, 0, s>>>(
        (const Tc *)a.src, a.sbox, (Tout *)a.dst, a.dbox, a.obox, a.axis, a.kfirst, a.klen, W, gw);
    note_launch();
    cudaError_t e = cudaGetLastError();
    if (gw) cudaFreeAsync(gw, s);
    return e;
}

cudaError_t launch_pass_box(const PassBoxArgs &a, cudaStream_t s)
{
    if (a.obox.count == 0) return cudaSuccess;
    if (!a.compute_f64) {
        if (a.out_type == IFX_F32) return pass_box_t<float, float>(a, s);
        if (a.out_type == IFX_F64) return pass_box_t<float, double>(a, s);
    } else {
        if (a.out_type == IFX_F64) return pass_box_t<double, double>(a, s);
        if (a.out_type == IFX_F32) return pass_box_t<double, float>(a, s);
    }
    return cudaErrorInvalidValue;
}

// =========================================================================
// Fused 2-D separable kernel.  One CTA computes a TX x TY output tile:
//  1. gather the (TX+kx-1) x (TY+ky-1) input tile through the border map,
//     converting to the compute type (FP32, or FP64 for Float64 images);
//  2. first pass over the whole tile height (or width), i.e. over the halo
//     the second pass needs -- the reference's cascade ranges;
//  3. second pass, store in the output eltype.
// The tile is TX = 64 or 128 wide for FP32, 32 or 64 for FP64 (a template
// parameter) and TY = 8..128 rows (a multiple of 8); the default is 64 x 64
// for FP32 and 32 x 32 for FP64, the autotuner may pick another.
// =========================================================================
template <class Tc> struct Sep2dTile;
template <> struct Sep2dTile<float> { static constexpr int TX = 64, TY = 64; };
template <> struct Sep2dTile<double> { static constexpr int TX = 32, TY = 32; };
constexpr int kSepNB = 8;

template <class Tc> struct Sep2dW { Tc wx[IFX_MAX_TAPS + 3]; Tc wy[IFX_MAX_TAPS + 3]; };


template <class Tc>
static size_t sep2d_smem(int kx, int ky, int x_first, int TX = Sep2dTile<Tc>::TX, int TY = Sep2dTile<Tc>::TY)
{
    size_t t, i;
    if (x_first) {
        t = (size_t)(TY + ky - 1) * (TX + up4(kx));
        i = (size_t)(TY + up4(ky)) * TX;
    } else {
        t = (size_t)(TY + up4(ky)) * (TX + kx - 1);
        i = (size_t)TY * (TX + up4(kx));
    }
    return (t + i + 2 * (IFX_MAX_TAPS + 3)) * sizeof(Tc);
}

// FP32 taps up to kCorrKmax: the unrolled chain with a fixed register per
// window value; otherwise (FP64, longer factors) the sliding window.
template <class Tc, int NB>
__device__ __forceinline__ void corr_tc(const Tc *p, int step, const Tc *w, int k, Tc *acc)
{
    if constexpr (sizeof(Tc) == 4) {
        if (k <= kCorrKmax) {
            corr_col<NB>(p, step, w, k, acc);
            return;
        }
    }
    corr_run<Tc, NB>(p, step, w, k, acc);
}

template <class Tin, class Tc, class Tout, int TX>
__global__ void __launch_bounds__(256)
k_sep2d(const Tin *__restrict__ img, Tout *__restrict__ out, int nx, int ny,
        int fx, int kx, int fy, int ky, int x_first, int style, Tc fill, bool norm, int TY,
        const __grid_constant__ Sep2dW<Tc> W)
{
    constexpr int NB = kSepNB, lx = TX == 32 ? 5 : (TX == 64 ? 6 : 7), ls = lx - 3;   // log2 TX, log2 segments
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Tc *sm = reinterpret_cast<Tc *>(smem_raw);
    const int kx4 = up4(kx), ky4 = up4(ky);
    Tc *wx = sm;
    Tc *wy = sm + (IFX_MAX_TAPS + 3);
    Tc *T = wy + (IFX_MAX_TAPS + 3);
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int t = tid; t < kx4; t += nth) wx[t] = W.wx[t];
    for (int t = tid; t < ky4; t += nth) wy[t] = W.wy[t];

    const int tx0 = blockIdx.x * TX, ty0 = blockIdx.y * TY;
    // tile geometry
    const int RT = x_first ? (TY + ky - 1) : (TY + ky4);
    const int CT = x_first ? (TX + kx4) : (TX + kx - 1);
    const int RV = TY + ky - 1, CV = TX + kx - 1;   // valid (image-backed) part
    Tc *I = T + (size_t)RT * CT;

    // 1. the input window: rows straight from the image when it lies inside
    //    (a warp per row, four loads in flight per lane), else gathered
    //    through the border map
    if (tx0 + fx >= 0 && tx0 + fx + CV <= nx && ty0 + fy >= 0 && ty0 + fy + RV <= ny) {
        const int lane = tid & 31, nw = nth >> 5;
        for (int r = tid >> 5; r < RT; r += nw) {
            const Tin *rp = img + (long long)(ty0 + fy + r) * nx + tx0 + fx;
            for (int c0 = 0; c0 < CT; c0 += 128) {
                Tc v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = c0 + lane + 32 * q;
                    v[q] = (r < RV && c < CV) ? cvt<Tc, Tin>(rp[c], norm) : Tc(0);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = c0 + lane + 32 * q;
                    if (c < CT) T[(size_t)r * CT + c] = v[q];
                }
            }
        }
    } else {
        gather_tile<8>(T, RT * CT, [&](int idx) -> Tc {
            const int r = idx / CT, c = idx - r * CT;
            if (r >= RV || c >= CV) return Tc(0);
            const int mx = map_index(tx0 + fx + c, nx, style);
            const int my = map_index(ty0 + fy + r, ny, style);
            return (mx < 0 || my < 0) ? fill : cvt<Tc, Tin>(img[(long long)my * nx + mx], norm);
        });
    }
    __syncthreads();

    Tc acc[NB];
    if (x_first) {
        // 2. x pass over RT rows -> I (RT rows valid, pad rows zero), row stride TX
        for (int it = tid; it < ((TY + ky4) << ls); it += nth) {
            const int r = it >> ls, c0 = (it & ((1 << ls) - 1)) * NB;
            if (r < RT) {
                corr_tc<Tc, NB>(T + (size_t)r * CT + c0, 1, wx, kx, acc);
#pragma unroll
                for (int i = 0; i < NB; ++i) I[(size_t)r * TX + c0 + i] = acc[i];
            } else {
#pragma unroll
                for (int i = 0; i < NB; ++i) I[(size_t)r * TX + c0 + i] = 0;
            }
        }
        __syncthreads();
        // 3. y pass down each column, 8 rows per item
        const int rsegs = TY / NB;
        for (int it = tid; it < (rsegs << lx); it += nth) {
            const int rs = it >> lx, c = it & (TX - 1), r0 = rs * NB;
            corr_tc<Tc, NB>(I + (size_t)r0 * TX + c, TX, wy, ky, acc);
            const int x = tx0 + c;
            if (x < nx) {
#pragma unroll
                for (int i = 0; i < NB; ++i) {
                    const int y = ty0 + r0 + i;
                    if (y < ny) out[(long long)y * nx + x] = out_cvt_alt<Tout>(acc[i], i);
                }
            }
        }
    } else {
        // 2. y pass down each of the CT columns -> I (TY rows, row stride TX+kx4)
        const int CI = TX + kx4;
        const int rsegs = TY / NB;
        for (int it = tid; it < CI * rsegs; it += nth) {
            const int rs = it / CI, c = it - rs * CI, r0 = rs * NB;
            if (c < CT) {
                corr_tc<Tc, NB>(T + (size_t)r0 * CT + c, CT, wy, ky, acc);
#pragma unroll
                for (int i = 0; i < NB; ++i) I[(size_t)(r0 + i) * CI + c] = acc[i];
            } else {
#pragma unroll
                for (int i = 0; i < NB; ++i) I[(size_t)(r0 + i) * CI + c] = 0;
            }
        }
        __syncthreads();
        // 3. x pass along rows
        for (int it = tid; it < (TY << ls); it += nth) {
            const int r = it >> ls, c0 = (it & ((1 << ls) - 1)) * NB;
            corr_tc<Tc, NB>(I + (size_t)r * CI + c0, 1, wx, kx, acc);
            const int y = ty0 + r;
            if (y < ny) {
#pragma unroll
                for (int i = 0; i < NB; ++i) {
                    const int x = tx0 + c0 + i;
                    if (x < nx) out[(long long)y * nx + x] = out_cvt_alt<Tout>(acc[i], i);
                }
            }
        }
    }
}

// The gather kernel's tile for `a`: the requested one when the kernel takes
// it (width 32, 64 or 128; height a multiple of 8 up to 128; shared memory
// within 200 KB), else the default.
template <class Tc> static void sep2d_gather_tile(const Sep2dArgs &a, int *tw, int *th)
{
    const int w = a.tile_w, h = a.tile_h;
    const bool wide_ok = sizeof(Tc) == 4 ? (w == 64 || w == 128) : (w == 32 || w == 64);
    if (wide_ok && h >= 8 && h <= 128 && h % 8 == 0 &&
        sep2d_smem<Tc>(a.kx, a.ky, a.x_first, w, h) <= 200 * 1024 && (a.ny + h - 1) / h <= 65535) {
        *tw = w;
        *th = h;
    } else {
        *tw = Sep2dTile<Tc>::TX;
        *th = Sep2dTile<Tc>::TY;
    }
}

template <class Tin, class Tc, class Tout>
static cudaError_t sep2d_t(const Sep2dArgs &a, cudaStream_t s)
{
    int TX, TY;
    sep2d_gather_tile<Tc>(a, &TX, &TY);
    Sep2dW<Tc> W;
    memset(&W, 0, sizeof W);
    for (int t = 0; t < a.kx; ++t) W.wx[t] = (Tc)a.wx[t];
    for (int t = 0; t < a.ky; ++t) W.wy[t] = (Tc)a.wy[t];
    const size_t smem = sep2d_smem<Tc>(a.kx, a.ky, a.x_first, TX, TY);
    constexpr int TW0 = Sep2dTile<Tc>::TX;          // the two widths: the default and twice it
    auto kern = TX == TW0 ? k_sep2d<Tin, Tc, Tout, TW0> : k_sep2d<Tin, Tc, Tout, 2 * TW0>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((a.nx + TX - 1) / TX, (a.ny + TY - 1) / TY);
    kern<<<grid, 256, smem, s>>>((const Tin *)a.img, (Tout *)a.out, a.nx, a.ny, a.fx, a.kx, a.fy,
                                 a.ky, a.x_first, a.style, (Tc)a.fill, a.in_type == IFX_N0F8, TY, W);
    note_launch();
    return cudaGetLastError();
}

// =========================================================================
// Fused 2-D separable kernel, persistent and fed by the Tensor Memory
// Accelerator (FP32 compute; Float32 or 8-bit images whose rows meet the copy
// engine's 16-byte rules; factors of at most kCorrKmax taps).  Each CTA walks
// tiles blockIdx.x, +gridDim.x, ...  Two input buffers alternate: when a
// tile starts, the bulk copy of the CTA's next tile (TX+kx-1 by TY+ky-1
// inputs) is issued into the other buffer, so it lands while both passes of
// this tile run.  Every tile arrives by the copy engine, whose cells outside
// the image are zeros; for tiles whose window leaves the image those cells
// then take the border's values in shared memory (rows, then columns, from
// in-image cells of the tile, or of the image where the window does not hold
// them), so only the halo strips cost index arithmetic.
//
// Shared-memory layout keeps the row passes free of bank conflicts: the tile
// grid is shifted so that every window starts on a 16-byte boundary,
// row pitches are 4 mod 8 floats, and each 8-lane phase of a warp reads 4 rows
// x 2 window starts with 16-byte loads.  The column pass runs on the packed
// FP32x2 pipe, on pairs of columns whose outputs store as one 8- or 16-byte
// word; the row pass stays scalar (packed output pairs need the shifted
// value pairs built by moves, which measured slower).  The passes are
// those of k_sep2d (cascade order, pass ranges); outputs of FP32 results
// widen exactly.
//
// Tiles are TX = 64 or 128 outputs wide (a 128-wide tile runs the 64-wide
// row-pass layout on each half, halves on alternate warps) and TY = 8..128
// rows (a multiple of 8).  The default is 64 wide and as tall as keeps three
// CTAs on an SM; the autotuner may pick another shape.
// =========================================================================
constexpr int kStTX = 64, kStTY = 64, kStNB = 16, kStNBY = 8, kStMaxTX = 128, kStMaxTY = 128;

// Two adjacent outputs of an FP32 result (8-byte store for Float32, 16-byte
// for Float64; the caller checks the alignment).  Float64: one value widens
// by the conversion instruction (the narrow FP64 pipe), the other in integer
// operations (the ALU pipe), so that neither pipe carries all the widening;
// both are exact (measured 3-4 % faster than either alone).
template <class To> __device__ __forceinline__ void store_pair(To *o, float2 v);
template <> __device__ __forceinline__ void store_pair<float>(float *o, float2 v)
{
    *reinterpret_cast<float2 *>(o) = v;
}
template <> __device__ __forceinline__ void store_pair<double>(double *o, float2 v)
{
    *reinterpret_cast<double2 *>(o) = make_double2((double)v.x, f32_to_f64(v.y));
}

__host__ __device__ inline size_t st_round128(size_t b) { return (b + 127) & ~(size_t)127; }
// smallest pitch >= n floats that is 4 mod 8
__host__ __device__ inline int st_pitch(int n) { int p = (n + 3) & ~3; return (p & 7) ? p : p + 4; }

struct SepTmaSmem {
    int boxw;                   // TMA box width (elements) = row pitch of the input buffer
    int st, si;                 // pitches of the 8-bit value tile and of the intermediate
    size_t raw, w, t, i, total;
};

__host__ __device__ inline SepTmaSmem sep_tma_smem(int kx, int ky, int x_first, int elt_bytes, int ty,
                                                   int tx = kStTX)
{
    SepTmaSmem L;
    const int RV = ty + ky - 1, CV = tx + kx - 1;
    // Windows start on 16-byte boundaries.  Float32: 3 floats of slack for
    // the 16-byte loads; 8-bit: codes are converted four at a time.
    L.boxw = elt_bytes == 4 ? st_pitch(CV + 3) : (CV + 3 + 15) / 16 * 16;
    L.st = st_pitch(CV + 3);
    L.si = x_first ? st_pitch(tx) : st_pitch(CV + 3);
    L.raw = st_round128((size_t)L.boxw * RV * elt_bytes);
    L.w = st_round128(2 * (IFX_MAX_TAPS + 3) * sizeof(float2) + 256 * sizeof(float));
    L.t = elt_bytes == 1 ? st_round128((size_t)RV * L.st * sizeof(float)) : 0;
    L.i = st_round128((size_t)(x_first ? RV : ty) * L.si * sizeof(float));
    L.total = 2 * L.raw + L.w + L.t + L.i;       // two input buffers: the next tile loads during this one
    return L;
}

// Poll budget of each tile's first wait for its copy.  A testing setting
// (ifx_debug_force_wait_timeout) sets it to 0, so that the wait gives up at
// once and the kernel takes its timeout path; the waits for copies still in
// flight on that path keep their full budget.
static __device__ unsigned g_first_wait_tma = kFirstWaitTma;

cudaError_t set_first_wait_tma(bool force_timeout)
{
    const unsigned v = force_timeout ? 0u : kFirstWaitTma;
    return cudaMemcpyToSymbol(g_first_wait_tma, &v, sizeof v);
}

template <class Tin, class Tout, int WSH>
__global__ void __launch_bounds__(256)
k_sep2d_tma(const __grid_constant__ CUtensorMap map, const Tin *__restrict__ img, Tout *__restrict__ out,
            int nx, int ny, int inx, int iny, int fx, int kx, int fy, int ky, int x_first, int style, float fill,
            bool norm, int shift, int ty, int tiles_x, int tiles_per_slice, int tiles, int pair_store, int *err,
            const __grid_constant__ Sep2dW<float> W)
{
    constexpr int NB = kStNB, NBY = kStNBY, wsh = WSH;
    constexpr int TX = kStTX << WSH;                        // 64 or 128
    const int TY = ty;                                      // a multiple of NBY, at most kStMaxTY
    constexpr int ALIGN = 16 / (int)sizeof(Tin);          // x granularity of a box start
    extern __shared__ __align__(128) unsigned char st_smem[];
    __shared__ __align__(8) uint64_t bar[2];
    __shared__ int src_row[kStMaxTY + kCorrKmax], src_col[kStMaxTX + kCorrKmax];   // border tiles' source maps
    constexpr int kSrcFill = -1;
    const int RV = TY + ky - 1, CV = TX + kx - 1;
    const SepTmaSmem L = sep_tma_smem(kx, ky, x_first, (int)sizeof(Tin), TY, TX);
    const int boxw = L.boxw;
    const unsigned first_tries = g_first_wait_tma;
    auto raw_buf = [&](int b) { return reinterpret_cast<Tin *>(st_smem + (size_t)b * L.raw); };
    unsigned char *rest = st_smem + 2 * L.raw;
    float *wxs = reinterpret_cast<float *>(rest);     // row-pass weights
    float2 *wy = reinterpret_cast<float2 *>(rest) + (IFX_MAX_TAPS + 3);   // column-pass (w, w) pairs
    float *lut = reinterpret_cast<float *>(wy + (IFX_MAX_TAPS + 3));   // 8-bit code -> value
    float *T = reinterpret_cast<float *>(rest + L.w);
    float *I = reinterpret_cast<float *>(rest + L.w + L.t);
    const int tid = threadIdx.x, nth = blockDim.x;
    const uint32_t box_bytes = (uint32_t)(boxw * RV * (int)sizeof(Tin));
    for (int t = tid; t < kx; t += nth) wxs[t] = W.wx[t];
    for (int t = tid; t < ky; t += nth) wy[t] = make_float2(W.wy[t], W.wy[t]);
    if (sizeof(Tin) == 1)
        for (int c = tid; c < 256; c += nth) lut[c] = to_c<float>((uint8_t)c, norm);
    if (tid == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        mbar_fence_init();
        tma_prefetch_map(&map);
    }
    __syncthreads();

    // tile t covers outputs x in [tx*TX - shift, +TX), y in [yt*TY, +TY) of
    // plane sl (a stack of planes of nx x ny, filtered each on its own)
    auto origin = [&](int t, int &px, int &py, int &sl) {
        sl = t / tiles_per_slice;
        const int u = t - sl * tiles_per_slice, yt = u / tiles_x, tx = u - yt * tiles_x;
        px = tx * TX - shift + fx;
        py = yt * TY + fy;
    };
    auto interior = [&](int t) {
        int px, py, sl;
        origin(t, px, py, sl);
        return px >= 0 && px + CV <= inx && py >= 0 && py + RV <= iny;
    };
    // input planes are inx x iny (the output's nx x ny, or a padded copy of
    // the input whose windows all lie inside)
    const long long plane_in = (long long)inx * iny, plane_out = (long long)nx * ny;
    // all threads call it (uniform); thread 0 issues the copy of tile t into
    // buffer b.  The buffer's previous readers finished before the block
    // barrier that ended the previous tile (after a proxy fence).
    uint32_t parity = 0;              // bit b: phase of bar[b] to wait for
    uint32_t pending = 0;             // bit b: a copy into buffer b is in flight
    auto prefetch = [&](int t, int b) {
        if (t < tiles) {
            if (tid == 0) {
                int px, py, sl;
                origin(t, px, py, sl);
                mbar_expect_tx(&bar[b], box_bytes);
                tma_load_3d(raw_buf(b), &map, px & ~(ALIGN - 1), py, sl, &bar[b]);
            }
            pending |= 1u << b;
        }
    };
    // row-pass item -> (row, window start) over `rows` rows: two warps cover 16
    // rows x 4 starts, each 8-lane phase 4 rows x 2 starts; the last rows go in
    // groups of 8 rows x 4 starts per warp, each phase 8 rows x 1 start (both
    // conflict-free for pitches 4 mod 8).  row_items(rows) items, whole warps,
    // per 64 columns; a 128-wide tile gives its halves to alternate warps.
    auto row_items = [&](int rows) { return (64 * (rows >> 4) + 32 * (((rows & 15) + 7) >> 3)) << wsh; };
    auto row_item = [&](int it, int rows, int &r, int &c0) {
        const int lane = it & 31, half = (it >> 5) & wsh, grp = it >> (5 + wsh), full = 2 * (rows >> 4);
        if (grp < full) {
            r = 16 * (grp >> 1) + 4 * (lane >> 3) + ((lane >> 1) & 3);
            c0 = NB * (2 * (grp & 1) + (lane & 1));
        } else {
            r = 8 * grp + (lane & 7);              // rows 8*full onwards, 8 per warp
            c0 = NB * (lane >> 3);
        }
        c0 += 64 * half;
    };

    int t = blockIdx.x;
    prefetch(t, 0);
    for (int n = 0; t < tiles; t += gridDim.x, ++n) {
        const int b = n & 1;
        Tin *raw = raw_buf(b);
        // the next tile loads into the other buffer while this one computes
        prefetch(t + gridDim.x, b ^ 1);
        int px, py, sl;
        origin(t, px, py, sl);
        const Tin *img_s = img + sl * plane_in;
        Tout *out_s = out + sl * plane_out;
        // a border tile's source maps (see below), while its copy is in flight;
        // the barrier after the wait publishes them
        const bool border = !interior(t);
        if (border) {
            for (int i = tid; i < RV + CV; i += nth) {
                const bool row = i < RV;
                const int w = row ? RV : CV, o = row ? py : px, j = row ? i : i - RV;
                const int m = map_index(o + j, row ? iny : inx, style);
                const int code = m < 0 ? kSrcFill : (m - o >= 0 && m - o < w ? m - o : -2 - m);
                (row ? src_row : src_col)[j] = code;
            }
        }
        // every tile arrives by the copy engine (cells outside the image as zeros)
        const uint32_t ph = (parity >> b) & 1u;
        const bool ok = mbar_wait_sleep(&bar[b], ph, first_tries);
        parity ^= 1u << b;
        pending &= ~(1u << b);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(err, 1);
                // copies may still land: give them time before the block exits
                mbar_wait_sleep(&bar[b], ph);
                if (pending & (1u << (b ^ 1))) mbar_wait_sleep(&bar[b ^ 1], (parity >> (b ^ 1)) & 1u);
            }
            return;
        }
        float *P;
        int SP;
        if (sizeof(Tin) == 4) {
            P = reinterpret_cast<float *>(raw);       // window starts aligned
            SP = boxw;
        } else {
            // codes -> values, four per thread (the box starts at the window)
            const int q4 = (CV + 3) >> 2;
            for (int idx = tid; idx < RV * q4; idx += nth) {
                const int r = idx / q4, c = 4 * (idx - r * q4);
                const uint32_t w4 = *reinterpret_cast<const uint32_t *>(
                    reinterpret_cast<const uint8_t *>(raw) + r * boxw + c);
                *reinterpret_cast<float4 *>(T + r * L.st + c) =
                    make_float4(lut[w4 & 0xFF], lut[(w4 >> 8) & 0xFF], lut[(w4 >> 16) & 0xFF], lut[w4 >> 24]);
            }
            P = T;
            SP = L.st;
        }
        if (border) {
            // border tile: the cells of the window outside the image take the
            // border's values, rows first (in-image columns), then columns (all
            // rows, corners included).  Sources are in-image cells: read from
            // the tile when the window holds them, from the image otherwise.
            // The border map runs once per window row and column, into
            // src_row / src_col: >= 0 the source's row (column) in the tile,
            // kSrcFill the fill value, <= -2 the image row (column) -2 - code.
            const int top = min(max(-py, 0), RV), bot = min(max(RV - (iny - py), 0), RV - top);
            const int lft = min(max(-px, 0), CV), rgt = min(max(CV - (inx - px), 0), CV - lft);
            if (sizeof(Tin) == 1) __syncthreads();        // the converted tile is complete
            const int ncin = CV - lft - rgt;
            for (int rr = tid >> 5; rr < top + bot; rr += nth >> 5) {
                const int r = rr < top ? rr : RV - bot + (rr - top), code = src_row[r];
                for (int c = lft + (tid & 31); c < lft + ncin; c += 32)
                    P[r * SP + c] = code >= 0          ? P[code * SP + c]
                                    : code == kSrcFill ? fill
                                                       : cvt<float, Tin>(img_s[(long long)(-2 - code) * inx + px + c], norm);
            }
            __syncthreads();
            // outside columns: 16 threads per row, rows in steps of nth / 16
            const int nco = lft + rgt;
            for (int r = tid >> 4; r < RV; r += nth >> 4) {
                for (int cc = tid & 15; cc < nco; cc += 16) {
                    const int c = cc < lft ? cc : CV - rgt + (cc - lft), code = src_col[c];
                    float v = fill;
                    if (code >= 0) {
                        v = P[r * SP + code];
                    } else if (code != kSrcFill) {
                        const int rc = src_row[r];
                        const int my = rc >= 0 ? py + rc : -2 - rc;
                        if (rc != kSrcFill) v = cvt<float, Tin>(img_s[(long long)my * inx + (-2 - code)], norm);
                    }
                    P[r * SP + c] = v;
                }
            }
        }
        fence_proxy_async();
        __syncthreads();

        const int tx0 = px - fx, ty0 = py - fy;
        // interior output tiles store without bounds tests, by pointer steps
        const bool full = tx0 >= 0 && tx0 + TX <= nx && ty0 + TY <= ny;
        // a tile at the right or bottom edge skips the items whose outputs all
        // fall outside the image (the last tile column may hold 1-3 columns)
        const int need_x = nx - tx0, need_y = ny - ty0;
        float acc[NB];
        if (x_first) {
            // x pass over the RV rows -> I (pitch si)
            for (int it = tid; it < row_items(RV); it += nth) {
                int r, c0;
                row_item(it, RV, r, c0);
                if (r >= RV || c0 >= need_x || r >= need_y + ky - 1) continue;
                corr_row4<NB>(P + (size_t)r * SP + c0, wxs, kx, acc);
                float4 *d = reinterpret_cast<float4 *>(I + (size_t)r * L.si + c0);
#pragma unroll
                for (int q = 0; q < NB / 4; ++q)
                    d[q] = make_float4(acc[4 * q], acc[4 * q + 1], acc[4 * q + 2], acc[4 * q + 3]);
            }
            fence_proxy_async();
            __syncthreads();
            // y pass down each column pair, NBY rows per item: a warp covers one
            // 64-wide row block (256 contiguous bytes of I per load)
            float2 ya[NBY];
            for (int it = tid; it < (TY / NBY) << (5 + wsh); it += nth) {
                const int rs = it >> (5 + wsh), c = 2 * (it & ((TX >> 1) - 1)), r0 = rs * NBY;
                if (c >= need_x || r0 >= need_y) continue;
                corr_col_x2<NBY>(I + (size_t)r0 * L.si + c, L.si, wy, ky, ya);
                const int x = tx0 + c;
                if (full && pair_store) {
                    Tout *o = out_s + (long long)(ty0 + r0) * nx + x;
#pragma unroll
                    for (int i = 0; i < NBY; ++i, o += nx) store_pair<Tout>(o, ya[i]);
                } else {
#pragma unroll
                    for (int i = 0; i < NBY; ++i) {
                        const int y = ty0 + r0 + i;
                        if (y >= ny) break;
                        Tout *o = out_s + (long long)y * nx + x;
                        if (x >= 0 && x < nx) o[0] = out_cvt<Tout>(ya[i].x);
                        if (x + 1 >= 0 && x + 1 < nx) o[1] = out_cvt<Tout>(ya[i].y);
                    }
                }
            }
        } else {
            // y pass down column pairs of the CV columns -> I (TY rows, pitch si);
            // the pair at CV-1 (CV odd) also fills column CV, inside the pitch
            float2 ya[NBY];
            for (int it = tid; it < ((CV + 1) >> 1) * (TY / NBY); it += nth) {
                const int cp = (CV + 1) >> 1, rs = it / cp, c = 2 * (it - rs * cp), r0 = rs * NBY;
                if (c >= need_x + kx - 1 || r0 >= need_y) continue;
                corr_col_x2<NBY>(P + (size_t)r0 * SP + c, SP, wy, ky, ya);
#pragma unroll
                for (int i = 0; i < NBY; ++i) *reinterpret_cast<float2 *>(I + (size_t)(r0 + i) * L.si + c) = ya[i];
            }
            fence_proxy_async();
            __syncthreads();
            // x pass along the TY rows (items cover whole 16-row groups: TY
            // may be 8 mod 16)
            for (int it = tid; it < row_items(TY); it += nth) {
                int r, c0;
                row_item(it, TY, r, c0);
                if (r >= TY || r >= need_y || c0 >= need_x) continue;
                corr_row4<NB>(I + (size_t)r * L.si + c0, wxs, kx, acc);
                const int y = ty0 + r;
                if (full) {
                    Tout *o = out_s + (long long)y * nx + tx0 + c0;
#pragma unroll
                    for (int i = 0; i < NB; ++i) o[i] = out_cvt_alt<Tout>(acc[i], i);
                } else if (y < ny) {
#pragma unroll
                    for (int i = 0; i < NB; ++i) {
                        const int x = tx0 + c0 + i;
                        if (x >= 0 && x < nx) out_s[(long long)y * nx + x] = out_cvt_alt<Tout>(acc[i], i);
                    }
                }
            }
        }
        // I and T are rewritten by the next tile
        __syncthreads();
    }
}

// Tile height: 64 rows, lowered in steps of 8 (to 32 at most) until three
// CTAs share an SM (the largest factors would otherwise leave two).
static int sep_tma_ty(int kx, int ky, int x_first, int elt_bytes)
{
    int ty = kStTY;
    while (ty > 32 && sep_tma_smem(kx, ky, x_first, elt_bytes, ty).total > 74 * 1024) ty -= kStNBY;
    return ty;
}

// The TMA kernel's tile for `a`: the requested shape when the kernel takes it
// (64 or 128 wide, a multiple of 8 rows up to 128, the box within the copy
// engine's 256 x 256 limit, shared memory within 200 KB), else the default
// (64 wide, sep_tma_ty rows, within 160 KB); false when neither fits.
template <class Tin> static bool sep_tma_tile(const Sep2dArgs &a, int *tx, int *ty, SepTmaSmem *L)
{
    if (a.kx > kCorrKmax || a.ky > kCorrKmax) return false;
    auto fits = [&](int w, int h, size_t cap) {
        *L = sep_tma_smem(a.kx, a.ky, a.x_first, (int)sizeof(Tin), h, w);
        return L->boxw <= 256 && h + a.ky - 1 <= 256 && L->total <= cap;
    };
    const int w = a.tile_w, h = a.tile_h;
    if ((w == kStTX || w == kStMaxTX) && h >= kStNBY && h <= kStMaxTY && h % kStNBY == 0 && fits(w, h, 200 * 1024)) {
        *tx = w;
        *ty = h;
        return true;
    }
    *tx = kStTX;
    *ty = sep_tma_ty(a.kx, a.ky, a.x_first, (int)sizeof(Tin));
    return fits(*tx, *ty, 160 * 1024);
}

template <class Tin, class Tout>
static bool sep2d_tma_t(const Sep2dArgs &a, cudaStream_t s, cudaError_t *e)
{
    int TX, ty;
    SepTmaSmem L;
    if (!sep_tma_tile<Tin>(a, &TX, &ty, &L)) return false;
    const int RV = ty + a.ky - 1;
    const int nsl = a.nsl > 1 ? a.nsl : 1;
    const int inx = a.in_nx > 0 ? a.in_nx : a.nx, iny = a.in_ny > 0 ? a.in_ny : a.ny;
    CUtensorMap map;
    const long long pitch = (long long)inx * (long long)sizeof(Tin);
    if (!tma_encode_3d(&map, a.img, (int)sizeof(Tin), inx, iny, nsl, pitch, pitch * iny, L.boxw, RV))
        return false;
    int dev = 0;
    if ((*e = cudaGetDevice(&dev)) != cudaSuccess) return true;
    int *err = tma_error_word(dev);
    if (!err) {
        *e = cudaErrorMemoryAllocation;
        return true;
    }
    Sep2dW<float> W;
    memset(&W, 0, sizeof W);
    for (int t = 0; t < a.kx; ++t) W.wx[t] = (float)a.wx[t];
    for (int t = 0; t < a.ky; ++t) W.wy[t] = (float)a.wy[t];
    auto kern = TX == kStMaxTX ? k_sep2d_tma<Tin, Tout, 1> : k_sep2d_tma<Tin, Tout, 0>;
    if ((*e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.total)) !=
        cudaSuccess)
        return true;
    // 8 warps; the row pass's last groups take a second round (blocks with a
    // warp for every group, 288-320 threads, measured slower)
    const int nthreads = 256;
    int sms = 0, per_sm = 1;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nthreads, L.total) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    // tiles shift left so that tile windows start on 16-byte boundaries
    constexpr int ALIGN = 16 / (int)sizeof(Tin);
    const int shift = ((a.fx % ALIGN) + ALIGN) % ALIGN;
    const int tiles_x = (a.nx + shift + TX - 1) / TX;
    const long long per_slice = (long long)tiles_x * ((a.ny + ty - 1) / ty);
    const long long tiles = per_slice * nsl;
    if (tiles > (1ll << 30)) return false;
    const long long slots = (long long)sms * per_sm;
    const int grid = (int)(tiles < slots ? tiles : slots);
    // interior output pairs (x even relative to the row start) store as one
    // 8- or 16-byte word when rows and the tile grid keep them aligned
    const int pair_store = (a.nx % 2 == 0) && (shift % 2 == 0) &&
                           ((uintptr_t)a.out % (2 * sizeof(Tout)) == 0);
    kern<<<grid, nthreads, L.total, s>>>(map, (const Tin *)a.img, (Tout *)a.out, a.nx, a.ny, inx, iny, a.fx, a.kx, a.fy,
                                    a.ky, a.x_first, a.style, (float)a.fill, a.in_type == IFX_N0F8, shift, ty,
                                    tiles_x, (int)per_slice, (int)tiles, pair_store, err, W);
    note_launch();
    *e = cudaGetLastError();
    return true;
}

// Whether the TMA tile kernel takes these arguments (the checks of
// sep2d_tma_t, without a launch).
template <class Tin> static bool sep2d_tma_fits(const Sep2dArgs &a)
{
    int TX, ty;
    SepTmaSmem L;
    if (!sep_tma_tile<Tin>(a, &TX, &ty, &L)) return false;
    const int RV = ty + a.ky - 1;
    const int nsl = a.nsl > 1 ? a.nsl : 1;
    const long long tiles = (long long)((a.nx + 16 + TX - 1) / TX) * ((a.ny + ty - 1) / ty) * nsl;
    const int inx = a.in_nx > 0 ? a.in_nx : a.nx, iny = a.in_ny > 0 ? a.in_ny : a.ny;
    CUtensorMap map;
    const long long pitch = (long long)inx * (long long)sizeof(Tin);
    return tiles <= (1ll << 30) &&
           tma_encode_3d(&map, a.img, (int)sizeof(Tin), inx, iny, nsl, pitch, pitch * iny, L.boxw, RV);
}

bool sep2d_tma_applies(const Sep2dArgs &a)
{
    if (a.compute_f64 || a.nx == 0 || a.ny == 0) return false;
    if (a.in_type == IFX_F32 && (a.out_type == IFX_F32 || a.out_type == IFX_F64)) return sep2d_tma_fits<float>(a);
    if (is8(a.in_type) && (a.out_type == IFX_F32 || a.out_type == IFX_F64)) return sep2d_tma_fits<uint8_t>(a);
    return false;
}

// true when the TMA kernel took the call (its launch status in *e); false
// when it does not apply (or variant 2 asks for the gather kernel) and
// k_sep2d runs instead.
static bool launch_sep2d_tma(const Sep2dArgs &a, cudaStream_t s, cudaError_t *e)
{
    if (a.compute_f64 || a.variant == 2) return false;
    const int it = a.in_type, ot = a.out_type;
    if (it == IFX_F32 && ot == IFX_F32) return sep2d_tma_t<float, float>(a, s, e);
    if (it == IFX_F32 && ot == IFX_F64) return sep2d_tma_t<float, double>(a, s, e);
    if (is8(it) && ot == IFX_F32) return sep2d_tma_t<uint8_t, float>(a, s, e);
    if (is8(it) && ot == IFX_F64) return sep2d_tma_t<uint8_t, double>(a, s, e);
    return false;
}

size_t sep2d_smem_bytes(int kx, int ky, int x_first, int f64)
{
    return f64 ? sep2d_smem<double>(kx, ky, x_first) : sep2d_smem<float>(kx, ky, x_first);
}

bool sep2d_tile_shape(const Sep2dArgs &a, int variant, int *tw, int *th)
{
    if (variant == 1) {
        if (!sep2d_tma_applies(a)) return false;
        SepTmaSmem L;
        return is8(a.in_type) ? sep_tma_tile<uint8_t>(a, tw, th, &L) : sep_tma_tile<float>(a, tw, th, &L);
    }
    if (a.nsl > 1) return false;
    if (a.compute_f64) sep2d_gather_tile<double>(a, tw, th);
    else sep2d_gather_tile<float>(a, tw, th);
    return true;
}

cudaError_t launch_sep2d(const Sep2dArgs &a, cudaStream_t s)
{
    if (a.nx == 0 || a.ny == 0) return cudaSuccess;
    cudaError_t e = cudaSuccess;
    if (launch_sep2d_tma(a, s, &e)) return e;
    // stacks of planes and padded inputs: TMA tile kernel only
    if (a.nsl > 1 || (a.in_nx > 0 && a.in_nx != a.nx) || (a.in_ny > 0 && a.in_ny != a.ny)) return cudaErrorInvalidValue;
    const int it = a.in_type, ot = a.out_type;
    if (!a.compute_f64) {
        if (it == IFX_F32 && ot == IFX_F32) return sep2d_t<float, float, float>(a, s);
        if (it == IFX_F32 && ot == IFX_F64) return sep2d_t<float, float, double>(a, s);
        if (is8(it) && ot == IFX_F32) return sep2d_t<uint8_t, float, float>(a, s);
        if (is8(it) && ot == IFX_F64) return sep2d_t<uint8_t, float, double>(a, s);
    } else {
        if (it == IFX_F64 && ot == IFX_F64) return sep2d_t<double, double, double>(a, s);
        if (it == IFX_F64 && ot == IFX_F32) return sep2d_t<double, double, float>(a, s);
    }
    return cudaErrorInvalidValue;
}

// =========================================================================
// Fused 3-D separable kernel (factors along axes 0, 1, 2 in that order), FP32.
// A CTA owns a TX x TY column of the volume and a chunk of ZC output slices.
// It sweeps the input slices the chunk needs (ZC + kz - 1 of them): each slice
// is gathered through the border map with its x/y halo, filtered along x over
// the halo rows and then along y, and the TX x TY result goes into a ring of
// kz slices in shared memory; once kz slices are in the ring, the z pass
// writes one output slice.  The x pass runs over the y halo and the x/y passes
// over the z halo, as pad-then-cascade does (src/imfilter.jl:385-457).
// =========================================================================
// Unrolled tap chain when the factor is short enough, the sliding loop otherwise.
template <int NB>
__device__ __forceinline__ void corr_any(const float *p, int step, const float *w, int k, float *acc)
{
    if (k <= kCorrKmax) corr_col<NB>(p, step, w, k, acc);
    else corr_run<float, NB>(p, step, w, k, acc);
}

constexpr int k3TX = 64, k3TY = 16, k3ZC = 32, k3MaxKz = 17;

struct Sep3dW { float wx[IFX_MAX_TAPS + 3], wy[IFX_MAX_TAPS + 3], wz[k3MaxKz]; };

__host__ __device__ inline size_t sep3d_smem_floats(int kx, int ky, int kz)
{
    return (size_t)(k3TY + ky - 1) * (k3TX + up4(kx)) + (size_t)(k3TY + ky - 1) * k3TX +
           (size_t)kz * k3TY * k3TX + 2 * (IFX_MAX_TAPS + 3) + k3MaxKz;
}

template <class Tin, class Tout>
__global__ void __launch_bounds__(256)
k_sep3d(const Tin *__restrict__ img, Tout *__restrict__ out, int nx, int ny, int nz, int fx, int kx,
        int fy, int ky, int fz, int kz, int style, float fill, bool norm, int zcd,
        const __grid_constant__ Sep3dW W)
{
    constexpr int TX = k3TX, TY = k3TY, NB = 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float *sm = reinterpret_cast<float *>(smem_raw);
    float *wx = sm, *wy = wx + IFX_MAX_TAPS + 3, *wz = wy + IFX_MAX_TAPS + 3;
    const int RT = TY + ky - 1, CT = TX + up4(kx), CV = TX + kx - 1;
    float *T = wz + k3MaxKz;
    float *I = T + RT * CT;
    float *ring = I + RT * TX;
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int t = tid; t < kx; t += nth) wx[t] = W.wx[t];
    for (int t = tid; t < ky; t += nth) wy[t] = W.wy[t];
    for (int t = tid; t < kz; t += nth) wz[t] = W.wz[t];
    const int tx0 = blockIdx.x * TX, ty0 = blockIdx.y * TY;
    const int zchunks = (nz + zcd - 1) / zcd;               // zcd output slices per chunk
    const int zc = blockIdx.z % zchunks, vol = blockIdx.z / zchunks;
    const int z0 = zc * zcd, z1 = min(nz, z0 + zcd);
    const long long vstride = (long long)nx * ny * nz;
    const Tin *src = img + vol * vstride;
    Tout *dst = out + vol * vstride;
    const long long plane = (long long)nx * ny;
    const int s_first = z0 + fz, s_last = z1 - 1 + fz + kz - 1;
    // the x/y window of every slice lies inside the image: no border map in x/y
    const bool inside_xy = tx0 + fx >= 0 && tx0 + fx + CV <= nx && ty0 + fy >= 0 && ty0 + fy + RT <= ny;
    const int lane = tid & 31, warp = tid >> 5, nw = nth >> 5;
    float acc[NB];
    for (int s = s_first; s <= s_last; ++s) {
        const int ms = map_index(s, nz, style);
        __syncthreads();                       // T and I free again
        // gather: warps take rows, lanes take columns (up to 4 column chunks in flight)
        if (inside_xy && ms >= 0) {
            const Tin *sp = src + (long long)ms * plane + (long long)(ty0 + fy) * nx + tx0 + fx;
            for (int r = warp; r < RT; r += nw) {
                const Tin *rp = sp + (long long)r * nx;
                float v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = lane + 32 * q;
                    v[q] = c < CV ? cvt<float, Tin>(rp[c], norm) : 0.0f;
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = lane + 32 * q;
                    if (c < CT) T[r * CT + c] = v[q];
                }
                for (int c = lane + 128; c < CT; c += 32) T[r * CT + c] = c < CV ? cvt<float, Tin>(rp[c], norm) : 0.0f;
            }
        } else {
            for (int r = warp; r < RT; r += nw) {
                const int my = map_index(ty0 + fy + r, ny, style);
                for (int c = lane; c < CT; c += 32) {
                    float v = 0.0f;
                    if (c < CV) {
                        const int mx = map_index(tx0 + fx + c, nx, style);
                        v = (mx < 0 || my < 0 || ms < 0)
                                ? fill
                                : cvt<float, Tin>(src[(long long)ms * plane + (long long)my * nx + mx], norm);
                    }
                    T[r * CT + c] = v;
                }
            }
        }
        __syncthreads();
        const int segs = TX / NB;
        for (int it = tid; it < RT * segs; it += nth) {
            const int r = it / segs, c0 = (it - r * segs) * NB;
            corr_any<NB>(T + r * CT + c0, 1, wx, kx, acc);
#pragma unroll
            for (int i = 0; i < NB; ++i) I[r * TX + c0 + i] = acc[i];
        }
        __syncthreads();
        float *slot = ring + ((s - s_first) % kz) * (TY * TX);
        constexpr int NBY = 4;                 // TX * TY / 4 items: one per thread
        for (int it = tid; it < TX * (TY / NBY); it += nth) {
            const int rs = it / TX, c = it - rs * TX, r0 = rs * NBY;
            corr_any<NBY>(I + r0 * TX + c, TX, wy, ky, acc);
#pragma unroll
            for (int i = 0; i < NBY; ++i) slot[(r0 + i) * TX + c] = acc[i];
        }
        __syncthreads();
        const int z = s - fz - (kz - 1);       // output slice completed by this input slice
        if (z >= z0) {
            const int slot0 = (z + fz - s_first) % kz;     // ring slot of tap 0
            for (int it = tid; it < TX * TY; it += nth) {
                const int r = it / TX, c = it - r * TX;
                const int x = tx0 + c, y = ty0 + r;
                float a = 0.0f;
                int sl = slot0;
                for (int t = 0; t < kz; ++t) {
                    a = fmaf(wz[t], ring[sl * (TY * TX) + it], a);
                    if (++sl == kz) sl = 0;
                }
                if (x < nx && y < ny) dst[(long long)z * plane + (long long)y * nx + x] = out_cvt<Tout>(a);
            }
        }
    }
}

template <class Tin, class Tout>
static cudaError_t sep3d_t(const Sep3dArgs &a, cudaStream_t s, int zcd)
{
    Sep3dW W;
    memset(&W, 0, sizeof W);
    for (int t = 0; t < a.kx; ++t) W.wx[t] = (float)a.wx[t];
    for (int t = 0; t < a.ky; ++t) W.wy[t] = (float)a.wy[t];
    for (int t = 0; t < a.kz; ++t) W.wz[t] = (float)a.wz[t];
    const size_t smem = sep3d_smem_floats(a.kx, a.ky, a.kz) * sizeof(float);
    auto kern = k_sep3d<Tin, Tout>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int zchunks = (a.nz + zcd - 1) / zcd;
    dim3 grid((a.nx + k3TX - 1) / k3TX, (a.ny + k3TY - 1) / k3TY, zchunks * a.nvol);
    kern<<<grid, 256, smem, s>>>((const Tin *)a.img, (Tout *)a.out, a.nx, a.ny, a.nz, a.fx, a.kx, a.fy,
                                 a.ky, a.fz, a.kz, a.style, (float)a.fill, a.in_type == IFX_N0F8, zcd, W);
    note_launch();
    return cudaGetLastError();
}

bool sep3d_supported(int kx, int ky, int kz, int nx, int ny, int nz, int nvol)
{
    const int zchunks = (nz + k3ZC - 1) / k3ZC;
    return kz <= k3MaxKz && kx <= 64 && ky <= 64 && (ny + k3TY - 1) / k3TY <= 65535 &&
           (long long)zchunks * nvol <= 65535 &&
           sep3d_smem_floats(kx, ky, kz) * sizeof(float) <= 200 * 1024;
}

cudaError_t launch_sep3d(const Sep3dArgs &a, cudaStream_t s, int zdepth)
{
    if ((long long)a.nx * a.ny * a.nz == 0 || a.nvol == 0) return cudaSuccess;
    // chunk depths from 4 to 256 slices whose chunk count fits the grid, else the default
    int zcd = k3ZC;
    if (zdepth >= 4 && zdepth <= 256 && (long long)((a.nz + zdepth - 1) / zdepth) * a.nvol <= 65535) zcd = zdepth;
    const int it = a.in_type, ot = a.out_type;
    if (it == IFX_F32 && ot == IFX_F32) return sep3d_t<float, float>(a, s, zcd);
    if (it == IFX_F32 && ot == IFX_F64) return sep3d_t<float, double>(a, s, zcd);
    if (is8(it) && ot == IFX_F32) return sep3d_t<uint8_t, float>(a, s, zcd);
    if (is8(it) && ot == IFX_F64) return sep3d_t<uint8_t, double>(a, s, zcd);
    return cudaErrorInvalidValue;
}

// =========================================================================
// 3-D separable path in two sweeps (the default where it applies): the z
// factor first, from the image into an FP32 volume, then the x and y factors
// of every z plane by the TMA tile kernel over the stack of planes, into the
// output.  Pad-then-cascade filters one fixed padded array, so the order of
// the factors only moves FP32 rounding.  The FP32 volume is the z-filtered
// PADDED array: its planes carry the x/y border (lx columns left, ly rows on
// top, and what the x/y windows reach past the far edges, the width rounded
// up to a multiple of 4), each halo cell the z filter of the column the
// border maps it to (Fill: of fill values).  The x/y sweep then reads every
// window inside a plane -- no border work in its tiles -- with window starts
// on 16-byte boundaries (lx makes fx + lx a multiple of 4).  Traffic: the
// image once, the padded FP32 volume twice, the output once.
//
// k_zpass: a thread computes kZNB consecutive z outputs of two adjacent
// padded x (FP32x2 pairs); threads take the padded plane's pairs in linear
// order (rows back to back: no partial blocks at the row ends); the z window
// goes through the border map (one map per plane, uniform), x and y through
// the border map once per thread.
// =========================================================================
constexpr int kZNB = 8, kZMax = 17;      // outputs per thread, longest z factor

struct ZpassW { float wz[kZMax]; };

// Geometry of the padded FP32 volume of the split path.
struct SplitGeo {
    int lx, ly;                           // left / top border columns and rows
    int nxp, nyp;                         // padded plane
    int fxp, fyp;                         // x / y window offsets in padded coordinates (>= 0)
};

static SplitGeo split_geo(const Sep3dArgs &a)
{
    SplitGeo g;
    g.lx = a.fx < 0 ? -a.fx : 0;
    g.lx += ((-(a.fx + g.lx)) % 4 + 4) % 4;              // fx + lx a multiple of 4
    g.fxp = a.fx + g.lx;
    g.nxp = (a.nx + g.fxp + a.kx - 1 + 3) & ~3;
    g.ly = a.fy < 0 ? -a.fy : 0;
    g.fyp = a.fy + g.ly;
    g.nyp = a.ny + g.fyp + a.ky - 1;
    return g;
}

size_t sep3d_split_tmp_bytes(const Sep3dArgs &a)
{
    const SplitGeo g = split_geo(a);
    return (size_t)g.nxp * g.nyp * a.nz * a.nvol * sizeof(float);
}

template <class Tin, bool PAIR>
__global__ void __launch_bounds__(256)
k_zpass(const Tin *__restrict__ img, float *__restrict__ out, int nx, int ny, int nz, int zblocks, int fz, int kz,
        int style, float fill, bool norm, int lx, int ly, int nxp, int nyp, const __grid_constant__ ZpassW W)
{
    constexpr int NB = kZNB;
    __shared__ float2 w2[kZMax];
    const int tid = threadIdx.x;
    for (int t = tid; t < kz; t += blockDim.x) w2[t] = make_float2(W.wz[t], W.wz[t]);
    __syncthreads();
    const long long lin = 2ll * ((long long)blockIdx.x * blockDim.x + tid);     // nxp is even
    if (lin >= (long long)nxp * nyp) return;
    const int yp = (int)(lin / nxp), xp = (int)(lin - (long long)yp * nxp);
    const int zb = blockIdx.y % zblocks, vol = blockIdx.y / zblocks, z0 = zb * NB;
    // the source columns of padded (xp, yp) and (xp + 1, yp); negative: fill
    const int my = map_index(yp - ly, ny, style);
    const int mx0 = map_index(xp - lx, nx, style), mx1 = map_index(xp + 1 - lx, nx, style);
    const bool in0 = my >= 0 && mx0 >= 0, in1 = my >= 0 && mx1 >= 0;
    // one 8-byte load for both when they are adjacent and the pair is aligned
    const bool pair = PAIR && in0 && in1 && mx1 == mx0 + 1 && (mx0 & 1) == 0;
    const long long plane = (long long)nx * ny;
    const long long base = (long long)vol * plane * nz + (long long)(in0 || in1 ? my : 0) * nx;
    auto at = [&](int j) -> float2 {
        const int ms = map_index(z0 + fz + j, nz, style);
        if (ms < 0) return make_float2(fill, fill);
        const Tin *p = img + base + (long long)ms * plane;
        if constexpr (PAIR && sizeof(Tin) == 4) {
            if (pair) return *reinterpret_cast<const float2 *>(p + mx0);
        } else if constexpr (PAIR) {
            if (pair) {
                const uchar2 u = *reinterpret_cast<const uchar2 *>(p + mx0);
                return make_float2(cvt<float, Tin>(u.x, norm), cvt<float, Tin>(u.y, norm));
            }
        }
        return make_float2(in0 ? cvt<float, Tin>(p[mx0], norm) : fill, in1 ? cvt<float, Tin>(p[mx1], norm) : fill);
    };
    // the whole window is loaded before any arithmetic: every load of the
    // thread is in flight at once (the sweep is bound by their latency)
    float2 v[NB + kZMax - 1], acc[NB];
#pragma unroll
    for (int j = 0; j < NB + kZMax - 1; ++j)
        if (j < NB + kz - 1) v[j] = at(j);
#pragma unroll
    for (int i = 0; i < NB; ++i) acc[i] = make_float2(0.0f, 0.0f);
#pragma unroll
    for (int t = 0; t < kZMax; ++t) {
        if (t >= kz) break;
        const float2 w = w2[t];
#pragma unroll
        for (int i = 0; i < NB; ++i) acc[i] = __ffma2_rn(w, v[i + t], acc[i]);
    }
    const long long pplane = (long long)nxp * nyp;
    float *o = out + (long long)vol * pplane * nz + (long long)z0 * pplane + (long long)yp * nxp + xp;
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        if (z0 + i >= nz) break;
        *reinterpret_cast<float2 *>(o + i * pplane) = acc[i];
    }
}

template <class Tin>
static cudaError_t zpass_t(const Sep3dArgs &a, float *tmp, cudaStream_t s)
{
    ZpassW W;
    memset(&W, 0, sizeof W);
    for (int t = 0; t < a.kz; ++t) W.wz[t] = (float)a.wz[t];
    const SplitGeo g = split_geo(a);
    const int zblocks = (a.nz + kZNB - 1) / kZNB;
    dim3 grid((unsigned)(((long long)g.nxp * g.nyp / 2 + 255) / 256), zblocks * a.nvol);
    const bool pair = a.nx % 2 == 0 && (uintptr_t)a.img % (2 * sizeof(Tin)) == 0;
    if (pair)
        k_zpass<Tin, true><<<grid, 256, 0, s>>>((const Tin *)a.img, tmp, a.nx, a.ny, a.nz, zblocks, a.fz, a.kz,
                                                a.style, (float)a.fill, a.in_type == IFX_N0F8, g.lx, g.ly, g.nxp,
                                                g.nyp, W);
    else
        k_zpass<Tin, false><<<grid, 256, 0, s>>>((const Tin *)a.img, tmp, a.nx, a.ny, a.nz, zblocks, a.fz,
                                                 a.kz, a.style, (float)a.fill, a.in_type == IFX_N0F8, g.lx, g.ly,
                                                 g.nxp, g.nyp, W);
    note_launch();
    return cudaGetLastError();
}

// The x/y sweep of the split path over the padded FP32 volume at `tmp`:
// every window needed lies inside its plane, so the border style of the sweep
// only touches cells that feed no output (Fill(0)).
static Sep2dArgs sep3d_xy_args(const Sep3dArgs &a, const float *tmp)
{
    const SplitGeo g = split_geo(a);
    Sep2dArgs b{};
    b.img = tmp;
    b.in_type = IFX_F32;
    b.out = a.out;
    b.out_type = a.out_type;
    b.nx = a.nx;
    b.ny = a.ny;
    b.in_nx = g.nxp;
    b.in_ny = g.nyp;
    b.fx = g.fxp;
    b.kx = a.kx;
    b.fy = g.fyp;
    b.ky = a.ky;
    b.wx = a.wx;
    b.wy = a.wy;
    b.x_first = 1;
    b.style = IFX_FILL;
    b.fill = 0.0;
    b.compute_f64 = 0;
    b.variant = 1;
    b.nsl = a.nz * a.nvol;
    return b;
}

bool sep3d_split_applies(const Sep3dArgs &a)
{
    if (!(a.in_type == IFX_F32 || is8(a.in_type)) || !(a.out_type == IFX_F32 || a.out_type == IFX_F64)) return false;
    if (a.kz > kZMax || a.kx > kCorrKmax || a.ky > kCorrKmax) return false;
    const SplitGeo g = split_geo(a);
    if ((long long)g.nxp * g.nyp * a.nz * a.nvol >= (1ll << 40)) return false;
    if ((long long)((a.nz + kZNB - 1) / kZNB) * a.nvol > 65535 || (long long)g.nxp * g.nyp / 2 / 256 >= (1ll << 31))
        return false;
    // the FP32 volume of cudaMalloc is 256-byte aligned: probe the x/y sweep with such a base
    Sep2dArgs b = sep3d_xy_args(a, reinterpret_cast<const float *>(uintptr_t(256)));
    return sep2d_tma_applies(b);
}

cudaError_t launch_sep3d_split(const Sep3dArgs &a, float *tmp, cudaStream_t s, int tw, int th)
{
    if ((long long)a.nx * a.ny * a.nz == 0 || a.nvol == 0) return cudaSuccess;
    cudaError_t e = is8(a.in_type) ? zpass_t<uint8_t>(a, tmp, s) : zpass_t<float>(a, tmp, s);
    if (e != cudaSuccess) return e;
    Sep2dArgs b = sep3d_xy_args(a, tmp);
    b.tile_w = tw;
    b.tile_h = th;
    return launch_sep2d(b, s);
}

// =========================================================================
// Fused 3-D gradients (imgradients with a 3-tap (derivative, smoothing) pair
// on all three axes, src/specialty.jl:39-53): gradient d is the cascade of
// the derivative along axis d and the smoothing along the other axes, in axis
// order (x, y, z), pad-then-cascade.  The three cascades share their passes:
// x gives Dx and Sx; y gives SyDx, DySx and SySx; z gives gx = Sz(SyDx),
// gy = Sz(DySx), gz = Dz(SySx).  A CTA owns a TX x TY column and a chunk of
// ZC output slices and marches over the chunk's input slices (ZC + 2): each is
// gathered through the border map with its x/y halo, the x pass runs over the
// halo rows, the y results go into a ring of three slices, and the z pass
// writes one output slice of all three gradients.  Every pass sums its three
// taps in order -1, 0, 1, as the reference's 1-D loop does.
// =========================================================================
constexpr int kG3TX = 32, kG3ZC = 32;
template <class Tc> constexpr int g3ty() { return sizeof(Tc) == 8 ? 8 : 16; }   // static smem < 48 KB

template <class Tc>
__device__ __forceinline__ Tc tap3(const Tc *w, Tc a, Tc b, Tc c)
{
    return fma(w[2], c, fma(w[1], b, w[0] * a));
}

// Sobel-structured pairs (derivative (-h, 0, h), smoothing (q, 2q, q), h and
// q powers of two, as KernelFactors.sobel's [-1,0,1]/2 and [1,2,1]/4): the
// passes sum unscaled, D = c - a (one addition) and S = (a + c) + 2b (an
// addition and an exact-doubling fma), and every gradient takes the common
// power-of-two factor h q^2 once at the end.  Scaling by a power of two is
// exact, so this reorders the reference's sums only (FP64 rounding,
// differences far inside the Float64 tolerance) and needs 14 instead of 26
// FP64 operations per voxel, the bound on this part's narrow FP64 pipe.
template <class Tc> __device__ __forceinline__ Tc sob_d(Tc a, Tc, Tc c) { return c - a; }
template <class Tc> __device__ __forceinline__ Tc sob_s(Tc a, Tc b, Tc c) { return fma(Tc(2), b, a + c); }

// v * 2^e for a power-of-two factor f = 2^e: exponent arithmetic when v and
// the result are normal numbers, the multiplication otherwise.
__device__ __forceinline__ double scale_pow2(double v, int e, double f)
{
    const long long b = __double_as_longlong(v);
    const int ex = (int)((b >> 52) & 0x7FF);
    if (ex > 0 && ex < 2047 && ex + e > 0 && ex + e < 2047) return __longlong_as_double(b + ((long long)e << 52));
    return v * f;
}
__device__ __forceinline__ float scale_pow2(float v, int, float f) { return v * f; }

template <class Tin, class Tc, class Tout, bool SOB>
__global__ void __launch_bounds__(256)
k_grad3d(const Tin *__restrict__ img, Tout *__restrict__ gx, Tout *__restrict__ gy, Tout *__restrict__ gz,
         int nx, int ny, int nz, Tc d0, Tc d1, Tc d2, Tc s0, Tc s1, Tc s2, int style, Tc fill, bool norm,
         int scale_exp, Tc scale)
{
    constexpr int TX = kG3TX, TY = g3ty<Tc>(), RT = TY + 2, CT = TX + 2;
    __shared__ Tc T[RT * CT];                   // input slice tile with x/y halo
    __shared__ Tc Dx[RT * TX], Sx[RT * TX];     // x pass over the halo rows
    __shared__ Tc ring[3][3][TY * TX];          // slot, (SyDx, DySx, SySx), pixel
    const Tc dw[3] = {d0, d1, d2}, sw[3] = {s0, s1, s2};
    const int tid = threadIdx.x, nth = blockDim.x;
    const int tx0 = blockIdx.x * TX, ty0 = blockIdx.y * TY;
    const int z0 = blockIdx.z * kG3ZC, z1 = min(nz, z0 + kG3ZC);
    const long long plane = (long long)nx * ny;
    for (int sl = z0 - 1; sl <= z1; ++sl) {
        const int ms = map_index(sl, nz, style);
        __syncthreads();                        // T, Dx, Sx free again
        gather_tile<4>(T, RT * CT, [&](int idx) -> Tc {
            const int r = idx / CT, c = idx - r * CT;
            const int mx = map_index(tx0 - 1 + c, nx, style);
            const int my = map_index(ty0 - 1 + r, ny, style);
            return (mx < 0 || my < 0 || ms < 0) ? fill
                   : cvt<Tc, Tin>(img[(long long)ms * plane + (long long)my * nx + mx], norm);
        });
        __syncthreads();
        for (int e = tid; e < RT * TX; e += nth) {
            const int r = e / TX, c = e - r * TX;
            const Tc *p = T + r * CT + c;
            if constexpr (SOB) {
                Dx[e] = sob_d(p[0], p[1], p[2]);
                Sx[e] = sob_s(p[0], p[1], p[2]);
            } else {
                Dx[e] = tap3(dw, p[0], p[1], p[2]);
                Sx[e] = tap3(sw, p[0], p[1], p[2]);
            }
        }
        __syncthreads();
        const int slot = (sl - (z0 - 1)) % 3;
        for (int e = tid; e < TY * TX; e += nth) {
            const int r = e / TX, c = e - r * TX;
            const int i0 = r * TX + c, i1 = i0 + TX, i2 = i1 + TX;
            if constexpr (SOB) {
                ring[slot][0][e] = sob_s(Dx[i0], Dx[i1], Dx[i2]);
                ring[slot][1][e] = sob_d(Sx[i0], Sx[i1], Sx[i2]);
                ring[slot][2][e] = sob_s(Sx[i0], Sx[i1], Sx[i2]);
            } else {
                ring[slot][0][e] = tap3(sw, Dx[i0], Dx[i1], Dx[i2]);
                ring[slot][1][e] = tap3(dw, Sx[i0], Sx[i1], Sx[i2]);
                ring[slot][2][e] = tap3(sw, Sx[i0], Sx[i1], Sx[i2]);
            }
        }
        __syncthreads();
        const int z = sl - 1;                   // output slice completed by this input slice
        if (z >= z0) {
            const int a = (z - 1 - (z0 - 1)) % 3, b = (z - (z0 - 1)) % 3, c3 = (z + 1 - (z0 - 1)) % 3;
            for (int e = tid; e < TY * TX; e += nth) {
                const int r = e / TX, c = e - r * TX;
                const int x = tx0 + c, y = ty0 + r;
                if (x >= nx || y >= ny) continue;
                const long long o = (long long)z * plane + (long long)y * nx + x;
                if constexpr (SOB) {
                    gx[o] = out_cvt<Tout>(scale_pow2(sob_s(ring[a][0][e], ring[b][0][e], ring[c3][0][e]),
                                                     scale_exp, scale));
                    gy[o] = out_cvt<Tout>(scale_pow2(sob_s(ring[a][1][e], ring[b][1][e], ring[c3][1][e]),
                                                     scale_exp, scale));
                    gz[o] = out_cvt<Tout>(scale_pow2(sob_d(ring[a][2][e], ring[b][2][e], ring[c3][2][e]),
                                                     scale_exp, scale));
                } else {
                    gx[o] = out_cvt<Tout>(tap3(sw, ring[a][0][e], ring[b][0][e], ring[c3][0][e]));
                    gy[o] = out_cvt<Tout>(tap3(sw, ring[a][1][e], ring[b][1][e], ring[c3][1][e]));
                    gz[o] = out_cvt<Tout>(tap3(dw, ring[a][2][e], ring[b][2][e], ring[c3][2][e]));
                }
            }
        }
    }
}

// Power of two 2^e with |e| < 64 (returns false otherwise).
static bool pow2_exp(double v, int *e)
{
    int ex = 0;
    const double m = std::frexp(std::fabs(v), &ex);
    if (m != 0.5 || ex - 1 < -63 || ex - 1 > 63) return false;
    *e = ex - 1;
    return true;
}

// Whether (d, s) are Sobel-structured, and the exponent of the common factor
// h q^2 (negative h folds its sign into the factor).
static bool sobel_structured(const Grad3dArgs &a, int *scale_exp, double *scale)
{
    int eh = 0, eq = 0;
    if (a.d[1] != 0.0 || a.d[0] != -a.d[2] || !pow2_exp(a.d[2], &eh)) return false;
    if (a.s[0] != a.s[2] || a.s[1] != 2.0 * a.s[0] || a.s[0] <= 0.0 || !pow2_exp(a.s[0], &eq)) return false;
    *scale_exp = eh + 2 * eq;
    *scale = a.d[2] * a.s[0] * a.s[0];
    return a.d[2] > 0.0;       // a negative factor would flip signs in the exponent path
}

template <class Tin, class Tc, class Tout>
static cudaError_t grad3d_t(const Grad3dArgs &a, cudaStream_t s)
{
    dim3 grid((a.nx + kG3TX - 1) / kG3TX, (a.ny + g3ty<Tc>() - 1) / g3ty<Tc>(), (a.nz + kG3ZC - 1) / kG3ZC);
    int se = 0;
    double sc = 1.0;
    if (sizeof(Tc) == 8 && sobel_structured(a, &se, &sc))
        k_grad3d<Tin, Tc, Tout, true><<<grid, 256, 0, s>>>(
            (const Tin *)a.img, (Tout *)a.out[0], (Tout *)a.out[1], (Tout *)a.out[2], a.nx, a.ny, a.nz,
            (Tc)a.d[0], (Tc)a.d[1], (Tc)a.d[2], (Tc)a.s[0], (Tc)a.s[1], (Tc)a.s[2], a.style, (Tc)a.fill,
            a.in_type == IFX_N0F8, se, (Tc)sc);
    else
        k_grad3d<Tin, Tc, Tout, false><<<grid, 256, 0, s>>>(
            (const Tin *)a.img, (Tout *)a.out[0], (Tout *)a.out[1], (Tout *)a.out[2], a.nx, a.ny, a.nz,
            (Tc)a.d[0], (Tc)a.d[1], (Tc)a.d[2], (Tc)a.s[0], (Tc)a.s[1], (Tc)a.s[2], a.style, (Tc)a.fill,
            a.in_type == IFX_N0F8, 0, (Tc)1);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_grad3d(const Grad3dArgs &a, cudaStream_t s)
{
    if ((long long)a.nx * a.ny * a.nz == 0) return cudaSuccess;
    if ((a.ny + 7) / 8 > 65535 || (a.nz + kG3ZC - 1) / kG3ZC > 65535) return cudaErrorInvalidValue;
    const int it = a.in_type, ot = a.out_type;
    if (a.compute_f64) {
        if (it == IFX_F64 && ot == IFX_F64) return grad3d_t<double, double, double>(a, s);
        if (it == IFX_F64 && ot == IFX_F32) return grad3d_t<double, double, float>(a, s);
        return cudaErrorInvalidValue;
    }
    if (it == IFX_F32 && ot == IFX_F64) return grad3d_t<float, float, double>(a, s);
    if (it == IFX_F32 && ot == IFX_F32) return grad3d_t<float, float, float>(a, s);
    if (is8(it) && ot == IFX_F64) return grad3d_t<uint8_t, float, double>(a, s);
    if (is8(it) && ot == IFX_F32) return grad3d_t<uint8_t, float, float>(a, s);
    return cudaErrorInvalidValue;
}

// =========================================================================
// Dense 2-D direct correlation on CUDA cores (src/imfilter.jl:624-669):
// out[x,y] = sum_{i,j} A[x+fx+i, y+fy+j] K[i,j].  A TX x TY tile plus halo is
// loaded row by row where it lies in the image, gathered through the border
// map elsewhere; each thread computes 8 consecutive x outputs, running the
// tap chain along every kernel row (unrolled for rows of up to 12 taps).
// =========================================================================
template <class Tc> struct Dense2dTile;
template <> struct Dense2dTile<float> { static constexpr int TX = 64, TY = 32; };
template <> struct Dense2dTile<double> { static constexpr int TX = 32, TY = 16; };

template <class Tc>
static size_t dense2d_smem(int kw, int kh)
{
    const int TX = Dense2dTile<Tc>::TX, TY = Dense2dTile<Tc>::TY;
    return ((size_t)(TY + kh - 1) * (TX + up4(kw)) + (size_t)kh * up4(kw)) * sizeof(Tc);
}

template <class Tin, class Tc, class Tout>
__global__ void __launch_bounds__(256)
k_dense2d(const Tin *__restrict__ img, Tout *__restrict__ out, int nx, int ny,
          int fx, int kw, int fy, int kh, int style, Tc fill, bool norm,
          const __grid_constant__ Weights<Tc, kMaxDenseTaps> W)
{
    constexpr int TX = Dense2dTile<Tc>::TX, TY = Dense2dTile<Tc>::TY, NB = 8;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    Tc *sm = reinterpret_cast<Tc *>(smem_raw);
    const int kw4 = up4(kw);
    const int CT = TX + kw4, RT = TY + kh - 1, CV = TX + kw - 1;
    Tc *T = sm;
    Tc *Ks = T + (size_t)RT * CT;
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int t = tid; t < kh * kw4; t += nth) {
        const int j = t / kw4, i = t - j * kw4;
        Ks[t] = i < kw ? W.w[j * kw + i] : (Tc)0;
    }
    const int tx0 = blockIdx.x * TX, ty0 = blockIdx.y * TY;
    if (tx0 + fx >= 0 && tx0 + fx + CV <= nx && ty0 + fy >= 0 && ty0 + fy + RT <= ny) {
        // the window lies in the image: rows straight from it (a warp per row,
        // four loads in flight per lane), no border map
        const int lane = tid & 31, nw = nth >> 5;
        for (int r = tid >> 5; r < RT; r += nw) {
            const Tin *rp = img + (long long)(ty0 + fy + r) * nx + tx0 + fx;
            for (int c0 = 0; c0 < CT; c0 += 128) {
                Tc v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = c0 + lane + 32 * q;
                    v[q] = c < CV ? cvt<Tc, Tin>(rp[c], norm) : Tc(0);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int c = c0 + lane + 32 * q;
                    if (c < CT) T[(size_t)r * CT + c] = v[q];
                }
            }
        }
    } else {
        gather_tile<8>(T, RT * CT, [&](int idx) -> Tc {
            const int r = idx / CT, c = idx - r * CT;
            if (c >= CV) return Tc(0);
            const int mx = map_index(tx0 + fx + c, nx, style);
            const int my = map_index(ty0 + fy + r, ny, style);
            return (mx < 0 || my < 0) ? fill : cvt<Tc, Tin>(img[(long long)my * nx + mx], norm);
        });
    }
    __syncthreads();
    const int segs = TX / NB;
    for (int it = tid; it < TY * segs; it += nth) {
        const int r = it / segs, c0 = (it - r * segs) * NB;
        Tc acc[NB], part[NB];
#pragma unroll
        for (int i = 0; i < NB; ++i) acc[i] = 0;
        for (int j = 0; j < kh; ++j) {
            // short rows: the unrolled chain; long rows: the 4-tap sliding form
            // (the unrolled chain measured 1.4-1.9x slower at 15 and 31 taps)
            if (kw <= 12) corr_tc<Tc, NB>(T + (size_t)(r + j) * CT + c0, 1, Ks + (size_t)j * kw4, kw, part);
            else corr_run<Tc, NB>(T + (size_t)(r + j) * CT + c0, 1, Ks + (size_t)j * kw4, kw, part);
#pragma unroll
            for (int i = 0; i < NB; ++i) acc[i] += part[i];
        }
        const int y = ty0 + r;
        if (y < ny) {
#pragma unroll
            for (int i = 0; i < NB; ++i) {
                const int x = tx0 + c0 + i;
                if (x < nx) out[(long long)y * nx + x] = (Tout)acc[i];
            }
        }
    }
}

template <class Tin, class Tc, class Tout>
static cudaError_t dense2d_t(const Dense2dArgs &a, cudaStream_t s)
{
    constexpr int TX = Dense2dTile<Tc>::TX, TY = Dense2dTile<Tc>::TY;
    static thread_local Weights<Tc, kMaxDenseTaps> W;   // large: keep off the host stack
    const int nt = a.kw * a.kh;
    for (int t = 0; t < nt; ++t) W.w[t] = (Tc)a.K[t];
    const size_t smem = dense2d_smem<Tc>(a.kw, a.kh);
    auto kern = k_dense2d<Tin, Tc, Tout>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((a.nx + TX - 1) / TX, (a.ny + TY - 1) / TY);
    kern<<<grid, 256, smem, s>>>((const Tin *)a.img, (Tout *)a.out, a.nx, a.ny, a.fx, a.kw, a.fy,
                                 a.kh, a.style, (Tc)a.fill, a.in_type == IFX_N0F8, W);
    note_launch();
    return cudaGetLastError();
}

size_t dense2d_smem_bytes(int kw, int kh, int f64)
{
    return f64 ? dense2d_smem<double>(kw, kh) : dense2d_smem<float>(kw, kh);
}

cudaError_t launch_dense2d(const Dense2dArgs &a, cudaStream_t s)
{
    if (a.nx == 0 || a.ny == 0) return cudaSuccess;
    const int it = a.in_type, ot = a.out_type;
    if (!a.compute_f64) {
        if (it == IFX_F32 && ot == IFX_F32) return dense2d_t<float, float, float>(a, s);
        if (it == IFX_F32 && ot == IFX_F64) return dense2d_t<float, float, double>(a, s);
        if (is8(it) && ot == IFX_F32) return dense2d_t<uint8_t, float, float>(a, s);
        if (is8(it) && ot == IFX_F64) return dense2d_t<uint8_t, float, double>(a, s);
    } else {
        if (it == IFX_F64 && ot == IFX_F64) return dense2d_t<double, double, double>(a, s);
        if (it == IFX_F64 && ot == IFX_F32) return dense2d_t<double, double, float>(a, s);
    }
    return cudaErrorInvalidValue;
}

// =========================================================================
// Dense N-d over a padded compute-type box (generic fallback for 1-D, 3-D and
// 4-D kernels).  Taps run column-major (axis 0 fastest) as in the reference.
// =========================================================================
template <class Tc, class Tout>
__global__ void k_dense_box(const Tc *__restrict__ src, Box S, Tout *__restrict__ out, Box O,
                            int4 ks, int4 kf, const __grid_constant__ Weights<Tc, kMaxDenseTaps> W)
{
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < O.count;
         p += (long long)gridDim.x * blockDim.x) {
        long long rem = p, so = 0;
#pragma unroll
        for (int d = 0; d < IFX_MAXD; ++d) {
            if (d < O.nd) {
                int c = O.lo[d] + (int)(rem % O.size[d]);
                rem /= O.size[d];
                so += (long long)(c - S.lo[d]) * S.stride[d];
            }
        }
        so += kf.x * S.stride[0] + kf.y * S.stride[1] + kf.z * S.stride[2] + kf.w * S.stride[3];
        Tc acc = 0;
        int t = 0;
        for (int l = 0; l < ks.w; ++l)
            for (int k = 0; k < ks.z; ++k)
                for (int j = 0; j < ks.y; ++j) {
                    const Tc *a = src + so + l * S.stride[3] + k * S.stride[2] + j * S.stride[1];
                    for (int i = 0; i < ks.x; ++i, ++t) acc = fma(a[i], W.w[t], acc);
                }
        out[p] = (Tout)acc;
    }
}

template <class Tc, class Tout>
static cudaError_t dense_box_t(const DenseBoxArgs &a, cudaStream_t s)
{
    static thread_local Weights<Tc, kMaxDenseTaps> W;
    int nt = 1;
    for (int d = 0; d < a.nd; ++d) nt *= a.ksize[d];
    for (int t = 0; t < nt; ++t) W.w[t] = (Tc)a.K[t];
    int4 ks = make_int4(a.ksize[0], a.nd > 1 ? a.ksize[1] : 1, a.nd > 2 ? a.ksize[2] : 1,
                        a.nd > 3 ? a.ksize[3] : 1);
    int4 kf = make_int4(a.kfirst[0], a.nd > 1 ? a.kfirst[1] : 0, a.nd > 2 ? a.kfirst[2] : 0,
                        a.nd > 3 ? a.kfirst[3] : 0);
    k_dense_box<Tc, Tout><<<grid_for(a.obox.count, 256), 256, 0, s>>>(
        (const Tc *)a.src, a.sbox, (Tout *)a.out, a.obox, ks, kf, W);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_dense_box(const DenseBoxArgs &a, cudaStream_t s)
{
    if (a.obox.count == 0) return cudaSuccess;
    if (!a.compute_f64) {
        if (a.out_type == IFX_F32) return dense_box_t<float, float>(a, s);
        if (a.out_type == IFX_F64) return dense_box_t<float, double>(a, s);
    } else {
        if (a.out_type == IFX_F64) return dense_box_t<double, double>(a, s);
        if (a.out_type == IFX_F32) return dense_box_t<double, float>(a, s);
    }
    return cudaErrorInvalidValue;
}

// =========================================================================
// Laplacian stencil (src/specialty.jl:3-17), exact: arithmetic in the output
// eltype TT with the reference's operation order and no fused multiply-add:
//   tmp = TT(-2n * A[I]); for each flagged axis: tmp += A[I+e]; tmp += A[I-e]
// =========================================================================
template <class TT> __device__ __forceinline__ TT lap_mul(TT a, TT b) { return a * b; }
template <> __device__ __forceinline__ float lap_mul<float>(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double lap_mul<double>(double a, double b) { return __dmul_rn(a, b); }
template <class TT> __device__ __forceinline__ TT lap_add(TT a, TT b) { return a + b; }
template <> __device__ __forceinline__ float lap_add<float>(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ double lap_add<double>(double a, double b) { return __dadd_rn(a, b); }

template <class TT> struct LapAcc { using type = TT; };
template <> struct LapAcc<int16_t> { using type = int; };

template <class Tin, class TT>
__global__ void k_laplacian(const Tin *__restrict__ img, TT *__restrict__ out, int nd, int4 n4,
                            int4 f4, int style, typename LapAcc<TT>::type fill, bool norm)
{
    using A = typename LapAcc<TT>::type;
    const int n[4] = {n4.x, n4.y, n4.z, n4.w};
    const int fl[4] = {f4.x, f4.y, f4.z, f4.w};
    long long total = (long long)n[0] * n[1] * n[2] * n[3];
    int cnt = 0;
#pragma unroll
    for (int d = 0; d < 4; ++d) cnt += fl[d];
    for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        int c[4];
        long long rem = p;
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            c[d] = (int)(rem % n[d]);
            rem /= n[d];
        }
        A tmp = lap_mul<A>((A)(-2 * cnt), cvt<A, Tin>(img[p], norm));
#pragma unroll
        for (int d = 0; d < 4; ++d) {
            if (d < nd && fl[d]) {
                long long st = 1;
                for (int e = 0; e < d; ++e) st *= n[e];
                const long long base = p - (long long)c[d] * st;
                int mp = map_index(c[d] + 1, n[d], style);
                int mm = map_index(c[d] - 1, n[d], style);
                A vp = mp < 0 ? fill : cvt<A, Tin>(img[base + (long long)mp * st], norm);
                A vm = mm < 0 ? fill : cvt<A, Tin>(img[base + (long long)mm * st], norm);
                tmp = lap_add<A>(tmp, vp);
                tmp = lap_add<A>(tmp, vm);
            }
        }
        out[p] = (TT)tmp;
    }
}
// 2-D tile version: the halo-1 tile is gathered once (border map applied),
// each output reads its 4 neighbours from shared memory; same operation order.
constexpr int kLapTX = 64, kLapTY = 32;

template <class Tin, class TT>
__global__ void __launch_bounds__(256)
k_lap2d(const Tin *__restrict__ img, TT *__restrict__ out, int nx, int ny, int fxl, int fyl,
        int style, typename LapAcc<TT>::type fill, bool norm)
{
    using A = typename LapAcc<TT>::type;
    constexpr int CT = kLapTX + 2, RT = kLapTY + 2;
    __shared__ A T[RT * CT];
    const int tx0 = blockIdx.x * kLapTX, ty0 = blockIdx.y * kLapTY;
    gather_tile<8>(T, RT * CT, [&](int idx) -> A {
        const int r = idx / CT, c = idx - r * CT;
        const int mx = map_index(tx0 - 1 + c, nx, style);
        const int my = map_index(ty0 - 1 + r, ny, style);
        return (mx < 0 || my < 0) ? fill : cvt<A, Tin>(img[(long long)my * nx + mx], norm);
    });
    __syncthreads();
    const A n2 = (A)(-2 * (fxl + fyl));
    for (int it = threadIdx.x; it < kLapTX * kLapTY; it += blockDim.x) {
        const int r = it / kLapTX, c = it - r * kLapTX;
        const int x = tx0 + c, y = ty0 + r;
        if (x >= nx || y >= ny) continue;
        const A *p = T + (r + 1) * CT + (c + 1);
        A tmp = lap_mul<A>(n2, p[0]);
        if (fxl) {
            tmp = lap_add<A>(tmp, p[1]);
            tmp = lap_add<A>(tmp, p[-1]);
        }
        if (fyl) {
            tmp = lap_add<A>(tmp, p[CT]);
            tmp = lap_add<A>(tmp, p[-CT]);
        }
        out[(long long)y * nx + x] = (TT)tmp;
    }
}

template <class Tin, class TT>
static cudaError_t laplacian_t(const LaplacianArgs &a, cudaStream_t s)
{
    if (a.nd <= 2) {
        const int nx = a.n[0], ny = a.nd > 1 ? a.n[1] : 1;
        dim3 grid((nx + kLapTX - 1) / kLapTX, (ny + kLapTY - 1) / kLapTY);
        k_lap2d<Tin, TT><<<grid, 256, 0, s>>>((const Tin *)a.img, (TT *)a.out, nx, ny, a.flags[0],
                                              a.nd > 1 ? a.flags[1] : 0, a.style,
                                              (typename LapAcc<TT>::type)a.fill, a.in_type == IFX_N0F8);
        note_launch();
        return cudaGetLastError();
    }
    int4 n = make_int4(a.n[0], a.nd > 1 ? a.n[1] : 1, a.nd > 2 ? a.n[2] : 1, a.nd > 3 ? a.n[3] : 1);
    int4 f = make_int4(a.flags[0], a.nd > 1 ? a.flags[1] : 0, a.nd > 2 ? a.flags[2] : 0,
                       a.nd > 3 ? a.flags[3] : 0);
    long long total = (long long)n.x * n.y * n.z * n.w;
    k_laplacian<Tin, TT><<<grid_for(total, 256), 256, 0, s>>>(
        (const Tin *)a.img, (TT *)a.out, a.nd, n, f, a.style,
        (typename LapAcc<TT>::type)a.fill, a.in_type == IFX_N0F8);
    note_launch();
    return cudaGetLastError();
}

cudaError_t launch_laplacian(const LaplacianArgs &a, cudaStream_t s)
{
    const int it = a.in_type, ot = a.out_type;
    if (it == IFX_F32 && ot == IFX_F32) return laplacian_t<float, float>(a, s);
    if (it == IFX_F32 && ot == IFX_F64) return laplacian_t<float, double>(a, s);
    if (it == IFX_F64 && ot == IFX_F64) return laplacian_t<double, double>(a, s);
    if (it == IFX_F64 && ot == IFX_F32) return laplacian_t<double, float>(a, s);
    if (is8(it) && ot == IFX_F32) return laplacian_t<uint8_t, float>(a, s);
    if (is8(it) && ot == IFX_F64) return laplacian_t<uint8_t, double>(a, s);
    if (is8(it) && ot == IFX_I16) return laplacian_t<uint8_t, int16_t>(a, s);
    return cudaErrorInvalidValue;
}

} // namespace ifx
