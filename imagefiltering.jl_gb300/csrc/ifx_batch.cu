// ifx_batch.cu -- the batched engine: many 2-D requests of different sizes,
// ops and borders in ONE persistent launch over a device tile work-queue.
//
// Each request is cut into output tiles (the tile shape depends on the op);
// the tiles of all requests of a batch form one global index space
// [0, total).  Resident CTAs take tile indices from an atomic counter, find
// the owning request by binary search over the requests' first tile indices
// and run the op's tile routine.  The descriptor upload, the counter reset and
// the kernel form a CUDA graph replayed once per batch (two graph slots
// alternate so a batch can be prepared while the previous one runs).
//
// Tile routines reproduce the standalone kernels' arithmetic:
//   factored  imfilter with two 1-D factors, axis 0 then axis 1
//             (src/imfilter.jl:385-457, 671-739), FP32
//   gradients imgradients with a 3-tap (derivative, smoothing) pair, both
//             outputs (src/specialty.jl:39-53), FP32
//   laplacian Kernel.Laplacian((true,true)), exact FP32 in the reference's
//             operation order (src/specialty.jl:3-17)
//   median    mapwindow(median!, img, (w,w)), bit-exact (src/mapwindow.jl:
//             123-131, 270-333); circular windows at the edges wrap inside
//             window-intersect-image, as copy_win! does
// Borders are resolved by the index map (src/border.jl:564-596) while the
// tile is gathered.
#include "ifx_internal.h"
#include "ifx_select.cuh"
#include "ifx_tma.cuh"
#include <algorithm>
#include <cstring>
#include <mutex>
#include <vector>

namespace ifx {

constexpr int kBatchMaxTaps = 36;     // factor taps (<= 33) rounded up to 4

struct BReq {
    int op, in_type, out_type, style;
    int nx, ny, tiles_x, win;
    int tw, th;                       // output tile of this request (see bt_tile_ok)
    long long tile_base, tile_end;    // this request's tiles: [tile_base, tile_end)
    const void *in;
    void *out0;
    void *out1;
    float fill;                       // value domain (N0f8: c/255)
    int fill_code;                    // 8-bit images: the fill code
    int kx, ky, fx, fy;
    float2 wx[kBatchMaxTaps];         // weights as (w, w) pairs: operands of the packed FP32x2 FMA
    float2 wy[kBatchMaxTaps];
};

struct BHdr {
    int nreq;
    int pad;
    long long total_tiles;
};

enum { BOP_FACTORED = 1, BOP_GRADIENTS = 2, BOP_LAPLACIAN = 3, BOP_MEDIAN = 4 };

// Default tile shapes (outputs per tile); each input window (tile + halo)
// fits one staging buffer of 64 rows x 400 bytes
constexpr int kFTX = 64, kFTY = 32;        // factored (halo up to 32 x 32)
constexpr int kGTX = 88, kGTY = 56;        // gradients / laplacian (halo 2 x 2); (88 + 2) * 4 + 15 <= kStagePitch
constexpr int kMUX = 256, kMUY = 56;       // 8-bit median
constexpr int kMFX = 64, kMFY = 56;        // float median
constexpr int kStageRowsMax = kFTY + 32, kStagePitchBytes = 400;

__host__ __device__ inline int bt_tile_w(int op, int in_type)
{
    if (op == BOP_MEDIAN) return (in_type == IFX_F32) ? kMFX : kMUX;
    return op == BOP_FACTORED ? kFTX : kGTX;
}
// Factored tiles are as tall as the staging rows allow for the y factor's
// taps, rounded down to a multiple of 8: 32 rows for 33 taps, 48 for 17, 56
// for 9 or 5, 64 for 1.
__host__ __device__ inline int bt_fact_h(int ky) { return (kFTY + 32 - (ky - 1)) & ~7; }

__host__ __device__ inline int bt_tile_h(int op, int in_type, int ky)
{
    if (op == BOP_FACTORED) return bt_fact_h(ky);
    if (op == BOP_MEDIAN) return (in_type == IFX_F32) ? kMFY : kMUY;
    return kGTY;
}

// Tile shapes the routines take besides the defaults: factored tiles a
// multiple of 64 wide (the routine runs 64-column blocks through its
// intermediate) and a multiple of 8 tall; gradient / Laplacian tiles a
// multiple of 88 wide and 56 tall; median tiles the defaults only.  The
// window (tile + halo, plus up to 15 bytes of row lead) must fit the staging
// buffer.
inline bool bt_tile_ok(int op, int in_type, int kx, int ky, int tw, int th)
{
    const int elt = in_type == IFX_F32 ? 4 : 1;
    if (tw <= 0 || th <= 0) return false;
    switch (op) {
    case BOP_FACTORED:
        return tw % kFTX == 0 && th % 8 == 0 && th + ky - 1 <= kStageRowsMax &&
               (tw + kx - 1) * elt + 15 <= kStagePitchBytes;
    case BOP_GRADIENTS:
    case BOP_LAPLACIAN: return tw % kGTX == 0 && th == kGTY && (tw + 2) * elt + 15 <= kStagePitchBytes;
    default: return tw == bt_tile_w(op, in_type) && th == bt_tile_h(op, in_type, ky);
    }
}

// Thread roles of k_batch: warp 0 is the producer (it looks tiles up and
// issues their copies); the other warps -- the consumers -- gather border
// windows and run the tile routines, synchronising among themselves with
// named barrier 1.
__device__ __forceinline__ int ct_id() { return (int)threadIdx.x - 32; }
__device__ __forceinline__ int ct_n() { return (int)blockDim.x - 32; }
__device__ __forceinline__ void ct_sync() { asm volatile("bar.sync 1, %0;" ::"r"(ct_n()) : "memory"); }
// Named barrier 1 with an AND over the consumers' predicates: every consumer
// gets the same answer (a per-thread result, such as a bounded wait that one
// thread gave up on, would otherwise split the consumers at the next barrier
// inside a tile routine).
__device__ __forceinline__ bool ct_all(bool v)
{
    uint32_t r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.u32 p, %1, 0;\n\tbar.red.and.pred q, 1, %2, p;\n\t"
                 "selp.u32 %0, 1, 0, q;\n\t}\n"
                 : "=r"(r) : "r"((uint32_t)v), "r"(ct_n()) : "memory");
    return r != 0;
}

// Division-free 2-D gather of a tile whose element (r, c) is load(r, c): warps
// take rows, lanes take columns; each thread issues up to 2 rows x 4 column
// chunks of loads before storing them, so 8 global loads are in flight.
template <class T, class F>
__device__ __forceinline__ void gather2d(T *dst, int rows, int cols, int pitch, F load)
{
    const int lane = threadIdx.x & 31, warp = ct_id() >> 5, nw = ct_n() >> 5;
    for (int r0 = warp; r0 < rows; r0 += 2 * nw) {
        T v[2][4];
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int r = r0 + a * nw, c = lane + 32 * b;
                v[a][b] = (r < rows && c < cols) ? load(r, c) : T(0);
            }
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int b = 0; b < 4; ++b) {
                const int r = r0 + a * nw, c = lane + 32 * b;
                if (r < rows && c < cols) dst[r * pitch + c] = v[a][b];
            }
        for (int c = lane + 128; c < cols; c += 32)          // wide tiles: the rest of the row
            for (int a = 0; a < 2; ++a) {
                const int r = r0 + a * nw;
                if (r < rows) dst[r * pitch + c] = load(r, c);
            }
    }
}


// ---------------------------------------------------------------- staging
// A tile's input window (rows x cols elements from image position (ox, oy))
// is staged raw -- Float32 values or 8-bit codes -- in a shared buffer of
// kStagePitch-byte rows: element (r, c) sits at byte r*kStagePitch + lead[r] +
// c*elt.  Interior windows arrive by one bulk copy per row (the row's 16-byte
// aligned superset; lead[r] is the row start's offset in it), issued one tile
// ahead so the copies land while the previous tile computes.  Windows that
// leave the image are gathered through the border map (lead 0).
constexpr int kStageRows = kStageRowsMax;              // factored with 33 taps
constexpr int kStagePitch = kStagePitchBytes;          // >= 15 + (64 + 32) * 4, multiple of 16
constexpr int kStageBytes = kStageRows * kStagePitch;
constexpr int kIPitch = kFTX + 4;                      // factored intermediate (floats)
static_assert((kGTX + 2) * 4 + 15 <= kStagePitch && kGTY + 2 <= kStageRows, "gradient tiles fit a stage");

struct TileGeo {
    int ox, oy, rows, cols, elt;
};

__device__ __forceinline__ TileGeo bt_geo(const BReq &R, int tx0, int ty0)
{
    const int elt = R.in_type == IFX_F32 ? 4 : 1;
    switch (R.op) {
    case BOP_FACTORED: return {tx0 + R.fx, ty0 + R.fy, R.th + R.ky - 1, R.tw + R.kx - 1, elt};
    case BOP_GRADIENTS:
    case BOP_LAPLACIAN: return {tx0 - 1, ty0 - 1, R.th + 2, R.tw + 2, elt};
    default: {
        const int h = R.win / 2;
        if (elt == 4) return {tx0 - h, ty0 - h, kMFY + R.win - 1, kMFX + R.win - 1, 4};
        return {tx0 - h, ty0 - h, kMUY + R.win - 1, kMUX + R.win - 1, 1};
    }
    }
}

// The window lies in the image and every row's aligned superset lies in the
// image's bytes (the base is 16-byte aligned).
__device__ __forceinline__ bool bt_bulk_ok(const BReq &R, const TileGeo &g)
{
    if (((uintptr_t)R.in & 15) || g.ox < 0 || g.oy < 0 || g.ox + g.cols > R.nx || g.oy + g.rows > R.ny)
        return false;
    const long long last = ((long long)(g.oy + g.rows - 1) * R.nx + g.ox) * g.elt;
    const long long end = (last & ~15ll) + (((last & 15) + (long long)g.cols * g.elt + 15) & ~15ll);
    return end <= (long long)R.nx * R.ny * g.elt;
}

__device__ __forceinline__ void bulk_copy(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(smem_addr(dst)), "l"((uint64_t)src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

// Warp 0: one bulk copy per row into `st`, all completing on *bar.
__device__ __forceinline__ void bt_issue_rows(const BReq &R, const TileGeo &g, unsigned char *st,
                                              unsigned char *lead, uint64_t *bar)
{
    const int lane = threadIdx.x & 31;
    uint32_t total = 0;
    for (int r = lane; r < g.rows; r += 32) {
        const long long off = ((long long)(g.oy + r) * R.nx + g.ox) * g.elt;
        const uint32_t ld = (uint32_t)(off & 15);
        total += (ld + (uint32_t)g.cols * g.elt + 15) & ~15u;
        lead[r] = (unsigned char)ld;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) total += __shfl_xor_sync(0xffffffffu, total, o);
    if (lane == 0) mbar_expect_tx(bar, total);
    __syncwarp();
    for (int r = lane; r < g.rows; r += 32) {
        const long long off = ((long long)(g.oy + r) * R.nx + g.ox) * g.elt;
        const uint32_t ld = (uint32_t)(off & 15);
        bulk_copy(st + r * kStagePitch, (const unsigned char *)R.in + (off - ld),
                  (ld + (uint32_t)g.cols * g.elt + 15) & ~15u, bar);
    }
}

// All threads: raw window through the border map (lead 0).
__device__ __forceinline__ void bt_gather_raw(const BReq &R, const TileGeo &g, unsigned char *st,
                                              unsigned char *lead)
{
    for (int r = ct_id(); r < g.rows; r += ct_n()) lead[r] = 0;
    const int nx = R.nx, ny = R.ny, style = R.style;
    if (g.elt == 4) {
        const float *img = (const float *)R.in;
        gather2d<float>(reinterpret_cast<float *>(st), g.rows, g.cols, kStagePitch / 4,
                        [&](int r, int c) -> float {
                            const int mx = map_index(g.ox + c, nx, style), my = map_index(g.oy + r, ny, style);
                            return (mx < 0 || my < 0) ? R.fill : img[(long long)my * nx + mx];
                        });
    } else {
        const uint8_t *img = (const uint8_t *)R.in;
        gather2d<uint8_t>(st, g.rows, g.cols, kStagePitch, [&](int r, int c) -> uint8_t {
            const int mx = map_index(g.ox + c, nx, style), my = map_index(g.oy + r, ny, style);
            return (mx < 0 || my < 0) ? (uint8_t)R.fill_code : img[(long long)my * nx + mx];
        });
    }
}

// Value of staged element (r, c) in the compute domain (the element type is a
// compile-time parameter of the tile routines).  8-bit codes convert in
// arithmetic -- N0f8 c/255 correctly rounded, UInt8 c -- rather than through
// a shared table, whose lookups by 32 lanes at random codes conflict on the
// banks; row pairs convert on the packed FP32x2 pipe.

template <class Tin> struct Rows;
template <> struct Rows<float> {
    const unsigned char *st;
    const unsigned char *lead;
    __device__ __forceinline__ Rows(const unsigned char *s, const unsigned char *l, const float *) : st(s), lead(l) {}
    __device__ __forceinline__ const float *row(int r) const
    {
        return reinterpret_cast<const float *>(st + r * kStagePitch + lead[r]);
    }
    __device__ __forceinline__ float val(const float *p, int c) const { return p[c]; }
};
template <> struct Rows<uint8_t> {
    const unsigned char *st;
    const unsigned char *lead;
    bool norm;                        // N0f8 (c/255) or UInt8 (c)
    __device__ __forceinline__ Rows(const unsigned char *s, const unsigned char *l, bool n)
        : st(s), lead(l), norm(n) {}
    __device__ __forceinline__ const uint8_t *row(int r) const { return st + r * kStagePitch + lead[r]; }
    __device__ __forceinline__ float val(const uint8_t *p, int c) const
    {
        return norm ? n0f8_to_f32(p[c]) : u8_to_f32(p[c]);
    }
    // elements c of two rows, as a pair
    __device__ __forceinline__ float2 val2(const uint8_t *p0, const uint8_t *p1, int c) const
    {
        const float2 f = __fadd2_rn(make_float2(__uint_as_float(0x4B000000u | p0[c]),
                                                __uint_as_float(0x4B000000u | p1[c])),
                                    make_float2(-8388608.0f, -8388608.0f));      // (2^23 + c) - 2^23
        if (!norm) return f;
        const float2 r = make_float2(1.0f / 255.0f, 1.0f / 255.0f);
        const float2 q = __fmul2_rn(f, r);                                        // as n0f8_to_f32, per lane
        return __ffma2_rn(__ffma2_rn(q, make_float2(-255.0f, -255.0f), f), r, q);
    }
};

// Output rows of a tile: element (x, y) of `out`; `full` tiles skip the bounds tests.
template <class Tout> struct OutTile {
    Tout *base;
    int nx, ny, tx0, ty0;
    bool full;
    __device__ __forceinline__ OutTile(const BReq &R, void *out, int x0, int y0, int tw, int th)
        : base((Tout *)out), nx(R.nx), ny(R.ny), tx0(x0), ty0(y0),
          full(x0 + tw <= R.nx && y0 + th <= R.ny) {}
    // NB outputs down column c from row r0
    template <int NB> __device__ __forceinline__ void col(int c, int r0, const float *v) const
    {
        const int x = tx0 + c;
        Tout *p = base + (long long)(ty0 + r0) * nx + x;
        if (full) {
#pragma unroll
            for (int i = 0; i < NB; ++i) p[(long long)i * nx] = out_cvt_alt<Tout>(v[i], i);
        } else if (x < nx) {
#pragma unroll
            for (int i = 0; i < NB; ++i)
                if (ty0 + r0 + i < ny) p[(long long)i * nx] = out_cvt_alt<Tout>(v[i], i);
        }
    }
    // N outputs along row r from column c0
    template <int N> __device__ __forceinline__ void row(int c0, int r, const float *v) const
    {
        const int y = ty0 + r;
        Tout *p = base + (long long)y * nx + tx0 + c0;
        if (full) {
#pragma unroll
            for (int i = 0; i < N; ++i) p[i] = out_cvt_alt<Tout>(v[i], i);
        } else if (y < ny) {
#pragma unroll
            for (int i = 0; i < N; ++i)
                if (tx0 + c0 + i < nx) p[i] = out_cvt_alt<Tout>(v[i], i);
        }
    }
};

// ---------------------------------------------------------------- factored
// acc[i] = sum_{t<k} w[t] src(i+t), i < NB, the window read through `at`
// (weights as (w, w) pairs; the first lane is used).
template <int NB, class F>
__device__ __forceinline__ void corr_fn(F at, const float2 *w, int k, float *acc)
{
    float v[NB + kCorrKmax - 1];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        v[i] = at(i);
        acc[i] = 0.0f;
    }
#pragma unroll
    for (int t = 0; t < kCorrKmax; ++t) {
        if (t >= k) break;
        if (t > 0) v[NB - 1 + t] = at(NB - 1 + t);
        const float wt = w[t].x;
#pragma unroll
        for (int i = 0; i < NB; ++i) acc[i] = fmaf(wt, v[i + t], acc[i]);
    }
}

// The same for two sources at once on the
// packed FP32x2 pipe: at(j) returns element j of both; each lane computes
// the fmaf chain of the scalar form, in the same order (the same bits).
template <int NB, class F>
__device__ __forceinline__ void corr_fn2(F at, const float2 *w, int k, float2 *acc)
{
    float2 v[NB + kCorrKmax - 1];
#pragma unroll
    for (int i = 0; i < NB; ++i) {
        v[i] = at(i);
        acc[i] = make_float2(0.0f, 0.0f);
    }
#pragma unroll
    for (int t = 0; t < kCorrKmax; ++t) {
        if (t >= k) break;
        if (t > 0) v[NB - 1 + t] = at(NB - 1 + t);
        const float2 wt = w[t];
#pragma unroll
        for (int i = 0; i < NB; ++i) acc[i] = __ffma2_rn(wt, v[i + t], acc[i]);
    }
}

// Factored tiles: the x pass over all rows of the window (the y halo) into
// the intermediate I, then the y pass down each column of I.  8-bit images
// run the x pass on row pairs on the packed FP32x2 pipe (codes convert two at
// a time there too); Float32 images run it one row
// per item (row pairs read rows 8 words apart, which share banks in this
// layout, and measured slower).  A window with an odd row count pairs its
// last row with itself (the copy lands in intermediate row `rows`, which is
// never read).  Every output is the fmaf chain of the reference's cascade
// order in both forms.
template <class Tin, class Tout>
__device__ void bt_factored(const BReq &R, int tx0, int ty0, const Rows<Tin> &S, float *I)
{
    constexpr int BW = kFTX, NB = 8;                 // 64-column blocks through the intermediate
    const int kx = R.kx, ky = R.ky, TY = R.th, rows = TY + ky - 1;
    const int tid = ct_id(), nth = ct_n();
    for (int cb = 0; cb < R.tw && tx0 + cb < R.nx; cb += BW) {
        if (cb > 0) ct_sync();                       // the previous block's y pass has read I
        if constexpr (sizeof(Tin) == 1) {
            const int pairs = (rows + 1) >> 1;
            float2 acc[NB];
            for (int it = tid; it < pairs * (BW / NB); it += nth) {
                const int r = 2 * (it >> 3), c0 = (it & 7) * NB;
                const auto *p0 = S.row(r) + cb + c0, *p1 = S.row(r + 1 < rows ? r + 1 : r) + cb + c0;
                corr_fn2<NB>([&](int j) { return S.val2(p0, p1, j); }, R.wx, kx, acc);
                float4 *d0 = reinterpret_cast<float4 *>(I + r * kIPitch + c0);
                float4 *d1 = reinterpret_cast<float4 *>(I + (r + 1) * kIPitch + c0);
#pragma unroll
                for (int q = 0; q < NB / 4; ++q) {
                    d0[q] = make_float4(acc[4 * q].x, acc[4 * q + 1].x, acc[4 * q + 2].x, acc[4 * q + 3].x);
                    d1[q] = make_float4(acc[4 * q].y, acc[4 * q + 1].y, acc[4 * q + 2].y, acc[4 * q + 3].y);
                }
            }
        } else {
            float acc[NB];
            for (int it = tid; it < rows * (BW / NB); it += nth) {
                const int r = it >> 3, c0 = (it & 7) * NB;
                const float *p = S.row(r) + cb + c0;
                corr_fn<NB>([&](int j) { return p[j]; }, R.wx, kx, acc);
#pragma unroll
                for (int i = 0; i < NB; ++i) I[r * kIPitch + c0 + i] = acc[i];
            }
        }
        ct_sync();
        // y pass down each column
        float acc[NB];
        const OutTile<Tout> O(R, R.out0, tx0 + cb, ty0, BW, TY);
        for (int it = tid; it < BW * (TY / NB); it += nth) {
            const int rs = it / BW, c = it - rs * BW, r0 = rs * NB;
            corr_fn<NB>([&](int j) { return I[(r0 + j) * kIPitch + c]; }, R.wy, ky, acc);
            O.template col<NB>(c, r0, acc);
        }
    }
}

// ---------------------------------------------------------------- gradients
// out0 = smooth_y(deriv_x), out1 = deriv_y(smooth_x) over a halo-1 window.
// Gradient and Laplacian tiles are R.tw wide: blocks of kGTX columns, items
// numbered across the blocks.
template <class Tin, class Tout>
__device__ void bt_gradients(const BReq &R, int tx0, int ty0, const Rows<Tin> &S)
{
    constexpr int TX = kGTX, TY = kGTY, NB = 8, PER = TX * (TY / NB);
    const int tid = ct_id(), nth = ct_n();
    const float d0 = R.wx[0].x, d1 = R.wx[1].x, d2 = R.wx[2].x;
    const float s0 = R.wy[0].x, s1 = R.wy[1].x, s2 = R.wy[2].x;
    const OutTile<Tout> O0(R, R.out0, tx0, ty0, R.tw, TY), O1(R, R.out1, tx0, ty0, R.tw, TY);
    for (int it = tid; it < (R.tw / TX) * PER; it += nth) {
        const int cb = it / PER, rem = it - cb * PER;
        const int rs = rem / TX, c = cb * TX + rem - rs * TX, r0 = rs * NB;
        float D[NB + 2], Sm[NB + 2];
#pragma unroll
        for (int j = 0; j < NB + 2; ++j) {
            const auto *p = S.row(r0 + j) + c;
            const float a0 = S.val(p, 0), a1 = S.val(p, 1), a2 = S.val(p, 2);
            D[j] = fmaf(d2, a2, fmaf(d1, a1, d0 * a0));
            Sm[j] = fmaf(s2, a2, fmaf(s1, a1, s0 * a0));
        }
        float g0[NB], g1[NB];
#pragma unroll
        for (int i = 0; i < NB; ++i) {
            g0[i] = fmaf(s2, D[i + 2], fmaf(s1, D[i + 1], s0 * D[i]));
            g1[i] = fmaf(d2, Sm[i + 2], fmaf(d1, Sm[i + 1], d0 * Sm[i]));
        }
        O0.template col<NB>(c, r0, g0);
        O1.template col<NB>(c, r0, g1);
    }
}

// ---------------------------------------------------------------- laplacian
// Kernel.Laplacian((true,true)) in the reference's operation order.
template <class Tin, class Tout>
__device__ void bt_laplacian(const BReq &R, int tx0, int ty0, const Rows<Tin> &S)
{
    constexpr int TX = kGTX, TY = kGTY, NB = 8, PER = TX * (TY / NB);
    const int tid = ct_id(), nth = ct_n();
    const OutTile<Tout> O(R, R.out0, tx0, ty0, R.tw, TY);
    for (int it = tid; it < (R.tw / TX) * PER; it += nth) {
        const int cb = it / PER, rem = it - cb * PER;
        const int rs = rem / TX, c = cb * TX + rem - rs * TX, r0 = rs * NB;
        float col[NB + 2], lft[NB], rgt[NB], res[NB];
#pragma unroll
        for (int j = 0; j < NB + 2; ++j) {
            const auto *p = S.row(r0 + j) + c;
            col[j] = S.val(p, 1);
            if (j >= 1 && j <= NB) {
                lft[j - 1] = S.val(p, 0);
                rgt[j - 1] = S.val(p, 2);
            }
        }
#pragma unroll
        for (int i = 0; i < NB; ++i) {
            float tmp = __fmul_rn(-4.0f, col[i + 1]);
            tmp = __fadd_rn(tmp, rgt[i]);
            tmp = __fadd_rn(tmp, lft[i]);
            tmp = __fadd_rn(tmp, col[i + 2]);
            res[i] = __fadd_rn(tmp, col[i]);
        }
        O.template col<NB>(c, r0, res);
    }
}

// ---------------------------------------------------------------- median
// Window value (i,j) of output (x,y) read from the image itself, with the
// window-relative map of copy_win! (needed for circular at the edges).
__device__ __forceinline__ int bt_win_index(const BReq &R, int x, int y, int i, int j, int h)
{
    const int of = x - h, ol = x + h, ofy = y - h, oly = y + h;
    const int ax = of > 0 ? of : 0, bx = ol < R.nx - 1 ? ol : R.nx - 1;
    const int ay = ofy > 0 ? ofy : 0, by = oly < R.ny - 1 ? oly : R.ny - 1;
    const int mx = map_index_in(of + i, ax, bx - ax + 1, R.style);
    const int my = map_index_in(ofy + j, ay, by - ay + 1, R.style);
    return my * R.nx + mx;
}

// Value of an 8-bit median code in the output eltype's domain: N0f8 -> c/255
// (Float32), UInt8 -> c.
__device__ __forceinline__ float code_value(uint32_t c, bool norm)
{
    return norm ? n0f8_to_f32(c) : (float)c;
}

// Median of the W x W window of output (x, y) read from the image through the
// window-relative map (circular windows at the edges).
template <int W>
__device__ __forceinline__ uint32_t bt_median_u8_at(const BReq &R, int x, int y)
{
    const uint8_t *img = (const uint8_t *)R.in;
    uint32_t v[W * W];
#pragma unroll
    for (int j = 0; j < W; ++j)
#pragma unroll
        for (int i = 0; i < W; ++i) v[j * W + i] = img[bt_win_index(R, x, y, i, j, W / 2)];
    net_sort<W * W, uint32_t>(v);
    return v[(W * W - 1) / 2];
}

// Circular images: outputs of the tile whose windows leave the image wrap
// inside window-intersect-image (copy_win!), not through the whole-image map
// the tile was staged with.  After the tile's blocks are stored, the consumer
// threads recompute those outputs one per thread, from the image (a per-block
// test instead would stall every warp that holds one such block).
template <class F>
__device__ __forceinline__ void bt_circular_edges(const BReq &R, int tx0, int ty0, int tw, int th, int h, F one)
{
    if (R.style != IFX_CIRCULAR) return;
    const EdgeRects E(tx0, ty0, tw, th, R.nx, R.ny, h, h, h, h);
    if (E.count == 0) return;
    ct_sync();                      // the blocks' stores of these outputs come first
    for (int e = ct_id(); e < E.count; e += ct_n()) {
        int x, y;
        E.at(e, x, y);
        one(x, y);
    }
}

template <int W, class Tout>
__device__ void bt_median_u8(const BReq &R, int tx0, int ty0, const Rows<uint8_t> &S)
{
    const int tid = ct_id();
    const int nx = R.nx, ny = R.ny;
    const bool norm = R.in_type == IFX_N0F8;
    const OutTile<Tout> O(R, R.out0, tx0, ty0, kMUX, kMUY);
    if constexpr (W == 5) {
        // Blocks of 8 x BH outputs per thread: two 4 x BH blocks side by side,
        // one in each 16-bit lane, through the generated 5 x 5 block network.
        constexpr int BH = MedBlock<5>::BH, BX = kMUX / 8, NBLK = BX * (kMUY / BH);
        for (int b = tid; b < NBLK; b += ct_n()) {
            const int lx = (b % BX) * 8, ly = (b / BX) * BH;
            if (tx0 + lx >= nx || ty0 + ly >= ny) continue;
            uint32_t in[BH + 4][8], out[BH][4];
#pragma unroll
            for (int r = 0; r < BH + 4; ++r) {
                const int off = S.lead[ly + r] + lx, a = off & ~3;
                const uint32_t *w = reinterpret_cast<const uint32_t *>(S.st + (ly + r) * kStagePitch + a);
                const uint32_t w0 = w[0], w1 = w[1], w2 = w[2], w3 = w[3];
                const uint32_t sel = 0x3210u + 0x1111u * (uint32_t)(off & 3);
                const uint32_t bytes[3] = {__byte_perm(w0, w1, sel), __byte_perm(w1, w2, sel),
                                           __byte_perm(w2, w3, sel)};
#pragma unroll
                for (int c = 0; c < 8; ++c) in[r][c] = lanes_c_c4(bytes, c);
            }
            median_block4<5, CxU16x2>(in, out);
#pragma unroll
            for (int j = 0; j < BH; ++j) {
                float v[8];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    v[q] = code_value(out[j][q] & 0xFFFFu, norm);
                    v[q + 4] = code_value(out[j][q] >> 16, norm);
                }
                O.template row<8>(lx, ly + j, v);
            }
        }
    } else {
        for (int step = tid >> 5; step < kMUY * (kMUX / 128); step += ct_n() >> 5) {
            const int ly = step % kMUY, lx = (step / kMUY) * 128 + (tid & 31) * 4;
            if (tx0 + lx >= nx || ty0 + ly >= ny) continue;
            // 3 x 3: shared column sorts
            uint32_t A[3], B[3];
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                const unsigned char *base = S.st + (ly + j) * kStagePitch;
                const int l = S.lead[ly + j];
                A[j] = load_word(base, l + lx);
                B[j] = load_word(base, l + lx + 4);
            }
            const uint32_t res = median3x3_u8x4(A, B);
            float v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = code_value((res >> (8 * q)) & 0xFFu, norm);
            O.template row<4>(lx, ly, v);
        }
    }
    bt_circular_edges(R, tx0, ty0, kMUX, kMUY, W / 2, [&](int x, int y) {
        ((Tout *)R.out0)[(long long)y * nx + x] = out_cvt<Tout>(code_value(bt_median_u8_at<W>(R, x, y), norm));
    });
}

template <int W, class Tout>
__device__ void bt_median_f32(const BReq &R, int tx0, int ty0, const Rows<float> &S)
{
    using SK = SortKey<float>;
    constexpr int h = W / 2, N = W * W;
    const int nx = R.nx, ny = R.ny;
    // staged values -> order-preserving keys, in place, once per element
    for (int e = ct_id(); e < (kMFY + W - 1) * (kMFX + W - 1); e += ct_n()) {
        const int r = e / (kMFX + W - 1), c = e - r * (kMFX + W - 1);
        float *q = const_cast<float *>(S.row(r)) + c;
        *reinterpret_cast<uint32_t *>(q) = SK::key(*q);
    }
    ct_sync();
    // blocks of 4 x BH outputs per thread through the generated block network
    constexpr int BH = MedBlock<W>::BH, BX = kMFX / 4, NBLK = BX * (kMFY / BH);
    static_assert(kMFY % BH == 0, "whole blocks per tile");
    const OutTile<Tout> O(R, R.out0, tx0, ty0, kMFX, kMFY);
    for (int b = ct_id(); b < NBLK; b += ct_n()) {
        const int lx = (b % BX) * 4, ly = (b / BX) * BH;
        if (tx0 + lx >= nx || ty0 + ly >= ny) continue;
        uint32_t in[BH + W - 1][W + 3], out[BH][4];
#pragma unroll
        for (int r = 0; r < BH + W - 1; ++r) {
            const uint32_t *rowk = reinterpret_cast<const uint32_t *>(S.row(ly + r)) + lx;
#pragma unroll
            for (int c = 0; c < W + 3; ++c) in[r][c] = rowk[c];
        }
        median_block4<W, CxKey32>(in, out);
#pragma unroll
        for (int j = 0; j < BH; ++j) {
            float v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) v[q] = SK::val(out[j][q]);
            O.template row<4>(lx, ly + j, v);
        }
    }
    bt_circular_edges(R, tx0, ty0, kMFX, kMFY, h, [&](int x, int y) {
        const float *img = (const float *)R.in;
        uint32_t k[N];
#pragma unroll
        for (int jj = 0; jj < W; ++jj)
#pragma unroll
            for (int ii = 0; ii < W; ++ii) k[jj * W + ii] = SK::key(img[bt_win_index(R, x, y, ii, jj, h)]);
        net_sort<N, uint32_t>(k);
        ((Tout *)R.out0)[(long long)y * nx + x] = out_cvt<Tout>(SK::val(k[(N - 1) / 2]));
    });
}

// Tile routine for the (element type, output type) pair of the request.
template <class Tin, class Tout>
__device__ __forceinline__ void bt_dispatch(const BReq &R, int tx0, int ty0, const Rows<Tin> &S, float *I)
{
    switch (R.op) {
    case BOP_FACTORED: bt_factored<Tin, Tout>(R, tx0, ty0, S, I); break;
    case BOP_GRADIENTS: bt_gradients<Tin, Tout>(R, tx0, ty0, S); break;
    case BOP_LAPLACIAN: bt_laplacian<Tin, Tout>(R, tx0, ty0, S); break;
    default:
        if constexpr (sizeof(Tin) == 4) {
            if (R.win == 3) bt_median_f32<3, Tout>(R, tx0, ty0, S);
            else bt_median_f32<5, Tout>(R, tx0, ty0, S);
        } else {
            if (R.win == 3) bt_median_u8<3, Tout>(R, tx0, ty0, S);
            else bt_median_u8<5, Tout>(R, tx0, ty0, S);
        }
    }
}

// ---------------------------------------------------------------- the kernel
constexpr int kReqTable = 1024;      // requests whose first tiles are searched in shared memory
// Pipeline shape: kBatchBufs staging buffers per CTA, so the windows of the
// next kBatchBufs-1 tiles are in flight while a tile computes; kBatchThreads
// threads (one producer warp, the rest consumers), kBatchCtas CTAs per SM
// (registers and shared memory allow it).
constexpr int kBatchBufs = 2, kBatchThreads = 288, kBatchCtas = 3;

// Poll budget of each tile's first wait for its copies; a testing setting
// (ifx_debug_force_wait_timeout) sets it to 0 so that the timeout path runs.
// The drain waits of that path keep their full budget.
static __device__ unsigned g_first_wait_batch = kFirstWaitBatch;

cudaError_t set_first_wait_batch(bool force_timeout)
{
    const unsigned v = force_timeout ? 0u : kFirstWaitBatch;
    return cudaMemcpyToSymbol(g_first_wait_batch, &v, sizeof v);
}

__global__ void __launch_bounds__(kBatchThreads, kBatchCtas)
k_batch(const unsigned char *__restrict__ desc, unsigned long long *counter, int *err)
{
    constexpr int NB = kBatchBufs;
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ long long s_tile[NB];
    __shared__ int s_base[kReqTable];
    __shared__ __align__(16) BReq s_req[NB];
    __shared__ __align__(8) uint64_t s_bar[NB];
    __shared__ unsigned char s_lead[NB][kStageRows];
    const BHdr *hdr = reinterpret_cast<const BHdr *>(desc);
    const BReq *reqs = reinterpret_cast<const BReq *>(desc + sizeof(BHdr));
    const long long total = hdr->total_tiles;
    const int nreq = hdr->nreq;
    const int ntab = nreq < kReqTable ? nreq : kReqTable;
    const int tid = threadIdx.x, warp = tid >> 5;
    const unsigned first_tries = g_first_wait_batch;
    float *I = reinterpret_cast<float *>(smem + NB * kStageBytes);
    for (int i = tid; i < ntab; i += blockDim.x) s_base[i] = (int)reqs[i].tile_base;
    __shared__ int s_bulk[NB];           // buffer b's window arrives by bulk copies
    long long ahead = 0;                 // thread 0: the next tile to hand out (already fetched)
    if (tid == 0) {
        for (int i = 0; i < NB; ++i) mbar_init(&s_bar[i], 1);
        mbar_fence_init();
        for (int i = 0; i < NB - 1; ++i) s_tile[i] = (long long)atomicAdd(counter, 1ULL);
        ahead = (long long)atomicAdd(counter, 1ULL);
    }
    __syncthreads();

    // Warp 0 only: looks tile t up, stages its descriptor in s_req[b] and, for an
    // interior window, issues its row copies into buffer b.  Consecutive tiles
    // mostly belong to one request: then the descriptor is copied from the
    // previously prepared buffer `pb` instead of searched for and fetched.  The
    // other warps meet the result after the next block barrier.
    auto prepare = [&](int b, long long t, int pb) {
        const int lane = tid & 31;
        if (t >= total) {
            if (lane == 0) s_bulk[b] = 0;
            return;
        }
        const int *src;
        if (pb >= 0 && t >= s_req[pb].tile_base && t < s_req[pb].tile_end) {
            src = reinterpret_cast<const int *>(&s_req[pb]);
        } else {
            int lo = 0, hi = ntab - 1;
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_base[mid] <= t) lo = mid;
                else hi = mid - 1;
            }
            if (lo == kReqTable - 1 && nreq > kReqTable) {
                hi = nreq - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (reqs[mid].tile_base <= t) lo = mid;
                    else hi = mid - 1;
                }
            }
            src = reinterpret_cast<const int *>(reqs + lo);
        }
        int *dst = reinterpret_cast<int *>(&s_req[b]);
        for (int i = lane; i < (int)(sizeof(BReq) / 4); i += 32) dst[i] = src[i];
        __syncwarp();
        const BReq &R = s_req[b];
        const int local = (int)(t - R.tile_base);
        const int by = local / R.tiles_x, bx = local - by * R.tiles_x;
        const TileGeo g = bt_geo(R, bx * R.tw, by * R.th);
        const bool bulk = bt_bulk_ok(R, g);
        if (bulk) bt_issue_rows(R, g, smem + b * kStageBytes, s_lead[b], &s_bar[b]);
        if (lane == 0) s_bulk[b] = bulk;
    };

    if (warp == 0)
        for (int i = 0; i < NB - 1; ++i) prepare(i, s_tile[i], i - 1);
    __syncthreads();

    uint32_t parity = 0;                 // per buffer: the phase awaited next
    for (int k = 0;; ++k) {
        const int b = k % NB;
        const long long t = s_tile[b];
        if (t >= total) break;
        bool ok = true;
        if (warp == 0) {
            // producer: tile k + NB - 1 into the buffer tile k - 1 used, while the
            // consumers run tile k
            const int nb = (k + NB - 1) % NB;
            long long tn = 0;
            if (tid == 0) {                    // the counter's latency hides behind a tile
                tn = ahead;
                ahead = (long long)atomicAdd(counter, 1ULL);
                s_tile[nb] = tn;               // read by every thread in iteration k + NB - 1
            }
            tn = __shfl_sync(0xffffffffu, tn, 0);
            prepare(nb, tn, (k + NB - 2) % NB);
        } else {
            const BReq &R = s_req[b];
            const int local = (int)(t - R.tile_base);
            const int by = local / R.tiles_x, bx = local - by * R.tiles_x;
            const int tx0 = bx * R.tw, ty0 = by * R.th;
            unsigned char *st = smem + b * kStageBytes;
            if (s_bulk[b]) {
                ok = ct_all(mbar_wait_bounded(&s_bar[b], (parity >> b) & 1u, first_tries));
            } else {
                bt_gather_raw(R, bt_geo(R, tx0, ty0), st, s_lead[b]);
                ct_sync();
            }
            if (ok) {
                const bool o64 = R.out_type == IFX_F64;
                if (R.in_type == IFX_F32) {
                    const Rows<float> S(st, s_lead[b], nullptr);
                    if (o64) bt_dispatch<float, double>(R, tx0, ty0, S, I);
                    else bt_dispatch<float, float>(R, tx0, ty0, S, I);
                } else {
                    const Rows<uint8_t> S(st, s_lead[b], R.in_type == IFX_N0F8);
                    if (o64) bt_dispatch<uint8_t, double>(R, tx0, ty0, S, I);
                    else bt_dispatch<uint8_t, float>(R, tx0, ty0, S, I);
                }
            }
            // buffer b is refilled by the bulk copies of a later tile
            fence_proxy_async();
        }
        if (s_bulk[b]) parity ^= 1u << b;
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(err, 1);
                // copies still in flight: wait (bounded) for them; buffer b's phase
                // was counted as consumed above
                const uint32_t ph = s_bulk[b] ? parity ^ (1u << b) : parity;
                for (int i = 0; i < NB; ++i)
                    if (s_bulk[i]) mbar_wait_bounded(&s_bar[i], (ph >> i) & 1u);
            }
            return;
        }
    }
}

constexpr size_t kBatchSmem = kBatchBufs * (size_t)kStageBytes + (size_t)kStageRows * kIPitch * sizeof(float);

// ---------------------------------------------------------------- host side
struct BatchSlot {
    unsigned char *host = nullptr;      // pinned staging
    unsigned char *dev = nullptr;
    unsigned long long *counter = nullptr;
    size_t cap = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaGraphNode_t copy_node = nullptr;
    cudaEvent_t done = nullptr;
    int grid = 0;
};

// Two descriptor slots used in turn: a launch first waits until the launch two
// before it has finished.  The serving loop relies on that wait to pace its
// admissions (uploads start about two batches ahead of their kernel); eight
// slots, which let it queue every upload at once, made a served stream of 1000
// requests 15 % slower, the early uploads taking link time from the downloads.
struct BatchEngine {
    std::mutex mu;
    int device = -1;
    int grid = 0;
    cudaStream_t capture = nullptr;
    BatchSlot slot[2];
    int next = 0;
    std::vector<BReq> reqs;
};

static cudaError_t slot_build(BatchEngine &E, BatchSlot &S, size_t cap)
{
    cudaError_t e;
    if (S.exec) cudaGraphExecDestroy(S.exec);
    if (S.graph) cudaGraphDestroy(S.graph);
    if (S.host) cudaFreeHost(S.host);
    if (S.dev) cudaFree(S.dev);
    if (S.counter) cudaFree(S.counter);
    if (S.done) cudaEventDestroy(S.done);
    S = BatchSlot();
    if ((e = cudaMallocHost(&S.host, cap)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&S.dev, cap)) != cudaSuccess) return e;
    if ((e = cudaMalloc(&S.counter, sizeof(unsigned long long))) != cudaSuccess) return e;
    if ((e = cudaEventCreateWithFlags(&S.done, cudaEventDisableTiming)) != cudaSuccess) return e;
    S.cap = cap;
    S.grid = E.grid;
    int *err = tma_error_word(E.device);     // allocated outside the capture
    if (!err) return cudaErrorMemoryAllocation;
    // graph: descriptor upload -> counter reset -> persistent kernel
    if ((e = cudaStreamBeginCapture(E.capture, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    cudaMemcpyAsync(S.dev, S.host, cap, cudaMemcpyHostToDevice, E.capture);
    cudaMemsetAsync(S.counter, 0, sizeof(unsigned long long), E.capture);
    k_batch<<<E.grid, kBatchThreads, kBatchSmem, E.capture>>>(S.dev, S.counter, err);
    if ((e = cudaStreamEndCapture(E.capture, &S.graph)) != cudaSuccess) return e;
    size_t n = 0;
    if ((e = cudaGraphGetNodes(S.graph, nullptr, &n)) != cudaSuccess) return e;
    std::vector<cudaGraphNode_t> nodes(n);
    if ((e = cudaGraphGetNodes(S.graph, nodes.data(), &n)) != cudaSuccess) return e;
    for (auto nd : nodes) {
        cudaGraphNodeType ty;
        cudaGraphNodeGetType(nd, &ty);
        if (ty == cudaGraphNodeTypeMemcpy) S.copy_node = nd;
    }
    if (!S.copy_node) return cudaErrorInvalidValue;
    return cudaGraphInstantiate(&S.exec, S.graph, 0);
}

static BatchEngine *g_engines[64];
static std::mutex g_engines_mu;

static cudaError_t engine_for(int device, BatchEngine **out)
{
    if (device < 0 || device >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_engines_mu);
    if (!g_engines[device]) {
        auto *E = new BatchEngine();
        E->device = device;
        cudaError_t e = cudaFuncSetAttribute(k_batch, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)kBatchSmem);
        if (e != cudaSuccess) return e;
        int per_sm = 0, sms = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, kBatchThreads, kBatchSmem);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        E->grid = (per_sm > 0 ? per_sm : 1) * sms;
        if ((e = cudaStreamCreateWithFlags(&E->capture, cudaStreamNonBlocking)) != cudaSuccess) return e;
        g_engines[device] = E;
    }
    *out = g_engines[device];
    return cudaSuccess;
}

int batch_grid(int device)
{
    BatchEngine *E;
    return engine_for(device, &E) == cudaSuccess ? E->grid : 0;
}

// The tile of a request: `force` when given, else the cached (tuned or
// pinned) choice of its key, when the routine takes it; else the default.
static int bt_key_win(const BReq &R) { return R.op == BOP_MEDIAN ? R.win : 0; }

static void bt_choose_tile(BReq &R, const TuneChoice *force)
{
    R.tw = bt_tile_w(R.op, R.in_type);
    R.th = bt_tile_h(R.op, R.in_type, R.ky);
    TuneChoice c;
    if (force) c = *force;
    else if (!autotune_lookup_batch(R.op, R.in_type, R.out_type, R.kx, R.ky, bt_key_win(R), &c)) return;
    if (bt_tile_ok(R.op, R.in_type, R.kx, R.ky, c.tile_w, c.tile_h)) {
        R.tw = c.tile_w;
        R.th = c.tile_h;
    }
}

// The tile shapes the tuner tries for a request's key: factored tiles 64,
// 128 or 256 wide (8-bit images: the staging rows hold them) at the tallest
// height and half of it; gradient / Laplacian tiles 88, 176 or 352 wide;
// median tiles are not tuned (their block networks fix the shape).
static std::vector<TuneChoice> bt_candidates(const BReq &R)
{
    std::vector<TuneChoice> out;
    if (R.op == BOP_FACTORED) {
        const int h0 = bt_fact_h(R.ky), hs[2] = {h0, (h0 / 2) & ~7};
        for (int w = kFTX; w <= 4 * kFTX; w *= 2)
            for (int h : hs)
                if (bt_tile_ok(R.op, R.in_type, R.kx, R.ky, w, h)) out.push_back(TuneChoice{0, 0, w, h, 0, 0.0f});
    } else if (R.op == BOP_GRADIENTS || R.op == BOP_LAPLACIAN) {
        for (int w = kGTX; w <= 4 * kGTX; w *= 2)
            if (bt_tile_ok(R.op, R.in_type, R.kx, R.ky, w, kGTY)) out.push_back(TuneChoice{0, 0, w, kGTY, 0, 0.0f});
    }
    return out;
}

// Fill `out` from a validated request list; returns the total tile count.
// The descriptor lists the requests grouped by tile routine (op, element
// type, window): tiles are handed out in descriptor order, so the CTAs that
// run at the same time mostly run the same code.  Outputs do not depend on
// the order.
long long batch_describe(const BatchItem *items, int n, std::vector<BReq> &out)
{
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    auto key = [&](int i) {
        const BatchItem &it = items[i];
        return (long long)it.op << 40 | (long long)it.in_type << 32 | (long long)it.window << 16 |
               (long long)(it.kx & 0xFFFF);
    };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return key(a) < key(b); });
    out.resize(n);
    long long base = 0;
    for (int i = 0; i < n; ++i) {
        const BatchItem &it = items[order[i]];
        BReq &R = out[i];
        memset(&R, 0, sizeof R);
        R.op = it.op;
        R.in_type = it.in_type;
        R.out_type = it.out_type;
        R.style = it.style;
        R.nx = it.nx;
        R.ny = it.ny;
        R.win = it.window;
        R.in = it.in;
        R.out0 = it.out0;
        R.out1 = it.out1;
        R.fill = (float)it.fill;
        R.fill_code = it.fill_code;
        R.kx = it.kx;
        R.ky = it.ky;
        R.fx = it.fx;
        R.fy = it.fy;
        for (int t = 0; t < it.kx && t < kBatchMaxTaps; ++t) R.wx[t] = make_float2((float)it.wx[t], (float)it.wx[t]);
        for (int t = 0; t < it.ky && t < kBatchMaxTaps; ++t) R.wy[t] = make_float2((float)it.wy[t], (float)it.wy[t]);
        bt_choose_tile(R, nullptr);
        R.tiles_x = (R.nx + R.tw - 1) / R.tw;
        const long long tiles = (long long)R.tiles_x * ((R.ny + R.th - 1) / R.th);
        R.tile_base = base;
        base += tiles;
        R.tile_end = base;
    }
    return base;
}

// Re-cuts the requests into tiles after their tile shapes changed.
static long long bt_assign(std::vector<BReq> &reqs)
{
    long long base = 0;
    for (BReq &R : reqs) {
        R.tiles_x = (R.nx + R.tw - 1) / R.tw;
        R.tile_base = base;
        base += (long long)R.tiles_x * ((R.ny + R.th - 1) / R.th);
        R.tile_end = base;
    }
    return base;
}

cudaError_t launch_batch(int device, const BatchItem *items, int n, cudaStream_t s, long long *tiles_out)
{
    BatchEngine *E;
    cudaError_t e = engine_for(device, &E);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(E->mu);
    const long long total = batch_describe(items, n, E->reqs);
    if (tiles_out) *tiles_out = total;
    if (total == 0) return cudaSuccess;
    const size_t bytes = sizeof(BHdr) + (size_t)n * sizeof(BReq);
    BatchSlot &S = E->slot[E->next];
    E->next ^= 1;
    if (S.cap < bytes || !S.exec) {
        if (S.done) cudaEventSynchronize(S.done);
        size_t cap = 1 << 20;
        while (cap < bytes) cap <<= 1;
        if ((e = slot_build(*E, S, cap)) != cudaSuccess) return e;
    }
    if ((e = cudaEventSynchronize(S.done)) != cudaSuccess) return e;   // staging free again
    BHdr h{n, 0, total};
    memcpy(S.host, &h, sizeof h);
    memcpy(S.host + sizeof(BHdr), E->reqs.data(), (size_t)n * sizeof(BReq));
    if ((e = cudaGraphExecMemcpyNodeSetParams1D(S.exec, S.copy_node, S.dev, S.host, bytes,
                                                cudaMemcpyHostToDevice)) != cudaSuccess)
        return e;
    if ((e = cudaGraphLaunch(S.exec, s)) != cudaSuccess) return e;
    note_launch();
    return cudaEventRecord(S.done, s);
}

// ---------------------------------------------------------------- plans
// A validated batch whose descriptors stay in device memory: each launch is one
// graph replay (counter reset + persistent kernel), with no host-side work.
struct BatchPlanImpl {
    int device = 0;
    unsigned char *dev = nullptr;
    unsigned long long *counter = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    long long tiles = 0;
    int n = 0;
    std::vector<BReq> reqs;           // the descriptors (host copy), for re-cutting after tuning
    bool tuned = false;               // the tuner ran (or had nothing to tune) for this plan
};

// Uploads header + descriptors of `reqs` to `dev` (synchronous).
static cudaError_t bt_upload(unsigned char *dev, const std::vector<BReq> &reqs, long long tiles)
{
    const size_t bytes = sizeof(BHdr) + reqs.size() * sizeof(BReq);
    std::vector<unsigned char> host(bytes);
    BHdr h{(int)reqs.size(), 0, tiles};
    memcpy(host.data(), &h, sizeof h);
    if (!reqs.empty()) memcpy(host.data() + sizeof(BHdr), reqs.data(), reqs.size() * sizeof(BReq));
    return cudaMemcpy(dev, host.data(), bytes, cudaMemcpyHostToDevice);
}

// A tile replaces the default only when it is at least this much faster.
constexpr float kBatchTuneMargin = 0.97f;

// The tuner on a plan's first launch (stream s): every key of the plan that
// has several candidate tiles and no cached choice is timed on the plan's
// own requests of that key -- a batch of just those, one warm-up and three
// timed launches per candidate, L2 overwritten before each -- and the
// fastest tile is cached (the default unless another is clearly faster).  Then the
// plan is re-cut with the cached tiles.  The timed batches write the
// requests' outputs, which the plan's launch then rewrites.
static cudaError_t plan_tune(BatchPlanImpl *P, cudaStream_t s)
{
    BatchEngine *E;
    cudaError_t e = engine_for(P->device, &E);
    if (e != cudaSuccess) return e;
    int *err = tma_error_word(P->device);
    if (!err) return cudaErrorMemoryAllocation;
    // keys in plan order, each with the indices of its requests
    std::vector<std::vector<int>> groups;
    for (int i = 0; i < P->n; ++i) {
        const BReq &R = P->reqs[i];
        bool found = false;
        for (auto &g : groups) {
            const BReq &Q = P->reqs[g[0]];
            if (Q.op == R.op && Q.in_type == R.in_type && Q.out_type == R.out_type && Q.kx == R.kx &&
                Q.ky == R.ky && bt_key_win(Q) == bt_key_win(R)) {
                g.push_back(i);
                found = true;
                break;
            }
        }
        if (!found) groups.push_back({i});
    }
    unsigned char *dev = nullptr;
    unsigned long long *counter = nullptr;
    TuneTimer tt;
    const size_t cap = sizeof(BHdr) + (size_t)P->n * sizeof(BReq);
    if ((e = cudaMalloc(&dev, cap)) == cudaSuccess && (e = cudaMalloc(&counter, sizeof *counter)) == cudaSuccess &&
        (e = tt.init()) == cudaSuccess && (e = cudaStreamSynchronize(s)) == cudaSuccess) {
        for (const auto &g : groups) {
            const BReq &R0 = P->reqs[g[0]];
            TuneChoice have;
            if (autotune_lookup_batch(R0.op, R0.in_type, R0.out_type, R0.kx, R0.ky, bt_key_win(R0), &have))
                continue;
            const std::vector<TuneChoice> cands = bt_candidates(R0);
            if (cands.size() < 2) continue;
            // the default tile first; another replaces it only when clearly faster
            BReq D = R0;
            bt_choose_tile(D, nullptr);
            TuneChoice def{0, 0, D.tw, D.th, 0, 0.0f}, best{0, 0, 0, 0, 0, 1e30f};
            for (int ci = -1; ci < (int)cands.size() && e == cudaSuccess; ++ci) {
                const TuneChoice c = ci < 0 ? def : cands[ci];
                if (ci >= 0 && c.tile_w == def.tile_w && c.tile_h == def.tile_h) continue;
                std::vector<BReq> sub;
                for (int i : g) {
                    sub.push_back(P->reqs[i]);
                    bt_choose_tile(sub.back(), &c);
                }
                const long long tiles = bt_assign(sub);
                if ((e = bt_upload(dev, sub, tiles)) != cudaSuccess) break;
                float ms = 0.0f;
                e = tt.time(
                    [&]() {
                        cudaMemsetAsync(counter, 0, sizeof *counter, s);
                        k_batch<<<E->grid, kBatchThreads, kBatchSmem, s>>>(dev, counter, err);
                        note_launch();
                        return cudaGetLastError();
                    },
                    s, &ms);
                if (e != cudaSuccess) break;
                if (ci < 0) def.ms = ms;
                if (ms < best.ms) {
                    best = c;
                    best.ms = ms;
                }
            }
            if (e != cudaSuccess) break;
            if (best.ms > kBatchTuneMargin * def.ms) best = def;
            autotune_store_batch(R0.op, R0.in_type, R0.out_type, R0.kx, R0.ky, bt_key_win(R0), best, true);
        }
    }
    if (dev) cudaFree(dev);
    if (counter) cudaFree(counter);
    if (e != cudaSuccess) return e;
    for (BReq &R : P->reqs) bt_choose_tile(R, nullptr);
    P->tiles = bt_assign(P->reqs);
    return bt_upload(P->dev, P->reqs, P->tiles);
}

cudaError_t plan_create(int device, const BatchItem *items, int n, void **out)
{
    BatchEngine *E;
    cudaError_t e = engine_for(device, &E);
    if (e != cudaSuccess) return e;
    auto *P = new BatchPlanImpl();
    P->device = device;
    P->n = n;
    P->tiles = batch_describe(items, n, P->reqs);
    const size_t bytes = sizeof(BHdr) + (size_t)n * sizeof(BReq);
    if ((e = cudaMalloc(&P->dev, bytes)) != cudaSuccess ||
        (e = cudaMalloc(&P->counter, sizeof(unsigned long long))) != cudaSuccess ||
        (e = bt_upload(P->dev, P->reqs, P->tiles)) != cudaSuccess) {
        plan_destroy(P);
        return e;
    }
    int *err = tma_error_word(E->device);    // allocated outside the capture
    if (!err) {
        plan_destroy(P);
        return cudaErrorMemoryAllocation;
    }
    std::lock_guard<std::mutex> lk(E->mu);
    if ((e = cudaStreamBeginCapture(E->capture, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        plan_destroy(P);
        return e;
    }
    cudaMemsetAsync(P->counter, 0, sizeof(unsigned long long), E->capture);
    k_batch<<<E->grid, kBatchThreads, kBatchSmem, E->capture>>>(P->dev, P->counter, err);
    if ((e = cudaStreamEndCapture(E->capture, &P->graph)) != cudaSuccess ||
        (e = cudaGraphInstantiate(&P->exec, P->graph, 0)) != cudaSuccess) {
        plan_destroy(P);
        return e;
    }
    *out = P;
    return cudaSuccess;
}

cudaError_t plan_launch(void *plan, cudaStream_t s, long long *tiles)
{
    auto *P = (BatchPlanImpl *)plan;
    if (!P->tuned && P->tiles > 0 && autotune_enabled()) {
        cudaError_t e = plan_tune(P, s);
        if (e != cudaSuccess) return e;
        P->tuned = true;
    }
    if (tiles) *tiles = P->tiles;
    if (P->tiles == 0) return cudaSuccess;
    cudaError_t e = cudaGraphLaunch(P->exec, s);
    if (e == cudaSuccess) note_launch();
    return e;
}

void plan_destroy(void *plan)
{
    auto *P = (BatchPlanImpl *)plan;
    if (!P) return;
    if (P->exec) cudaGraphExecDestroy(P->exec);
    if (P->graph) cudaGraphDestroy(P->graph);
    if (P->dev) cudaFree(P->dev);
    if (P->counter) cudaFree(P->counter);
    delete P;
}

} // namespace ifx
