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
#include <cstring>
#include <mutex>
#include <vector>

namespace ifx {

constexpr int kBatchMaxTaps = 36;     // factor taps (<= 33) rounded up to 4

struct BReq {
    int op, in_type, out_type, style;
    int nx, ny, tiles_x, win;
    long long tile_base;
    const void *in;
    void *out0;
    void *out1;
    float fill;                       // value domain (N0f8: c/255)
    int fill_code;                    // 8-bit images: the fill code
    int kx, ky, fx, fy;
    float wx[kBatchMaxTaps];
    float wy[kBatchMaxTaps];
};

struct BHdr {
    int nreq;
    int pad;
    long long total_tiles;
};

enum { BOP_FACTORED = 1, BOP_GRADIENTS = 2, BOP_LAPLACIAN = 3, BOP_MEDIAN = 4 };

// tile shapes (outputs per tile)
constexpr int kFTX = 64, kFTY = 32;        // factored / gradients / laplacian
constexpr int kMUX = 128, kMUY = 32;       // 8-bit median (4 pixels per thread, 4 rows)
constexpr int kMFX = 64, kMFY = 32;        // float median (8 pixels per thread)

__host__ __device__ inline int bt_tile_w(int op, int in_type)
{
    if (op == BOP_MEDIAN) return (in_type == IFX_F32) ? kMFX : kMUX;
    return kFTX;
}
__host__ __device__ inline int bt_tile_h(int op, int in_type)
{
    if (op == BOP_MEDIAN) return (in_type == IFX_F32) ? kMFY : kMUY;
    return kFTY;
}

__device__ __forceinline__ float bt_load(const BReq &R, int x, int y)
{
    const int mx = map_index(x, R.nx, R.style);
    const int my = map_index(y, R.ny, R.style);
    if (mx < 0 || my < 0) return R.fill;
    const long long o = (long long)my * R.nx + mx;
    if (R.in_type == IFX_F32) return ((const float *)R.in)[o];
    const uint8_t c = ((const uint8_t *)R.in)[o];
    return R.in_type == IFX_N0F8 ? __fdiv_rn((float)c, 255.0f) : (float)c;
}

__device__ __forceinline__ void bt_store(const BReq &R, void *out, int x, int y, float v)
{
    if (x >= R.nx || y >= R.ny) return;
    const long long o = (long long)y * R.nx + x;
    if (R.out_type == IFX_F64) ((double *)out)[o] = (double)v;
    else ((float *)out)[o] = v;
}

// Division-free 2-D gather of a tile whose element (r, c) is load(r, c): warps
// take rows, lanes take columns; each thread issues up to 2 rows x 4 column
// chunks of loads before storing them, so 8 global loads are in flight.
template <class T, class F>
__device__ __forceinline__ void gather2d(T *dst, int rows, int cols, int pitch, F load)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
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

// N0f8 codes as Float32 (c/255 correctly rounded), one table per CTA.
__shared__ float s_n0f8[256];

// Gather the (rows x cols) float tile whose element (r, c) is the image value
// at (ox + c, oy + r) through the border map; columns >= cv are zero.  Tiles
// whose source box lies inside the image skip the map; the element type
// branch is taken once per tile.
__device__ __forceinline__ void bt_gather_f(const BReq &R, float *T, int rows, int cols, int pitch,
                                            int cv, int ox, int oy)
{
    const bool inside = ox >= 0 && oy >= 0 && ox + cv <= R.nx && oy + rows <= R.ny;
    const int nx = R.nx;
    if (R.in_type == IFX_F32) {
        const float *img = (const float *)R.in;
        if (inside)
            gather2d<float>(T, rows, cols, pitch, [&](int r, int c) -> float {
                return c < cv ? img[(long long)(oy + r) * nx + ox + c] : 0.0f;
            });
        else
            gather2d<float>(T, rows, cols, pitch, [&](int r, int c) -> float {
                if (c >= cv) return 0.0f;
                const int mx = map_index(ox + c, nx, R.style), my = map_index(oy + r, R.ny, R.style);
                return (mx < 0 || my < 0) ? R.fill : img[(long long)my * nx + mx];
            });
    } else {
        const uint8_t *img = (const uint8_t *)R.in;
        const bool norm = R.in_type == IFX_N0F8;
        if (inside)
            gather2d<float>(T, rows, cols, pitch, [&](int r, int c) -> float {
                if (c >= cv) return 0.0f;
                const uint8_t v = img[(long long)(oy + r) * nx + ox + c];
                return norm ? s_n0f8[v] : (float)v;
            });
        else
            gather2d<float>(T, rows, cols, pitch, [&](int r, int c) -> float {
                if (c >= cv) return 0.0f;
                const int mx = map_index(ox + c, nx, R.style), my = map_index(oy + r, R.ny, R.style);
                if (mx < 0 || my < 0) return R.fill;
                const uint8_t v = img[(long long)my * nx + mx];
                return norm ? s_n0f8[v] : (float)v;
            });
    }
}

// ---------------------------------------------------------------- factored
__device__ void bt_factored(const BReq &R, int tx0, int ty0, float *sm)
{
    constexpr int TX = kFTX, TY = kFTY, NB = 8;
    const int kx = R.kx, ky = R.ky, kx4 = up4(kx), ky4 = up4(ky);
    float *wx = sm, *wy = sm + kBatchMaxTaps, *T = sm + 2 * kBatchMaxTaps;
    const int RT = TY + ky - 1, CT = TX + kx4, CV = TX + kx - 1;
    float *I = T + RT * CT;
    const int tid = threadIdx.x, nth = blockDim.x;
    if (tid < kx) wx[tid] = R.wx[tid];
    if (tid < ky) wy[tid] = R.wy[tid];
    bt_gather_f(R, T, RT, CT, CT, CV, tx0 + R.fx, ty0 + R.fy);
    __syncthreads();
    float acc[NB];
    const int segs = TX / NB;
    for (int it = tid; it < RT * segs; it += nth) {
        const int r = it / segs, c0 = (it - r * segs) * NB;
        corr_run<float, NB>(T + r * CT + c0, 1, wx, kx, acc);
#pragma unroll
        for (int i = 0; i < NB; ++i) I[r * TX + c0 + i] = acc[i];
    }
    (void)ky4;
    __syncthreads();
    for (int it = tid; it < TX * (TY / NB); it += nth) {
        const int rs = it / TX, c = it - rs * TX, r0 = rs * NB;
        corr_run<float, NB>(I + r0 * TX + c, TX, wy, ky, acc);
#pragma unroll
        for (int i = 0; i < NB; ++i) bt_store(R, R.out0, tx0 + c, ty0 + r0 + i, acc[i]);
    }
}

__host__ __device__ inline int bt_factored_smem_floats(int kx, int ky)
{
    return 2 * kBatchMaxTaps + (kFTY + ky - 1) * (kFTX + up4(kx)) + (kFTY + ky - 1) * kFTX;
}

// ---------------------------------------------------------------- gradients
// out0 = smooth_y(deriv_x), out1 = deriv_y(smooth_x) over a halo-1 tile.
__device__ void bt_gradients(const BReq &R, int tx0, int ty0, float *sm)
{
    constexpr int TX = kFTX, TY = kFTY, NB = 8, CT = TX + 2, RT = TY + 2;
    float *T = sm;
    const int tid = threadIdx.x, nth = blockDim.x;
    bt_gather_f(R, T, RT, CT, CT, CT, tx0 - 1, ty0 - 1);
    __syncthreads();
    const float d0 = R.wx[0], d1 = R.wx[1], d2 = R.wx[2];
    const float s0 = R.wy[0], s1 = R.wy[1], s2 = R.wy[2];
    for (int it = tid; it < TX * (TY / NB); it += nth) {
        const int rs = it / TX, c = it - rs * TX, r0 = rs * NB;
        float D[NB + 2], S[NB + 2];
#pragma unroll
        for (int j = 0; j < NB + 2; ++j) {
            const float *row = T + (r0 + j) * CT + c;
            D[j] = fmaf(d2, row[2], fmaf(d1, row[1], d0 * row[0]));
            S[j] = fmaf(s2, row[2], fmaf(s1, row[1], s0 * row[0]));
        }
#pragma unroll
        for (int i = 0; i < NB; ++i) {
            const float g0 = fmaf(s2, D[i + 2], fmaf(s1, D[i + 1], s0 * D[i]));
            const float g1 = fmaf(d2, S[i + 2], fmaf(d1, S[i + 1], d0 * S[i]));
            bt_store(R, R.out0, tx0 + c, ty0 + r0 + i, g0);
            bt_store(R, R.out1, tx0 + c, ty0 + r0 + i, g1);
        }
    }
}

// ---------------------------------------------------------------- laplacian
__device__ void bt_laplacian(const BReq &R, int tx0, int ty0, float *sm)
{
    constexpr int TX = kFTX, TY = kFTY, CT = TX + 2, RT = TY + 2;
    float *T = sm;
    const int tid = threadIdx.x, nth = blockDim.x;
    bt_gather_f(R, T, RT, CT, CT, CT, tx0 - 1, ty0 - 1);
    __syncthreads();
    for (int it = tid; it < TX * TY; it += nth) {
        const int r = it / TX, c = it - r * TX;
        const float *p = T + (r + 1) * CT + (c + 1);
        float tmp = __fmul_rn(-4.0f, p[0]);
        tmp = __fadd_rn(tmp, p[1]);
        tmp = __fadd_rn(tmp, p[-1]);
        tmp = __fadd_rn(tmp, p[CT]);
        tmp = __fadd_rn(tmp, p[-CT]);
        bt_store(R, R.out0, tx0 + c, ty0 + r, tmp);
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

template <int W>
__device__ void bt_median_u8(const BReq &R, int tx0, int ty0, uint8_t *tile)
{
    constexpr int CT = ((kMUX + W - 1 + 3) & ~3) + 4, RT = kMUY + W - 1, h = W / 2;
    gather2d<uint8_t>(tile, RT, CT, CT, [&](int r, int c) -> uint8_t {
        if (c >= kMUX + W - 1) return 0;
        const int mx = map_index(tx0 - h + c, R.nx, R.style);
        const int my = map_index(ty0 - h + r, R.ny, R.style);
        return (mx < 0 || my < 0) ? (uint8_t)R.fill_code
                                  : ((const uint8_t *)R.in)[(long long)my * R.nx + mx];
    });
    __syncthreads();
    const int tid = threadIdx.x;
    const int lx = (tid & 31) * 4;
    const uint32_t rank4 = 0x01010101u * (uint32_t)((W * W + 1) / 2);
    const bool norm = R.in_type == IFX_N0F8;
    for (int ly = tid >> 5; ly < kMUY; ly += blockDim.x >> 5) {
        const int x0 = tx0 + lx, y = ty0 + ly;
        if (x0 >= R.nx || y >= R.ny) continue;
        uint32_t w[W * W];
        const bool edge = R.style == IFX_CIRCULAR &&
                          (x0 < h || x0 + 3 >= R.nx - h || y < h || y >= R.ny - h);
        if (!edge) {
#pragma unroll
            for (int j = 0; j < W; ++j)
#pragma unroll
                for (int i = 0; i < W; ++i) w[j * W + i] = load_word(tile + (ly + j) * CT, lx + i);
        } else {
            const uint8_t *img = (const uint8_t *)R.in;
#pragma unroll
            for (int j = 0; j < W; ++j)
#pragma unroll
                for (int i = 0; i < W; ++i) {
                    uint32_t word = 0;
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int x = x0 + q < R.nx ? x0 + q : R.nx - 1;
                        word |= (uint32_t)img[bt_win_index(R, x, y, i, j, h)] << (8 * q);
                    }
                    w[j * W + i] = word;
                }
        }
        uint32_t res = 0;
#pragma unroll
        for (int b = 7; b >= 0; --b) {
            const uint32_t trial = res | (0x01010101u << b);
            uint32_t cnt = 0;
#pragma unroll
            for (int k = 0; k < W * W; ++k) cnt = count_lt(cnt, w[k], trial);
            const uint32_t below = __vcmpltu4(cnt, rank4);
            res = (trial & below) | (res & ~below);
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            const uint8_t code = (uint8_t)(res >> (8 * q));
            bt_store(R, R.out0, x0 + q, y, norm ? __fdiv_rn((float)code, 255.0f) : (float)code);
        }
    }
}

template <int W>
__device__ void bt_median_f32(const BReq &R, int tx0, int ty0, float *tile)
{
    using SK = SortKey<float>;
    constexpr int CT = kMFX + W - 1, RT = kMFY + W - 1, h = W / 2, N = W * W;
    gather2d<float>(tile, RT, CT, CT, [&](int r, int c) -> float {
        const int mx = map_index(tx0 - h + c, R.nx, R.style);
        const int my = map_index(ty0 - h + r, R.ny, R.style);
        return (mx < 0 || my < 0) ? R.fill : ((const float *)R.in)[(long long)my * R.nx + mx];
    });
    __syncthreads();
    for (int p = threadIdx.x; p < kMFX * kMFY; p += blockDim.x) {
        const int lx = p % kMFX, ly = p / kMFX, x = tx0 + lx, y = ty0 + ly;
        if (x >= R.nx || y >= R.ny) continue;
        const bool edge = R.style == IFX_CIRCULAR && (x < h || x >= R.nx - h || y < h || y >= R.ny - h);
        uint32_t v[N];
        if (!edge) {
#pragma unroll
            for (int j = 0; j < W; ++j)
#pragma unroll
                for (int i = 0; i < W; ++i) v[j * W + i] = SK::key(tile[(ly + j) * CT + lx + i]);
        } else {
            const float *img = (const float *)R.in;
#pragma unroll
            for (int j = 0; j < W; ++j)
#pragma unroll
                for (int i = 0; i < W; ++i) v[j * W + i] = SK::key(img[bt_win_index(R, x, y, i, j, h)]);
        }
        net_sort<N, uint32_t>(v);
        bt_store(R, R.out0, x, y, SK::val(v[(N - 1) / 2]));
    }
}

// ---------------------------------------------------------------- the kernel
constexpr int kReqTable = 2048;      // requests whose first tiles are searched in shared memory

__global__ void __launch_bounds__(256, 3)
k_batch(const unsigned char *__restrict__ desc, unsigned long long *counter)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ long long s_tile;
    __shared__ int s_base[kReqTable];
    __shared__ __align__(16) BReq s_req;
    const BHdr *hdr = reinterpret_cast<const BHdr *>(desc);
    const BReq *reqs = reinterpret_cast<const BReq *>(desc + sizeof(BHdr));
    const long long total = hdr->total_tiles;
    const int nreq = hdr->nreq;
    const int ntab = nreq < kReqTable ? nreq : kReqTable;
    for (int i = threadIdx.x; i < ntab; i += blockDim.x) s_base[i] = (int)reqs[i].tile_base;
    s_n0f8[threadIdx.x & 255] = __fdiv_rn((float)(threadIdx.x & 255), 255.0f);
    long long next = 0;
    if (threadIdx.x == 0) next = (long long)atomicAdd(counter, 1ULL);
    for (;;) {
        if (threadIdx.x == 0) {
            s_tile = next;
            next = (long long)atomicAdd(counter, 1ULL);   // in flight while this tile runs
        }
        __syncthreads();
        const long long t = s_tile;
        if (t >= total) break;
        // owning request: binary search over first tiles (shared table, then global)
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
        {   // the descriptor, one word per thread
            const int *src = reinterpret_cast<const int *>(reqs + lo);
            int *dst = reinterpret_cast<int *>(&s_req);
            for (int i = threadIdx.x; i < (int)(sizeof(BReq) / 4); i += blockDim.x) dst[i] = src[i];
        }
        __syncthreads();
        const BReq &R = s_req;
        const int local = (int)(t - R.tile_base);
        const int by = local / R.tiles_x, bx = local - by * R.tiles_x;
        const int tw = bt_tile_w(R.op, R.in_type), th = bt_tile_h(R.op, R.in_type);
        const int tx0 = bx * tw, ty0 = by * th;
        switch (R.op) {
        case BOP_FACTORED: bt_factored(R, tx0, ty0, reinterpret_cast<float *>(smem)); break;
        case BOP_GRADIENTS: bt_gradients(R, tx0, ty0, reinterpret_cast<float *>(smem)); break;
        case BOP_LAPLACIAN: bt_laplacian(R, tx0, ty0, reinterpret_cast<float *>(smem)); break;
        default:
            if (R.in_type == IFX_F32) {
                if (R.win == 3) bt_median_f32<3>(R, tx0, ty0, reinterpret_cast<float *>(smem));
                else bt_median_f32<5>(R, tx0, ty0, reinterpret_cast<float *>(smem));
            } else {
                if (R.win == 3) bt_median_u8<3>(R, tx0, ty0, smem);
                else bt_median_u8<5>(R, tx0, ty0, smem);
            }
        }
        __syncthreads();
    }
}

constexpr size_t kBatchSmem = (size_t)(2 * kBatchMaxTaps + (kFTY + 32) * (kFTX + 36) + (kFTY + 32) * kFTX) * 4;

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
    // graph: descriptor upload -> counter reset -> persistent kernel
    if ((e = cudaStreamBeginCapture(E.capture, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return e;
    cudaMemcpyAsync(S.dev, S.host, cap, cudaMemcpyHostToDevice, E.capture);
    cudaMemsetAsync(S.counter, 0, sizeof(unsigned long long), E.capture);
    k_batch<<<E.grid, 256, kBatchSmem, E.capture>>>(S.dev, S.counter);
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
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, 256, kBatchSmem);
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

// Fill `out` from a validated request list; returns the total tile count.
long long batch_describe(const BatchItem *items, int n, std::vector<BReq> &out)
{
    out.resize(n);
    long long base = 0;
    for (int i = 0; i < n; ++i) {
        const BatchItem &it = items[i];
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
        for (int t = 0; t < it.kx && t < kBatchMaxTaps; ++t) R.wx[t] = (float)it.wx[t];
        for (int t = 0; t < it.ky && t < kBatchMaxTaps; ++t) R.wy[t] = (float)it.wy[t];
        const int tw = bt_tile_w(R.op, R.in_type), th = bt_tile_h(R.op, R.in_type);
        R.tiles_x = (R.nx + tw - 1) / tw;
        const long long tiles = (long long)R.tiles_x * ((R.ny + th - 1) / th);
        R.tile_base = base;
        base += tiles;
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
};

cudaError_t plan_create(int device, const BatchItem *items, int n, void **out)
{
    BatchEngine *E;
    cudaError_t e = engine_for(device, &E);
    if (e != cudaSuccess) return e;
    auto *P = new BatchPlanImpl();
    P->device = device;
    P->n = n;
    std::vector<BReq> reqs;
    P->tiles = batch_describe(items, n, reqs);
    const size_t bytes = sizeof(BHdr) + (size_t)n * sizeof(BReq);
    std::vector<unsigned char> host(bytes);
    BHdr h{n, 0, P->tiles};
    memcpy(host.data(), &h, sizeof h);
    if (n) memcpy(host.data() + sizeof(BHdr), reqs.data(), (size_t)n * sizeof(BReq));
    if ((e = cudaMalloc(&P->dev, bytes)) != cudaSuccess ||
        (e = cudaMalloc(&P->counter, sizeof(unsigned long long))) != cudaSuccess ||
        (e = cudaMemcpy(P->dev, host.data(), bytes, cudaMemcpyHostToDevice)) != cudaSuccess) {
        plan_destroy(P);
        return e;
    }
    std::lock_guard<std::mutex> lk(E->mu);
    if ((e = cudaStreamBeginCapture(E->capture, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) {
        plan_destroy(P);
        return e;
    }
    cudaMemsetAsync(P->counter, 0, sizeof(unsigned long long), E->capture);
    k_batch<<<E->grid, 256, kBatchSmem, E->capture>>>(P->dev, P->counter);
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
