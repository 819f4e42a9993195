// ifx_tma.cu -- host side of the TMA helpers: tensor-map encoding through the
// driver entry point (no link-time dependency on libcuda) and the per-device
// error word of kernels with bounded waits.
#include "ifx_internal.h"
#include "ifx_tma.cuh"
#include <cudaTypedefs.h>
#include <mutex>

namespace ifx {

static PFN_cuTensorMapEncodeTiled_v12000 encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    });
    return fn;
}

bool tma_encode_3d(CUtensorMap *map, const void *base, int elt_bytes, long long nx, long long ny, long long nz,
                   long long pitch_bytes, long long plane_bytes, int box_w, int box_h)
{
    if (elt_bytes != 1 && elt_bytes != 4) return false;
    if (((uintptr_t)base & 15) || (pitch_bytes & 15) || pitch_bytes <= 0 || (plane_bytes & 15) ||
        plane_bytes < pitch_bytes * ny)
        return false;
    if (nx <= 0 || ny <= 0 || nz <= 0 || nx > (1ll << 31) || ny > (1ll << 31) || nz > (1ll << 31)) return false;
    if (box_w < 1 || box_w > 256 || box_h < 1 || box_h > 256 || (box_w * elt_bytes) % 16) return false;
    auto fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
    cuuint64_t strides[2] = {(cuuint64_t)pitch_bytes, (cuuint64_t)plane_bytes};
    cuuint32_t box[3] = {(cuuint32_t)box_w, (cuuint32_t)box_h, 1};
    cuuint32_t estr[3] = {1, 1, 1};
    const CUtensorMapDataType dt = elt_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT8;
    return fn(map, dt, 3, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
              CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

static int *g_err_word[64];
static std::mutex g_err_mu;

int *tma_error_word(int device)
{
    if (device < 0 || device >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(g_err_mu);
    if (!g_err_word[device]) {
        int *p = nullptr;
        if (cudaMalloc(&p, sizeof(int)) != cudaSuccess) return nullptr;
        if (cudaMemset(p, 0, sizeof(int)) != cudaSuccess) {
            cudaFree(p);
            return nullptr;
        }
        g_err_word[device] = p;
    }
    return g_err_word[device];
}

int kernel_timeout_take(int device) { return tma_error_take(device); }

int tma_error_take(int device)
{
    if (device < 0 || device >= 64) return 0;
    int *p;
    {
        std::lock_guard<std::mutex> lk(g_err_mu);
        p = g_err_word[device];
    }
    if (!p) return 0;
    int h = 0;
    cudaMemcpy(&h, p, sizeof(int), cudaMemcpyDeviceToHost);
    if (h) cudaMemset(p, 0, sizeof(int));
    return h;
}

} // namespace ifx
