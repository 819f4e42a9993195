// ifx_noalloc.cu -- ifx_imfilter_factored_noalloc: the separable cascade for
// callers that cannot allocate device memory on the filtering path, such as a
// real-time frame loop that must not stall on cudaMalloc/cudaFree (both can
// synchronize the whole device) or an application that reserves its entire
// device-memory budget when it starts.
//
// The regular entry point (ifx_imfilter_factored) takes the generic pipeline's
// two intermediate buffers from scratch that its context allocates and grows.
// This variant runs the same pipeline with both buffers carved out of one
// fixed array, `g_noalloc_scratch`, compiled into the library: every GPU that
// loads the library holds these kNoAllocScratchBytes until the process exits.
// It calls no cudaMalloc, cudaFree or other allocating routine, needs no
// context, and accepts device arrays only (host arrays would need staging
// buffers).
//
// Set-up: the first call on a device, with that device current, looks up the
// array's device address (cudaGetSymbolAddress) and keeps it; make that first
// call before any stream capture starts.  A failed look-up is not kept: the
// next call tries again.  The arrays (and the stream, if one is given) must
// belong to the current device, since the scratch used is that device's.  All calls on a device share
// the one array and leave the last call's contents in it.  Nothing needs to
// start at zero: the pipeline writes every scratch element before reading it.
// Calls whose work overlaps on the GPU (different streams, or the same array
// used from several host threads) race on the scratch: order them.
#include "ifx_internal.h"
#include <cstdio>
#include <mutex>

namespace ifx {

constexpr size_t kNoAllocScratchBytes = 32u << 20;     // 32 MiB per device

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

constexpr int kMaxDevices = 64;
static std::mutex g_setup_mu;
static void *g_scratch_addr[kMaxDevices];

// Device address of g_noalloc_scratch on device `dev` (the current device).
// In host code the symbol's name only stands for the array; the kernels need
// this address.  Only a successful look-up is kept.
static int scratch_address(int dev, void **addr)
{
    if (dev < 0 || dev >= kMaxDevices) return set_error(IFX_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (!g_scratch_addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            (void)cudaGetLastError();
            char m[260];
            snprintf(m, sizeof m, "cudaGetSymbolAddress of the fixed scratch failed on device %d: %s (make "
                     "the first call on a device outside stream capture)", dev, cudaGetErrorString(e));
            return set_error(IFX_ERR_CUDA, m);
        }
        g_scratch_addr[dev] = p;
    }
    *addr = g_scratch_addr[dev];
    return IFX_OK;
}

} // namespace ifx

using namespace ifx;

extern "C" {

uint64_t ifx_noalloc_scratch_bytes(void) { return (uint64_t)kNoAllocScratchBytes; }

int ifx_imfilter_factored_noalloc(ifx_array_t *out, const ifx_array_t *img, int32_t nfactors,
                                  const ifx_factor_t *factors, const ifx_border_t *border,
                                  void *stream)
{
    IFX_RANGE("ifx_imfilter_factored_noalloc");
    std::vector<Fac> facs;
    double fill;
    bool nothing;
    int rc = factored_prepare(out, img, nfactors, factors, border, facs, &fill, &nothing);
    if (rc || nothing) return rc;
    for (const Fac &f : facs)
        if (f.len > IFX_MAX_TAPS)           // longer factors need a device weight buffer
            return set_error(IFX_ERR_UNSUPPORTED, "the allocation-free entry point takes factors of up to "
                                                  "129 taps (IFX_MAX_TAPS)");
    int dev = -1;
    cudaError_t ge = cudaGetDevice(&dev);
    if (ge != cudaSuccess) {
        char m[160];
        snprintf(m, sizeof m, "cudaGetDevice failed: %s", cudaGetErrorString(ge));
        return set_error(IFX_ERR_CUDA, m);
    }
    if ((rc = check_device_array(*img, dev, "img")) || (rc = check_device_array(*out, dev, "out")))
        return rc;
    const cudaStream_t s = (cudaStream_t)stream;
    if (s) {
        int sdev = -1;
        if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) {
            (void)cudaGetLastError();
            return set_error(IFX_ERR_ARGUMENT, "stream: not a valid CUDA stream");
        }
        if (sdev != dev) {
            char m[160];
            snprintf(m, sizeof m, "the stream belongs to device %d but device %d is current", sdev, dev);
            return set_error(IFX_ERR_ARGUMENT, m);
        }
    }
    if (facs.empty()) {                          // copy kernels only: a conversion, no scratch
        PadBoxArgs pa;
        pa.img = img->data;
        pa.in_type = img->eltype;
        pa.dst = out->data;
        pa.out_type = out->eltype;
        pa.nd = img->ndim;
        int lo[IFX_MAXD] = {0, 0, 0, 0}, sz[IFX_MAXD];
        for (int d = 0; d < IFX_MAXD; ++d) {
            pa.n[d] = d < img->ndim ? (int)img->size[d] : 1;
            sz[d] = pa.n[d];
        }
        pa.box = make_box(img->ndim, lo, sz);
        pa.style = IFX_REPLICATE;
        pa.fill = 0.0;
        const cudaError_t e = launch_pad_box(pa, s);
        return e == cudaSuccess ? IFX_OK : set_error(IFX_ERR_CUDA, cudaGetErrorString(e));
    }
    size_t need_a = 0, need_b = 0;
    generic_cascade_sizes(*img, facs, &need_a, &need_b);
    const size_t a_bytes = (need_a + 255) / 256 * 256;
    if (a_bytes + need_b > kNoAllocScratchBytes) {
        char m[240];
        snprintf(m, sizeof m, "this filter needs %zu bytes of scratch; the fixed scratch of the "
                 "allocation-free entry point holds %zu bytes (use ifx_imfilter_factored)",
                 a_bytes + need_b, (size_t)kNoAllocScratchBytes);
        return set_error(IFX_ERR_NOMEM, m);
    }
    void *base = nullptr;
    if ((rc = scratch_address(dev, &base))) return rc;
    unsigned char *bufA = (unsigned char *)base;
    unsigned char *bufB = need_b ? bufA + a_bytes : nullptr;
    return generic_cascade_run(s, *img, img->data, *out, out->data, facs, border->style, fill, bufA, bufB);
}

} // extern "C"
