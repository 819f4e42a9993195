// ifx_api.cu -- the C ABI (include/ifx_gb300.h): argument validation with the
// reference's error classes, host<->device staging, scratch management and
// dispatch to the sm_103a kernels.  No CPU compute path exists: every result
// is produced by a kernel of this library.
#include "ifx_internal.h"
#include "ifx_tma.cuh"
#include <atomic>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

namespace ifx {

static std::atomic<uint64_t> g_launches{0};
void note_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

size_t dense2d_smem_bytes(int kw, int kh, int f64);

static thread_local std::string t_err;

static int fail(int code, const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    static const char *cls[] = {"", "ArgumentError: ", "DimensionMismatch: ", "ErrorException: ",
                                "CUDA error: ", "OutOfMemory: ", "Timeout: ", "Unsupported: "};
    t_err = std::string(code >= 0 && code <= 7 ? cls[code] : "") + buf;
    return code;
}

#define IFX_CUDA(call)                                                                         \
    do {                                                                                       \
        cudaError_t e_ = (call);                                                               \
        if (e_ != cudaSuccess) return fail(IFX_ERR_CUDA, "%s (%s:%d)", cudaGetErrorString(e_), \
                                           __FILE__, __LINE__);                                \
    } while (0)

static size_t elsize(int t)
{
    switch (t) {
    case IFX_F32: return 4;
    case IFX_F64: return 8;
    case IFX_N0F8:
    case IFX_U8: return 1;
    case IFX_I16: return 2;
    default: return 0;
    }
}
static bool is8(int t) { return t == IFX_N0F8 || t == IFX_U8; }
// Element sizes of every eltype ifx_convert takes (the filters take the ones
// elsize knows).
static size_t conv_elsize(int t)
{
    switch (t) {
    case IFX_I8: return 1;
    case IFX_U16:
    case IFX_N0F16: return 2;
    case IFX_I32: return 4;
    case IFX_I64: return 8;
    default: return elsize(t);
    }
}

// ------------------------------------------------------------------ context
struct Slot {
    void *ptr = nullptr;
    size_t cap = 0;
};

} // namespace ifx

struct ifx_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::mutex mu;
    ifx::Slot slots[32];
};

namespace ifx {

enum { kSlotIn = 0, kSlotOut = 1, kSlotTmp = 12 };

static int slot_get(ifx_context *c, int i, size_t bytes, void **out)
{
    Slot &s = c->slots[i];
    if (s.cap < bytes) {
        if (s.ptr) {
            IFX_CUDA(cudaDeviceSynchronize());
            IFX_CUDA(cudaFree(s.ptr));
            s.ptr = nullptr;
            s.cap = 0;
        }
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&s.ptr, want);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            s.ptr = nullptr;
            return fail(IFX_ERR_NOMEM, "device allocation of %zu bytes failed", want);
        }
        s.cap = want;
    }
    *out = s.ptr;
    return IFX_OK;
}

// ------------------------------------------------------------------ arrays
static long long numel(const ifx_array_t &a)
{
    long long n = 1;
    for (int d = 0; d < a.ndim; ++d) n *= a.size[d];
    return n;
}

static int check_array(const ifx_array_t *a, const char *name, int values_per_elem = 1, bool any_eltype = false)
{
    if (!a) return fail(IFX_ERR_ARGUMENT, "%s is NULL", name);
    if (a->ndim < 1 || a->ndim > IFX_MAX_DIMS)
        return fail(IFX_ERR_ARGUMENT, "%s: ndims %d not in 1..%d", name, a->ndim, IFX_MAX_DIMS);
    if ((any_eltype ? conv_elsize(a->eltype) : elsize(a->eltype)) == 0)
        return fail(IFX_ERR_ARGUMENT, "%s: eltype %d is not taken here%s", name, a->eltype,
                    conv_elsize(a->eltype) ? " (convert it with ifx_convert first)" : "");
    long long s = 1;
    for (int d = 0; d < a->ndim; ++d) {
        if (a->size[d] < 0) return fail(IFX_ERR_ARGUMENT, "%s: negative size", name);
        if (a->size[d] > (1LL << 30))
            return fail(IFX_ERR_UNSUPPORTED, "%s: axis %d longer than 2^30", name, d);
        if (a->size[d] > 1 && a->stride[d] != s)
            return fail(IFX_ERR_ARGUMENT, "%s: only dense column-major arrays are supported "
                        "(axis %d stride %lld, expected %lld)", name, d, (long long)a->stride[d], s);
        s *= a->size[d];
    }
    (void)values_per_elem;
    if (s > 0 && !a->data) return fail(IFX_ERR_ARGUMENT, "%s: data is NULL", name);
    return IFX_OK;
}

static int check_same_axes(const ifx_array_t &out, const ifx_array_t &img)
{
    if (out.ndim != img.ndim)
        return fail(IFX_ERR_DIMENSION, "output has %d dimensions, input %d", out.ndim, img.ndim);
    for (int d = 0; d < img.ndim; ++d)
        if (out.size[d] != img.size[d] || out.first[d] != img.first[d])
            return fail(IFX_ERR_DIMENSION, "output indices disagree with the input's on axis %d "
                        "(%lld:%lld vs %lld:%lld)", d + 1, (long long)out.first[d],
                        (long long)(out.first[d] + out.size[d] - 1), (long long)img.first[d],
                        (long long)(img.first[d] + img.size[d] - 1));
    return IFX_OK;
}

static bool is_device_ptr(const void *p)
{
    if (!p) return false;
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, p);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

// Device allocations seen by one call, as [base, end) ranges from the driver's
// cuMemGetAddressRange: arrays inside a known allocation need no further
// pointer query, and an array must end inside the allocation it starts in.
typedef int (*PfnAddressRange)(unsigned long long *base, size_t *size, unsigned long long dptr);

static PfnAddressRange address_range_fn()
{
    static PfnAddressRange fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (PfnAddressRange)p;
        (void)cudaGetLastError();
    });
    return fn;
}

struct DevRanges {
    std::vector<std::pair<uintptr_t, uintptr_t>> r;
    // true when [p, p+bytes) lies in device memory
    bool holds(const void *p, size_t bytes)
    {
        const uintptr_t a = (uintptr_t)p, e = a + (bytes ? bytes : 1);
        for (auto &x : r)
            if (a >= x.first && e <= x.second) return true;
        if (!is_device_ptr(p)) return false;
        PfnAddressRange fn = address_range_fn();
        unsigned long long base = 0;
        size_t size = 0;
        if (fn && fn(&base, &size, (unsigned long long)a) == 0) {
            r.push_back({(uintptr_t)base, (uintptr_t)(base + size)});
            return e <= (uintptr_t)(base + size);
        }
        return is_device_ptr((const char *)p + (bytes ? bytes - 1 : 0));
    }
};

// Staging of one call's arrays: host arrays are copied to scratch slots.
struct Call {
    ifx_context *ctx;
    cudaStream_t s;
    bool host = false;                  // any host array -> synchronous call
    struct Back { void *host; void *dev; size_t bytes; };
    std::vector<Back> back;
    int next_slot = kSlotIn;

    int input(const ifx_array_t &a, const void **dptr, size_t bytes_override = 0)
    {
        const size_t bytes = bytes_override ? bytes_override : (size_t)numel(a) * elsize(a.eltype);
        if (bytes == 0 || is_device_ptr(a.data)) {
            *dptr = a.data;
            return IFX_OK;
        }
        host = true;
        void *d;
        int rc = slot_get(ctx, next_slot++, bytes, &d);
        if (rc) return rc;
        IFX_CUDA(cudaMemcpyAsync(d, a.data, bytes, cudaMemcpyHostToDevice, s));
        *dptr = d;
        return IFX_OK;
    }
    int output(const ifx_array_t &a, void **dptr, size_t bytes_override = 0)
    {
        const size_t bytes = bytes_override ? bytes_override : (size_t)numel(a) * elsize(a.eltype);
        if (bytes == 0 || is_device_ptr(a.data)) {
            *dptr = a.data;
            return IFX_OK;
        }
        host = true;
        void *d;
        int rc = slot_get(ctx, next_slot++, bytes, &d);
        if (rc) return rc;
        back.push_back({a.data, d, bytes});
        *dptr = d;
        return IFX_OK;
    }
    int finish()
    {
        IFX_CUDA(cudaGetLastError());
        for (auto &b : back) IFX_CUDA(cudaMemcpyAsync(b.host, b.dev, b.bytes, cudaMemcpyDeviceToHost, s));
        if (host) IFX_CUDA(cudaStreamSynchronize(s));
        return IFX_OK;
    }
};

static int begin(ifx_context *ctx, void *stream, Call &c)
{
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    IFX_CUDA(cudaSetDevice(ctx->device));
    c.ctx = ctx;
    c.s = stream ? (cudaStream_t)stream : ctx->stream;
    return IFX_OK;
}

// ------------------------------------------------------------------ borders
static int check_border(const ifx_border_t *b)
{
    if (!b) return fail(IFX_ERR_ARGUMENT, "border is NULL");
    if (b->style < IFX_REPLICATE || b->style > IFX_FILL)
        return fail(IFX_ERR_ARGUMENT, "border style %d not a recognized border", b->style);
    return IFX_OK;
}

// The reference builds every padindex table, so reflect on a length-1 axis is
// a DivideError (src/border.jl:581-586: period 2n-2 == 0).
static int check_reflect(const ifx_border_t *b, const ifx_array_t &img)
{
    if (b->style != IFX_REFLECT) return IFX_OK;
    for (int d = 0; d < img.ndim; ++d)
        if (img.size[d] == 1)
            return fail(IFX_ERR_ERROR, "DivideError: integer division error (reflect padding of a "
                        "length-1 axis %d)", d + 1);
    return IFX_OK;
}

// Padding needed per axis (src/border.jl:614-621, 637-641) against an explicit
// Pad/Fill (src/imfilter.jl:604-615 raises DimensionMismatch when too small).
static int check_padding(const ifx_border_t *b, const ifx_array_t &img, const long long *pfirst,
                         const long long *plast)
{
    if (!b->explicit_pad) return IFX_OK;
    for (int d = 0; d < img.ndim; ++d) {
        long long need_lo = pfirst[d] < 0 ? -pfirst[d] : 0;
        long long need_hi = plast[d] > 0 ? plast[d] : 0;
        if (b->lo[d] < need_lo || b->hi[d] < need_hi)
            return fail(IFX_ERR_DIMENSION, "requested indices and kernel indices %lld:%lld do not "
                        "agree with indices of padded input (axis %d padded by %lld,%lld)",
                        pfirst[d], plast[d], d + 1, (long long)b->lo[d], (long long)b->hi[d]);
    }
    return IFX_OK;
}

// Fill value in the element domain of type t (8-bit: the code).
static int fill_for(const ifx_border_t *b, int t, double *out)
{
    double v = b->style == IFX_FILL ? b->fill_value : 0.0;
    if (is8(t)) {
        double code = t == IFX_N0F8 ? v * 255.0 : v;
        double r = std::nearbyint(code);
        if (!(r >= 0.0 && r <= 255.0) || std::fabs(r - code) > 1e-6)
            return fail(IFX_ERR_ARGUMENT, "Cannot convert elements of border=Fill(%g) to the 8-bit "
                        "image eltype", v);
        *out = r;
        return IFX_OK;
    }
    *out = v;
    return IFX_OK;
}

// Fill converted as BorderArray does (to the image eltype, src/borderarray.jl:
// 11-20), then expressed in the destination's domain: the 8-bit code for 8-bit
// destinations, the numeric value otherwise.
static int image_fill(const ifx_border_t *b, int img_type, int dst_type, double *out)
{
    double v;
    int rc = fill_for(b, img_type, &v);
    if (rc) return rc;
    if (is8(img_type) && !is8(dst_type)) v = img_type == IFX_N0F8 ? v / 255.0 : v;
    *out = v;
    return IFX_OK;
}

static Box image_box(const ifx_array_t &a)
{
    int lo[IFX_MAXD] = {0, 0, 0, 0}, sz[IFX_MAXD];
    for (int d = 0; d < IFX_MAXD; ++d) sz[d] = d < a.ndim ? (int)a.size[d] : 1;
    return make_box(a.ndim, lo, sz);
}

// ------------------------------------------------------------------ cascade

// The generic pipeline: the padded box [sum first, n-1+sum last] in the
// compute type (buffer A), then one pass per factor over the index range the
// later passes still need, alternating between buffers B and A (the padded
// box is no longer needed once the first pass has read it); the last pass
// writes the output.  Every element a pass reads was written before, so the
// buffers need no initialisation.
static void generic_cascade_boxes(const ifx_array_t &imgd, const std::vector<Fac> &facs, Box *pad,
                                  std::vector<Box> *outs)
{
    const int nd = imgd.ndim;
    long long pfirst[IFX_MAXD] = {0, 0, 0, 0}, plast[IFX_MAXD] = {0, 0, 0, 0};
    for (auto &f : facs) {
        pfirst[f.axis] += f.first;
        plast[f.axis] += f.first + f.len - 1;
    }
    int blo[IFX_MAXD], bsz[IFX_MAXD], slo[IFX_MAXD], shi[IFX_MAXD];
    for (int d = 0; d < IFX_MAXD; ++d) {
        const int n = d < nd ? (int)imgd.size[d] : 1;
        blo[d] = d < nd ? (int)pfirst[d] : 0;
        bsz[d] = d < nd ? (int)(n + plast[d] - pfirst[d]) : 1;
        slo[d] = blo[d];
        shi[d] = blo[d] + bsz[d] - 1;
    }
    *pad = make_box(nd, blo, bsz);
    outs->clear();
    for (auto &f : facs) {
        slo[f.axis] -= f.first;
        shi[f.axis] -= f.first + f.len - 1;
        int olo[IFX_MAXD], osz[IFX_MAXD];
        for (int d = 0; d < IFX_MAXD; ++d) {
            olo[d] = slo[d];
            osz[d] = shi[d] - slo[d] + 1;
        }
        outs->push_back(make_box(nd, olo, osz));
    }
}

// Bytes of buffers A and B the generic pipeline needs.
void generic_cascade_sizes(const ifx_array_t &imgd, const std::vector<Fac> &facs, size_t *a, size_t *b)
{
    const size_t cs = imgd.eltype == IFX_F64 ? 8 : 4;
    Box pad;
    std::vector<Box> outs;
    generic_cascade_boxes(imgd, facs, &pad, &outs);
    size_t na = (size_t)pad.count * cs, nb = 0;
    for (size_t q = 0; q + 1 < outs.size(); ++q) {        // intermediate results: B, A, B, ...
        const size_t bytes = (size_t)outs[q].count * cs;
        if (q % 2 == 0) nb = bytes > nb ? bytes : nb;
        else na = bytes > na ? bytes : na;
    }
    *a = na;
    *b = nb;
}

int generic_cascade_run(cudaStream_t s, const ifx_array_t &imgd, const void *img,
                        const ifx_array_t &outd, void *out, const std::vector<Fac> &facs, int style,
                        double fill, void *bufA, void *bufB)
{
    const int nd = imgd.ndim;
    const int ct = imgd.eltype == IFX_F64 ? IFX_F64 : IFX_F32;
    int n[IFX_MAXD];
    for (int d = 0; d < IFX_MAXD; ++d) n[d] = d < nd ? (int)imgd.size[d] : 1;
    Box cur;
    std::vector<Box> outs;
    generic_cascade_boxes(imgd, facs, &cur, &outs);
    PadBoxArgs pa{img, imgd.eltype, bufA, ct, nd, {n[0], n[1], n[2], n[3]}, cur, style, fill};
    IFX_CUDA(launch_pad_box(pa, s));
    const void *src = bufA;
    for (size_t q = 0; q < facs.size(); ++q) {
        const Fac &f = facs[q];
        const bool last = q + 1 == facs.size();
        void *dst = last ? out : (q % 2 == 0 ? bufB : bufA);
        const Box db = last ? image_box(imgd) : outs[q];
        PassBoxArgs pb{src, cur, dst, db, last ? outd.eltype : ct, outs[q], f.axis, f.first, f.len, f.w,
                       ct == IFX_F64};
        IFX_CUDA(launch_pass_box(pb, s));
        src = dst;
        cur = db;
    }
    return IFX_OK;
}


static bool is_copy(const ifx_factor_t &f)
{
    return f.length == 1 && f.first == 0 && f.weights[0] == 1.0;
}

// Cascade over device arrays.  img/out are device pointers.
static int run_cascade(Call &c, const ifx_array_t &imgd, const void *img, const ifx_array_t &outd,
                       void *out, const std::vector<Fac> &facs, const ifx_border_t *border,
                       int tmp_slot_base)
{
    const int nd = imgd.ndim;
    const int ct = imgd.eltype == IFX_F64 ? IFX_F64 : IFX_F32;   // compute type
    const size_t cs = elsize(ct);
    double fill;
    int rc = image_fill(border, imgd.eltype, ct, &fill);
    if (rc) return rc;
    int n[IFX_MAXD];
    for (int d = 0; d < IFX_MAXD; ++d) n[d] = d < nd ? (int)imgd.size[d] : 1;

    if (facs.empty()) {   // all copies: convert into out
        PadBoxArgs pa{img, imgd.eltype, out, outd.eltype, nd, {n[0], n[1], n[2], n[3]},
                      image_box(imgd), IFX_REPLICATE, 0.0};
        IFX_CUDA(launch_pad_box(pa, c.s));
        return IFX_OK;
    }

    // fast path: 1-D / 2-D with at most one factor per axis -> fused tile kernel
    bool fused = nd <= 2 && facs.size() <= 2 &&
                 !(facs.size() == 2 && facs[0].axis == facs[1].axis);
    if (fused) {
        static const double one = 1.0;
        Fac fx{0, 0, 1, &one}, fy{1, 0, 1, &one};
        int x_first = 1;
        for (size_t i = 0; i < facs.size(); ++i) (facs[i].axis == 0 ? fx : fy) = facs[i];
        // Two factors: pad-then-cascade commutes (only FP32 rounding moves), and
        // the FP32 kernels run the x pass first whatever the factor order -- their
        // last pass then stores down columns, coalesced (the y pass first measured
        // 2-2.5x slower in the TMA kernel: its last pass stores along rows, a
        // row per lane).  FP64 keeps the kernel order; the autotuner may choose.
        if (facs.size() == 2) x_first = ct == IFX_F64 ? facs[0].axis == 0 : 1;
        else x_first = facs[0].axis == 0 ? 1 : 0;
        if (fx.len > IFX_MAX_TAPS || fy.len > IFX_MAX_TAPS ||
            sep2d_smem_bytes(fx.len, fy.len, x_first, ct == IFX_F64) > 200 * 1024)
            fused = false;
        if (fused) {
            Sep2dArgs a{img, imgd.eltype, out, outd.eltype, n[0], nd > 1 ? n[1] : 1,
                        fx.first, fx.len, fy.first, fy.len, fx.w, fy.w, x_first,
                        border->style, fill, ct == IFX_F64};
            IFX_CUDA(launch_sep2d_tuned(a, c.s, !c.host));
            return IFX_OK;
        }
    }

    // 3-D with one factor per axis in axis order: the z sweep into an FP32
    // volume and the x/y TMA sweep over its planes (the default), or the fused
    // z-marching kernel (rows off the copy engine's rules, long z factors, or
    // the autotuner's choice)
    if (nd == 3 && ct == IFX_F32 && facs.size() == 3 && facs[0].axis == 0 && facs[1].axis == 1 &&
        facs[2].axis == 2) {
        Sep3dArgs a{img, imgd.eltype, out, outd.eltype, n[0], n[1], n[2], 1,
                    facs[0].first, facs[0].len, facs[1].first, facs[1].len, facs[2].first, facs[2].len,
                    facs[0].w, facs[1].w, facs[2].w, border->style, fill};
        const bool split = sep3d_split_applies(a);
        const bool fused = sep3d_supported(facs[0].len, facs[1].len, facs[2].len, n[0], n[1], n[2], 1);
        if (split || fused) {
            // the FP32 volume only when the split sweeps may run: no cached
            // choice of the fused kernel
            TuneChoice ch;
            const bool fused_cached = fused && autotune_lookup3(a, &ch) && ch.variant == 2;
            void *vol = nullptr;
            if (split && !fused_cached) {
                rc = slot_get(c.ctx, tmp_slot_base, sep3d_split_tmp_bytes(a), &vol);
                if (rc) return rc;
            }
            IFX_CUDA(launch_sep3d_tuned(a, static_cast<float *>(vol), c.s, !c.host));
            return IFX_OK;
        }
    }
    // generic: materialise the padded box in the compute type, then passes
    size_t need_a = 0, need_b = 0;
    generic_cascade_sizes(imgd, facs, &need_a, &need_b);
    void *bufA, *bufB = nullptr;
    rc = slot_get(c.ctx, tmp_slot_base, need_a, &bufA);
    if (rc) return rc;
    if (need_b && (rc = slot_get(c.ctx, tmp_slot_base + 1, need_b, &bufB))) return rc;
    return generic_cascade_run(c.s, imgd, img, outd, out, facs, border->style, fill, bufA, bufB);
}

static int check_filter_types(const ifx_array_t &img, const ifx_array_t &out)
{
    if (img.eltype == IFX_I16) return fail(IFX_ERR_UNSUPPORTED, "Int16 images are not supported");
    if (out.eltype != IFX_F32 && out.eltype != IFX_F64)
        return fail(IFX_ERR_UNSUPPORTED, "linear filters write Float32 or Float64 outputs");
    return IFX_OK;
}

// Validation of one batched request (also used by the server, which accepts
// host arrays and stages them itself).  Fills `it` with the request's own
// pointers and weights.
int request_item(const ifx_request_t &q, int i, bool need_device, BatchItem &it, DevRanges *dr)
{
    int rc;
    if ((rc = check_array(&q.img, "img")) || (rc = check_border(&q.border))) return rc;
    if (q.img.ndim != 2) return fail(IFX_ERR_UNSUPPORTED, "request %d: batched requests are 2-D", i);
    const int et = q.img.eltype;
    if (et != IFX_F32 && !is8(et))
        return fail(IFX_ERR_UNSUPPORTED, "request %d: batched images are Float32, N0f8 or UInt8", i);
    const int nout = q.op == IFX_OP_GRADIENTS2D ? 2 : 1;
    if (q.op < IFX_OP_FACTORED2D || q.op > IFX_OP_MEDIAN2D)
        return fail(IFX_ERR_ARGUMENT, "request %d: unknown op %d", i, q.op);
    for (int o = 0; o < nout; ++o) {
        if ((rc = check_array(&q.out[o], "out")) || (rc = check_same_axes(q.out[o], q.img))) return rc;
        const int ot = q.out[o].eltype;
        if (ot != IFX_F32 && ot != IFX_F64)
            return fail(IFX_ERR_UNSUPPORTED, "request %d: outputs are Float32 or Float64", i);
        if (need_device && !(dr ? dr->holds(q.out[o].data, (size_t)numel(q.out[o]) * elsize(ot))
                                : is_device_ptr(q.out[o].data)))
            return fail(IFX_ERR_ARGUMENT, "request %d: batched outputs must be device memory", i);
    }
    if (q.out[0].eltype != (nout == 2 ? q.out[1].eltype : q.out[0].eltype))
        return fail(IFX_ERR_UNSUPPORTED, "request %d: both gradients need one eltype", i);
    if (need_device && !(dr ? dr->holds(q.img.data, (size_t)numel(q.img) * elsize(et))
                            : is_device_ptr(q.img.data)))
        return fail(IFX_ERR_ARGUMENT, "request %d: batched images must be device memory", i);
    if (q.border.explicit_pad)
        return fail(IFX_ERR_UNSUPPORTED, "request %d: explicit padding sizes in a batch", i);
    if ((rc = check_reflect(&q.border, q.img))) return rc;
    memset(&it, 0, sizeof it);
    it.op = q.op;
    it.in_type = et;
    it.out_type = q.out[0].eltype;
    it.style = q.border.style;
    it.nx = (int)q.img.size[0];
    it.ny = (int)q.img.size[1];
    it.in = q.img.data;
    it.out0 = q.out[0].data;
    it.out1 = nout == 2 ? q.out[1].data : nullptr;
    double code = 0.0;
    if ((rc = fill_for(&q.border, et, &code))) return rc;
    it.fill_code = is8(et) ? (int)code : 0;
    it.fill = et == IFX_N0F8 ? (double)((float)code / 255.0f) : code;
    if (et == IFX_F32) it.fill = (double)(float)code;
    if (q.op == IFX_OP_FACTORED2D) {
        for (int a = 0; a < 2; ++a)
            if (q.taps[a] < 1 || q.taps[a] > 33 || !q.weights[a] || q.first[a] < -4096 || q.first[a] > 4096)
                return fail(IFX_ERR_UNSUPPORTED, "request %d: batched factors have 1..33 taps", i);
        it.kx = q.taps[0];
        it.ky = q.taps[1];
        it.fx = (int)q.first[0];
        it.fy = (int)q.first[1];
        it.wx = q.weights[0];
        it.wy = q.weights[1];
    } else if (q.op == IFX_OP_GRADIENTS2D) {
        if (q.taps[0] != 3 || q.taps[1] != 3 || q.first[0] != -1 || q.first[1] != -1 ||
            !q.weights[0] || !q.weights[1])
            return fail(IFX_ERR_UNSUPPORTED, "request %d: batched gradients use 3-tap centred pairs", i);
        it.kx = it.ky = 3;
        it.fx = it.fy = -1;
        it.wx = q.weights[0];
        it.wy = q.weights[1];
    } else if (q.op == IFX_OP_LAPLACIAN2D) {
        if (it.out_type != IFX_F32 || (is8(et) && et != IFX_N0F8))
            return fail(IFX_ERR_UNSUPPORTED, "request %d: batched Laplacian writes Float32", i);
    } else {
        if (q.window != 3 && q.window != 5)
            return fail(IFX_ERR_UNSUPPORTED, "request %d: batched median windows are 3 or 5", i);
        it.window = q.window;
    }
    return IFX_OK;
}

int set_error(int code, const char *msg) { return fail(code, "%s", msg); }

static int collect_factors(const ifx_array_t &img, int32_t nf, const ifx_factor_t *factors,
                           std::vector<Fac> &facs, long long *pfirst, long long *plast)
{
    if (nf < 0 || (nf > 0 && !factors)) return fail(IFX_ERR_ARGUMENT, "bad factor list");
    for (int d = 0; d < IFX_MAXD; ++d) pfirst[d] = plast[d] = 0;
    for (int i = 0; i < nf; ++i) {
        const ifx_factor_t &f = factors[i];
        if (f.axis < 0 || f.axis >= img.ndim)
            return fail(IFX_ERR_DIMENSION, "factor %d filters axis %d of a %d-dimensional image",
                        i + 1, f.axis + 1, img.ndim);
        if (f.length < 1 || f.length > kMaxFactorTaps)
            return fail(IFX_ERR_UNSUPPORTED, "factor %d has %d taps (1..%d supported)", i + 1,
                        f.length, kMaxFactorTaps);
        if (!f.weights) return fail(IFX_ERR_ARGUMENT, "factor %d has no weights", i + 1);
        if (f.first < -(1 << 20) || f.first > (1 << 20))
            return fail(IFX_ERR_UNSUPPORTED, "factor offset out of range");
        pfirst[f.axis] += f.first;
        plast[f.axis] += f.first + f.length - 1;
        if (!is_copy(f)) facs.push_back({f.axis, (int)f.first, f.length, f.weights});
    }
    return IFX_OK;
}

// Validation of ifx_imfilter_factored's arguments (shared with the
// fixed-scratch variant): kept factors in `facs`, the fill value in the
// compute type's domain, *nothing = true when there is no element to write.
int factored_prepare(const ifx_array_t *out, const ifx_array_t *img, int32_t nfactors,
                     const ifx_factor_t *factors, const ifx_border_t *border, std::vector<Fac> &facs,
                     double *fill, bool *nothing)
{
    int rc;
    *nothing = false;
    if ((rc = check_array(img, "img")) || (rc = check_array(out, "out")) || (rc = check_border(border)))
        return rc;
    if ((rc = check_same_axes(*out, *img)) || (rc = check_filter_types(*img, *out))) return rc;
    long long pfirst[IFX_MAXD], plast[IFX_MAXD];
    if ((rc = collect_factors(*img, nfactors, factors, facs, pfirst, plast))) return rc;
    if (border->explicit_pad && (rc = check_padding(border, *img, pfirst, plast))) return rc;
    if (numel(*img) == 0) {
        *nothing = true;
        return IFX_OK;
    }
    if ((rc = check_reflect(border, *img))) return rc;
    const int ct = img->eltype == IFX_F64 ? IFX_F64 : IFX_F32;
    return image_fill(border, img->eltype, ct, fill);
}

bool is_device_array(const void *p) { return is_device_ptr(p); }

int check_device_array(const ifx_array_t &a, int device, const char *name)
{
    const void *p = a.data;
    const size_t bytes = (size_t)numel(a) * elsize(a.eltype);
    cudaPointerAttributes attr;
    if (!p || cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return fail(IFX_ERR_ARGUMENT, "%s: device arrays only (host arrays would need staging buffers)", name);
    }
    if (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)
        return fail(IFX_ERR_ARGUMENT, "%s: device arrays only (host arrays would need staging buffers)", name);
    if (attr.type == cudaMemoryTypeDevice && attr.device != device)
        return fail(IFX_ERR_ARGUMENT, "%s lives on device %d but device %d is current: make the array's "
                    "device current before the call", name, attr.device, device);
    DevRanges r;
    if (!r.holds(p, bytes))
        return fail(IFX_ERR_ARGUMENT, "%s: the array's %zu bytes run past the end of its device allocation",
                    name, bytes);
    return IFX_OK;
}

} // namespace ifx

using namespace ifx;

// =========================================================================
// C ABI
// =========================================================================
extern "C" {

int ifx_abi_version(void) { return IFX_ABI_VERSION; }

const char *ifx_last_error(void) { return t_err.c_str(); }

uint64_t ifx_launch_count(void) { return g_launches.load(); }

int ifx_create(ifx_context_t **ctx, int device)
{
    IFX_RANGE("ifx_create");
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "ctx is NULL");
    *ctx = nullptr;
    int ndev = 0;
    IFX_CUDA(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return fail(IFX_ERR_ARGUMENT, "device %d out of range", device);
    IFX_CUDA(cudaSetDevice(device));
    auto *c = new ifx_context();
    c->device = device;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return fail(IFX_ERR_CUDA, "%s", cudaGetErrorString(e));
    }
    *ctx = c;
    return IFX_OK;
}

int ifx_destroy(ifx_context_t *ctx)
{
    IFX_RANGE("ifx_destroy");
    if (!ctx) return IFX_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto &s : ctx->slots)
        if (s.ptr) cudaFree(s.ptr);
    cudaStreamDestroy(ctx->stream);
    delete ctx;
    return IFX_OK;
}

int ifx_synchronize(ifx_context_t *ctx, void *stream)
{
    IFX_RANGE("ifx_synchronize");
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    IFX_CUDA(cudaSetDevice(ctx->device));
    IFX_CUDA(cudaStreamSynchronize(stream ? (cudaStream_t)stream : ctx->stream));
    if (kernel_timeout_take(ctx->device))
        return fail(IFX_ERR_TIMEOUT, "a kernel's bounded wait for its copies or tensor-core work ran out");
    return IFX_OK;
}

int ifx_debug_force_wait_timeout(ifx_context_t *ctx, int32_t on)
{
    IFX_RANGE("ifx_debug_force_wait_timeout");
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    IFX_CUDA(cudaSetDevice(ctx->device));
    IFX_CUDA(cudaDeviceSynchronize());
    IFX_CUDA(set_first_wait_tma(on != 0));
    IFX_CUDA(set_first_wait_batch(on != 0));
    return IFX_OK;
}

int ifx_padarray(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                 const ifx_border_t *border, void *stream)
{
    IFX_RANGE("ifx_padarray");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_array(out, "out")) || (rc = check_border(border)))
        return rc;
    if (!border->explicit_pad)
        return fail(IFX_ERR_ARGUMENT, "border lacks the proper padding sizes for an array with %d "
                    "dimensions", img->ndim);
    if (out->ndim != img->ndim) return fail(IFX_ERR_DIMENSION, "output dimensionality differs");
    for (int d = 0; d < img->ndim; ++d) {
        if (border->lo[d] < 0 || border->hi[d] < 0)
            return fail(IFX_ERR_ARGUMENT, "negative padding");
        if (out->size[d] != img->size[d] + border->lo[d] + border->hi[d])
            return fail(IFX_ERR_DIMENSION, "output size on axis %d must be lo+n+hi", d + 1);
    }
    if (is8(out->eltype) != is8(img->eltype) && is8(out->eltype))
        return fail(IFX_ERR_UNSUPPORTED, "padarray to an 8-bit eltype from a float eltype");
    if (out->eltype == IFX_I16 || img->eltype == IFX_I16)
        return fail(IFX_ERR_UNSUPPORTED, "Int16 arrays");
    if (numel(*out) == 0) return IFX_OK;
    if (numel(*img) == 0) return fail(IFX_ERR_ERROR, "cannot pad an empty array");
    if ((rc = check_reflect(border, *img))) return rc;
    double fill;
    if ((rc = image_fill(border, img->eltype, out->eltype, &fill))) return rc;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout))) return rc;
    int lo[IFX_MAXD], sz[IFX_MAXD], n[IFX_MAXD];
    for (int d = 0; d < IFX_MAXD; ++d) {
        lo[d] = d < img->ndim ? -(int)border->lo[d] : 0;
        sz[d] = d < img->ndim ? (int)out->size[d] : 1;
        n[d] = d < img->ndim ? (int)img->size[d] : 1;
    }
    PadBoxArgs pa{din, img->eltype, dout, out->eltype, img->ndim, {n[0], n[1], n[2], n[3]},
                  make_box(img->ndim, lo, sz), border->style, fill};
    IFX_CUDA(launch_pad_box(pa, c.s));
    return c.finish();
}


int ifx_imfilter_factored(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                          int32_t nfactors, const ifx_factor_t *factors,
                          const ifx_border_t *border, void *stream)
{
    IFX_RANGE("ifx_imfilter_factored");
    std::vector<Fac> facs;
    double fill;
    bool nothing;
    int rc = factored_prepare(out, img, nfactors, factors, border, facs, &fill, &nothing);
    if (rc || nothing) return rc;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout))) return rc;
    if ((rc = run_cascade(c, *img, din, *out, dout, facs, border, kSlotTmp))) return rc;
    return c.finish();
}

static int fft_geometry(const ifx_array_t &img, const ifx_array_t &out, const int64_t *ksize,
                        const int64_t *kfirst, FftArgs &f, int *lo, int *sz);
static int fft_body(ifx_context_t *ctx, Call &c, const ifx_array_t &img, const void *din, void *dout,
                    const double *kernel, const ifx_border_t *border, FftArgs &f, const int *lo, const int *sz);
static bool fft_cheaper(const ifx_array_t &img, const ifx_array_t &out, const int64_t *ksize, bool tc_ok);

int ifx_imfilter_dense(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                       const double *kernel, const int64_t *ksize, const int64_t *kfirst,
                       const ifx_border_t *border, int32_t method, void *stream)
{
    IFX_RANGE("ifx_imfilter_dense");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_array(out, "out")) || (rc = check_border(border)))
        return rc;
    if ((rc = check_same_axes(*out, *img)) || (rc = check_filter_types(*img, *out))) return rc;
    if (!kernel || !ksize || !kfirst) return fail(IFX_ERR_ARGUMENT, "kernel arrays are NULL");
    const int nd = img->ndim;
    long long kn = 1, pfirst[IFX_MAXD] = {0, 0, 0, 0}, plast[IFX_MAXD] = {0, 0, 0, 0};
    for (int d = 0; d < nd; ++d) {
        if (ksize[d] < 1) return fail(IFX_ERR_ARGUMENT, "empty kernel");
        kn *= ksize[d];
        pfirst[d] = kfirst[d];
        plast[d] = kfirst[d] + ksize[d] - 1;
    }
    if (method < 0 || method > 2) return fail(IFX_ERR_ARGUMENT, "method %d", method);
    if (kn > kMaxDenseTaps && method != 0)
        return fail(IFX_ERR_UNSUPPORTED, "dense kernel with %lld taps (at most %d)", kn, kMaxDenseTaps);
    if (border->explicit_pad && (rc = check_padding(border, *img, pfirst, plast))) return rc;
    if (numel(*img) == 0) return IFX_OK;
    if ((rc = check_reflect(border, *img))) return rc;
    const bool tc_ok = nd <= 2 && dense_tc_supported(img->eltype, (int)ksize[0], nd > 1 ? (int)ksize[1] : 1);
    // The automatic method takes the tensor cores only for sign-definite
    // kernels (smoothing kernels: every weight >= 0, or every weight <= 0).
    // Their BF16 hi/lo products carry errors of about 2^-17 of each term; with
    // weights of one sign these average out, while kernels of mixed signs whose
    // sum nearly cancels reached 1.2e-5 normwise at 31 x 31 (two of twelve
    // N(0,1) kernels normalised to sum 1), above the 1e-5 bound: those take the
    // CUDA cores (reference precision) unless the tensor cores are asked for.
    bool sign_definite = true;
    if (method == 0 && tc_ok) {
        bool pos = false, neg = false;
        for (long long i = 0; i < kn; ++i) {
            pos |= kernel[i] > 0.0;
            neg |= kernel[i] < 0.0;
        }
        sign_definite = !(pos && neg);
    }
    const bool tc_auto = tc_ok && sign_definite;
    if (method == 2 && !tc_ok)
        return fail(IFX_ERR_UNSUPPORTED, "the tensor-core path takes 2-D Float32/8-bit images and "
                    "kernels up to 33 wide and 40 tall");
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout))) return rc;
    // automatic: the FFT when it is estimated well below the direct kernels
    // and every element is finite (the reference's filter_algorithm,
    // src/imfilter.jl:1200-1206, also falls back to FIR for non-finite images)
    if (method == 0 && !border->explicit_pad && (kn > kMaxDenseTaps || fft_cheaper(*img, *out, ksize, tc_auto)) &&
        fft_available()) {
        FftArgs f;
        int lo[IFX_MAXD], sz[IFX_MAXD];
        if (fft_geometry(*img, *out, ksize, kfirst, f, lo, sz) == IFX_OK) {
            void *buf;
            if ((rc = slot_get(ctx, 20, 16, &buf))) return rc;
            IFX_CUDA(cudaMemsetAsync(buf, 0, 16, c.s));
            IFX_CUDA(launch_maxabs(din, img->eltype, numel(*img), (unsigned long long *)buf, c.s));
            unsigned long long h[2] = {0, 0};
            IFX_CUDA(cudaMemcpyAsync(h, buf, 16, cudaMemcpyDeviceToHost, c.s));
            IFX_CUDA(cudaStreamSynchronize(c.s));
            double m;
            memcpy(&m, &h[0], 8);
            if (!h[1] && std::isfinite(m)) {
                if ((rc = fft_body(ctx, c, *img, din, dout, kernel, border, f, lo, sz))) return rc;
                return c.finish();
            }
        }
    }
    if (kn > kMaxDenseTaps)
        return fail(IFX_ERR_UNSUPPORTED, "dense kernel with %lld taps (at most %d for the direct kernels; "
                    "the FFT needs a finite image of at most 3 dimensions)", kn, kMaxDenseTaps);
    const int ct = img->eltype == IFX_F64 ? IFX_F64 : IFX_F32;
    double fill;
    if ((rc = image_fill(border, img->eltype, ct, &fill))) return rc;
    int n[IFX_MAXD];
    for (int d = 0; d < IFX_MAXD; ++d) n[d] = d < nd ? (int)img->size[d] : 1;
    // automatic: tensor cores for sign-definite 2-D kernels of 11 x 11 and larger
    // (faster than the CUDA-core kernel there)
    const bool use_tc = method == 2 || (method == 0 && tc_auto && ksize[0] >= 11 && nd > 1 && ksize[1] >= 11);
    if (use_tc) {
        Dense2dArgs a{din, img->eltype, dout, out->eltype, n[0], nd > 1 ? n[1] : 1,
                      (int)kfirst[0], (int)ksize[0], nd > 1 ? (int)kfirst[1] : 0,
                      nd > 1 ? (int)ksize[1] : 1, kernel, border->style, fill, 0};
        IFX_CUDA(launch_dense_tc(a, c.s, ctx->device));
        if ((rc = c.finish())) return rc;
        if (c.host && kernel_timeout_take(ctx->device))
            return fail(IFX_ERR_TIMEOUT, "tensor-core kernel: a bounded wait ran out");
        return IFX_OK;
    }
    if (nd <= 2 && dense2d_smem_bytes((int)ksize[0], nd > 1 ? (int)ksize[1] : 1, ct == IFX_F64) <=
                       200 * 1024) {
        Dense2dArgs a{din, img->eltype, dout, out->eltype, n[0], nd > 1 ? n[1] : 1,
                      (int)kfirst[0], (int)ksize[0], nd > 1 ? (int)kfirst[1] : 0,
                      nd > 1 ? (int)ksize[1] : 1, kernel, border->style, fill, ct == IFX_F64};
        IFX_CUDA(launch_dense2d(a, c.s));
        return c.finish();
    }
    int blo[IFX_MAXD], bsz[IFX_MAXD];
    for (int d = 0; d < IFX_MAXD; ++d) {
        blo[d] = d < nd ? (int)pfirst[d] : 0;
        bsz[d] = d < nd ? (int)(n[d] + plast[d] - pfirst[d]) : 1;
    }
    Box pb = make_box(nd, blo, bsz);
    void *buf;
    if ((rc = slot_get(ctx, kSlotTmp, (size_t)pb.count * elsize(ct), &buf))) return rc;
    PadBoxArgs pa{din, img->eltype, buf, ct, nd, {n[0], n[1], n[2], n[3]}, pb, border->style, fill};
    IFX_CUDA(launch_pad_box(pa, c.s));
    DenseBoxArgs da;
    memset(&da, 0, sizeof da);
    da.src = buf;
    da.sbox = pb;
    da.out = dout;
    da.out_type = out->eltype;
    da.obox = image_box(*img);
    da.nd = nd;
    for (int d = 0; d < IFX_MAXD; ++d) {
        da.ksize[d] = d < nd ? (int)ksize[d] : 1;
        da.kfirst[d] = d < nd ? (int)kfirst[d] : 0;
    }
    da.K = kernel;
    da.compute_f64 = ct == IFX_F64;
    IFX_CUDA(launch_dense_box(da, c.s));
    return c.finish();
}

int ifx_imfilter_laplacian(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                           const int32_t *flags, const ifx_border_t *border, void *stream)
{
    IFX_RANGE("ifx_imfilter_laplacian");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_array(out, "out")) || (rc = check_border(border)))
        return rc;
    if ((rc = check_same_axes(*out, *img))) return rc;
    if (!flags) return fail(IFX_ERR_ARGUMENT, "flags is NULL");
    const int it = img->eltype, ot = out->eltype;
    const bool ok = (it == IFX_F32 || it == IFX_F64) ? (ot == IFX_F32 || ot == IFX_F64)
                    : is8(it) ? (ot == IFX_F32 || ot == IFX_F64 || ot == IFX_I16) : false;
    if (!ok) return fail(IFX_ERR_UNSUPPORTED, "Laplacian from eltype %d to %d", it, ot);
    long long pf[IFX_MAXD] = {0, 0, 0, 0}, pl[IFX_MAXD] = {0, 0, 0, 0};
    for (int d = 0; d < img->ndim; ++d) {
        pf[d] = flags[d] ? -1 : 0;
        pl[d] = flags[d] ? 1 : 0;
    }
    if (border->explicit_pad && (rc = check_padding(border, *img, pf, pl))) return rc;
    if (numel(*img) == 0) return IFX_OK;
    if ((rc = check_reflect(border, *img))) return rc;
    double fill;
    if ((rc = image_fill(border, it, ot, &fill))) return rc;
    if (it == IFX_N0F8 && ot == IFX_F32)        // Float32(N0f8): code/255 rounded once in FP32
        fill = (double)((float)std::nearbyint(fill * 255.0) / 255.0f);
    if (ot == IFX_I16 && fill != std::nearbyint(fill))
        return fail(IFX_ERR_ARGUMENT, "Cannot convert elements of border=Fill(%g)", fill);
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout))) return rc;
    LaplacianArgs a;
    memset(&a, 0, sizeof a);
    a.img = din;
    a.in_type = it;
    a.out = dout;
    a.out_type = ot;
    a.nd = img->ndim;
    for (int d = 0; d < IFX_MAXD; ++d) {
        a.n[d] = d < img->ndim ? (int)img->size[d] : 1;
        a.flags[d] = d < img->ndim ? (flags[d] != 0) : 0;
    }
    a.style = border->style;
    a.fill = fill;
    IFX_CUDA(launch_laplacian(a, c.s));
    return c.finish();
}

int ifx_imgradients(ifx_context_t *ctx, ifx_array_t *outs, const ifx_array_t *img,
                    const double *deriv, const double *smooth, int32_t length, int64_t first,
                    const int32_t *extended, const ifx_border_t *border, void *stream)
{
    IFX_RANGE("ifx_imgradients");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_border(border))) return rc;
    if (!outs || !deriv || !smooth || !extended) return fail(IFX_ERR_ARGUMENT, "NULL argument");
    if (length < 1 || length > IFX_MAX_TAPS) return fail(IFX_ERR_UNSUPPORTED, "gradient length");
    const int nd = img->ndim;
    for (int d = 0; d < nd; ++d) {
        if ((rc = check_array(&outs[d], "outs[d]")) || (rc = check_same_axes(outs[d], *img)) ||
            (rc = check_filter_types(*img, outs[d])))
            return rc;
    }
    // per-gradient factor lists (gradfactors, src/kernelfactors.jl:598-604)
    static const double one = 1.0;
    std::vector<std::vector<ifx_factor_t>> lists(nd);
    for (int d = 0; d < nd; ++d)
        for (int e = 0; e < nd; ++e) {
            ifx_factor_t f;
            f.axis = e;
            if (!extended[e]) {
                f.length = 1;
                f.first = 0;
                f.weights = &one;
            } else {
                f.length = length;
                f.first = first;
                f.weights = e == d ? deriv : smooth;
            }
            lists[d].push_back(f);
        }
    for (int d = 0; d < nd; ++d) {
        std::vector<Fac> facs;
        long long pfirst[IFX_MAXD], plast[IFX_MAXD];
        if ((rc = collect_factors(*img, nd, lists[d].data(), facs, pfirst, plast))) return rc;
        if (border->explicit_pad && (rc = check_padding(border, *img, pfirst, plast))) return rc;
    }
    if (numel(*img) == 0) return IFX_OK;
    if ((rc = check_reflect(border, *img))) return rc;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    if ((rc = c.input(*img, &din))) return rc;
    // 3-D, 3-tap pair on every axis, one output eltype: the fused sweep
    if (nd == 3 && length == 3 && first == -1 && extended[0] && extended[1] && extended[2] &&
        outs[1].eltype == outs[0].eltype && outs[2].eltype == outs[0].eltype && img->eltype != IFX_I16) {
        Grad3dArgs g{};
        g.img = din;
        g.in_type = img->eltype;
        for (int d = 0; d < 3; ++d)
            if ((rc = c.output(outs[d], &g.out[d]))) return rc;
        g.out_type = outs[0].eltype;
        g.nx = (int)img->size[0];
        g.ny = (int)img->size[1];
        g.nz = (int)img->size[2];
        for (int t = 0; t < 3; ++t) {
            g.d[t] = deriv[t];
            g.s[t] = smooth[t];
        }
        g.compute_f64 = img->eltype == IFX_F64;
        g.style = border->style;
        if ((rc = image_fill(border, img->eltype, g.compute_f64 ? IFX_F64 : IFX_F32, &g.fill))) return rc;
        IFX_CUDA(launch_grad3d(g, c.s));
        return c.finish();
    }
    for (int d = 0; d < nd; ++d) {
        void *dout;
        if ((rc = c.output(outs[d], &dout))) return rc;
        std::vector<Fac> facs;
        long long pfirst[IFX_MAXD], plast[IFX_MAXD];
        collect_factors(*img, nd, lists[d].data(), facs, pfirst, plast);
        if ((rc = run_cascade(c, *img, din, outs[d], dout, facs, border, kSlotTmp))) return rc;
    }
    return c.finish();
}

// mapwindow's copy_win! builds padindex tables relative to window-intersect-
// image; with reflect a length-1 intersection is the reference's DivideError.
static int check_window_reflect(const ifx_border_t *b, const ifx_array_t &img, const int *wf,
                                const int *wl)
{
    if (!b || b->style != IFX_REFLECT) return IFX_OK;
    bool edges = false;
    for (int d = 0; d < img.ndim; ++d)
        if (wf[d] < 0 || wf[d] + wl[d] - 1 > 0) edges = true;
    if (!edges) return IFX_OK;
    for (int d = 0; d < img.ndim; ++d) {
        long long n = img.size[d], a = wf[d], b2 = wf[d] + wl[d] - 1;
        long long m = n;
        if (b2 + 1 < m) m = b2 + 1;
        if (1 - a < m) m = 1 - a;
        if (wl[d] < m) m = wl[d];
        if (m <= 1)
            return fail(IFX_ERR_ERROR, "DivideError: integer division error (reflect window of "
                        "length 1 on axis %d)", d + 1);
    }
    return IFX_OK;
}

int ifx_mapwindow_median(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                         const int64_t *wfirst, const int64_t *wlen, const ifx_border_t *border,
                         void *stream)
{
    IFX_RANGE("ifx_mapwindow_median");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_array(out, "out")) || (rc = check_border(border)))
        return rc;
    if ((rc = check_same_axes(*out, *img))) return rc;
    if (!wfirst || !wlen) return fail(IFX_ERR_ARGUMENT, "window is NULL");
    const int nd = img->ndim;
    int wf[IFX_MAXD] = {0, 0, 0, 0}, wl[IFX_MAXD] = {1, 1, 1, 1};
    long long m = 1;
    for (int d = 0; d < nd; ++d) {
        if (wlen[d] < 1) return fail(IFX_ERR_ARGUMENT, "empty window");
        if (wfirst[d] > 0 || wfirst[d] + wlen[d] - 1 < 0)
            return fail(IFX_ERR_UNSUPPORTED, "windows must contain offset 0");
        wf[d] = (int)wfirst[d];
        wl[d] = (int)wlen[d];
        m *= wlen[d];
    }
    if (m > 256) return fail(IFX_ERR_UNSUPPORTED, "median window of %lld values (at most 256)", m);
    const int it = img->eltype, ot = out->eltype;
    if (it == IFX_I16 || ot == IFX_I16) return fail(IFX_ERR_UNSUPPORTED, "Int16 median");
    if (!is8(it) && is8(ot)) return fail(IFX_ERR_UNSUPPORTED, "float median into 8-bit output");
    if (numel(*img) == 0) return IFX_OK;
    if ((rc = check_window_reflect(border, *img, wf, wl))) return rc;
    double fill;
    if ((rc = fill_for(border, it, &fill))) return rc;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout))) return rc;
    MedianArgs a;
    memset(&a, 0, sizeof a);
    a.img = din;
    a.in_type = it;
    a.out = dout;
    a.out_type = ot;
    a.nd = nd;
    for (int d = 0; d < IFX_MAXD; ++d) {
        a.n[d] = d < nd ? (int)img->size[d] : 1;
        a.wfirst[d] = wf[d];
        a.wlen[d] = wl[d];
    }
    a.style = border->style;
    a.fill = fill;
    IFX_CUDA(launch_median(a, c.s));
    return c.finish();
}

int ifx_mapwindow_extrema(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                          const int64_t *wfirst, const int64_t *wlen, const ifx_border_t *border,
                          int32_t which, void *stream)
{
    IFX_RANGE("ifx_mapwindow_extrema");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_array(out, "out"))) return rc;
    if (border && (rc = check_border(border))) return rc;
    if ((rc = check_same_axes(*out, *img))) return rc;
    if (which < 0 || which > 2) return fail(IFX_ERR_ARGUMENT, "which must be 0, 1 or 2");
    if (!wlen) return fail(IFX_ERR_ARGUMENT, "window is NULL");
    if (out->eltype != img->eltype)
        return fail(IFX_ERR_ARGUMENT, "extrema output eltype must equal the input eltype");
    if (img->eltype == IFX_I16) return fail(IFX_ERR_UNSUPPORTED, "Int16 extrema");
    const int nd = img->ndim;
    int a0[IFX_MAXD], a1[IFX_MAXD], wf[IFX_MAXD], wl[IFX_MAXD];
    for (int d = 0; d < nd; ++d) {
        if (wlen[d] < 1) return fail(IFX_ERR_ARGUMENT, "empty window");
        if (border) {
            if (!wfirst) return fail(IFX_ERR_ARGUMENT, "window first is NULL");
            a0[d] = (int)wfirst[d];
            a1[d] = (int)(wfirst[d] + wlen[d] - 1);
            if (a0[d] > 0 || a1[d] < 0) return fail(IFX_ERR_UNSUPPORTED, "windows must contain offset 0");
        } else {
            const int w = (int)wlen[d];
            a0[d] = -(w >> 1);
            a1[d] = w - 1 - (w >> 1);
        }
        wf[d] = a0[d];
        wl[d] = a1[d] - a0[d] + 1;
    }
    if (numel(*img) == 0) return IFX_OK;
    if ((rc = check_window_reflect(border, *img, wf, wl))) return rc;
    double fill = 0.0;
    const int use_fill = border && border->style == IFX_FILL;
    if (use_fill && (rc = fill_for(border, img->eltype, &fill))) return rc;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const size_t es = elsize(img->eltype);
    const size_t N = (size_t)numel(*img);
    const void *din;
    void *dout;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout, which == 0 ? 2 * N * es : 0)))
        return rc;
    if (nd == 2 && (img->eltype == IFX_N0F8 || img->eltype == IFX_U8) && wl[0] == wl[1] && a0[0] == a0[1]) {
        cudaError_t e;
        if (launch_extrema2d_u8(din, dout, (int)img->size[0], (int)img->size[1], wl[0], a0[0], use_fill, fill,
                                which, c.s, &e)) {
            IFX_CUDA(e);
            return c.finish();
        }
    }
    void *planes[4] = {nullptr, nullptr, nullptr, nullptr};
    if (nd > 1)
        for (int i = 0; i < (nd > 2 ? 4 : 2); ++i)
            if ((rc = slot_get(ctx, kSlotTmp + i, N * es, &planes[i]))) return rc;
    const void *smin = din, *smax = din;
    for (int d = 0; d < nd; ++d) {
        const bool last = d == nd - 1;
        ExtremaPassArgs a;
        memset(&a, 0, sizeof a);
        a.src_min = smin;
        a.src_max = smax;
        a.type = img->eltype;
        a.nd = nd;
        for (int e = 0; e < IFX_MAXD; ++e) a.n[e] = e < nd ? (int)img->size[e] : 1;
        a.axis = d;
        a.a0 = a0[d];
        a.a1 = a1[d];
        a.use_fill = use_fill;
        a.fill = fill;
        a.want_min = which != 2;
        a.want_max = which != 1;
        if (last) {
            a.dst_interleaved = which == 0;
            a.dst_min = dout;
            a.dst_max = dout;
        } else {
            void *pm = planes[(d & 1) * 2], *px = planes[(d & 1) * 2 + 1];
            a.dst_min = pm;
            a.dst_max = px;
            smin = pm;
            smax = px;
        }
        IFX_CUDA(launch_extrema_pass(a, c.s));
    }
    return c.finish();
}

int ifx_batch_run(ifx_context_t *ctx, const ifx_request_t *reqs, int32_t n, int64_t *tiles,
                  void *stream)
{
    IFX_RANGE("ifx_batch_run");
    if (n < 0 || (n > 0 && !reqs)) return fail(IFX_ERR_ARGUMENT, "bad request list");
    if (tiles) *tiles = 0;
    std::vector<BatchItem> items((size_t)n);
    DevRanges ranges;
    for (int i = 0; i < n; ++i) {
        int rc = request_item(reqs[i], i, true, items[i], &ranges);
        if (rc) return rc;
    }
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    IFX_CUDA(cudaSetDevice(ctx->device));
    long long t = 0;
    IFX_CUDA(launch_batch(ctx->device, items.data(), n, stream ? (cudaStream_t)stream : ctx->stream, &t));
    if (tiles) *tiles = t;
    return IFX_OK;
}

struct ifx_batch_plan {
    int device;
    void *impl;
};

int ifx_batch_plan_create(ifx_context_t *ctx, const ifx_request_t *reqs, int32_t n,
                          ifx_batch_plan_t **plan)
{
    IFX_RANGE("ifx_batch_plan_create");
    if (!plan) return fail(IFX_ERR_ARGUMENT, "plan is NULL");
    *plan = nullptr;
    if (n < 0 || (n > 0 && !reqs)) return fail(IFX_ERR_ARGUMENT, "bad request list");
    std::vector<BatchItem> items((size_t)n);
    DevRanges ranges;
    for (int i = 0; i < n; ++i) {
        int rc = request_item(reqs[i], i, true, items[i], &ranges);
        if (rc) return rc;
    }
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    IFX_CUDA(cudaSetDevice(ctx->device));
    void *impl = nullptr;
    IFX_CUDA(plan_create(ctx->device, items.data(), n, &impl));
    *plan = new ifx_batch_plan{ctx->device, impl};
    return IFX_OK;
}

int ifx_batch_plan_launch(ifx_batch_plan_t *plan, int64_t *tiles, void *stream)
{
    IFX_RANGE("ifx_batch_plan_launch");
    if (!plan) return fail(IFX_ERR_ARGUMENT, "plan is NULL");
    long long t = 0;
    IFX_CUDA(plan_launch(plan->impl, (cudaStream_t)stream, &t));
    if (tiles) *tiles = t;
    return IFX_OK;
}

int ifx_batch_plan_destroy(ifx_batch_plan_t *plan)
{
    IFX_RANGE("ifx_batch_plan_destroy");
    if (!plan) return IFX_OK;
    cudaSetDevice(plan->device);
    plan_destroy(plan->impl);
    delete plan;
    return IFX_OK;
}

// ---------------------------------------------------------------- autotuner
int ifx_autotune(ifx_context_t *ctx, int32_t enable, const char *cache_path)
{
    IFX_RANGE("ifx_autotune");
    (void)ctx;
    autotune_set(enable != 0, cache_path);
    return IFX_OK;
}

int ifx_autotune_choice(ifx_context_t *ctx, int32_t in_type, int32_t out_type, int32_t kx, int32_t ky,
                        int32_t fill, int64_t nx, int64_t ny, int32_t *x_first, int32_t *variant, double *ms)
{
    IFX_RANGE("ifx_autotune_choice");
    (void)ctx;
    if (!x_first || !variant) return fail(IFX_ERR_ARGUMENT, "NULL output");
    TuneChoice ch;
    if (!autotune_lookup_key(TUNE_SEP2D, in_type, out_type, kx, ky, 1, fill, nx, ny, 1, &ch))
        return fail(IFX_ERR_ARGUMENT, "no tuned choice for this key");
    *x_first = ch.x_first;
    *variant = ch.variant;
    if (ms) *ms = ch.ms;
    return IFX_OK;
}

static int check_tune_key(int32_t path, const int32_t *taps, const int64_t *size)
{
    if (path != IFX_TUNE_SEP2D && path != IFX_TUNE_SEP3D) return fail(IFX_ERR_ARGUMENT, "unknown tuner path");
    if (!taps || !size) return fail(IFX_ERR_ARGUMENT, "NULL key");
    for (int d = 0; d < 3; ++d)
        if (taps[d] < 1 || size[d] < 0) return fail(IFX_ERR_ARGUMENT, "bad key: taps >= 1, sizes >= 0");
    return IFX_OK;
}

int ifx_autotune_lookup(ifx_context_t *ctx, int32_t path, int32_t in_type, int32_t out_type, const int32_t *taps,
                        int32_t fill, const int64_t *size, ifx_tune_choice_t *choice)
{
    IFX_RANGE("ifx_autotune_lookup");
    (void)ctx;
    int rc;
    if ((rc = check_tune_key(path, taps, size))) return rc;
    if (!choice) return fail(IFX_ERR_ARGUMENT, "NULL output");
    TuneChoice ch;
    if (!autotune_lookup_key(path, in_type, out_type, taps[0], taps[1], taps[2], fill, size[0], size[1], size[2],
                             &ch))
        return fail(IFX_ERR_ARGUMENT, "no tuned choice for this key");
    choice->variant = ch.variant;
    choice->x_first = ch.x_first;
    choice->tile_w = ch.tile_w;
    choice->tile_h = ch.tile_h;
    choice->depth = ch.depth;
    choice->ms = ch.ms;
    return IFX_OK;
}

int ifx_autotune_pin(ifx_context_t *ctx, int32_t path, int32_t in_type, int32_t out_type, const int32_t *taps,
                     int32_t fill, const int64_t *size, const ifx_tune_choice_t *choice)
{
    IFX_RANGE("ifx_autotune_pin");
    (void)ctx;
    int rc;
    if ((rc = check_tune_key(path, taps, size))) return rc;
    if (!choice) return fail(IFX_ERR_ARGUMENT, "NULL choice");
    const ifx_tune_choice_t &c = *choice;
    if (c.variant != 1 && c.variant != 2) return fail(IFX_ERR_ARGUMENT, "variant must be 1 or 2");
    if (c.x_first != 0 && c.x_first != 1) return fail(IFX_ERR_ARGUMENT, "x_first must be 0 or 1");
    if (c.tile_w < 0 || c.tile_h < 0 || c.depth < 0) return fail(IFX_ERR_ARGUMENT, "negative tile or depth");
    autotune_pin_key(path, in_type, out_type, taps[0], taps[1], taps[2], fill, size[0], size[1], size[2],
                     TuneChoice{c.variant, c.x_first, c.tile_w, c.tile_h, c.depth, (float)c.ms});
    return IFX_OK;
}

// The batched engine's key as its requests hold it: factored (taps x, taps y),
// gradients (3, 3), Laplacian and median no taps, the window for medians only.
static int batch_tune_key(int32_t op, int32_t in_type, int32_t out_type, int32_t *kx, int32_t *ky, int32_t *win)
{
    if (op < IFX_OP_FACTORED2D || op > IFX_OP_MEDIAN2D) return fail(IFX_ERR_ARGUMENT, "unknown op %d", op);
    if (in_type != IFX_F32 && !is8(in_type)) return fail(IFX_ERR_ARGUMENT, "batched images are Float32 or 8-bit");
    if (out_type != IFX_F32 && out_type != IFX_F64) return fail(IFX_ERR_ARGUMENT, "outputs are Float32 or Float64");
    if (op == IFX_OP_GRADIENTS2D) *kx = *ky = 3;
    else if (op != IFX_OP_FACTORED2D) *kx = *ky = 0;
    if (op != IFX_OP_MEDIAN2D) *win = 0;
    return IFX_OK;
}

int ifx_batch_autotune_lookup(ifx_context_t *ctx, int32_t op, int32_t in_type, int32_t out_type, int32_t kx,
                              int32_t ky, int32_t window, ifx_tune_choice_t *choice)
{
    IFX_RANGE("ifx_batch_autotune_lookup");
    (void)ctx;
    int rc;
    if ((rc = batch_tune_key(op, in_type, out_type, &kx, &ky, &window))) return rc;
    if (!choice) return fail(IFX_ERR_ARGUMENT, "NULL output");
    TuneChoice ch;
    if (!autotune_lookup_batch(op, in_type, out_type, kx, ky, window, &ch))
        return fail(IFX_ERR_ARGUMENT, "no tuned choice for this key");
    *choice = ifx_tune_choice_t{ch.variant, ch.x_first, ch.tile_w, ch.tile_h, ch.depth, ch.ms};
    return IFX_OK;
}

int ifx_batch_autotune_pin(ifx_context_t *ctx, int32_t op, int32_t in_type, int32_t out_type, int32_t kx,
                           int32_t ky, int32_t window, const ifx_tune_choice_t *choice)
{
    IFX_RANGE("ifx_batch_autotune_pin");
    (void)ctx;
    int rc;
    if ((rc = batch_tune_key(op, in_type, out_type, &kx, &ky, &window))) return rc;
    if (!choice) return fail(IFX_ERR_ARGUMENT, "NULL choice");
    if (choice->tile_w < 0 || choice->tile_h < 0) return fail(IFX_ERR_ARGUMENT, "negative tile");
    autotune_store_batch(op, in_type, out_type, kx, ky, window,
                         TuneChoice{0, 0, choice->tile_w, choice->tile_h, 0, (float)choice->ms}, false);
    return IFX_OK;
}

int ifx_autotune_clear(ifx_context_t *ctx)
{
    IFX_RANGE("ifx_autotune_clear");
    (void)ctx;
    autotune_clear();
    return IFX_OK;
}

// ---------------------------------------------------------------- Algorithm.IIR()
int ifx_imfilter_iir(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img, int32_t nfactors,
                     const ifx_iir_t *factors, const ifx_border_t *border, void *stream)
{
    IFX_RANGE("ifx_imfilter_iir");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_array(out, "out")) || (rc = check_border(border)))
        return rc;
    if ((rc = check_same_axes(*out, *img))) return rc;
    if (img->eltype == IFX_I16) return fail(IFX_ERR_UNSUPPORTED, "Int16 images are not supported");
    if (out->eltype != IFX_F32 && out->eltype != IFX_F64)
        return fail(IFX_ERR_UNSUPPORTED, "IIR filtering writes Float32 or Float64 outputs");
    if (nfactors < 0 || nfactors > 64 || (nfactors > 0 && !factors))
        return fail(IFX_ERR_ARGUMENT, "nfactors %d", nfactors);
    const int nd = img->ndim;
    for (int f = 0; f < nfactors; ++f) {
        const int ax = factors[f].axis;
        if (ax < 0 || ax >= nd)
            return fail(IFX_ERR_DIMENSION, "cannot have more kernels than dimensions (factor along axis %d of a "
                        "%d-d image)", ax + 1, nd);
    }
    const long long total = numel(*img);
    if (total == 0) return IFX_OK;
    for (int f = 0; f < nfactors; ++f) {
        const int ax = factors[f].axis;
        if (img->size[ax] <= 3)
            return fail(IFX_ERR_DIMENSION, "size %lld of img along dimension %d is too small for filtering "
                        "with IIR kernel of length 3", (long long)img->size[ax], ax + 1);
    }
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout))) return rc;
    if (nfactors == 0) {                                  // every factor was a copy: convert
        PadBoxArgs pa{din, img->eltype, dout, out->eltype, nd, {0, 0, 0, 0}, image_box(*img), IFX_REPLICATE, 0.0};
        for (int d = 0; d < IFX_MAXD; ++d) pa.n[d] = d < nd ? (int)img->size[d] : 1;
        IFX_CUDA(launch_pad_box(pa, c.s));
        return c.finish();
    }
    long long st[IFX_MAXD];
    long long s = 1;
    for (int d = 0; d < IFX_MAXD; ++d) {
        st[d] = s;
        s *= d < nd ? img->size[d] : 1;
    }
    for (int f = 0; f < nfactors; ++f) {
        const ifx_iir_t &k = factors[f];
        IirArgs a;
        memset(&a, 0, sizeof a);
        a.src = f == 0 ? din : dout;
        a.src_type = f == 0 ? img->eltype : out->eltype;
        a.dst = dout;
        a.dst_type = out->eltype;
        a.L = img->size[k.axis];
        a.inner = st[k.axis];
        a.lines = total / a.L;
        for (int j = 0; j < 3; ++j) {
            a.a[j] = k.a[j];
            a.b[j] = k.b[j];
        }
        for (int j = 0; j < 9; ++j) a.M[j] = k.M[j];
        a.scale = k.scale;
        // 1 - sum(a) and 1 - sum(b) in the kernel's float type
        a.om_a = k.coef_f32 ? (double)(1.0f - (float)k.asum) : 1.0 - k.asum;
        a.om_b = k.coef_f32 ? (double)(1.0f - (float)k.bsum) : 1.0 - k.bsum;
        a.edge = border->style == IFX_FILL;
        a.fill = border->style == IFX_FILL ? border->fill_value : 0.0;
        a.compute_f64 = out->eltype == IFX_F64 || !k.coef_f32;
        IFX_CUDA(launch_iir(a, c.s));
    }
    return c.finish();
}

// ---------------------------------------------------------------- Algorithm.FFT()
// The padfft sizes (src/border.jl:245-248) and the padded box of an FFT
// filter; 0 or an error code.
static int fft_geometry(const ifx_array_t &img, const ifx_array_t &out, const int64_t *ksize,
                        const int64_t *kfirst, FftArgs &f, int *lo, int *sz)
{
    const int nd = img.ndim;
    if (nd > 3) return fail(IFX_ERR_UNSUPPORTED, "Algorithm.FFT() on more than 3 dimensions");
    f = FftArgs{};
    f.nd = nd;
    f.kn = 1;
    f.Ptotal = 1;
    f.total = numel(img);
    for (int d = 0; d < IFX_MAXD; ++d) {
        f.n[d] = d < nd ? img.size[d] : 1;
        f.ksize[d] = d < nd ? (int)ksize[d] : 1;
        if (f.ksize[d] < 1) return fail(IFX_ERR_ARGUMENT, "empty kernel");
        f.P[d] = d < nd ? fft_size(f.n[d], f.ksize[d]) : 1;
        if (f.P[d] > (1ll << 30)) return fail(IFX_ERR_UNSUPPORTED, "FFT size too large");
        lo[d] = d < nd ? (int)kfirst[d] : 0;               // padded box: image indices kfirst .. kfirst+P-1
        sz[d] = (int)f.P[d];
        f.kn *= f.ksize[d];
        f.Ptotal *= f.P[d];
    }
    f.Pc = f.Ptotal / f.P[0] * (f.P[0] / 2 + 1);
    f.out_type = out.eltype;
    f.compute_f64 = out.eltype == IFX_F64;
    if (out.eltype != IFX_F32 && out.eltype != IFX_F64)
        return fail(IFX_ERR_UNSUPPORTED, "Algorithm.FFT() writes Float32 or Float64 outputs");
    return IFX_OK;
}

// Pad, transform, multiply, invert and crop on the call's stream (the
// arguments are checked and the context is locked by the caller).
static int fft_body(ifx_context_t *ctx, Call &c, const ifx_array_t &img, const void *din, void *dout,
                    const double *kernel, const ifx_border_t *border, FftArgs &f, const int *lo, const int *sz)
{
    int rc;
    if (!fft_available()) return fail(IFX_ERR_UNSUPPORTED, "Algorithm.FFT() needs cuFFT (libcufft), not found");
    const int ct = f.compute_f64 ? IFX_F64 : IFX_F32;
    const size_t es = elsize(ct), cs = 2 * es;
    double fill = 0.0;
    if ((rc = image_fill(border, img.eltype, ct, &fill))) return rc;
    f.out = dout;
    void *kd;
    if ((rc = slot_get(ctx, kSlotTmp, (size_t)f.Ptotal * es, &f.padded)) ||
        (rc = slot_get(ctx, kSlotTmp + 1, (size_t)f.Ptotal * es, &f.krn)) ||
        (rc = slot_get(ctx, kSlotTmp + 2, (size_t)f.Pc * cs, &f.specA)) ||
        (rc = slot_get(ctx, kSlotTmp + 3, (size_t)f.Pc * cs, &f.specK)) ||
        (rc = slot_get(ctx, kSlotTmp + 4, (size_t)f.kn * sizeof(double), &kd)))
        return rc;
    IFX_CUDA(cudaMemcpyAsync(kd, kernel, (size_t)f.kn * sizeof(double), cudaMemcpyHostToDevice, c.s));
    f.Kdev = (const double *)kd;
    int n[IFX_MAXD];
    for (int d = 0; d < IFX_MAXD; ++d) n[d] = (int)f.n[d];
    PadBoxArgs pa{din, img.eltype, f.padded, ct, f.nd, {n[0], n[1], n[2], n[3]}, make_box(f.nd, lo, sz),
                  border->style, fill};
    IFX_CUDA(launch_pad_box(pa, c.s));
    const int r = launch_fft(f, c.s);
    if (r == -1) return fail(IFX_ERR_CUDA, "cuFFT plan or transform failed");
    if (r == -2) IFX_CUDA(cudaGetLastError());
    if (r) return fail(IFX_ERR_UNSUPPORTED, "Algorithm.FFT(): unsupported eltypes");
    return IFX_OK;
}

// Automatic choice between the direct kernels and the FFT for a dense kernel:
// estimated times from the measured rates of both on GB300 (direct F32 about
// 16e12 taps/s on CUDA cores, FP64 about 1e12; cuFFT about 37 ps per padded
// element in F32, twice that in F64, plus about 30 us of launches), with the
// FFT taken only when it is estimated at under half the direct time.
static bool fft_cheaper(const ifx_array_t &img, const ifx_array_t &out, const int64_t *ksize, bool tc_ok)
{
    if (img.ndim > 3 || (out.eltype != IFX_F32 && out.eltype != IFX_F64)) return false;
    double npix = 1, taps = 1, P = 1;
    for (int d = 0; d < img.ndim; ++d) {
        npix *= (double)img.size[d];
        taps *= (double)ksize[d];
        P *= (double)fft_size(img.size[d], ksize[d]);
    }
    const bool f64 = img.eltype == IFX_F64;
    double direct = npix * taps / (f64 ? 1.0e12 : 16.0e12);
    if (tc_ok && !f64 && ksize[0] >= 11 && img.ndim > 1 && ksize[1] >= 11) direct *= 0.45;   // tensor cores
    const double fft = 30e-6 + P * (out.eltype == IFX_F64 ? 74e-12 : 37e-12);
    return fft < 0.5 * direct;
}

int ifx_imfilter_fft(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img, const double *kernel,
                     const int64_t *ksize, const int64_t *kfirst, const ifx_border_t *border, void *stream)
{
    IFX_RANGE("ifx_imfilter_fft");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_array(out, "out")) || (rc = check_border(border)))
        return rc;
    if ((rc = check_same_axes(*out, *img)) || (rc = check_filter_types(*img, *out))) return rc;
    if (!kernel || !ksize || !kfirst) return fail(IFX_ERR_ARGUMENT, "kernel arrays are NULL");
    if (border->style == IFX_FILL && border->explicit_pad)
        return fail(IFX_ERR_UNSUPPORTED, "Algorithm.FFT() pads to its own sizes: give Fill(v) without widths");
    if (border->style != IFX_FILL && border->explicit_pad)
        return fail(IFX_ERR_UNSUPPORTED, "Algorithm.FFT() pads to its own sizes: give Pad(style) without widths");
    FftArgs f;
    int lo[IFX_MAXD], sz[IFX_MAXD];
    if ((rc = fft_geometry(*img, *out, ksize, kfirst, f, lo, sz))) return rc;
    if (f.total == 0) return IFX_OK;
    if ((rc = check_reflect(border, *img))) return rc;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout))) return rc;
    if ((rc = fft_body(ctx, c, *img, din, dout, kernel, border, f, lo, sz))) return rc;
    return c.finish();
}

// ---------------------------------------------------------------- blob_LoG pieces
int ifx_imfilter_factored_sum(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img, int32_t nterms,
                              int32_t nfactors, const ifx_factor_t *factors, double scale,
                              const ifx_border_t *border, void *stream)
{
    IFX_RANGE("ifx_imfilter_factored_sum");
    int rc;
    if (nterms < 1 || nfactors < 1 || !factors) return fail(IFX_ERR_ARGUMENT, "no terms");
    if ((rc = check_array(out, "out"))) return rc;
    if (out->eltype != IFX_F32 && out->eltype != IFX_F64)
        return fail(IFX_ERR_UNSUPPORTED, "sums of separable terms write Float32 or Float64");
    std::vector<std::vector<Fac>> terms(nterms);
    double fill = 0.0;
    for (int t = 0; t < nterms; ++t) {
        bool nothing = false;
        if ((rc = factored_prepare(out, img, nfactors, factors + (size_t)t * nfactors, border, terms[t], &fill,
                                   &nothing)))
            return rc;
        if (nothing) {
            if (numel(*img) == 0) return IFX_OK;
            return fail(IFX_ERR_UNSUPPORTED, "term %d is a copy: give it as a 1-tap factor", t);
        }
    }
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout, *tmp = nullptr;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*out, &dout))) return rc;
    const size_t bytes = (size_t)numel(*out) * elsize(out->eltype);
    if (nterms > 1 && (rc = slot_get(ctx, kSlotTmp + 8, bytes, &tmp))) return rc;
    for (int t = 0; t < nterms; ++t) {
        if ((rc = run_cascade(c, *img, din, *out, t == 0 ? dout : tmp, terms[t], border, kSlotTmp))) return rc;
        if (t > 0) IFX_CUDA(launch_sum_scale(dout, tmp, out->eltype, numel(*out), scale, t == nterms - 1, c.s));
    }
    if (nterms == 1 && scale != 1.0) {       // one term: scale it (sum with a zero term)
        if ((rc = slot_get(ctx, kSlotTmp + 8, bytes, &tmp))) return rc;
        IFX_CUDA(cudaMemsetAsync(tmp, 0, bytes, c.s));
        IFX_CUDA(launch_sum_scale(dout, tmp, out->eltype, numel(*out), scale, 1, c.s));
    }
    return c.finish();
}

int ifx_findlocalextrema(ifx_context_t *ctx, const ifx_array_t *img, const int32_t *window, const int32_t *edges,
                         int32_t minima, int64_t *indices, double *values, int64_t capacity, int64_t *count,
                         void *stream)
{
    IFX_RANGE("ifx_findlocalextrema");
    int rc;
    if ((rc = check_array(img, "img"))) return rc;
    if (!window || !edges || !count || (capacity > 0 && (!indices || !values)))
        return fail(IFX_ERR_ARGUMENT, "NULL argument");
    if (img->eltype == IFX_I16) return fail(IFX_ERR_UNSUPPORTED, "Int16 images are not supported");
    LeArgs a{};
    a.eltype = img->eltype;
    a.nd = img->ndim;
    a.total = numel(*img);
    a.minima = minima != 0;
    for (int d = 0; d < IFX_MAXD; ++d) a.n[d] = 1;
    for (int d = 0; d < a.nd; ++d) {
        if (window[d] < 1) return fail(IFX_ERR_ARGUMENT, "window sizes must be positive");
        a.n[d] = img->size[d];
        a.half[d] = window[d] >> 1;
        a.lo[d] = edges[d] ? 0 : 1;                          // clippedinds(R0, !edges)
        a.hi[d] = (int)(img->size[d] - 1 - (edges[d] ? 0 : 1));
    }
    *count = 0;
    if (a.total == 0) return IFX_OK;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    if ((rc = c.input(*img, &a.img))) return rc;
    const long long nb = localextrema_blocks(a.total);
    void *counts, *total, *didx, *dval;
    const long long cap = capacity > 0 ? capacity : 1;
    if ((rc = slot_get(ctx, 19, (size_t)nb * 8, &counts)) || (rc = slot_get(ctx, 20, 16, &total)) ||
        (rc = slot_get(ctx, 21, (size_t)cap * 8, &didx)) || (rc = slot_get(ctx, 22, (size_t)cap * 8, &dval)))
        return rc;
    IFX_CUDA(launch_localextrema(a, (unsigned long long *)counts, (unsigned long long *)total, (long long *)didx,
                                 (double *)dval, capacity, c.s));
    unsigned long long found = 0;
    IFX_CUDA(cudaMemcpyAsync(&found, total, 8, cudaMemcpyDeviceToHost, c.s));
    IFX_CUDA(cudaStreamSynchronize(c.s));
    *count = (int64_t)found;
    const long long k = (long long)found < capacity ? (long long)found : capacity;
    if (k > 0) {
        IFX_CUDA(cudaMemcpyAsync(indices, didx, (size_t)k * 8, cudaMemcpyDeviceToHost, c.s));
        IFX_CUDA(cudaMemcpyAsync(values, dval, (size_t)k * 8, cudaMemcpyDeviceToHost, c.s));
    }
    if ((rc = c.finish())) return rc;
    IFX_CUDA(cudaStreamSynchronize(c.s));
    return IFX_OK;
}

int ifx_convert(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img, void *stream)
{
    IFX_RANGE("ifx_convert");
    int rc;
    if ((rc = check_array(img, "img", 1, true)) || (rc = check_array(out, "out", 1, true))) return rc;
    if ((rc = check_same_axes(*out, *img))) return rc;
    const int st = img->eltype, dt = out->eltype;
    const bool to_int = dt == IFX_U8 || dt == IFX_I8 || dt == IFX_I16 || dt == IFX_U16 || dt == IFX_I32 ||
                        dt == IFX_I64;
    if (!(to_int || dt == IFX_F32 || dt == IFX_F64) && dt != st)
        return fail(IFX_ERR_UNSUPPORTED, "conversion to N0f8/N0f16 is not supported (from eltype %d)", st);
    const long long n = numel(*img);
    if (n == 0) return IFX_OK;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dout, *flag;
    if ((rc = c.input(*img, &din, (size_t)n * conv_elsize(st))) ||
        (rc = c.output(*out, &dout, (size_t)n * conv_elsize(dt))))
        return rc;
    if (dt == st) {
        if (dout != din) IFX_CUDA(cudaMemcpyAsync(dout, din, (size_t)n * conv_elsize(st), cudaMemcpyDeviceToDevice, c.s));
        return c.finish();
    }
    if ((rc = slot_get(ctx, 24, 16, &flag))) return rc;
    if (to_int) IFX_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), c.s));
    IFX_CUDA(launch_convert(din, st, dout, dt, n, (int *)flag, c.s));
    int bad = 0;
    if (to_int) IFX_CUDA(cudaMemcpyAsync(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost, c.s));
    if ((rc = c.finish())) return rc;
    if (to_int) {
        IFX_CUDA(cudaStreamSynchronize(c.s));
        if (bad)
            return fail(IFX_ERR_ARGUMENT, "InexactError: a value is not an integer inside the range of "
                        "the output's eltype");
    }
    return IFX_OK;
}

int ifx_maxabs(ifx_context_t *ctx, const ifx_array_t *img, double *result, void *stream)
{
    IFX_RANGE("ifx_maxabs");
    int rc;
    if ((rc = check_array(img, "img"))) return rc;
    if (!result) return fail(IFX_ERR_ARGUMENT, "result is NULL");
    if (img->eltype == IFX_I16) return fail(IFX_ERR_UNSUPPORTED, "Int16 images are not supported");
    *result = 0.0;
    if (numel(*img) == 0) return IFX_OK;
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *buf;
    if ((rc = c.input(*img, &din)) || (rc = slot_get(ctx, 20, 16, &buf))) return rc;
    IFX_CUDA(cudaMemsetAsync(buf, 0, 16, c.s));
    IFX_CUDA(launch_maxabs(din, img->eltype, numel(*img), (unsigned long long *)buf, c.s));
    unsigned long long h[2] = {0, 0};
    IFX_CUDA(cudaMemcpyAsync(h, buf, 16, cudaMemcpyDeviceToHost, c.s));
    if ((rc = c.finish())) return rc;
    IFX_CUDA(cudaStreamSynchronize(c.s));
    double m;
    memcpy(&m, &h[0], 8);
    *result = h[1] ? std::nan("") : m;
    return IFX_OK;
}

// ---------------------------------------------------------------- NA()
int ifx_na_prepare(ifx_context_t *ctx, ifx_array_t *zeroed, ifx_array_t *valid, const ifx_array_t *img,
                   int32_t na, int32_t *has_na, void *stream)
{
    IFX_RANGE("ifx_na_prepare");
    int rc;
    if ((rc = check_array(img, "img")) || (rc = check_array(zeroed, "zeroed")) ||
        (rc = check_array(valid, "valid")))
        return rc;
    if ((rc = check_same_axes(*zeroed, *img)) || (rc = check_same_axes(*valid, *img))) return rc;
    if (!has_na) return fail(IFX_ERR_ARGUMENT, "has_na is NULL");
    if (na < IFX_NA_ISNAN || na > IFX_NA_NONE) return fail(IFX_ERR_ARGUMENT, "unknown NA predicate %d", na);
    if ((zeroed->eltype != IFX_F32 && zeroed->eltype != IFX_F64) ||
        (valid->eltype != IFX_F32 && valid->eltype != IFX_F64))
        return fail(IFX_ERR_UNSUPPORTED, "NA filtering works in Float32 or Float64");
    if (img->eltype == IFX_I16) return fail(IFX_ERR_UNSUPPORTED, "Int16 images are not supported");
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *din;
    void *dz, *dv, *flag;
    if ((rc = c.input(*img, &din)) || (rc = c.output(*zeroed, &dz)) || (rc = c.output(*valid, &dv))) return rc;
    if ((rc = slot_get(ctx, 23, sizeof(int), &flag))) return rc;
    IFX_CUDA(cudaMemsetAsync(flag, 0, sizeof(int), c.s));
    IFX_CUDA(launch_na_prepare(din, img->eltype, dz, zeroed->eltype, dv, valid->eltype, numel(*img), na,
                               (int *)flag, c.s));
    int h = 0;
    IFX_CUDA(cudaMemcpyAsync(&h, flag, sizeof(int), cudaMemcpyDeviceToHost, c.s));
    if ((rc = c.finish())) return rc;
    IFX_CUDA(cudaStreamSynchronize(c.s));      // has_na is read on the host
    *has_na = h;
    return IFX_OK;
}

int ifx_na_divide(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *den, void *stream)
{
    IFX_RANGE("ifx_na_divide");
    int rc;
    if ((rc = check_array(out, "out")) || (rc = check_array(den, "den")) || (rc = check_same_axes(*out, *den)))
        return rc;
    if ((out->eltype != IFX_F32 && out->eltype != IFX_F64) || (den->eltype != IFX_F32 && den->eltype != IFX_F64))
        return fail(IFX_ERR_UNSUPPORTED, "NA normalisation works in Float32 or Float64");
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    const void *dd;
    void *dout;
    // out is read and written: stage it as an input and copy it back
    if ((rc = c.input(*out, (const void **)&dout)) || (rc = c.input(*den, &dd))) return rc;
    if (c.host && !is_device_ptr(out->data)) c.back.push_back({out->data, dout, (size_t)numel(*out) * elsize(out->eltype)});
    IFX_CUDA(launch_na_divide(dout, out->eltype, dd, den->eltype, numel(*out), c.s));
    return c.finish();
}

int ifx_na_normalize_separable(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *sums, void *stream)
{
    IFX_RANGE("ifx_na_normalize_separable");
    int rc;
    if ((rc = check_array(out, "out"))) return rc;
    if (!sums) return fail(IFX_ERR_ARGUMENT, "sums is NULL");
    if (out->eltype != IFX_F32 && out->eltype != IFX_F64)
        return fail(IFX_ERR_UNSUPPORTED, "NA normalisation works in Float32 or Float64");
    const int nd = out->ndim;
    for (int d = 0; d < nd; ++d) {
        if ((rc = check_array(&sums[d], "sums[d]"))) return rc;
        if (sums[d].eltype != IFX_F64 || sums[d].ndim != 1 || sums[d].size[0] != out->size[d])
            return fail(IFX_ERR_DIMENSION, "sums[%d] must be a Float64 vector of length %lld", d,
                        (long long)out->size[d]);
    }
    if (!ctx) return fail(IFX_ERR_ARGUMENT, "context is NULL");
    std::lock_guard<std::mutex> lk(ctx->mu);
    Call c;
    if ((rc = begin(ctx, stream, c))) return rc;
    void *dout;
    if ((rc = c.input(*out, (const void **)&dout))) return rc;
    if (c.host && !is_device_ptr(out->data)) c.back.push_back({out->data, dout, (size_t)numel(*out) * elsize(out->eltype)});
    const double *f[IFX_MAXD] = {};
    long long n[IFX_MAXD] = {};
    for (int d = 0; d < nd; ++d) {
        const void *p;
        if ((rc = c.input(sums[d], &p))) return rc;
        f[d] = (const double *)p;
        n[d] = out->size[d];
    }
    IFX_CUDA(launch_na_normalize(dout, out->eltype, numel(*out), f, n, nd, c.s));
    return c.finish();
}

} // extern "C"
