// ifx_internal.h -- launch descriptors shared between the C-ABI layer
// (ifx_api.cu) and the kernel files.  Host-side only types; no torch.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include <functional>
#include <vector>
#include "ifx_common.cuh"

#include <nvtx3/nvToolsExt.h>

namespace ifx {

// NVTX range around a public entry point (a no-op unless a profiler attaches)
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};
#define IFX_RANGE(name) ::ifx::NvtxRange ifx_nvtx_range_(name)

constexpr int kMaxDenseTaps = 3600;      // dense kernels passed by value (60x60)

// Weights by value (kernel parameter space is 32 KB on sm_70+ with CUDA 12.1+).
template <class Tc, int N> struct Weights { Tc w[N]; };

// Generic N-d box pipeline --------------------------------------------------
struct PadBoxArgs {
    const void *img; int in_type;          // ifx_eltype of img
    void *dst; int out_type;               // ifx_eltype of dst (compute type or output eltype)
    int nd; int n[IFX_MAXD];               // image sizes
    Box box;                               // dst box in image index space
    int style; double fill;                // fill already in dst's value domain (code for 8-bit)
};
cudaError_t launch_pad_box(const PadBoxArgs &a, cudaStream_t s);

// Longest 1-D factor: the fused kernels take up to IFX_MAX_TAPS (weights in
// the launch parameters), the generic pass kernel up to this many (weights in
// device memory beyond IFX_MAX_TAPS).
constexpr int kMaxFactorTaps = 4095;

struct PassBoxArgs {
    const void *src; Box sbox;             // compute-type buffer
    void *dst; Box dbox; int out_type;     // dst buffer (compute type, or the output eltype)
    Box obox;                              // region to compute (inside dbox)
    int axis, kfirst, klen;
    const double *w;                       // host weights (copied into the launch)
    int compute_f64;
};
cudaError_t launch_pass_box(const PassBoxArgs &a, cudaStream_t s);

// Fused 2-D separable tile kernel -------------------------------------------
struct Sep2dArgs {
    const void *img; int in_type;
    void *out; int out_type;
    int nx, ny;
    int fx, kx, fy, ky;                    // x factor: first, taps; y factor: first, taps
    const double *wx, *wy;                 // host weights
    int x_first;                           // pass order
    int style; double fill;                // fill in value domain
    int compute_f64;
    int variant;                           // 0: automatic, 1: TMA tile kernel where it applies, 2: gather kernel
    int nsl;                               // planes of nx x ny stacked at img/out, filtered each on its own
                                           // (0 or 1: one; more: TMA tile kernel only)
    int tile_w, tile_h;                    // output tile (0: the kernel's default); shapes a kernel
                                           // cannot take fall back to its default
    int in_nx, in_ny;                      // input planes (0: nx x ny); larger: a padded input whose
                                           // windows (offsets fx, fy) lie inside (TMA tile kernel only)
};
cudaError_t launch_sep2d(const Sep2dArgs &a, cudaStream_t s);
bool sep2d_tma_applies(const Sep2dArgs &a);
size_t sep2d_smem_bytes(int kx, int ky, int x_first, int f64);
// the tile shape each kernel of the fused 2-D path would run for `a`
// (variant 1: TMA tile kernel, 2: gather kernel); false when it cannot run it
bool sep2d_tile_shape(const Sep2dArgs &a, int variant, int *tw, int *th);

// Fused 3-D separable kernel (factors on axes 0, 1, 2 in that order; FP32) ---
struct Sep3dArgs {
    const void *img; int in_type;          // nvol volumes back to back
    void *out; int out_type;
    int nx, ny, nz, nvol;
    int fx, kx, fy, ky, fz, kz;
    const double *wx, *wy, *wz;
    int style; double fill;
};
bool sep3d_supported(int kx, int ky, int kz, int nx, int ny, int nz, int nvol);
// zdepth: output slices per z chunk of the fused kernel (0: default; the z
// halo of kz - 1 input slices is filtered once per chunk)
cudaError_t launch_sep3d(const Sep3dArgs &a, cudaStream_t s, int zdepth = 0);
// the split 3-D path (z sweep into a padded FP32 volume of
// sep3d_split_tmp_bytes at tmp, then the x/y TMA sweep over its planes, in
// tiles of tw x th when given); applies needs no device memory
bool sep3d_split_applies(const Sep3dArgs &a);
size_t sep3d_split_tmp_bytes(const Sep3dArgs &a);       // the split path's padded FP32 volume
cudaError_t launch_sep3d_split(const Sep3dArgs &a, float *tmp, cudaStream_t s, int tw = 0, int th = 0);

// The autotuner (ifx_tune.cu) -------------------------------------------------
// A tuned choice: variant (2-D: 1 TMA tile kernel, 2 gather kernel; 3-D: 1
// split sweeps, 2 fused z-marching kernel), pass order, output tile shape,
// z chunk depth, and the time it was tuned at.
struct TuneChoice {
    int variant, x_first, tile_w, tile_h, depth;
    float ms;
};
enum { TUNE_SEP2D = 0, TUNE_SEP3D = 1, TUNE_BATCH = 2 };
// Times tuner candidates with L2 overwritten before each timed launch.
struct TuneTimer {
    void *flush = nullptr;
    size_t flush_bytes = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t init();
    ~TuneTimer();
    cudaError_t time(const std::function<cudaError_t()> &run, cudaStream_t s, float *ms);
};
void autotune_set(bool enable, const char *path);
bool autotune_enabled();
bool autotune_lookup(const Sep2dArgs &a, TuneChoice *c);
bool autotune_lookup3(const Sep3dArgs &a, TuneChoice *c);
// key fields as the public API gives them (path, eltypes, taps, Fill, extents)
bool autotune_lookup_key(int path, int in_type, int out_type, int kx, int ky, int kz, int fill, long long nx,
                         long long ny, long long nz, TuneChoice *c);
void autotune_pin_key(int path, int in_type, int out_type, int kx, int ky, int kz, int fill, long long nx,
                      long long ny, long long nz, const TuneChoice &c);
void autotune_clear();
// the batched engine's tile per (op, eltypes, taps, median window): a cached
// choice (tile_w, tile_h) and storing one (persist: written to the cache file)
bool autotune_lookup_batch(int op, int in_type, int out_type, int kx, int ky, int win, TuneChoice *c);
void autotune_store_batch(int op, int in_type, int out_type, int kx, int ky, int win, const TuneChoice &c,
                          bool persist);
// the fused 2-D separable filter of `a`, tuned (device_arrays: tuning allowed)
cudaError_t launch_sep2d_tuned(Sep2dArgs a, cudaStream_t s, bool device_arrays);
// the 3-D separable filter of `a`: the cached choice, or (tuner enabled,
// device arrays) every candidate timed; tmp: the split path's FP32 volume
// (nullptr when the split path does not apply)
cudaError_t launch_sep3d_tuned(const Sep3dArgs &a, float *tmp, cudaStream_t s, bool device_arrays);

// Fused 3-D gradients (3-tap derivative / smoothing pair, all axes extended):
// the three imgradients outputs from one sweep -----------------------------
struct Grad3dArgs {
    const void *img; int in_type;
    void *out[3]; int out_type;
    int nx, ny, nz;
    double d[3], s[3];                     // derivative and smoothing taps (first index -1)
    int style; double fill;
    int compute_f64;
};
cudaError_t launch_grad3d(const Grad3dArgs &a, cudaStream_t s);

// Triggs-Sdika IIR passes ------------------------------------------------------------
// One pass along an axis of a contiguous column-major array: `lines` lines of
// `L` elements with element stride `inner` (line l = o * inner + p starts at
// o * inner * L + p).  src may equal dst (in place).  Coefficients hold the
// values of the kernel's own float type; om_a = 1 - asum and om_b = 1 - bsum
// are evaluated in that type.  edge 0: boundary values from the lines' end
// elements (Pad), 1: `fill` (Fill, already in dst's eltype).
struct IirArgs {
    const void *src; int src_type;
    void *dst; int dst_type;
    long long L, inner, lines;
    double a[3], b[3], scale, M[9], om_a, om_b;
    int edge; double fill;
    int compute_f64;
};
cudaError_t launch_iir(const IirArgs &a, cudaStream_t s);

// Algorithm.FFT() (cuFFT, loaded at run time) ---------------------------------------
struct FftArgs {
    int nd;
    long long n[IFX_MAXD], P[IFX_MAXD];   // image sizes, padded (FFT) sizes
    int ksize[IFX_MAXD];
    long long kn, Ptotal, Pc, total;      // kernel taps, padded elements, spectrum elements, outputs
    const double *Kdev;                   // kernel on the device, column-major
    void *padded, *krn, *specA, *specK;   // compute-type work buffers
    void *out; int out_type;
    int compute_f64;
};
bool fft_available();
long long fft_size(long long l, long long lk);
int launch_fft(const FftArgs &f, cudaStream_t s);   // 0 ok, -1 cuFFT, -2 CUDA, -3 no cuFFT

// blob_LoG pieces ---------------------------------------------------------------
struct LeArgs {
    const void *img;
    int eltype;
    int nd;
    long long n[IFX_MAXD];
    int half[IFX_MAXD];             // window >> 1
    int lo[IFX_MAXD], hi[IFX_MAXD]; // candidate range per axis (edges)
    long long total;
    int minima;
};

cudaError_t launch_localextrema(const LeArgs &a, unsigned long long *counts, unsigned long long *total,
                                long long *idx, double *val, long long capacity, cudaStream_t s);
long long localextrema_blocks(long long total);
cudaError_t launch_maxabs(const void *img, int eltype, long long n, unsigned long long *out, cudaStream_t s);
cudaError_t launch_sum_scale(void *out, const void *term, int eltype, long long n, double scale, int last,
                             cudaStream_t s);

// NA() pieces -----------------------------------------------------------------
cudaError_t launch_na_prepare(const void *img, int it, void *z, int zt, void *v, int vt, long long n, int na,
                              int *flag, cudaStream_t s);
cudaError_t launch_na_divide(void *out, int ot, const void *den, int dt, long long n, cudaStream_t s);
cudaError_t launch_na_normalize(void *out, int ot, long long total, const double *const *f, const long long *n,
                                int nd, cudaStream_t s);

// Dense --------------------------------------------------------------------
struct Dense2dArgs {
    const void *img; int in_type;
    void *out; int out_type;
    int nx, ny;
    int fx, kw, fy, kh;                    // K axes: x first/size, y first/size
    const double *K;                       // column-major kh? no: K[i + kw*j], i along x
    int style; double fill;
    int compute_f64;
};
cudaError_t launch_dense2d(const Dense2dArgs &a, cudaStream_t s);
// tcgen05 tensor-core path (2-D, kernels up to 33 wide and 40 tall)
bool dense_tc_supported(int in_type, int kw, int kh);
cudaError_t launch_dense_tc(const Dense2dArgs &a, cudaStream_t s, int device);
// Bounded waits that ran out in a kernel launched on `device` since the last
// call (reads and clears the device's error word).
int kernel_timeout_take(int device);

struct DenseBoxArgs {                      // N-d dense over a padded compute-type box
    const void *src; Box sbox;
    void *out; int out_type; Box obox;     // obox == image box (lo 0)
    int nd; int ksize[IFX_MAXD]; int kfirst[IFX_MAXD];
    const double *K;
    int compute_f64;
};
cudaError_t launch_dense_box(const DenseBoxArgs &a, cudaStream_t s);

// Laplacian ---------------------------------------------------------------
struct LaplacianArgs {
    const void *img; int in_type;
    void *out; int out_type;               // also the arithmetic type
    int nd; int n[IFX_MAXD]; int flags[IFX_MAXD];
    int style; double fill;                // fill in value domain of the output type
};
cudaError_t launch_laplacian(const LaplacianArgs &a, cudaStream_t s);

// Rank filters --------------------------------------------------------------
struct MedianArgs {
    const void *img; int in_type;
    void *out; int out_type;
    int nd; int n[IFX_MAXD];
    int wfirst[IFX_MAXD], wlen[IFX_MAXD];
    int style; double fill;                // fill: code for 8-bit inputs, value otherwise
};
cudaError_t launch_median(const MedianArgs &a, cudaStream_t s);

struct ExtremaPassArgs {                   // one separable min/max pass along `axis`
    const void *src_min, *src_max;         // src (input image for pass 0: both == img)
    void *dst_min, *dst_max;               // may be the final interleaved output
    int type;                              // element type of src and dst (F32/F64/U8)
    int nd; int n[IFX_MAXD];
    int axis, a0, a1;                      // window offsets a0..a1 along axis
    int use_fill; double fill;             // Fill border: fill joins windows leaving the image
    int dst_interleaved;                   // 1: dst_min points to (min,max) pairs
    int want_min, want_max;
};
cudaError_t launch_extrema_pass(const ExtremaPassArgs &a, cudaStream_t s);
// Element conversion (ifx_convert): *bad set when an integer target cannot hold a value.
cudaError_t launch_convert(const void *src, int st, void *dst, int dt, long long n, int *bad, cudaStream_t s);
// 8-bit 2-D extrema of square w x w windows (first offset a0 on both axes) in
// one launch; false when w has no compiled tile kernel.  which: 0 interleaved
// (min, max), 1 min, 2 max.
bool launch_extrema2d_u8(const void *img, void *out, int nx, int ny, int w, int a0, int use_fill, double fill,
                         int which, cudaStream_t s, cudaError_t *e);

// Separable cascade, generic pipeline (shared with the fixed-scratch entry) ---
struct Fac { int axis, first, len; const double *w; };
int factored_prepare(const ifx_array_t *out, const ifx_array_t *img, int32_t nfactors,
                     const ifx_factor_t *factors, const ifx_border_t *border, std::vector<Fac> &facs,
                     double *fill, bool *nothing);
void generic_cascade_sizes(const ifx_array_t &imgd, const std::vector<Fac> &facs, size_t *a, size_t *b);
int generic_cascade_run(cudaStream_t s, const ifx_array_t &imgd, const void *img,
                        const ifx_array_t &outd, void *out, const std::vector<Fac> &facs, int style,
                        double fill, void *bufA, void *bufB);
bool is_device_array(const void *p);
// IFX_OK when the array's bytes are device (or managed) memory inside one
// allocation and, for device memory, on `device`; IFX_ERR_ARGUMENT otherwise.
int check_device_array(const ifx_array_t &a, int device, const char *name);

// Batched engine -------------------------------------------------------------
struct BatchItem {                         // one validated 2-D request, device pointers
    int op, in_type, out_type, style;      // op: 1 factored, 2 gradients, 3 laplacian, 4 median
    int nx, ny, window;
    const void *in;
    void *out0, *out1;
    double fill;                           // value domain
    int fill_code;                         // 8-bit images
    int kx, ky, fx, fy;                    // factored: x/y factors; gradients: deriv/smooth (3, -1)
    const double *wx, *wy;
};
cudaError_t launch_batch(int device, const BatchItem *items, int n, cudaStream_t s, long long *tiles);
int batch_grid(int device);
cudaError_t plan_create(int device, const BatchItem *items, int n, void **plan);
cudaError_t plan_launch(void *plan, cudaStream_t s, long long *tiles);
void plan_destroy(void *plan);
// Validates one batched request and fills `it` (the request's own pointers).
struct DevRanges;
int request_item(const ifx_request_t &q, int index, bool need_device, BatchItem &it,
                 DevRanges *ranges = nullptr);
// Sets the calling thread's ifx_last_error() message; returns code.
int set_error(int code, const char *msg);

} // namespace ifx
