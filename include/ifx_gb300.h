/*
 * ifx_gb300.h -- C ABI of the GB300 (sm_103a) FIR and rank-filter library.
 *
 * This is the drop-in boundary for ImageFiltering.jl's FIR / rank-filter path.
 * A Julia method for a new algorithm tag `Algorithm.GB300 <: Alg` runs the
 * reference's dispatch steps 1-4 unchanged (output eltype, kernel factoring,
 * border resolution, output allocation: src/imfilter.jl:1-49, 204-254) and
 * then `ccall`s one entry point below in place of the padded-copy + CPU loop
 * backend.  Every entry point names the reference method it replaces
 * (paths relative to the ImageFiltering.jl v0.7.12 tree).
 *
 * Conventions
 *  - Arrays are column-major with axis 0 = Julia axis 1 (contiguous).  Only
 *    dense arrays are accepted: stride[0] == 1, stride[d] == stride[d-1]*size[d-1].
 *  - `data` may be host memory (plain or pinned) or device memory of the
 *    context's device.  Host arrays are staged through the library's own
 *    device buffers and the call returns when the result is back in host
 *    memory.  When every array is device memory the work is only enqueued on
 *    `stream` (NULL = the context's stream) and the call returns at once.
 *  - Return value: IFX_OK or an ifx_status; ifx_last_error() gives the
 *    message of the calling thread's last failure.  Status codes map to the
 *    reference's exception classes (ArgumentError, DimensionMismatch, error).
 *  - No C++ exceptions cross this boundary and no torch types appear in it.
 */
#ifndef IFX_GB300_H
#define IFX_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define IFX_ABI_VERSION 1
#define IFX_MAX_DIMS 4
#define IFX_MAX_TAPS 129          /* longest 1-D factor of the fused kernels; the generic
                                     N-d pipeline takes factors of up to 4095 taps */

typedef enum {
    IFX_OK = 0,
    IFX_ERR_ARGUMENT = 1,          /* ArgumentError   (src/border.jl:147-156, 250-256) */
    IFX_ERR_DIMENSION = 2,         /* DimensionMismatch (src/imfilter.jl:604-615)      */
    IFX_ERR_ERROR = 3,             /* error(...) / DivideError (src/mapwindow.jl:133-137,
                                      src/border.jl:581-586 with a length-1 axis)      */
    IFX_ERR_CUDA = 4,              /* a CUDA runtime call failed                        */
    IFX_ERR_NOMEM = 5,             /* device or host allocation failed / over the cap   */
    IFX_ERR_TIMEOUT = 6,           /* a bounded wait ran out                            */
    IFX_ERR_UNSUPPORTED = 7,       /* a case this path does not implement               */
    IFX_ERR_CANCELLED = 8          /* a served request cancelled before it ran          */
} ifx_status;

typedef enum {                     /* element types of arrays crossing the ABI          */
    IFX_F32 = 0,                   /* Float32 / Gray{Float32}                           */
    IFX_F64 = 1,                   /* Float64 / Gray{Float64}                           */
    IFX_N0F8 = 2,                  /* N0f8 / Gray{N0f8}: 8-bit code c means c/255       */
    IFX_U8 = 3,                    /* UInt8: 8-bit code c means c                       */
    IFX_I16 = 4,                   /* Int16 (Laplacian of UInt8, src/imfilter.jl:1139)  */
    /* element types that only ifx_convert takes (the filters take the types above) */
    IFX_I8 = 5,                    /* Int8                                               */
    IFX_U16 = 6,                   /* UInt16                                             */
    IFX_I32 = 7,                   /* Int32                                              */
    IFX_I64 = 8,                   /* Int64 / Int                                        */
    IFX_N0F16 = 9                  /* N0f16 / Gray{N0f16}: 16-bit code c means c/65535   */
} ifx_eltype;

typedef enum {                     /* border styles (src/border.jl:136-248, 465-555)    */
    IFX_REPLICATE = 0,
    IFX_CIRCULAR = 1,
    IFX_SYMMETRIC = 2,             /* dcba|abcd|dcba: edge duplicated (border.jl:574-580) */
    IFX_REFLECT = 3,               /* dcb|abcd|cba: edge not repeated (border.jl:581-586) */
    IFX_FILL = 4                   /* Fill(value)                                        */
} ifx_style;

typedef struct ifx_array {
    void *data;
    int32_t eltype;                /* ifx_eltype */
    int32_t ndim;                  /* 1 .. IFX_MAX_DIMS */
    int64_t size[IFX_MAX_DIMS];
    int64_t stride[IFX_MAX_DIMS];  /* in elements */
    int64_t first[IFX_MAX_DIMS];   /* first index of each axis (1 for Array, any for OffsetArray) */
} ifx_array_t;

typedef struct ifx_border {
    int32_t style;                 /* ifx_style */
    int32_t explicit_pad;          /* 0: Pad{0}/Fill{T,0}, amounts come from the kernel
                                      (src/border.jl:236-237, 614-621);
                                      1: Pad{N}/Fill{T,N} with lo/hi below, which must
                                      cover the kernel (DimensionMismatch otherwise)  */
    int64_t lo[IFX_MAX_DIMS];
    int64_t hi[IFX_MAX_DIMS];
    double fill_value;             /* Fill value, already converted to the image eltype
                                      (src/borderarray.jl:11-20)                        */
} ifx_border_t;

typedef struct ifx_factor {        /* one ReshapedOneD factor (src/kernelfactors.jl:52-131) */
    int32_t axis;                  /* 0-based axis it filters along (Npre)               */
    int32_t length;                /* taps, 1 .. 4095 (fused kernels up to IFX_MAX_TAPS) */
    int64_t first;                 /* kernel index of the first tap (OffsetArray axes)   */
    const double *weights;         /* host memory, `length` values                       */
} ifx_factor_t;

typedef struct ifx_context ifx_context_t;

/* ---- context ------------------------------------------------------------- */
int ifx_abi_version(void);
int ifx_create(ifx_context_t **ctx, int device);
int ifx_destroy(ifx_context_t *ctx);
const char *ifx_last_error(void);
/* Number of this library's kernel launches made by the calling process so far. */
uint64_t ifx_launch_count(void);
int ifx_synchronize(ifx_context_t *ctx, void *stream);
/* Testing aid, no counterpart in the reference: on != 0 makes the first wait
 * of every tile of the copy-fed kernels (the TMA-fed separable kernel and the
 * batched engine) on the context's device give up at once, so that the
 * kernels take their timeout path (they wait, with their full bound, for the
 * copies still in flight, record the timeout and return) and the next
 * ifx_synchronize reports IFX_ERR_TIMEOUT; on == 0 restores the default
 * bounds.  No GPU fault is involved. */
int ifx_debug_force_wait_timeout(ifx_context_t *ctx, int32_t on);

/* ---- a1: border index maps ------------------------------------------------
 * padarray(T, img, border) (src/border.jl:324-331 -> borderarray.jl:179-196,
 * index maps src/border.jl:564-596).  out has sizes lo+n+hi per axis and the
 * output eltype; its first indices are img.first - lo. */
int ifx_padarray(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                 const ifx_border_t *border, void *stream);

/* ---- a2/a3: separable cascade ---------------------------------------------
 * imfilter!(r::AbstractResource{GB300}, out, img, kernel::Tuple{ReshapedOneD...},
 * border) -- replaces the padded copy (src/imfilter.jl:331-341), the cascade
 * scheduler (385-457, tiled 460-564) and the 1-D loops (671-739).  Results
 * equal pad-then-cascade: each pass covers the halo that later passes need,
 * so Fill borders behave as in the reference.  Copy factors are skipped. */
int ifx_imfilter_factored(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                          int32_t nfactors, const ifx_factor_t *factors,
                          const ifx_border_t *border, void *stream);

/* ---- a4: dense kernel -------------------------------------------------------
 * imfilter! with a single dense (non-separable) kernel, the `(dummy, K)` case
 * after factorkernel (src/imfilter.jl:1159-1184) -> __imfilter_inbounds!
 * (src/imfilter.jl:624-669).  K is column-major with sizes ksize and first
 * indices kfirst (host memory).  method: 0 = automatic (tensor cores for
 * sign-definite 2-D kernels -- every weight >= 0, or every weight <= 0 -- of
 * 11 x 11 and larger that they take, CUDA cores otherwise, and the
 * FFT path of ifx_imfilter_fft when its estimated time is under half the
 * direct one -- large kernels, Float64 images -- or the kernel has more than
 * 3600 taps, provided every image element is finite; that check reads one
 * flag back, so the call waits for its stream then),
 * 1 = FP32/FP64 CUDA cores, 2 = tcgen05 tensor cores (BF16 hi/lo split, three
 * products, FP32 accumulation; 2-D Float32 and 8-bit images, kernels up to
 * 33 wide and 40 tall; up to about 1.5e-5 normwise for kernels of mixed
 * signs whose sum nearly cancels, which the automatic method keeps off them). */
int ifx_imfilter_dense(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                       const double *kernel, const int64_t *ksize, const int64_t *kfirst,
                       const ifx_border_t *border, int32_t method, void *stream);

/* ---- a5: Laplacian stencil --------------------------------------------------
 * imfilter(img, Kernel.Laplacian(flags), border) (src/specialty.jl:3-17,
 * src/kernel.jl:341-391).  Exact: the same operation order in the output
 * eltype (Float32, Float64 or Int16). */
int ifx_imfilter_laplacian(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                           const int32_t *flags, const ifx_border_t *border, void *stream);

/* ---- a6: imgradients --------------------------------------------------------
 * imgradients(img, kernelfun, border) for factored gradient kernels
 * (src/specialty.jl:39-53, gradfactors src/kernelfactors.jl:598-602): output d
 * is the cascade with `deriv` along axis d and `smooth` along every other
 * extended axis.  outs holds img.ndim arrays.  extended[d] == 0 gives a copy
 * factor on axis d (kdim, src/kernelfactors.jl:604). */
int ifx_imgradients(ifx_context_t *ctx, ifx_array_t *outs, const ifx_array_t *img,
                    const double *deriv, const double *smooth, int32_t length, int64_t first,
                    const int32_t *extended, const ifx_border_t *border, void *stream);

/* ---- a8: median -------------------------------------------------------------
 * mapwindow(median!, img, window; border) (src/mapwindow.jl:75-85, 123-131,
 * 270-333).  Window offsets wfirst .. wfirst+wlen-1 per axis, odd lengths
 * only for Dims windows (resolve_window, 133-137: the host checks).  The
 * selected value is written in out's eltype (8-bit inputs: code/255 for N0f8,
 * code for UInt8).  Bit-exact. */
int ifx_mapwindow_median(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                         const int64_t *wfirst, const int64_t *wlen,
                         const ifx_border_t *border, void *stream);

/* ---- a9: extrema ------------------------------------------------------------
 * which = 0: extrema -> out holds (min,max) pairs (Tuple{T,T} layout, 2 values
 *            per element); 1: minimum; 2: maximum.
 * border == NULL: mapwindow(extrema, A, window::Dims) without keywords, the
 *   Lemire filter (src/mapwindow.jl:337-338, 388-473): window offsets
 *   -(w>>1) .. w-1-(w>>1), truncated at the edges, even w allowed (wfirst is
 *   ignored and may be NULL).
 * border != NULL: the generic window path with that border (src/mapwindow.jl:
 *   270-333): Pad styles take values inside window-intersect-image only, Fill
 *   adds the fill value where the window leaves the image.  Bit-exact. */
int ifx_mapwindow_extrema(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img,
                          const int64_t *wfirst, const int64_t *wlen,
                          const ifx_border_t *border, int32_t which, void *stream);

/* ---- autotuner --------------------------------------------------------------
 * Two paths of ifx_imfilter_factored are tuned.
 *  IFX_TUNE_SEP2D, the fused 2-D separable path (at most one factor per axis
 *  of a 1-D or 2-D image): the tile kernel (variant 1: TMA-fed, 2: gather),
 *  the pass order (x_first), and the output tile's width and height (tile_w x
 *  tile_h outputs; the staged window adds the kx - 1 / ky - 1 halo, so the
 *  shape sets the halo's share of every copy and pass).  TMA tiles: 64 or 128
 *  wide, 8-128 rows; gather tiles: 32, 64 or 128 wide, 8-128 rows.
 *  IFX_TUNE_SEP3D, one factor per axis of a volume: variant 1 the split
 *  sweeps (z factor into an FP32 volume, then the x/y TMA sweep with its
 *  tile shape), variant 2 the fused z-marching kernel, whose `depth` output
 *  slices per chunk amortise the kz - 1 halo slices each chunk re-filters.
 * With the tuner enabled, the first device-array call per key (path, input
 * and output eltypes, taps, Fill or Pad, floor(log2(elements)), FP64
 * arithmetic) times every applicable candidate on its stream and keeps the
 * fastest; choices are cached in memory and, when cache_path is given, in
 * that text file (loaded here, appended as keys are tuned).  Cached choices
 * apply whether or not the tuner is enabled; a cached shape a kernel cannot
 * take runs as the kernel's default.  The tuner and its cache are
 * process-wide.  (No reference counterpart: the reference sizes its FIRTiled
 * tiles by a fixed rule, TiledIteration's padded_tilesize,
 * src/imfilter.jl:1200-1206, 1273-1278.) */
#define IFX_TUNE_SEP2D 0
#define IFX_TUNE_SEP3D 1
typedef struct ifx_tune_choice {
    int32_t variant;               /* see above                                          */
    int32_t x_first;               /* 2-D: 1 the x pass first                            */
    int32_t tile_w, tile_h;        /* output tile (0: the kernel's default)             */
    int32_t depth;                 /* 3-D fused: output slices per chunk (0: default)    */
    double ms;                     /* time per call when tuned (pinned: as given)        */
} ifx_tune_choice_t;
int ifx_autotune(ifx_context_t *ctx, int32_t enable, const char *cache_path);
/* The cached 2-D choice for a key: x_first (1: the x pass first), variant (1:
 * TMA tile kernel, 2: gather kernel) and its time in ms; IFX_ERR_ARGUMENT when
 * the key has not been tuned. */
int ifx_autotune_choice(ifx_context_t *ctx, int32_t in_type, int32_t out_type, int32_t kx, int32_t ky,
                        int32_t fill, int64_t nx, int64_t ny, int32_t *x_first, int32_t *variant, double *ms);
/* The cached choice of either path: taps[3] = x, y, z taps (1 for absent
 * axes), size[3] = the array's extents (1 for absent axes); IFX_ERR_ARGUMENT
 * when the key has not been tuned. */
int ifx_autotune_lookup(ifx_context_t *ctx, int32_t path, int32_t in_type, int32_t out_type, const int32_t *taps,
                        int32_t fill, const int64_t *size, ifx_tune_choice_t *choice);
/* Sets the choice for a key (replacing a cached one; not written to the cache
 * file): the next calls with that key run it. */
int ifx_autotune_pin(ifx_context_t *ctx, int32_t path, int32_t in_type, int32_t out_type, const int32_t *taps,
                     int32_t fill, const int64_t *size, const ifx_tune_choice_t *choice);
/* Forgets every cached and pinned choice (the cache file is left as it is). */
int ifx_autotune_clear(ifx_context_t *ctx);
/* The batched engine (ifx_batch_plan_launch): with the tuner enabled, a
 * plan's first launch times, for every key of its requests without a cached
 * choice (op, image and output eltypes, taps -- factored: the two factors'
 * taps, gradients: 3, 3, others ignored -- and the median window), the
 * candidate output tiles on the plan's own requests of that key, and caches
 * the fastest; later plans and ifx_batch_run / the server use cached tiles.
 * Candidates: factored tiles 64, 128 or 256 wide (8-bit images; Float32
 * rows hold 64) at the tallest height the staging rows allow for the y
 * factor and half of it; gradient and Laplacian tiles 88, 176 or 352 wide
 * (8-bit images).  Median tiles are fixed.  tile_w / tile_h of the choice;
 * a tile the engine cannot take runs as the default. */
int ifx_batch_autotune_lookup(ifx_context_t *ctx, int32_t op, int32_t in_type, int32_t out_type, int32_t kx,
                              int32_t ky, int32_t window, ifx_tune_choice_t *choice);
int ifx_batch_autotune_pin(ifx_context_t *ctx, int32_t op, int32_t in_type, int32_t out_type, int32_t kx,
                           int32_t ky, int32_t window, const ifx_tune_choice_t *choice);

/* ---- Algorithm.IIR(): Triggs-Sdika recursive filters ---------------------------
 * One factor per pass, a KernelFactors.TriggsSdika (src/kernelfactors.jl:
 * 462-505): forward coefficients a, backward coefficients b, the right-edge
 * matrix M (row-major), scale, and sum(a), sum(b) -- all values of the
 * kernel's float type (coef_f32 = 1 for Float32 kernels). */
typedef struct ifx_iir {
    int32_t axis;                  /* 0-based axis the factor filters along */
    int32_t coef_f32;              /* 1: Float32 coefficients, 0: Float64   */
    double a[3], b[3];
    double scale;
    double M[9];
    double asum, bsum;
} ifx_iir_t;

/* imfilter! with a cascade of Triggs-Sdika factors (src/imfilter.jl:892-900,
 * 961-1092; ReshapedOneD factors through the cascade of 385-457, whose IIR
 * padding is empty): each factor filters the previous result along its axis,
 * over whole lines, in place in `out`.  Arithmetic in promote(eltype(out),
 * coefficient type), intermediate results rounded to eltype(out), the
 * reference's operation order.  The border gives the boundary values: Pad
 * (any style; the padding of an IIR cascade is empty, so the boundary values
 * are the lines' end elements) or Fill(v) (v converted to eltype(out)).
 * Lines of 3 or fewer elements are a DimensionMismatch.  out may be img
 * (same eltype). */
int ifx_imfilter_iir(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img, int32_t nfactors,
                     const ifx_iir_t *factors, const ifx_border_t *border, void *stream);

/* ---- a4 with Algorithm.FFT() --------------------------------------------------
 * imfilter! with Algorithm.FFT() (src/imfilter.jl:776-884): each axis of length
 * l is padded with the border to nextprod([2,3], l + ksize) elements (padfft,
 * src/border.jl:239-248, 551-555) and the image is correlated with the dense
 * kernel (sizes ksize, first indices kfirst, column-major, host memory)
 * through real FFTs in the output's precision (cuFFT, loaded at run time;
 * IFX_ERR_UNSUPPORTED without it).  Pad/Fill must not carry explicit widths.
 * The reference selects this algorithm for kernels longer than 30
 * (filter_algorithm, src/imfilter.jl:1200-1206). */
int ifx_imfilter_fft(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img, const double *kernel,
                     const int64_t *ksize, const int64_t *kfirst, const ifx_border_t *border, void *stream);

/* ---- blob_LoG pieces --------------------------------------------------------
 * ifx_imfilter_factored_sum: out = scale * sum over nterms separable terms of
 * their cascades (term t = factors[t*nfactors .. t*nfactors+nfactors-1], each
 * like ifx_imfilter_factored), in out's eltype (Float32/Float64).  A
 * Laplacian of Gaussian is the sum over axes d of the second derivative of
 * the Gaussian along d times the Gaussian along the others (Kernel.LoG,
 * src/kernel.jl:325-339); multiLoG (src/extrema.jl:87-98) scales it by -sigma.
 * ifx_findlocalextrema: findlocalmaxima / findlocalminima
 * (src/extrema.jl:100-159) on an array of up to 4 dimensions: indices[k] are
 * the 0-based column-major linear indices of the elements greater (smaller)
 * than every other element of the window (window[d] >> 1 on each side, parts
 * outside the array skipped), in column-major order, values[k] their values;
 * edges[d] == 0 leaves out the first and last index of axis d.  *count is the
 * number found (only min(count, capacity) are written).  Synchronous.
 * ifx_maxabs: maximum(abs, img) (NaN if an element is NaN).  Synchronous. */
int ifx_imfilter_factored_sum(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img, int32_t nterms,
                              int32_t nfactors, const ifx_factor_t *factors, double scale,
                              const ifx_border_t *border, void *stream);
int ifx_findlocalextrema(ifx_context_t *ctx, const ifx_array_t *img, const int32_t *window, const int32_t *edges,
                         int32_t minima, int64_t *indices, double *values, int64_t capacity, int64_t *count,
                         void *stream);
int ifx_maxabs(ifx_context_t *ctx, const ifx_array_t *img, double *result, void *stream);

/* ---- element conversion -----------------------------------------------------
 * out .= convert.(eltype(out), img) (the eltype conversions around the
 * reference's imfilter!: its padded copy in the filter type,
 * src/border.jl:324-331, and the store of each result, src/imfilter.jl:
 * 660-666), same axes.  To Float32/Float64 from any eltype above: the value
 * (N0f8 c/255 and N0f16 c/65535 correctly rounded; integers exactly, or
 * rounded to nearest for Float32 beyond 2^24).  To an integer type: every
 * value must be an integer in the type's range (N0f8/N0f16 values are at 0
 * and 1 only), else IFX_ERR_ARGUMENT (Julia's InexactError); such calls are
 * synchronous (the check is read back).  To N0f8/N0f16: from the same eltype
 * only (a copy); other conversions to them return IFX_ERR_UNSUPPORTED. */
int ifx_convert(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *img, void *stream);

/* ---- NA() borders ---------------------------------------------------------
 * The non-filter steps of NA filtering (_imfilter_na!, src/imfilter.jl:280-318;
 * imfilter_na_inseparable! / imfilter_na_separable! 1094-1130;
 * normalize_separable! / normalize_dims! 1234-1250); the filters are
 * ifx_imfilter_factored / ifx_imfilter_dense with a Fill(0) border.
 * ifx_na_prepare: zeroed = img with NA elements set to 0 (in zeroed's eltype,
 * N0f8 as c/255), valid = 1 where img is not NA and 0 where it is, *has_na =
 * whether any element is NA; the predicate is isnan, !isfinite or never
 * (8-bit images have no NA elements).  Synchronous (has_na is read back).
 * ifx_na_divide: out[I] = out[I] / den[I], the quotient in Float64.
 * ifx_na_normalize_separable: out[I] = ((out[I] / sums[0][i0]) / sums[1][i1])
 * ..., in Float64; sums[d] is a Float64 vector of length size[d] (the 1-D
 * filter of ones along axis d with Fill(0)). */
#define IFX_NA_ISNAN 0
#define IFX_NA_NOTFINITE 1
#define IFX_NA_NONE 2
int ifx_na_prepare(ifx_context_t *ctx, ifx_array_t *zeroed, ifx_array_t *valid, const ifx_array_t *img,
                   int32_t na, int32_t *has_na, void *stream);
int ifx_na_divide(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *den, void *stream);
int ifx_na_normalize_separable(ifx_context_t *ctx, ifx_array_t *out, const ifx_array_t *sums, void *stream);

/* ---- separable cascade without allocation ------------------------------------
 * No counterpart in the reference: an allocation-free form of
 * ifx_imfilter_factored for callers that cannot allocate device memory on
 * the filtering path (a real-time frame loop that must not stall on
 * cudaMalloc/cudaFree, which can synchronize the device; an application that
 * reserves its whole device-memory budget at start-up).  Same results and
 * arguments as ifx_imfilter_factored without the context; arrays must be
 * device memory of the current device; work is enqueued on `stream`.
 * Its intermediate buffers live in one fixed device array of
 * ifx_noalloc_scratch_bytes() bytes (32 MiB) compiled into the library, held
 * by every GPU that loads the library until exit; a filter needing more is
 * rejected with IFX_ERR_NOMEM.  The first call on a device looks up that
 * array's address (make it before any stream capture starts).  All calls share
 * the array: calls that overlap on the GPU race. */
uint64_t ifx_noalloc_scratch_bytes(void);
int ifx_imfilter_factored_noalloc(ifx_array_t *out, const ifx_array_t *img, int32_t nfactors,
                                  const ifx_factor_t *factors, const ifx_border_t *border,
                                  void *stream);

/* ---- batched engine: many 2-D requests in one persistent launch --------------
 * The requests of a batch are cut into output tiles that resident CTAs take
 * from one device work-queue; a CUDA graph replays the descriptor upload and
 * the launch.  Every array must be device memory (IFX_ERR_ARGUMENT
 * otherwise); the work is enqueued on `stream` and the call returns at once.
 * Results equal the single-request entry points:
 *   IFX_OP_FACTORED2D  ifx_imfilter_factored with factors (axis 0, axis 1),
 *                      each at most 33 taps; FP32 arithmetic
 *   IFX_OP_GRADIENTS2D ifx_imgradients with a 3-tap pair at first index -1
 *                      (weights[0] = derivative, weights[1] = smoothing)
 *   IFX_OP_LAPLACIAN2D ifx_imfilter_laplacian, flags (1,1), Float32 output
 *   IFX_OP_MEDIAN2D    ifx_mapwindow_median, window 3x3 or 5x5
 * Images are Float32, N0f8 or UInt8; outputs Float32 or Float64. */
typedef enum {
    IFX_OP_FACTORED2D = 1,
    IFX_OP_GRADIENTS2D = 2,
    IFX_OP_LAPLACIAN2D = 3,
    IFX_OP_MEDIAN2D = 4
} ifx_op;

typedef struct ifx_request {
    int32_t op;                    /* ifx_op */
    int32_t window;                /* IFX_OP_MEDIAN2D: 3 or 5 */
    ifx_array_t img;
    ifx_array_t out[2];            /* out[1] is used by IFX_OP_GRADIENTS2D only */
    ifx_border_t border;
    int32_t taps[2];
    int64_t first[2];
    const double *weights[2];      /* host memory */
} ifx_request_t;

/* Runs the batch; *tiles receives the number of tiles (may be NULL). */
int ifx_batch_run(ifx_context_t *ctx, const ifx_request_t *reqs, int32_t n, int64_t *tiles,
                  void *stream);

/* A batch validated once, with its descriptors kept in device memory, for
 * workloads that run the same requests (the same arrays, new contents) many
 * times.  Each launch is one CUDA graph replay on `stream`.  Launches of one
 * plan must not overlap on the device (they share its tile counter); the
 * arrays must outlive the plan. */
typedef struct ifx_batch_plan ifx_batch_plan_t;
int ifx_batch_plan_create(ifx_context_t *ctx, const ifx_request_t *reqs, int32_t n,
                          ifx_batch_plan_t **plan);
int ifx_batch_plan_launch(ifx_batch_plan_t *plan, int64_t *tiles, void *stream);
int ifx_batch_plan_destroy(ifx_batch_plan_t *plan);

/* ---- serving: continuous batching of requests as they arrive ---------------
 * ifx_server_submit returns at once with a ticket.  An engine thread admits
 * queued requests in arrival order while the device bytes they need (staged
 * host images and host outputs; device arrays are used in place and cost
 * nothing) fit under hbm_cap_bytes, uploads host images on a copy stream,
 * packs admitted requests into batched launches (at most max_batch each, at
 * most max_inflight batches on the device at once), copies host outputs back
 * and frees their device memory.  Requests use the ifx_request_t forms of
 * ifx_batch_run; the weights are copied at submit.  Latency is measured from
 * submit to results in place (host outputs copied back). */
typedef struct ifx_server ifx_server_t;

typedef struct ifx_server_config {
    int64_t hbm_cap_bytes;         /* device bytes held by admitted requests, at most */
    int32_t max_batch;             /* requests per batched launch */
    int32_t max_inflight;          /* batched launches on the device at once */
} ifx_server_config_t;

typedef struct ifx_server_metrics {
    uint64_t submitted, completed, failed, batches;
    uint64_t pixels;               /* pixels of completed requests */
    double p50_latency_s, p99_latency_s, max_latency_s;
    double busy_s;                 /* first submit -> last completion */
    int64_t hbm_in_use, hbm_peak;
    int32_t queue_depth;           /* submitted, not yet admitted */
    uint64_t deferred_free;        /* admissions held back because the device's free
                                      memory (less a 256 MiB reserve) was short */
} ifx_server_metrics_t;

int ifx_server_create(ifx_context_t *ctx, const ifx_server_config_t *cfg, ifx_server_t **srv);
int ifx_server_submit(ifx_server_t *srv, const ifx_request_t *req, uint64_t *ticket);
/* IFX_ERR_TIMEOUT when the request is not done within timeout_s; *status gets
 * the request's own status when it is. */
int ifx_server_wait(ifx_server_t *srv, uint64_t ticket, double timeout_s, int32_t *status);
int ifx_server_drain(ifx_server_t *srv, double timeout_s);
/* Cancels a request that has not joined a launched batch: it completes with
 * IFX_ERR_CANCELLED (counted as failed) and its device memory is released;
 * IFX_ERR_ARGUMENT when the ticket is unknown, done or already launched. */
int ifx_server_cancel(ifx_server_t *srv, uint64_t ticket);
/* paused != 0: requests are still admitted (and uploaded) but no new batch
 * launches until the server is resumed (paused = 0); batches already launched
 * finish.  For maintenance windows and for tests that need requests to wait. */
int ifx_server_pause(ifx_server_t *srv, int32_t paused);
/* Failure injection on the host, for tests: the next `count` batched launches
 * are reported as failed launches without running their kernel; their
 * requests complete with IFX_ERR_CUDA and the server keeps serving. */
int ifx_server_inject_launch_error(ifx_server_t *srv, int32_t count);
int ifx_server_metrics(ifx_server_t *srv, ifx_server_metrics_t *m);
int ifx_server_reset_metrics(ifx_server_t *srv);
int ifx_server_destroy(ifx_server_t *srv);

#ifdef __cplusplus
}
#endif
#endif /* IFX_GB300_H */
