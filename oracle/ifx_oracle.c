/*
 * ifx_oracle.c -- CPU restatement of ImageFiltering.jl's FIR and rank-filter
 * path, in FP64.  THIS IS TEST INFRASTRUCTURE: only the tests, the smoke check
 * and the CPU-baseline leg of the benchmark load it, as the checker.  The
 * product path (the CUDA library) never calls into this file.
 *
 * Every routine follows the reference loops step by step, in the same
 * summation order, and cites the reference file:line it restates (paths are
 * relative to the ImageFiltering.jl v0.7.12 source tree):
 *
 *   ora_padindex        src/border.jl:564-596      (padindex: mod-based index maps)
 *   ora_padarray        src/border.jl:324-352,      (padarray -> BorderArray -> copy!)
 *                       src/borderarray.jl:179-196
 *   ora_imfilter_cascade src/imfilter.jl:331-341    (pad whole image once, accumulated padding)
 *                       src/imfilter.jl:385-457     (cascade over shrinking index ranges)
 *                       src/imfilter.jl:671-739     (1-D factor loops, sequential tap sum)
 *                       src/border.jl:614-684       (calculate_padding / expand / shrink)
 *   ora_imfilter_dense  src/imfilter.jl:624-669     (dense loop, column-major tap order)
 *   ora_laplacian       src/specialty.jl:3-17       (Laplacian stencil, -2n*A[I] then pairs)
 *   ora_mapwindow_*     src/mapwindow.jl:123-131, 270-333 (median_fast!, mapwindow_kernel!,
 *                       copy_win! with padindex relative to window-intersect-image)
 *   ora_extrema_trunc   src/mapwindow.jl:388-473    (Lemire wedge: min/max over the window
 *                       truncated at the edges; even windows allowed)
 *   ora_imfilter_iir    src/imfilter.jl:961-1092    (Triggs-Sdika passes with their border
 *                       initialisation, cascaded along the factors' axes)
 *
 * Arrays are column-major (axis 0 contiguous, i.e. Julia's axis 1), at most
 * ORA_MAXD dimensions, with 0-based indices; Julia's OffsetArray first indices
 * only shift axes and are handled by the caller.  Compile with
 * -ffp-contract=off so that no multiply-add is fused (the reference loops
 * `tmp += a*k` are not contracted).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <pthread.h>

#define ORA_MAXD 4

enum { ORA_REPLICATE = 0, ORA_CIRCULAR = 1, ORA_SYMMETRIC = 2, ORA_REFLECT = 3, ORA_FILL = 4 };
enum { ORA_OK = 0, ORA_EARG = 1, ORA_EDIM = 2, ORA_EERR = 3, ORA_ENOMEM = 5 };

static int g_threads = 1;
void ora_set_threads(int n) { g_threads = n < 1 ? 1 : n; }
int ora_get_threads(void) { return g_threads; }

static int64_t mod64(int64_t x, int64_t m) { int64_t r = x % m; return r < 0 ? r + m : r; }

/* ---------------------------------------------------------------------------
 * padindex (src/border.jl:564-596).  Writes into idx[0 .. lo+n+hi) the source
 * index (0-based, in [0,n)) for padded positions -lo .. n-1+hi.
 *   replicate: clamp                                  (border.jl:566-571)
 *   circular : modrange over the image axis           (border.jl:573)
 *   symmetric: table [0..n-1, n-1..0], period 2n      (border.jl:574-580)
 *   reflect  : table [0..n-1, n-2..1], period 2n-2    (border.jl:581-586)
 * A zero-length period (symmetric n=0, reflect n<=1) is a DivideError in the
 * reference; it is reported as ORA_EERR.
 * ------------------------------------------------------------------------- */
int ora_padindex(int style, int64_t lo, int64_t n, int64_t hi, int64_t *idx)
{
    int64_t total = lo + n + hi;
    if (style == ORA_REPLICATE) {
        if (n <= 0 && total > 0) return ORA_EERR;
        for (int64_t p = 0; p < total; ++p) {
            int64_t x = p - lo;
            idx[p] = x < 0 ? 0 : (x > n - 1 ? n - 1 : x);
        }
        return ORA_OK;
    }
    if (style == ORA_CIRCULAR) {
        if (n <= 0) return total > 0 ? ORA_EERR : ORA_OK;
        for (int64_t p = 0; p < total; ++p) idx[p] = mod64(p - lo, n);
        return ORA_OK;
    }
    if (style == ORA_SYMMETRIC) {
        int64_t period = 2 * n;
        if (period <= 0) return ORA_EERR;
        for (int64_t p = 0; p < total; ++p) {
            int64_t r = mod64(p - lo, period);
            idx[p] = r < n ? r : period - 1 - r;
        }
        return ORA_OK;
    }
    if (style == ORA_REFLECT) {
        int64_t period = 2 * n - 2;
        if (period <= 0) return ORA_EERR;
        for (int64_t p = 0; p < total; ++p) {
            int64_t r = mod64(p - lo, period);
            idx[p] = r < n ? r : period - r;
        }
        return ORA_OK;
    }
    return ORA_EARG;
}

/* strides of a dense column-major array */
static void col_strides(int nd, const int64_t *sz, int64_t *st)
{
    int64_t s = 1;
    for (int d = 0; d < nd; ++d) { st[d] = s; s *= sz[d]; }
}
static int64_t prod(int nd, const int64_t *sz)
{
    int64_t p = 1;
    for (int d = 0; d < nd; ++d) p *= sz[d];
    return p;
}

/* ---------------------------------------------------------------------------
 * padarray (src/border.jl:324-352, src/borderarray.jl:179-196): the padded
 * copy with axes [-lo_d, n_d-1+hi_d].  Pad styles copy through padindex
 * (copydata!); Fill writes `fill` everywhere and then the image in the middle.
 * out has sizes lo_d+n_d+hi_d.
 * ------------------------------------------------------------------------- */
int ora_padarray(int nd, const int64_t *n, const double *img,
                 int style, double fill, const int64_t *lo, const int64_t *hi,
                 double *out)
{
    if (nd < 1 || nd > ORA_MAXD) return ORA_EARG;
    int64_t psz[ORA_MAXD], pst[ORA_MAXD], ist[ORA_MAXD];
    for (int d = 0; d < nd; ++d) psz[d] = lo[d] + n[d] + hi[d];
    col_strides(nd, psz, pst);
    col_strides(nd, n, ist);
    int64_t total = prod(nd, psz);
    if (style == ORA_FILL) {
        for (int64_t p = 0; p < total; ++p) {
            int64_t rem = p, src = 0;
            int inside = 1;
            for (int d = 0; d < nd; ++d) {
                int64_t c = rem % psz[d] - lo[d];
                rem /= psz[d];
                if (c < 0 || c >= n[d]) { inside = 0; break; }
                src += c * ist[d];
            }
            out[p] = inside ? img[src] : fill;
        }
        return ORA_OK;
    }
    int64_t *maps[ORA_MAXD] = {0};
    int rc = ORA_OK;
    for (int d = 0; d < nd; ++d) {
        maps[d] = (int64_t *)malloc(sizeof(int64_t) * (size_t)(psz[d] > 0 ? psz[d] : 1));
        if (!maps[d]) { rc = ORA_ENOMEM; goto done; }
        rc = ora_padindex(style, lo[d], n[d], hi[d], maps[d]);
        if (rc) goto done;
    }
    for (int64_t p = 0; p < total; ++p) {
        int64_t rem = p, src = 0;
        for (int d = 0; d < nd; ++d) {
            int64_t c = rem % psz[d];
            rem /= psz[d];
            src += maps[d][c] * ist[d];
        }
        out[p] = img[src];
    }
done:
    for (int d = 0; d < nd; ++d) free(maps[d]);
    return rc;
}

/* ---------------------------------------------------------------------------
 * One FIR pass of a 1-D factor along `axis` (src/imfilter.jl:705-739):
 *   for Ipost, for i, for Ipre:  tmp = 0; for j in taps: tmp += A[Ipre,i+j,Ipost]*k[j]
 * A lives on box [alo, alo+asz), the result on box [olo, olo+osz) of the same
 * index space; the result box is written into `dst` laid out on `dbox`.
 * Threads split the outermost non-unit axis, like FIRTiled's task partition
 * (src/imfilter.jl:486-500); each output value is computed identically.
 * ------------------------------------------------------------------------- */
typedef struct {
    int nd, axis;
    const double *A; const int64_t *alo, *asz;
    double *D; const int64_t *dlo, *dsz;
    const int64_t *olo, *osz;
    const double *k; int64_t kfirst, klen;
    int64_t t0, t1;   /* range over the split axis */
    int split;
} pass_job;

static void *pass_worker(void *arg)
{
    pass_job *J = (pass_job *)arg;
    int nd = J->nd;
    int64_t ast[ORA_MAXD] = {0}, dst[ORA_MAXD] = {0};
    col_strides(nd, J->asz, ast);
    col_strides(nd, J->dsz, dst);
    int64_t cnt[ORA_MAXD], lo[ORA_MAXD];
    for (int d = 0; d < nd; ++d) { lo[d] = J->olo[d]; cnt[d] = J->osz[d]; }
    lo[J->split] = J->olo[J->split] + J->t0;
    cnt[J->split] = J->t1 - J->t0;
    int64_t total = prod(nd, cnt);
    int64_t astep = ast[J->axis];
    for (int64_t p = 0; p < total; ++p) {
        int64_t rem = p, aoff = 0, doff = 0;
        for (int d = 0; d < nd; ++d) {
            int64_t c = lo[d] + rem % cnt[d];
            rem /= cnt[d];
            aoff += (c - J->alo[d]) * ast[d];
            doff += (c - J->dlo[d]) * dst[d];
        }
        const double *a = J->A + aoff + J->kfirst * astep;
        double tmp = 0.0;
        for (int64_t j = 0; j < J->klen; ++j) tmp += a[j * astep] * J->k[j];
        J->D[doff] = tmp;
    }
    return NULL;
}

static void run_pass(pass_job *base)
{
    int nd = base->nd;
    /* split the outermost axis with >1 element */
    int split = nd - 1;
    while (split > 0 && base->osz[split] <= 1) --split;
    base->split = split;
    int64_t len = base->osz[split];
    int nt = g_threads;
    if (nt > len) nt = (int)(len > 0 ? len : 1);
    if (nt <= 1) { base->t0 = 0; base->t1 = len; pass_worker(base); return; }
    pthread_t th[256];
    pass_job jobs[256];
    if (nt > 256) nt = 256;
    int64_t chunk = (len + nt - 1) / nt;
    int launched = 0;
    for (int t = 0; t < nt; ++t) {
        jobs[t] = *base;
        jobs[t].t0 = t * chunk;
        jobs[t].t1 = (t + 1) * chunk < len ? (t + 1) * chunk : len;
        if (jobs[t].t0 >= jobs[t].t1) break;
        pthread_create(&th[t], NULL, pass_worker, &jobs[t]);
        ++launched;
    }
    for (int t = 0; t < launched; ++t) pthread_join(th[t], NULL);
}

/* ---------------------------------------------------------------------------
 * imfilter with a tuple of 1-D factors (src/imfilter.jl:331-341, 385-457):
 *  1. padding = accumulate_padding over all factors (border.jl:614-621);
 *     lo = max(0,-sum first), hi = max(0, sum last) per axis (border.jl:637-641)
 *  2. A = padarray(img, Pad/Fill(lo,hi))
 *  3. indsstep = shrink(expand(axes(img), padding), k1); each pass filters
 *     into a fresh buffer over indsstep, then indsstep = shrink(indsstep, k_next);
 *     the last pass writes over axes(img).
 * Factor f runs along axis[f], taps k[off[f] .. off[f]+len[f]) with kernel
 * indices kfirst[f] .. kfirst[f]+len[f]-1.  A factor that is a copy (one tap
 * at index 0 equal to 1, src/imfilter.jl:1252-1255) is skipped, as iscopy does.
 * ------------------------------------------------------------------------- */
int ora_imfilter_cascade(int nd, const int64_t *n, const double *img,
                         int nf, const int32_t *axis, const int64_t *kfirst,
                         const int64_t *klen, const double *kdata,
                         int style, double fill, double *out)
{
    if (nd < 1 || nd > ORA_MAXD || nf < 0 || nf > 64) return ORA_EARG;
    int64_t koff[64];
    int64_t o = 0;
    for (int f = 0; f < nf; ++f) {
        if (axis[f] < 0 || axis[f] >= nd || klen[f] < 1) return ORA_EARG;
        koff[f] = o; o += klen[f];
    }
    int64_t N = prod(nd, n);
    /* drop copy kernels */
    int keep[64], nk = 0;
    for (int f = 0; f < nf; ++f) {
        int copy = (klen[f] == 1 && kfirst[f] == 0 && kdata[koff[f]] == 1.0);
        if (!copy) keep[nk++] = f;
    }
    if (N == 0) return ORA_OK;
    if (nk == 0) { memcpy(out, img, sizeof(double) * (size_t)N); return ORA_OK; }
    int64_t pfirst[ORA_MAXD] = {0}, plast[ORA_MAXD] = {0};
    for (int f = 0; f < nf; ++f) {      /* calculate_padding includes copies too (axes 0:0) */
        pfirst[axis[f]] += kfirst[f];
        plast[axis[f]] += kfirst[f] + klen[f] - 1;
    }
    int64_t lo[ORA_MAXD], hi[ORA_MAXD], psz[ORA_MAXD], plo[ORA_MAXD];
    for (int d = 0; d < nd; ++d) {
        lo[d] = pfirst[d] < 0 ? -pfirst[d] : 0;
        hi[d] = plast[d] > 0 ? plast[d] : 0;
        psz[d] = lo[d] + n[d] + hi[d];
        plo[d] = -lo[d];
    }
    double *A = (double *)malloc(sizeof(double) * (size_t)prod(nd, psz));
    if (!A) return ORA_ENOMEM;
    int rc = ora_padarray(nd, n, img, style, fill, lo, hi, A);
    if (rc) { free(A); return rc; }
    /* step ranges: expand(axes(img), padding) then shrink by each kept kernel */
    int64_t slo[ORA_MAXD], shi[ORA_MAXD];
    for (int d = 0; d < nd; ++d) { slo[d] = pfirst[d]; shi[d] = n[d] - 1 + plast[d]; }
    const double *cur = A;
    int64_t clo[ORA_MAXD], csz[ORA_MAXD];
    for (int d = 0; d < nd; ++d) { clo[d] = plo[d]; csz[d] = psz[d]; }
    double *owned = A;
    for (int q = 0; q < nk; ++q) {
        int f = keep[q];
        int ax = axis[f];
        slo[ax] -= kfirst[f];
        shi[ax] -= kfirst[f] + klen[f] - 1;
        int64_t olo[ORA_MAXD], osz[ORA_MAXD];
        for (int d = 0; d < nd; ++d) {
            olo[d] = slo[d];
            osz[d] = shi[d] - slo[d] + 1;
            if (q == nk - 1) {     /* intersect with axes(out) */
                int64_t a = olo[d] > 0 ? olo[d] : 0;
                int64_t b = shi[d] < n[d] - 1 ? shi[d] : n[d] - 1;
                olo[d] = a; osz[d] = b - a + 1;
            }
            if (osz[d] < 0) osz[d] = 0;
        }
        double *D;
        int64_t dlo[ORA_MAXD], dsz[ORA_MAXD];
        if (q == nk - 1) {
            D = out;
            for (int d = 0; d < nd; ++d) { dlo[d] = 0; dsz[d] = n[d]; }
        } else {
            for (int d = 0; d < nd; ++d) { dlo[d] = olo[d]; dsz[d] = osz[d]; }
            D = (double *)malloc(sizeof(double) * (size_t)(prod(nd, dsz) > 0 ? prod(nd, dsz) : 1));
            if (!D) { free(owned); return ORA_ENOMEM; }
        }
        pass_job job;
        memset(&job, 0, sizeof job);
        job.nd = nd; job.axis = ax;
        job.A = cur; job.alo = clo; job.asz = csz;
        job.D = D; job.dlo = dlo; job.dsz = dsz;
        job.olo = olo; job.osz = osz;
        job.k = kdata + koff[f]; job.kfirst = kfirst[f]; job.klen = klen[f];
        if (prod(nd, osz) > 0) run_pass(&job);
        if (owned) free(owned);
        owned = (q == nk - 1) ? NULL : D;
        cur = D;
        for (int d = 0; d < nd; ++d) { clo[d] = dlo[d]; csz[d] = dsz[d]; }
    }
    return ORA_OK;
}

/* ---------------------------------------------------------------------------
 * Dense N-d kernel (src/imfilter.jl:624-669): pad by the kernel's axes, then
 *   out[I] = sum over J (column-major: axis 0 fastest) of A[I+J]*K[J],
 * accumulated sequentially from 0.  K has sizes ksz, first indices kfirst.
 * Threads split the outermost axis of the output.
 * ------------------------------------------------------------------------- */
typedef struct {
    int nd; const int64_t *n; const double *A; const int64_t *psz, *lo;
    const double *K; const int64_t *ksz, *kfirst; double *out;
    int64_t t0, t1;
} dense_job;

static void *dense_worker(void *arg)
{
    dense_job *J = (dense_job *)arg;
    int nd = J->nd;
    int64_t ast[ORA_MAXD], ost[ORA_MAXD];
    col_strides(nd, J->psz, ast);
    col_strides(nd, J->n, ost);
    int64_t kn = prod(nd, J->ksz);
    int64_t *koffs = (int64_t *)malloc(sizeof(int64_t) * (size_t)kn);
    for (int64_t t = 0; t < kn; ++t) {
        int64_t rem = t, off = 0;
        for (int d = 0; d < nd; ++d) {
            int64_t c = rem % J->ksz[d] + J->kfirst[d];
            rem /= J->ksz[d];
            off += c * ast[d];
        }
        koffs[t] = off;
    }
    int64_t cnt[ORA_MAXD];
    for (int d = 0; d < nd; ++d) cnt[d] = J->n[d];
    cnt[nd - 1] = J->t1 - J->t0;
    int64_t total = prod(nd, cnt);
    for (int64_t p = 0; p < total; ++p) {
        int64_t rem = p, aoff = 0, ooff = 0;
        for (int d = 0; d < nd; ++d) {
            int64_t c = rem % cnt[d];
            rem /= cnt[d];
            if (d == nd - 1) c += J->t0;
            aoff += (c + J->lo[d]) * ast[d];
            ooff += c * ost[d];
        }
        const double *a = J->A + aoff;
        double tmp = 0.0;
        for (int64_t t = 0; t < kn; ++t) tmp += a[koffs[t]] * J->K[t];
        J->out[ooff] = tmp;
    }
    free(koffs);
    return NULL;
}

int ora_imfilter_dense(int nd, const int64_t *n, const double *img,
                       const int64_t *ksz, const int64_t *kfirst, const double *K,
                       int style, double fill, double *out)
{
    if (nd < 1 || nd > ORA_MAXD) return ORA_EARG;
    if (prod(nd, n) == 0) return ORA_OK;
    int64_t lo[ORA_MAXD], hi[ORA_MAXD], psz[ORA_MAXD];
    for (int d = 0; d < nd; ++d) {
        int64_t f = kfirst[d], l = kfirst[d] + ksz[d] - 1;
        lo[d] = f < 0 ? -f : 0;
        hi[d] = l > 0 ? l : 0;
        psz[d] = lo[d] + n[d] + hi[d];
    }
    double *A = (double *)malloc(sizeof(double) * (size_t)prod(nd, psz));
    if (!A) return ORA_ENOMEM;
    int rc = ora_padarray(nd, n, img, style, fill, lo, hi, A);
    if (rc) { free(A); return rc; }
    int64_t len = n[nd - 1];
    int nt = g_threads;
    if (nt > len) nt = (int)len;
    if (nt < 1) nt = 1;
    if (nt > 256) nt = 256;
    pthread_t th[256];
    dense_job jobs[256];
    int64_t chunk = (len + nt - 1) / nt;
    int launched = 0;
    for (int t = 0; t < nt; ++t) {
        dense_job j = { nd, n, A, psz, lo, K, ksz, kfirst, out, t * chunk,
                        (t + 1) * chunk < len ? (t + 1) * chunk : len };
        if (j.t0 >= j.t1) break;
        jobs[t] = j;
        if (nt == 1) { dense_worker(&jobs[t]); launched = 0; break; }
        pthread_create(&th[t], NULL, dense_worker, &jobs[t]);
        ++launched;
    }
    for (int t = 0; t < launched; ++t) pthread_join(th[t], NULL);
    free(A);
    return ORA_OK;
}

/* ---------------------------------------------------------------------------
 * Laplacian stencil (src/specialty.jl:3-17) with padding axes(L) = -1:1 on the
 * flagged axes (src/kernel.jl:384).  The arithmetic type is the output
 * eltype (src/imfilter.jl:1134-1139); three variants keep the exact rounding:
 *   ora_laplacian_f64: Float64,  ora_laplacian_f32: Float32,
 *   ora_laplacian_i64: integer (Int16 outputs fit for 8-bit inputs).
 *   tmp = convert(TT, -n*A[I]); for each flagged axis: tmp += A[I+e]; tmp += A[I-e]
 * ------------------------------------------------------------------------- */
#define LAPLACIAN_BODY(T)                                                         \
    if (nd < 1 || nd > ORA_MAXD) return ORA_EARG;                                 \
    if (prod(nd, n) == 0) return ORA_OK;                                          \
    int64_t lo[ORA_MAXD], hi[ORA_MAXD], psz[ORA_MAXD], ast[ORA_MAXD], ost[ORA_MAXD]; \
    int cnt = 0;                                                                  \
    for (int d = 0; d < nd; ++d) {                                                \
        lo[d] = hi[d] = flags[d] ? 1 : 0;                                         \
        cnt += flags[d] ? 1 : 0;                                                  \
        psz[d] = n[d] + lo[d] + hi[d];                                            \
    }                                                                             \
    double *A = (double *)malloc(sizeof(double) * (size_t)prod(nd, psz));        \
    if (!A) return ORA_ENOMEM;                                                    \
    int rc = ora_padarray(nd, n, img, style, fill, lo, hi, A);                    \
    if (rc) { free(A); return rc; }                                               \
    col_strides(nd, psz, ast);                                                    \
    col_strides(nd, n, ost);                                                      \
    int64_t total = prod(nd, n);                                                  \
    for (int64_t p = 0; p < total; ++p) {                                         \
        int64_t rem = p, aoff = 0;                                                \
        for (int d = 0; d < nd; ++d) {                                            \
            int64_t c = rem % n[d];                                               \
            rem /= n[d];                                                          \
            aoff += (c + lo[d]) * ast[d];                                         \
        }                                                                         \
        T tmp = (T)(-(2 * cnt)) * (T)A[aoff];                                     \
        for (int d = 0; d < nd; ++d) {                                            \
            if (!flags[d]) continue;                                              \
            tmp = tmp + (T)A[aoff + ast[d]];                                      \
            tmp = tmp + (T)A[aoff - ast[d]];                                      \
        }                                                                         \
        out[p] = (double)tmp;                                                     \
    }                                                                             \
    free(A);                                                                      \
    return ORA_OK;

int ora_laplacian_f64(int nd, const int64_t *n, const double *img, const int32_t *flags,
                      int style, double fill, double *out) { LAPLACIAN_BODY(double) }
int ora_laplacian_f32(int nd, const int64_t *n, const double *img, const int32_t *flags,
                      int style, double fill, double *out) { LAPLACIAN_BODY(float) }
int ora_laplacian_i64(int nd, const int64_t *n, const double *img, const int32_t *flags,
                      int style, double fill, double *out) { LAPLACIAN_BODY(int64_t) }

/* ---------------------------------------------------------------------------
 * Window gathering for mapwindow (src/mapwindow.jl:270-333).
 * For output pixel I and window offsets wfirst..wfirst+wlen-1 per axis:
 *  - Pad styles: copy_win! maps each axis with padindex relative to
 *    inner = window-intersect-image (mapwindow.jl:311-314), so every value
 *    comes from inside the truncated window;
 *  - Fill: values outside the image are the fill value (mapwindow.jl:325-333).
 * Interior windows (mapwindow.jl:286-292) are the same as the padindex gather
 * with zero padding, so one routine covers both.
 * ------------------------------------------------------------------------- */
static int gather_window(int nd, const int64_t *n, const int64_t *ist, const double *img,
                         const int64_t *I, const int64_t *wfirst, const int64_t *wlen,
                         int style, double fill, double *buf, int64_t *scratch)
{
    /* scratch holds per-axis index maps, wlen[d] entries each */
    int64_t *maps[ORA_MAXD];
    int64_t *s = scratch;
    for (int d = 0; d < nd; ++d) {
        maps[d] = s;
        s += wlen[d];
        int64_t of = I[d] + wfirst[d], ol = of + wlen[d] - 1;
        if (style == ORA_FILL) {
            for (int64_t t = 0; t < wlen[d]; ++t) {
                int64_t c = of + t;
                maps[d][t] = (c < 0 || c >= n[d]) ? -1 : c;
            }
            continue;
        }
        int64_t inf = of > 0 ? of : 0, inl = ol < n[d] - 1 ? ol : n[d] - 1;
        if (inl < inf) return ORA_EERR;       /* empty intersection */
        int64_t lo = inf - of, hi = ol - inl;
        int rc = ora_padindex(style, lo, inl - inf + 1, hi, maps[d]);
        if (rc) return rc;
        for (int64_t t = 0; t < wlen[d]; ++t) maps[d][t] += inf;
    }
    int64_t wn = prod(nd, wlen);
    for (int64_t t = 0; t < wn; ++t) {
        int64_t rem = t, off = 0;
        int outside = 0;
        for (int d = 0; d < nd; ++d) {
            int64_t c = maps[d][rem % wlen[d]];
            rem /= wlen[d];
            if (c < 0) { outside = 1; break; }
            off += c * ist[d];
        }
        buf[t] = outside ? fill : img[off];
    }
    return ORA_OK;
}

static void sort_doubles(double *v, int64_t m)
{
    for (int64_t i = 1; i < m; ++i) {     /* insertion sort: windows are small */
        double x = v[i];
        int64_t j = i - 1;
        while (j >= 0 && v[j] > x) { v[j + 1] = v[j]; --j; }
        v[j + 1] = x;
    }
}

/* median_fast! (src/mapwindow.jl:123-128): partialsort! at (first+last)/2 of
 * the vectorised window, i.e. the ((1+m) div 2)-th smallest of m values. */
int ora_mapwindow_median(int nd, const int64_t *n, const double *img,
                         const int64_t *wfirst, const int64_t *wlen,
                         int style, double fill, double *out)
{
    if (nd < 1 || nd > ORA_MAXD) return ORA_EARG;
    int64_t ist[ORA_MAXD];
    col_strides(nd, n, ist);
    int64_t wn = prod(nd, wlen), ms = 0;
    for (int d = 0; d < nd; ++d) ms += wlen[d];
    double *buf = (double *)malloc(sizeof(double) * (size_t)(wn > 0 ? wn : 1));
    int64_t *scr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ms > 0 ? ms : 1));
    if (!buf || !scr) { free(buf); free(scr); return ORA_ENOMEM; }
    int64_t total = prod(nd, n);
    int rc = ORA_OK;
    for (int64_t p = 0; p < total && !rc; ++p) {
        int64_t I[ORA_MAXD], rem = p;
        for (int d = 0; d < nd; ++d) { I[d] = rem % n[d]; rem /= n[d]; }
        rc = gather_window(nd, n, ist, img, I, wfirst, wlen, style, fill, buf, scr);
        if (rc) break;
        sort_doubles(buf, wn);
        out[p] = buf[(wn + 1) / 2 - 1];
    }
    free(buf); free(scr);
    return rc;
}

/* Generic mapwindow with extrema / minimum / maximum and a border
 * (src/mapwindow.jl:75-85, 270-333 with Base.extrema on the window). */
int ora_mapwindow_extrema(int nd, const int64_t *n, const double *img,
                          const int64_t *wfirst, const int64_t *wlen,
                          int style, double fill, double *out_min, double *out_max)
{
    if (nd < 1 || nd > ORA_MAXD) return ORA_EARG;
    int64_t ist[ORA_MAXD];
    col_strides(nd, n, ist);
    int64_t wn = prod(nd, wlen), ms = 0;
    for (int d = 0; d < nd; ++d) ms += wlen[d];
    double *buf = (double *)malloc(sizeof(double) * (size_t)(wn > 0 ? wn : 1));
    int64_t *scr = (int64_t *)malloc(sizeof(int64_t) * (size_t)(ms > 0 ? ms : 1));
    if (!buf || !scr) { free(buf); free(scr); return ORA_ENOMEM; }
    int64_t total = prod(nd, n);
    int rc = ORA_OK;
    for (int64_t p = 0; p < total && !rc; ++p) {
        int64_t I[ORA_MAXD], rem = p;
        for (int d = 0; d < nd; ++d) { I[d] = rem % n[d]; rem /= n[d]; }
        rc = gather_window(nd, n, ist, img, I, wfirst, wlen, style, fill, buf, scr);
        if (rc) break;
        double mn = buf[0], mx = buf[0];
        for (int64_t t = 1; t < wn; ++t) {
            if (buf[t] < mn) mn = buf[t];
            if (buf[t] > mx) mx = buf[t];
        }
        if (out_min) out_min[p] = mn;
        if (out_max) out_max[p] = mx;
    }
    free(buf); free(scr);
    return rc;
}

/* Lemire extrema filter (src/mapwindow.jl:388-473): per axis d, the window of
 * width w covers offsets -(w>>1) .. w-1-(w>>1), truncated at the array edges
 * (the wedge only ever holds in-range indices).  Even widths are allowed.
 * The min/max of a box is the same whether taken axis by axis or at once, so
 * this takes it directly over the truncated box. */
int ora_extrema_trunc(int nd, const int64_t *n, const double *img, const int64_t *w,
                      double *out_min, double *out_max)
{
    if (nd < 1 || nd > ORA_MAXD) return ORA_EARG;
    int64_t ist[ORA_MAXD];
    col_strides(nd, n, ist);
    int64_t total = prod(nd, n);
    for (int64_t p = 0; p < total; ++p) {
        int64_t I[ORA_MAXD], a[ORA_MAXD], b[ORA_MAXD], cnt[ORA_MAXD], rem = p;
        for (int d = 0; d < nd; ++d) {
            I[d] = rem % n[d]; rem /= n[d];
            int64_t wd = w[d] < 1 ? 1 : w[d];
            a[d] = I[d] - (wd >> 1);
            b[d] = I[d] + wd - 1 - (wd >> 1);
            if (a[d] < 0) a[d] = 0;
            if (b[d] > n[d] - 1) b[d] = n[d] - 1;
            cnt[d] = b[d] - a[d] + 1;
        }
        int64_t m = prod(nd, cnt);
        double mn = 0, mx = 0;
        for (int64_t t = 0; t < m; ++t) {
            int64_t r2 = t, off = 0;
            for (int d = 0; d < nd; ++d) { off += (a[d] + r2 % cnt[d]) * ist[d]; r2 /= cnt[d]; }
            double v = img[off];
            if (t == 0 || v < mn) mn = v;
            if (t == 0 || v > mx) mx = v;
        }
        if (out_min) out_min[p] = mn;
        if (out_max) out_max[p] = mx;
    }
    return ORA_OK;
}

/* Fast 8-bit median used only for the CPU baseline timing: the same window
 * gather as ora_mapwindow_median, but a 256-bin count selects the median. */
int ora_mapwindow_median_u8(int nd, const int64_t *n, const uint8_t *img,
                            const int64_t *wfirst, const int64_t *wlen,
                            int style, double fill, uint8_t *out, int64_t row0, int64_t row1)
{
    if (nd != 2) return ORA_EARG;
    int64_t wn = wlen[0] * wlen[1];
    int64_t *m0 = (int64_t *)malloc(sizeof(int64_t) * (size_t)wlen[0]);
    int64_t *m1 = (int64_t *)malloc(sizeof(int64_t) * (size_t)wlen[1]);
    if (!m0 || !m1) { free(m0); free(m1); return ORA_ENOMEM; }
    int rank = (int)((wn + 1) / 2);
    uint8_t fv = (uint8_t)fill;
    for (int64_t y = row0; y < row1; ++y) {
        for (int64_t x = 0; x < n[0]; ++x) {
            int64_t I[2] = { x, y };
            int64_t *maps[2] = { m0, m1 };
            for (int d = 0; d < 2; ++d) {
                int64_t of = I[d] + wfirst[d], ol = of + wlen[d] - 1;
                if (style == ORA_FILL) {
                    for (int64_t t = 0; t < wlen[d]; ++t) {
                        int64_t c = of + t;
                        maps[d][t] = (c < 0 || c >= n[d]) ? -1 : c;
                    }
                    continue;
                }
                int64_t inf = of > 0 ? of : 0, inl = ol < n[d] - 1 ? ol : n[d] - 1;
                ora_padindex(style, inf - of, inl - inf + 1, ol - inl, maps[d]);
                for (int64_t t = 0; t < wlen[d]; ++t) maps[d][t] += inf;
            }
            int hist[256];
            memset(hist, 0, sizeof hist);
            for (int64_t j = 0; j < wlen[1]; ++j)
                for (int64_t i = 0; i < wlen[0]; ++i) {
                    int64_t a = m0[i], b = m1[j];
                    hist[(a < 0 || b < 0) ? fv : img[a + b * n[0]]]++;
                }
            int acc = 0, v = 0;
            while (v < 255 && acc + hist[v] < rank) acc += hist[v++];
            out[x + y * n[0]] = (uint8_t)v;
        }
    }
    free(m0); free(m1);
    return ORA_OK;
}

typedef struct {
    const int64_t *n; const uint8_t *img; const int64_t *wfirst, *wlen;
    int style; double fill; uint8_t *out; int64_t r0, r1;
} med_job;

static void *med_worker(void *arg)
{
    med_job *J = (med_job *)arg;
    ora_mapwindow_median_u8(2, J->n, J->img, J->wfirst, J->wlen, J->style, J->fill,
                            J->out, J->r0, J->r1);
    return NULL;
}

/* Threaded driver for the 8-bit median over rows [row0,row1) of a 2-D image. */
int ora_mapwindow_median_u8_mt(const int64_t *n, const uint8_t *img,
                               const int64_t *wfirst, const int64_t *wlen,
                               int style, double fill, uint8_t *out, int64_t row0, int64_t row1)
{
    int64_t len = row1 - row0;
    int nt = g_threads;
    if (nt > len) nt = (int)(len > 0 ? len : 1);
    if (nt > 256) nt = 256;
    pthread_t th[256];
    med_job jobs[256];
    int64_t chunk = (len + nt - 1) / nt;
    int launched = 0;
    for (int t = 0; t < nt; ++t) {
        med_job j = { n, img, wfirst, wlen, style, fill, out, row0 + t * chunk,
                      row0 + ((t + 1) * chunk < len ? (t + 1) * chunk : len) };
        if (j.r0 >= j.r1) break;
        jobs[t] = j;
        pthread_create(&th[t], NULL, med_worker, &jobs[t]);
        ++launched;
    }
    for (int t = 0; t < launched; ++t) pthread_join(th[t], NULL);
    return ORA_OK;
}

/* ------------------------------------------------------------------ IIR
 * One Triggs-Sdika pass (order 3 forward, order 3 backward) along a line of
 * length L with element stride st, x -> y (x == y allowed):
 * _imfilter_dim! (src/imfilter.jl:961-1030) with _leftborder!
 * (src/imfilter.jl:1033-1045), _rightborder! (1057-1084) and rightΔu
 * (1087-1092).  ab = a1 a2 a3 b1 b2 b3; M row-major 3x3; edge 0 = Pad
 * (boundary values are the line's end elements), 1 = Fill(fill).
 *
 * Types as in the reference: the arithmetic runs in CT = promote(eltype(out),
 * coefficient type) (iir_line_f64 / iir_line_f32), every stored result is
 * rounded to eltype(out) (s32: Float32), sum(a) and sum(b) are taken in the
 * coefficients' type (c32: Float32).  x and y hold the values as doubles. */
#define ORA_IIR_LINE(NAME, CT)                                                                        \
static void NAME(const double *x, double *y, int64_t L, int64_t st, const double *ab, double scale_,  \
                 const double *M_, int edge, double fill_, int s32, int c32)                          \
{                                                                                                     \
    const CT a[3] = {(CT)ab[0], (CT)ab[1], (CT)ab[2]}, b[3] = {(CT)ab[3], (CT)ab[4], (CT)ab[5]};      \
    CT M[9];                                                                                          \
    for (int r = 0; r < 9; ++r) M[r] = (CT)M_[r];                                                     \
    const CT scale = (CT)scale_;                                                                      \
    const CT om_a = c32 ? (CT)(1.0f - (((float)ab[0] + (float)ab[1]) + (float)ab[2]))                 \
                        : (CT)(1.0 - ((ab[0] + ab[1]) + ab[2]));                                      \
    const CT om_b = c32 ? (CT)(1.0f - (((float)ab[3] + (float)ab[4]) + (float)ab[5]))                 \
                        : (CT)(1.0 - ((ab[3] + ab[4]) + ab[5]));                                      \
    const CT fill = s32 ? (CT)(float)fill_ : (CT)fill_;                                               \
    const CT iminus = edge ? fill : (CT)x[0];                                                         \
    const CT uminus = iminus / om_a;                                                                  \
    for (int n = 1; n <= 3; ++n) {                 /* the left border */                              \
        const int64_t i = n - 1;                                                                      \
        CT tmp = (CT)x[i * st];                                                                       \
        for (int j = 1; j <= n - 1; ++j) tmp += a[j - 1] * (CT)y[(i - j) * st];                       \
        for (int j = n; j <= 3; ++j) tmp += a[j - 1] * uminus;                                        \
        y[i * st] = s32 ? (double)(float)tmp : (double)tmp;                                           \
    }                                                                                                 \
    for (int64_t i = 3; i <= L - 2; ++i) {         /* forward, the last point omitted */              \
        CT tmp = (CT)x[i * st];                                                                       \
        for (int j = 1; j <= 3; ++j) tmp += a[j - 1] * (CT)y[(i - j) * st];                           \
        y[i * st] = s32 ? (double)(float)tmp : (double)tmp;                                           \
    }                                                                                                 \
    const CT iplus = edge ? fill : (CT)x[(L - 1) * st]; /* read before the last point is written */   \
    {                                                                                                 \
        const int64_t i = L - 1;                                                                      \
        CT tmp = (CT)x[i * st];                                                                       \
        for (int j = 1; j <= 3; ++j) tmp += a[j - 1] * (CT)y[(i - j) * st];                           \
        y[i * st] = s32 ? (double)(float)tmp : (double)tmp;                                           \
    }                                                                                                 \
    const CT uplus = iplus / om_a;                                                                    \
    const CT vplus = uplus / om_b;                                                                    \
    const CT du[3] = {(CT)y[(L - 1) * st] - uplus, (CT)y[(L - 2) * st] - uplus,                       \
                      (CT)y[(L - 3) * st] - uplus};                                                   \
    CT vright[3];                                                                                     \
    for (int r = 0; r < 3; ++r)                                                                       \
        vright[r] = (M[3 * r] * du[0] + M[3 * r + 1] * du[1] + M[3 * r + 2] * du[2]) + vplus;         \
    y[(L - 1) * st] = s32 ? (double)(float)vright[0] : (double)vright[0];                             \
    int n = 1;                                                                                        \
    for (int64_t i = L - 2; i >= L - 3; --i) {     /* propagate inward from the right edge */         \
        ++n;                                                                                          \
        CT tmp = (CT)y[i * st];                                                                       \
        for (int j = 1; j <= n - 1; ++j) tmp += b[j - 1] * (CT)y[(i + j) * st];                       \
        for (int j = n; j <= 3; ++j) tmp += b[j - 1] * vright[j - n + 1];                             \
        y[i * st] = s32 ? (double)(float)tmp : (double)tmp;                                           \
    }                                                                                                 \
    for (int64_t i = L - 4; i >= 0; --i) {         /* backward */                                     \
        CT tmp = (CT)y[i * st];                                                                       \
        for (int j = 1; j <= 3; ++j) tmp += b[j - 1] * (CT)y[(i + j) * st];                           \
        y[i * st] = s32 ? (double)(float)tmp : (double)tmp;                                           \
    }                                                                                                 \
    for (int64_t i = 0; i < L; ++i) {                                                                 \
        const CT v = (CT)y[i * st] * scale;                                                           \
        y[i * st] = s32 ? (double)(float)v : (double)v;                                               \
    }                                                                                                 \
}
ORA_IIR_LINE(iir_line_f64, double)
ORA_IIR_LINE(iir_line_f32, float)

/* An IIR cascade (src/imfilter.jl:385-457 with the IIR stage of 427-435 and
 * the zero-width padding of src/border.jl:640-652): every factor filters the
 * previous stage's result along its axis over the whole array.  nf factors
 * with axis[f], ab[6f..6f+5], scale[f], M[9f..9f+8].  img holds the values of
 * the first stage's input already converted to eltype(out).  arith: 0 =
 * Float64 arithmetic and storage, 1 = Float32 arithmetic and storage,
 * 2 = Float64 arithmetic with Float32 storage; c32: Float32 coefficients.  A
 * line of 3 or fewer elements along a filtered axis is a DimensionMismatch
 * (src/imfilter.jl:971-977). */
int ora_imfilter_iir(int nd, const int64_t *n, const double *img, int nf, const int32_t *axis,
                     const double *ab, const double *scale, const double *M, int edge, double fill,
                     int arith, int c32, double *out)
{
    if (nd < 1 || nd > ORA_MAXD) return ORA_EARG;
    int64_t st[ORA_MAXD];
    col_strides(nd, n, st);
    const int64_t total = prod(nd, n);
    memcpy(out, img, (size_t)total * sizeof(double));
    const int s32 = arith != 0;
    for (int f = 0; f < nf; ++f) {
        const int ax = axis[f];
        if (ax < 0 || ax >= nd) return ORA_EDIM;
        const int64_t L = n[ax];
        if (total == 0) continue;
        if (L <= 3) return ORA_EDIM;
        const int64_t inner = st[ax], outer = total / (inner * L);
        for (int64_t o = 0; o < outer; ++o)
            for (int64_t p = 0; p < inner; ++p) {
                double *line = out + o * inner * L + p;
                if (arith == 1)
                    iir_line_f32(line, line, L, inner, ab + 6 * f, scale[f], M + 9 * f, edge, fill, s32, c32);
                else
                    iir_line_f64(line, line, L, inner, ab + 6 * f, scale[f], M + 9 * f, edge, fill, s32, c32);
            }
    }
    return ORA_OK;
}
