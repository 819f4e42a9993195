// ifx_tune.cu -- the autotuner of the separable paths.
//
// Every candidate below leaves the result within the FP32 tolerance (the
// pass order and the z strategy only move FP32 rounding; tile shapes and
// chunk depths do not change any output's arithmetic) and changes the speed:
//
//  2-D (the fused 2-D separable path, ifx_imfilter_factored with one factor
//  per axis): the tile kernel (persistent TMA-fed, or gather-based), the
//  order of the two passes (axis order), and the output tile shape -- its
//  width and height, which set how much of each staged window is halo
//  ((kx - 1) columns and (ky - 1) rows around TX x TY outputs) and how many
//  CTAs share an SM.
//  3-D (one factor per axis of a volume): the split sweeps (z factor into an
//  FP32 volume, then the TMA x/y sweep, with its tile shape) or the fused
//  z-marching kernel with its chunk depth -- the output slices a CTA walks,
//  over which the kz - 1 halo slices, filtered along x and y once per chunk,
//  are amortised.
//  Batched engine (ifx_batch.cu tunes it, on a plan's first launch): the tile
//  shape of each (op, eltypes, taps) group of requests, stored here under the
//  key (TUNE_BATCH, eltypes, kx, ky, median window, op).
//
// With the tuner enabled, the first device-array call for a key
//   (path, input eltype, output eltype, x / y / z taps, Fill or Pad,
//    size class = floor(log2(elements)), FP64 arithmetic)
// times the default and every applicable candidate on the call's stream (one
// warm-up and three timed launches each, CUDA events, L2 overwritten before
// each timed launch), keeps the fastest -- the default unless another is at
// least 3 % faster -- and runs it; later calls with the key take the cached
// choice without timing.  Choices
// persist in a text cache file, one line per key, loaded when the tuner is
// enabled and appended as keys are tuned.  Host arrays are never tuned
// (their time is the copies'); with the tuner disabled cached choices still
// apply.  A choice may also be pinned by the caller.
#include "ifx_internal.h"
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

namespace ifx {

namespace {

// (path, in, out, kx, ky, kz, fill, size class, f64)
using TuneKey = std::tuple<int, int, int, int, int, int, int, int, int>;

struct Tuner {
    std::mutex mu;
    std::map<TuneKey, TuneChoice> cache;
    bool enabled = false;
    std::string path;
};

Tuner &tuner()
{
    static Tuner t;
    return t;
}

int size_class(long long n)
{
    int c = 0;
    while (n > 1) {
        n >>= 1;
        ++c;
    }
    return c;
}

TuneKey make_key(int path, int in_type, int out_type, int kx, int ky, int kz, int fill, long long n, int f64)
{
    return TuneKey{path, in_type, out_type, kx, ky, kz, fill ? 1 : 0, size_class(n), f64};
}

TuneKey key_of(const Sep2dArgs &a)
{
    return make_key(TUNE_SEP2D, a.in_type, a.out_type, a.kx, a.ky, 0, a.style == IFX_FILL,
                    (long long)a.nx * a.ny, a.compute_f64);
}

TuneKey key_of(const Sep3dArgs &a)
{
    return make_key(TUNE_SEP3D, a.in_type, a.out_type, a.kx, a.ky, a.kz, a.style == IFX_FILL,
                    (long long)a.nx * a.ny * a.nz * a.nvol, 0);
}

// Cache file lines: "t2" and the nine key fields, then variant, x_first,
// tile_w, tile_h, depth and the time in ms.  Other lines are skipped.
void load_file(Tuner &T)
{
    if (T.path.empty()) return;
    FILE *f = fopen(T.path.c_str(), "r");
    if (!f) return;
    char line[512];
    while (fgets(line, sizeof line, f)) {
        int k[9], v[5];
        float ms;
        if (sscanf(line, "t2 %d %d %d %d %d %d %d %d %d %d %d %d %d %d %f", &k[0], &k[1], &k[2], &k[3], &k[4],
                   &k[5], &k[6], &k[7], &k[8], &v[0], &v[1], &v[2], &v[3], &v[4], &ms) != 15)
            continue;
        T.cache[TuneKey{k[0], k[1], k[2], k[3], k[4], k[5], k[6], k[7], k[8]}] =
            TuneChoice{v[0], v[1], v[2], v[3], v[4], ms};
    }
    fclose(f);
}

void append_file(const Tuner &T, const TuneKey &k, const TuneChoice &c)
{
    if (T.path.empty()) return;
    FILE *f = fopen(T.path.c_str(), "a");
    if (!f) return;
    fprintf(f, "t2 %d %d %d %d %d %d %d %d %d %d %d %d %d %d %.6f\n", std::get<0>(k), std::get<1>(k),
            std::get<2>(k), std::get<3>(k), std::get<4>(k), std::get<5>(k), std::get<6>(k), std::get<7>(k),
            std::get<8>(k), c.variant, c.x_first, c.tile_w, c.tile_h, c.depth, c.ms);
    fclose(f);
}

bool lookup(const TuneKey &k, TuneChoice *c)
{
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lk(T.mu);
    auto it = T.cache.find(k);
    if (it == T.cache.end()) return false;
    *c = it->second;
    return true;
}

void store(const TuneKey &k, const TuneChoice &c)
{
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lk(T.mu);
    if (T.cache.find(k) != T.cache.end()) return;
    T.cache[k] = c;
    append_file(T, k, c);
}

} // namespace

// Candidate timing: one warm-up launch, then three timed launches, each
// after L2 is overwritten (a device buffer twice the L2 size is cleared), so
// that every timed launch reads its inputs from HBM as a call on fresh data
// does; the mean of the three, in ms.
cudaError_t TuneTimer::init()
{
    cudaError_t e;
    int dev = 0, l2 = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, dev);
    flush_bytes = 2 * (size_t)(l2 > 0 ? l2 : (64 << 20));
    if ((e = cudaMalloc(&flush, flush_bytes)) != cudaSuccess) return e;
    if ((e = cudaEventCreate(&e0)) != cudaSuccess) return e;
    return cudaEventCreate(&e1);
}

TuneTimer::~TuneTimer()
{
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (flush) cudaFree(flush);
}

cudaError_t TuneTimer::time(const std::function<cudaError_t()> &run, cudaStream_t s, float *ms)
{
    cudaError_t e;
    if ((e = run()) != cudaSuccess) return e;
    float total = 0.0f;
    for (int r = 0; r < 3; ++r) {
        if ((e = cudaMemsetAsync(flush, r, flush_bytes, s)) != cudaSuccess) return e;
        if ((e = cudaEventRecord(e0, s)) != cudaSuccess) return e;
        if ((e = run()) != cudaSuccess) return e;
        if ((e = cudaEventRecord(e1, s)) != cudaSuccess || (e = cudaEventSynchronize(e1)) != cudaSuccess) return e;
        float t = 0.0f;
        if ((e = cudaEventElapsedTime(&t, e0, e1)) != cudaSuccess) return e;
        total += t;
    }
    *ms = total / 3.0f;
    return cudaSuccess;
}

namespace {

// The 2-D candidates: per kernel and pass order, the distinct tile shapes the
// kernel takes (a requested shape it cannot take runs as its default, so
// shapes are deduplicated by what would run).
std::vector<TuneChoice> sep2d_candidates(const Sep2dArgs &a)
{
    static const int tma_w[] = {64, 128}, tma_h[] = {16, 32, 48, 64, 96, 128};
    static const int g_w[] = {32, 64, 128}, g_h[] = {16, 32, 64};   // widths the kernel does not take dedupe away
    std::vector<TuneChoice> out;
    for (int variant = 1; variant <= 2; ++variant) {
        for (int order = 1; order >= 0; --order) {
            Sep2dArgs c = a;
            c.x_first = order;
            c.variant = variant;
            if (variant == 2 && sep2d_smem_bytes(c.kx, c.ky, c.x_first, c.compute_f64) > 200 * 1024) continue;
            const int *ws = variant == 1 ? tma_w : g_w, *hs = variant == 1 ? tma_h : g_h;
            const int nw = variant == 1 ? 2 : 3, nh = variant == 1 ? 6 : 3;
            for (int i = -1; i < nw; ++i)                  // i = -1: the kernel's default shape
                for (int j = 0; j < nh; ++j) {
                    c.tile_w = i < 0 ? 0 : ws[i];
                    c.tile_h = i < 0 ? 0 : hs[j];
                    int tw, th;
                    if (!sep2d_tile_shape(c, variant, &tw, &th)) continue;
                    bool dup = false;
                    for (const TuneChoice &o : out)
                        dup |= o.variant == variant && o.x_first == order && o.tile_w == tw && o.tile_h == th;
                    if (!dup) out.push_back(TuneChoice{variant, order, tw, th, 0, 0.0f});
                }
        }
    }
    return out;
}

} // namespace

void autotune_set(bool enable, const char *path)
{
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lk(T.mu);
    T.enabled = enable;
    T.path = path ? path : "";
    load_file(T);
}

bool autotune_enabled()
{
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lk(T.mu);
    return T.enabled;
}

void autotune_clear()
{
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lk(T.mu);
    T.cache.clear();
}

bool autotune_lookup_batch(int op, int in_type, int out_type, int kx, int ky, int win, TuneChoice *c)
{
    return lookup(TuneKey{TUNE_BATCH, in_type, out_type, kx, ky, win, op, 0, 0}, c);
}

void autotune_store_batch(int op, int in_type, int out_type, int kx, int ky, int win, const TuneChoice &c,
                          bool persist)
{
    const TuneKey k{TUNE_BATCH, in_type, out_type, kx, ky, win, op, 0, 0};
    if (persist) {
        store(k, c);
        return;
    }
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lk(T.mu);
    T.cache[k] = c;
}

bool autotune_lookup(const Sep2dArgs &a, TuneChoice *c) { return lookup(key_of(a), c); }
bool autotune_lookup3(const Sep3dArgs &a, TuneChoice *c) { return lookup(key_of(a), c); }

bool autotune_lookup_key(int path, int in_type, int out_type, int kx, int ky, int kz, int fill, long long nx,
                         long long ny, long long nz, TuneChoice *c)
{
    return lookup(make_key(path, in_type, out_type, kx, ky, path == TUNE_SEP3D ? kz : 0, fill, nx * ny * nz,
                           path == TUNE_SEP2D && in_type == IFX_F64),
                  c);
}

void autotune_pin_key(int path, int in_type, int out_type, int kx, int ky, int kz, int fill, long long nx,
                      long long ny, long long nz, const TuneChoice &c)
{
    const TuneKey k = make_key(path, in_type, out_type, kx, ky, path == TUNE_SEP3D ? kz : 0, fill, nx * ny * nz,
                               path == TUNE_SEP2D && in_type == IFX_F64);
    Tuner &T = tuner();
    std::lock_guard<std::mutex> lk(T.mu);
    T.cache[k] = c;                      // pinned choices replace the cached one, and are not written out
}

static Sep2dArgs with_choice(Sep2dArgs a, const TuneChoice &c)
{
    a.x_first = c.x_first;
    a.variant = c.variant;
    a.tile_w = c.tile_w;
    a.tile_h = c.tile_h;
    return a;
}

// A candidate replaces the default only when it is at least this much faster
// (timing noise does not move a key off the default).
constexpr float kTuneMargin = 0.97f;

cudaError_t launch_sep2d_tuned(Sep2dArgs a, cudaStream_t s, bool device_arrays)
{
    TuneChoice ch;
    if (autotune_lookup(a, &ch)) return launch_sep2d(with_choice(a, ch), s);
    if (!autotune_enabled() || !device_arrays) return launch_sep2d(a, s);
    TuneTimer tt;
    cudaError_t e;
    if ((e = tt.init()) != cudaSuccess) return e;
    // the default first (the kernel and tile an untuned call runs, written out)
    TuneChoice def{sep2d_tma_applies(a) ? 1 : 2, a.x_first, 0, 0, 0, 0.0f};
    {
        Sep2dArgs d = a;
        d.variant = def.variant;
        if (!sep2d_tile_shape(d, def.variant, &def.tile_w, &def.tile_h)) def.tile_w = def.tile_h = 0;
    }
    if ((e = tt.time([&] { return launch_sep2d(with_choice(a, def), s); }, s, &def.ms)) != cudaSuccess) return e;
    TuneChoice best = def;
    for (const TuneChoice &c : sep2d_candidates(a)) {
        const Sep2dArgs ca = with_choice(a, c);
        float ms;
        if ((e = tt.time([&] { return launch_sep2d(ca, s); }, s, &ms)) != cudaSuccess) return e;
        if (ms < best.ms) {
            best = c;
            best.ms = ms;
        }
    }
    if (best.ms > kTuneMargin * def.ms) best = def;
    store(key_of(a), best);
    return launch_sep2d(with_choice(a, best), s);    // the result of the chosen candidate is the call's
}

cudaError_t launch_sep3d_tuned(const Sep3dArgs &a, float *tmp, cudaStream_t s, bool device_arrays)
{
    const bool split = tmp != nullptr;                 // the caller checked sep3d_split_applies
    const bool fused = sep3d_supported(a.kx, a.ky, a.kz, a.nx, a.ny, a.nz, a.nvol);
    auto run = [&](const TuneChoice &c) -> cudaError_t {
        if (c.variant == 2 && fused) return launch_sep3d(a, s, c.depth);
        if (split) return launch_sep3d_split(a, tmp, s, c.tile_w, c.tile_h);
        return launch_sep3d(a, s, c.depth);
    };
    TuneChoice ch{split ? 1 : 2, 1, 0, 0, 0, 0.0f};
    if (autotune_lookup3(a, &ch) || !autotune_enabled() || !device_arrays) return run(ch);
    std::vector<TuneChoice> cands;
    if (split) {
        static const int sw[] = {64, 64, 128, 128}, sh[] = {32, 64, 32, 64};
        cands.push_back(TuneChoice{1, 1, 0, 0, 0, 0.0f});                  // the default x/y tile
        for (int i = 0; i < 4; ++i) cands.push_back(TuneChoice{1, 1, sw[i], sh[i], 0, 0.0f});
    }
    if (fused) {
        static const int zd[] = {8, 16, 32, 64, 128};
        for (int d : zd)
            if (d < 2 * a.nz || d == 8) cands.push_back(TuneChoice{2, 1, 0, 0, d, 0.0f});
    }
    TuneTimer tt;
    cudaError_t e;
    if ((e = tt.init()) != cudaSuccess) return e;
    TuneChoice def = ch;                                // the default: split where it applies
    if ((e = tt.time([&] { return run(def); }, s, &def.ms)) != cudaSuccess) return e;
    TuneChoice best = def;
    for (const TuneChoice &c : cands) {
        float ms;
        if ((e = tt.time([&] { return run(c); }, s, &ms)) != cudaSuccess) return e;
        if (ms < best.ms) {
            best = c;
            best.ms = ms;
        }
    }
    if (best.ms > kTuneMargin * def.ms) best = def;
    store(key_of(a), best);
    return run(best);
}

} // namespace ifx
