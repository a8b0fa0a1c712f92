// C ABI entry points (include/mermake_gb300.h): context, scratch, and the
// drivers that chain the kernels of deconv.cu / wiener.cu / maxima.cu.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <atomic>
#include <map>
#include <mutex>
#include <utility>

#include "deconv.cuh"

namespace {
thread_local char g_err[1024] = "";

enum Slot { WS_SPEC = 0, WS_RES, WS_TMP, WS_VOL, WS_CAND, WS_SMALL, WS_SELECT, WS_N };
}  // namespace

static std::atomic<unsigned long long> g_launches{0};
void mm_launch_counter_add() { g_launches.fetch_add(1, std::memory_order_relaxed); }

int mm_set_smem(const void *fn, size_t bytes) {
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> done;
    int dev = 0;
    MM_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    size_t &cur = done[{dev, fn}];
    if (bytes <= cur) return MM_OK;
    MM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    cur = bytes;
    return MM_OK;
}
unsigned long long mm_launch_counter_get() { return g_launches.load(); }

void mm_set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

// Per-stage timing: when enabled, every stage launch is bracketed by CUDA
// events on the launching stream; elapsed times are collected when the
// records are read (or the record buffer fills), together with the stage's
// algorithmic bytes (the minimum DRAM traffic its function needs).
enum Stage { ST_ROWS_FWD = 0, ST_COLS_FWD, ST_ZPASS, ST_COLS_INV, ST_ROWS_INV, ST_BLUR_X, ST_MAKE_RAW,
             ST_MAXIMA_FIT, ST_SUMSQ, ST_WIENER, ST_N };
static const char *kStageNames[ST_N] = {"rows_fwd", "cols_fwd", "zpass", "cols_inv", "rows_inv_blur_y",
                                        "blur_x_sub", "make_raw", "maxima_fit", "sumsq", "wiener"};
constexpr int kMaxRec = 1024;

struct Prof {
    bool on = false;
    int n = 0;
    cudaEvent_t ev0[kMaxRec], ev1[kMaxRec];
    int stage[kMaxRec];
    double bytes[kMaxRec];
    bool created = false;
    double ms[ST_N] = {};
    double tot_bytes[ST_N] = {};
    long long launches[ST_N] = {};
};

struct mm_ctx {
    std::mutex mu;
    void *ws[WS_N] = {};
    size_t ws_bytes[WS_N] = {};
    unsigned *h_counters = nullptr;  // pinned: [0] candidates, [1] rows, [2] rows (2nd set)
    int device = 0;
    int blur_mode = MM_BLUR_AUTO;    // mm_ctx_set_option(MM_OPT_BLUR_MODE)
    int zform = MM_ZFORM_AUTO;       // mm_ctx_set_option(MM_OPT_ZFORM)
    bool used = false;               // a call has used the scratch ...
    cudaStream_t last_stream = nullptr;  // ... on this stream
    std::atomic<unsigned long long> scratch_total{0};  // device bytes of scratch held
    Prof prof;
};

namespace {

int prof_collect(mm_ctx *c) {
    Prof &p = c->prof;
    for (int i = 0; i < p.n; ++i) {
        MM_CUDA_TRY(cudaEventSynchronize(p.ev1[i]));
        float ms = 0.f;
        MM_CUDA_TRY(cudaEventElapsedTime(&ms, p.ev0[i], p.ev1[i]));
        p.ms[p.stage[i]] += ms;
        p.tot_bytes[p.stage[i]] += p.bytes[i];
        p.launches[p.stage[i]] += 1;
    }
    p.n = 0;
    return MM_OK;
}

// RAII bracket around one stage launch
struct StageTimer {
    mm_ctx *c;
    int idx = -1;
    cudaStream_t st;
    StageTimer(mm_ctx *c_, int stage, double bytes, cudaStream_t st_) : c(c_), st(st_) {
        Prof &p = c->prof;
        if (!p.on) return;
        if (p.n == kMaxRec) prof_collect(c);
        idx = p.n++;
        p.stage[idx] = stage;
        p.bytes[idx] = bytes;
        cudaEventRecord(p.ev0[idx], st);
    }
    ~StageTimer() {
        if (idx >= 0) cudaEventRecord(c->prof.ev1[idx], st);
    }
};

// Scratch slot s of at least `bytes`, grown (never shrunk) in stream order on
// the calling stream st: the old buffer is freed and the new one allocated on
// st (cudaFreeAsync / cudaMallocAsync), so growing does not wait for the rest
// of the device.  Earlier work of this context on st is ordered before the
// free; when the context's previous call ran on another stream, the device is
// synchronised first, as that work may still read the old buffer.
int ws_get(mm_ctx *c, Slot s, size_t bytes, void **out, cudaStream_t st) {
    if (bytes == 0) bytes = 16;
    if (c->ws_bytes[s] < bytes) {
        if (c->ws[s]) {
            if (c->used && c->last_stream != st) MM_CUDA_TRY(cudaDeviceSynchronize());
            MM_CUDA_TRY(cudaFreeAsync(c->ws[s], st));
            c->scratch_total.fetch_sub(c->ws_bytes[s]);
            c->ws[s] = nullptr;
            c->ws_bytes[s] = 0;
        }
        // grow with headroom so that slowly growing requests do not thrash
        size_t want = bytes + bytes / 8;
        cudaError_t e = cudaMallocAsync(&c->ws[s], want, st);
        if (e != cudaSuccess) {
            cudaGetLastError();
            e = cudaMallocAsync(&c->ws[s], bytes, st);
            want = bytes;
        }
        if (e != cudaSuccess) {
            cudaGetLastError();
            c->ws[s] = nullptr;
            mm_set_error("allocation of %zu bytes of scratch failed: %s", bytes, cudaGetErrorString(e));
            return MM_ENOMEM;
        }
        c->ws_bytes[s] = want;
        c->scratch_total.fetch_add(want);
    }
    c->used = true;
    c->last_stream = st;
    *out = c->ws[s];
    return MM_OK;
}

// small device scratch: counters and reduction cells
struct Small {
    unsigned cand;       // candidate count
    unsigned rows;       // kept rows (set 1)
    unsigned rows2;      // kept rows (set 2)
    unsigned overflow;   // largest candidate count that did not fit
    unsigned err;        // a kernel gave up a bounded wait (MM_ETIMEOUT)
    unsigned pad0_;
    double sumsq;
    float div;
    float pad_;
    double parts[MM_SUM_PARTS];  // per-block partial sums (fixed-order reductions)
};

int small_get(mm_ctx *c, Small **out, cudaStream_t st) {
    void *p;
    const bool fresh = c->ws[WS_SMALL] == nullptr;
    int rc = ws_get(c, WS_SMALL, sizeof(Small), &p, st);
    if (rc) return rc;
    if (fresh) MM_CUDA_TRY(cudaMemsetAsync(p, 0, sizeof(Small), st));  // counters and the error flag start at zero
    *out = (Small *)p;
    return MM_OK;
}

// A kernel's bounded wait gave up (Small::err, read back with the counters):
// clears the flag and reports MM_ETIMEOUT.
int timeout_seen(Small *sm, unsigned err, cudaStream_t st) {
    if (!err) return MM_OK;
    MM_CUDA_TRY(cudaMemsetAsync(&sm->err, 0, sizeof(unsigned), st));
    mm_set_error("a kernel gave up waiting for its shared-memory copies");
    return MM_ETIMEOUT;
}

int ntiles_of(const TileGeom &g) {
    int nx = (g.X + g.ts - 1) / g.ts;
    int n = nx * g.ny;
    // zip(tiles, psf_ffts) truncates when several spectra are given (deconvolver.py:110, 116)
    if (g.npsf > 1 && g.npsf < n) n = g.npsf;
    return n;
}

int fill_geom(TileGeom &g, int Z, int X, int Y, long long isz, long long isx, long long fsx, int ts, int zpad,
              int ov, int npsf) {
    MM_REQUIRE(Z > 0 && X > 0 && Y > 0, "empty channel (%d, %d, %d)", Z, X, Y);
    MM_REQUIRE(Z < 65536 && X < 65536 && Y < 65536, "channel dimensions must be < 65536");
    MM_REQUIRE(ts > 0, "tile_size must be positive");
    MM_REQUIRE(ov >= 0, "overlap must be >= 0");
    MM_REQUIRE(zpad >= 1, "zpad must be >= 1 (the reference's [zpad:-zpad] crop is empty for zpad = 0)");
    MM_REQUIRE(npsf >= 1, "need at least one Wiener spectrum");
    g.Z = Z; g.X = X; g.Y = Y;
    g.isz = isz; g.isx = isx; g.fsx = fsx;
    g.ts = ts; g.ov = ov; g.zpad = zpad;
    g.P = ts + 2 * ov;
    g.H = g.P / 2 + 1;
    g.Zp = Z + 2 * zpad;
    MM_REQUIRE(g.P <= MM_FFT_MAXN && g.Zp <= MM_FFT_MAXN, "padded tile (%d, %d) exceeds the FFT length limit %d",
               g.Zp, g.P, MM_FFT_MAXN);
    g.ny = (Y + ts - 1) / ts;
    g.t0 = 0; g.nt = 0;
    g.npsf = npsf;
    g.ntot = 0;
    g.ntot = ntiles_of(g);
    return MM_OK;
}


// Whether a call may fold the blur subtraction into the z step (the
// spectrum times 1 - D(kx) D(ky), mm_blur_response_get): the z step runs from
// the z kernel, and every voxel the caller reads lies at least delta (the
// box half-width) from the tile's edges, where the truncated box mean of the
// reference equals the circular one.  `reach` is how far inside the overlap
// the caller reads: the stitched centres start at the overlap (reach 0); the
// kept spots of a hyb tile have centroids inside it and read their maxima and
// fit neighbourhoods, at most delta_fit + max(delta, delta_fit) closer to the
// edge.
// The z step of a batch: MM_ZFORM_REGISTERS (k_zth_apply over one shared
// spectrum, else k_zpt_apply with a kernel per tile), _SHARED (k_zop_apply),
// _DIRECT (k_zconv) or _TRANSFORMS (k_zpass).  The context's MM_OPT_ZFORM
// choice when the batch qualifies for it (a z kernel, one spectrum for the
// shared and tensor forms, the forms' shape limits), else the first of
// registers, shared, direct and transforms that qualifies, the shared-spectrum
// matrix forms only for batches of at least MM_ZOP_MIN_TILES tiles.  A
// register-form batch split into tile chunks (deeper tiles: each chunk reloads
// the z kernel and rounds its tiles up to whole thread groups) gives way to
// the shared-memory form where that form takes the depth.
bool zth_takes(const TileGeom &g, bool forced) {
    if (g.npsf != 1 || g.nt < (forced ? 1 : MM_ZOP_MIN_TILES)) return false;
    const int chunks = mm_zth_supported(g.Z, g.zpad, g.nt, (long long)g.P * g.H);
    return chunks == 1 || (chunks > 1 && (forced || mm_zop_supported(g.Z, g.zpad) == 0));
}

int zform_of(const mm_ctx *c, const TileGeom &g, const float2 *zop) {
    const long long plane = (long long)g.P * g.H;
    // forced: the context's own choice, which takes any batch the form takes
    auto ok = [&](int f, bool forced) {
        const int min_tiles = forced ? 1 : MM_ZOP_MIN_TILES;
        switch (f) {
            case MM_ZFORM_REGISTERS: {
                if (!zop) return false;
                // one spectrum and a batch the shared-spectrum forms take: the
                // per-tile form only where k_zth_apply does not take it
                if (g.npsf == 1 && g.nt >= min_tiles && mm_zop_supported(g.Z, g.zpad) != 0)
                    return zth_takes(g, forced);
                return zth_takes(g, forced) || mm_zpt_supported(g.Z, g.zpad, g.nt, plane) != 0;
            }
            case MM_ZFORM_SHARED:
                return zop && g.npsf == 1 && g.nt >= min_tiles && mm_zop_supported(g.Z, g.zpad) != 0;
            case MM_ZFORM_TENSOR:
                return zop && g.npsf == 1 && g.nt >= min_tiles && mm_zmma_supported(g.Z, g.zpad, g.nt, plane) != 0;
            case MM_ZFORM_DIRECT: return zop && mm_zconv_supported(g.Z, g.zpad) != 0;
            default: return true;
        }
    };
    if (c->zform != MM_ZFORM_AUTO && ok(c->zform, true)) return c->zform;
    for (int f : {MM_ZFORM_REGISTERS, MM_ZFORM_SHARED, MM_ZFORM_DIRECT})
        if (ok(f, false)) return f;
    return MM_ZFORM_TRANSFORMS;
}

bool fold_allowed(const mm_ctx *c, const TileGeom &g, int blur_radius, const float2 *zop, bool driver, int reach) {
    if (blur_radius < 0 || !zop || c->blur_mode == MM_BLUR_EXACT) return false;
    if (!driver && c->blur_mode != MM_BLUR_SPECTRAL) return false;
    return zform_of(c, g, zop) != MM_ZFORM_TRANSFORMS && g.ov - reach >= blur_radius / 2 + 1 &&
           2 * (blur_radius / 2) + 1 <= g.P;
}

// tile_wise core for tiles [g.t0, g.t0 + g.nt); fold: the blur subtraction
// runs as a factor of the z step's output (fold_allowed) instead of the y and
// x box means of the result
//
// win: with the blur folded, the caller reads only a window of each tile (a
// driver's keep band, win >= 0 its reach, or the stitched centre, win == -1):
// the inverse y pass then transforms and writes only the rows and columns of
// that window (k_rows_inv_win).  win < -1: whole tiles.
int run_tiles(mm_ctx *c, TileGeom g, const void *image, int dtype, const float *flat, const float2 *W,
              const float2 *zop, int blur_radius, float *res_out, float *raw_out, float *stitch, long long osz,
              long long osx, cudaStream_t st, bool fold = false, int win = -2) {
    const long long plane_c = (long long)g.P * g.H;
    const long long tile_c = (long long)g.Z * plane_c;
    const long long tile_r = (long long)g.Z * g.P * g.P;
    void *spec, *res, *tmp = nullptr;
    int rc;
    const int delta = blur_radius >= 0 ? blur_radius / 2 : -1;
    const float *fresp = nullptr;
    if (fold && delta >= 0 && (rc = mm_blur_response_get(g.P, delta, &fresp))) return rc;
    // the box means still to take on the result
    const int rdelta = fresp ? -1 : delta;
    if ((rc = ws_get(c, WS_SPEC, sizeof(float2) * tile_c * g.nt, &spec, st))) return rc;
    res = res_out;
    if (!res && (rc = ws_get(c, WS_RES, sizeof(float) * tile_r * g.nt, &res, st))) return rc;
    if (rdelta >= 0 && (rc = ws_get(c, WS_TMP, sizeof(float) * tile_r * g.nt, &tmp, st))) return rc;
    float2 *S = (float2 *)spec;
    const long long wstride = (long long)g.Zp * plane_c;
    // algorithmic bytes of each stage for this batch (its inputs read once, outputs written once)
    double in_b = 0;
    for (int t = g.t0; t < g.t0 + g.nt; ++t) {
        TileDesc d = mm_tile_desc(g, t);
        in_b += (double)g.Z * d.xd * d.yd * (dtype == MM_DTYPE_U16 ? 2 : 4) + (flat ? 4.0 * d.xd * d.yd : 0.0);
    }
    const double spec_b = 8.0 * tile_c * g.nt, real_b = 4.0 * tile_r * g.nt, w_b = 8.0 * wstride * g.nt;
    {
        StageTimer t(c, ST_ROWS_FWD, in_b + spec_b, st);
        if ((rc = mm_launch_rows_fwd_img(g, image, dtype, flat, S, st))) return rc;
    }
    {
        StageTimer t(c, ST_COLS_FWD, 2 * spec_b, st);
        if ((rc = mm_launch_cols(S, g.P, g.H, g.H, plane_c, g.nt * g.Z, false, st))) return rc;
    }
    const int zform = zform_of(c, g, zop);
    if (zform == MM_ZFORM_TENSOR) {
        // the matrix applied on the tensor cores; the z kernel is read once per batch
        Small *sm;
        if ((rc = small_get(c, &sm, st))) return rc;
        StageTimer t(c, ST_ZPASS, 2 * spec_b + 8.0 * wstride, st);
        if ((rc = mm_launch_zmma_apply(S, zop, g.Z, g.zpad, g.Zp, plane_c, g.nt, fresp, &sm->err, st))) return rc;
    } else if (zform == MM_ZFORM_REGISTERS && zth_takes(g, c->zform == MM_ZFORM_REGISTERS)) {
        // the matrix formed in registers, operands staged by TMA; the z kernel
        // is read once per batch
        Small *sm;
        if ((rc = small_get(c, &sm, st))) return rc;
        StageTimer t(c, ST_ZPASS, 2 * spec_b + 8.0 * wstride, st);
        if ((rc = mm_launch_zth_apply(S, zop, g.Z, g.zpad, g.Zp, plane_c, g.nt, fresp, &sm->err, st))) return rc;
    } else if (zform == MM_ZFORM_REGISTERS) {
        // the same with each tile's own z kernel, read once per tile
        Small *sm;
        if ((rc = small_get(c, &sm, st))) return rc;
        StageTimer t(c, ST_ZPASS, 2 * spec_b + (g.npsf == 1 ? 8.0 * wstride : w_b), st);
        if ((rc = mm_launch_zpt_apply(S, zop, wstride, g.Z, g.zpad, g.Zp, plane_c, g.t0, g.nt, g.npsf, fresp,
                                      &sm->err, st)))
            return rc;
    } else if (zform == MM_ZFORM_SHARED) {
        // the z kernel (Zp per frequency, the size of W) is read once per batch
        StageTimer t(c, ST_ZPASS, 2 * spec_b + 8.0 * wstride, st);
        if ((rc = mm_launch_zop_apply(S, zop, g.Z, g.zpad, g.Zp, plane_c, g.nt, fresp, st))) return rc;
    } else if (zform == MM_ZFORM_DIRECT) {
        // each tile's z kernel read once (once per batch when shared)
        StageTimer t(c, ST_ZPASS, 2 * spec_b + (g.npsf == 1 ? 8.0 * wstride : w_b), st);
        if ((rc = mm_launch_zconv(S, zop, wstride, g.Z, g.zpad, g.Zp, plane_c, g.t0, g.nt, g.npsf, fresp, st)))
            return rc;
    } else {
        MM_REQUIRE(!fresp, "the blur fold needs the z kernel");
        StageTimer t(c, ST_ZPASS, 2 * spec_b + w_b, st);
        if ((rc = mm_launch_zpass(g, S, W, wstride, st))) return rc;
    }
    {
        StageTimer t(c, ST_COLS_INV, 2 * spec_b, st);
        if ((rc = mm_launch_cols(S, g.P, g.H, g.H, plane_c, g.nt * g.Z, true, st))) return rc;
    }
    // with the blur folded and only the centre read, the stitched buffer is
    // written straight from the inverse pass
    const bool direct_stitch = fresp && win == -1 && !res_out && stitch;
    if (fresp && win >= -1 && !res_out) {
        StageTimer t(c, ST_ROWS_INV, spec_b + real_b, st);
        if ((rc = mm_launch_rows_inv_win(S, g, win, (float *)res, direct_stitch ? stitch : nullptr, osz, osx, st)))
            return rc;
    } else {
        StageTimer t(c, ST_ROWS_INV, spec_b + real_b * (rdelta >= 0 ? 2 : 1), st);
        if ((rc = mm_launch_rows_inv(S, g.nt * g.Z * g.P, g.P, g.H, (float *)res, (float *)tmp, rdelta, st)))
            return rc;
    }
    if (rdelta >= 0 || (stitch && !direct_stitch)) {
        // with no box mean left to take, only the stitch: the result is final
        // in res already and is not written back
        StageTimer t(c, ST_BLUR_X, (rdelta >= 0 ? 3 : 2) * real_b, st);
        if ((rc = mm_launch_blur_x_sub(g, (float *)res, (float *)tmp, rdelta, rdelta >= 0 ? (float *)res : nullptr,
                                       stitch, osz, osx, st)))
            return rc;
    }
    if (raw_out) {
        StageTimer t(c, ST_MAKE_RAW, in_b + real_b, st);
        if ((rc = mm_launch_make_raw(g, image, dtype, flat, raw_out, st))) return rc;
    }
    return MM_OK;
}

}  // namespace

extern "C" {

int mm_abi_version(void) { return 1; }

const char *mm_last_error(void) { return g_err; }

int mm_ctx_create(mm_ctx **out) {
    MM_REQUIRE(out != nullptr, "null output pointer");
    mm_ctx *c = new mm_ctx();
    MM_CUDA_TRY(cudaGetDevice(&c->device));
    if (cudaMallocHost(&c->h_counters, 16 * sizeof(unsigned)) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        mm_set_error("cudaMallocHost for counters failed");
        return MM_ENOMEM;
    }
    int rc = mm_maxima_ensure_init(0);
    if (rc) {
        cudaFreeHost(c->h_counters);
        delete c;
        return rc;
    }
    *out = c;
    return MM_OK;
}

int mm_ctx_destroy(mm_ctx *c) {
    if (!c) return MM_OK;
    cudaDeviceSynchronize();
    if (c->prof.created)
        for (int i = 0; i < kMaxRec; ++i) {
            cudaEventDestroy(c->prof.ev0[i]);
            cudaEventDestroy(c->prof.ev1[i]);
        }
    for (int s = 0; s < WS_N; ++s)
        if (c->ws[s]) cudaFreeAsync(c->ws[s], 0);
    cudaStreamSynchronize(0);
    if (c->h_counters) cudaFreeHost(c->h_counters);
    delete c;
    return MM_OK;
}

int mm_ctx_scratch_bytes(const mm_ctx *c, uint64_t *bytes) {
    MM_REQUIRE(c && bytes, "null argument");
    *bytes = c->scratch_total.load();
    return MM_OK;
}

int mm_wiener_spectrum(mm_ctx *c, const float *psf, int pz, int px, int py, int tile_height, int tile_size,
                       int zpad, int overlap, float beta, void *W, void *stream) {
    MM_REQUIRE(c && psf && W, "null argument");
    MM_REQUIRE(pz > 0 && px > 0 && py > 0, "empty PSF");
    MM_REQUIRE(tile_height > 0 && tile_size > 0 && zpad >= 0 && overlap >= 0, "bad tile geometry");
    std::lock_guard<std::mutex> lock(c->mu);
    cudaStream_t st = (cudaStream_t)stream;
    const int nz = tile_height + 2 * zpad, nx = tile_size + 2 * overlap;
    MM_REQUIRE(nz <= MM_FFT_MAXN && nx <= MM_FFT_MAXN, "padded PSF exceeds the FFT length limit");
    const int H = nx / 2 + 1;
    void *vol, *spec;
    Small *sm;
    int rc;
    if ((rc = ws_get(c, WS_VOL, sizeof(float) * (size_t)nz * nx * nx, &vol, st))) return rc;
    if ((rc = ws_get(c, WS_SPEC, sizeof(float2) * (size_t)nz * nx * H, &spec, st))) return rc;
    if ((rc = small_get(c, &sm, st))) return rc;
    StageTimer tm(c, ST_WIENER, 4.0 * nz * nx * nx + 8.0 * nz * nx * H, st);
    return mm_wiener_build_impl(psf, pz, px, py, tile_height, tile_size, zpad, overlap, beta, (float2 *)W,
                                (float *)vol, (float2 *)spec, &sm->sumsq, sm->parts, st);
}

int mm_wiener_zop(mm_ctx *c, const void *W, int tile_height, int zpad, int tile_size, int overlap, void *zop,
                  void *stream) {
    MM_REQUIRE(c && W && zop, "null argument");
    MM_REQUIRE(tile_height > 0 && tile_size > 0 && zpad >= 0 && overlap >= 0, "bad tile geometry");
    MM_REQUIRE(mm_zconv_supported(tile_height, zpad), "z kernel needs 1 <= zpad, tile height <= 128 and Zp <= %d",
               MM_ZOP_MAX_ZP);
    std::lock_guard<std::mutex> lock(c->mu);
    cudaStream_t st = (cudaStream_t)stream;
    const int Zp = tile_height + 2 * zpad, P = tile_size + 2 * overlap;
    const long long plane = (long long)P * (P / 2 + 1);
    StageTimer tm(c, ST_WIENER, 16.0 * Zp * plane, st);
    return mm_zker_build_impl((const float2 *)W, Zp, plane, (float2 *)zop, st);
}

int mm_zkernel_supported(int tile_height, int zpad) { return mm_zconv_supported(tile_height, zpad); }

int mm_deconv_tiles(mm_ctx *c, const void *image, int image_dtype, int Z, int X, int Y, int64_t isz, int64_t isx,
                    const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size, int zpad,
                    int overlap, int tile_begin, int tile_count, int blur_radius, float *res_out, float *raw_out,
                    float *stitch_out, int64_t osz, int64_t osx, void *stream) {
    MM_REQUIRE(c && image && W, "null argument");
    TileGeom g;
    int rc = fill_geom(g, Z, X, Y, isz, isx, fsx, tile_size, zpad, overlap, npsf);
    if (rc) return rc;
    const int nt = ntiles_of(g);
    MM_REQUIRE(tile_begin >= 0 && tile_count >= 0 && tile_begin + tile_count <= nt,
               "tiles [%d, %d) outside the %d tiles of the channel", tile_begin, tile_begin + tile_count, nt);
    MM_REQUIRE(!stitch_out || overlap >= 1, "stitching needs overlap >= 1");
    MM_REQUIRE(image_dtype == MM_DTYPE_U16 || image_dtype == MM_DTYPE_F32, "image_dtype must be uint16 or float32");
    if (tile_count == 0) return MM_OK;
    g.t0 = tile_begin;
    g.nt = tile_count;
    std::lock_guard<std::mutex> lock(c->mu);
    const bool fold = fold_allowed(c, g, blur_radius, (const float2 *)zop, false, 0);
    return run_tiles(c, g, image, image_dtype, flat, (const float2 *)W, (const float2 *)zop, blur_radius, res_out,
                     raw_out, stitch_out, osz, osx, (cudaStream_t)stream, fold);
}

int mm_find_local_maxima(mm_ctx *c, const float *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                         const void *raw, int raw_dtype, int64_t rsz, int64_t rsx, float threshold, int delta,
                         int delta_fit, float sigmaZ, float sigmaXY, float norm_div, int negate, float *out,
                         uint32_t out_cap, uint32_t *count, void *stream) {
    MM_REQUIRE(c && image && raw && count, "null argument");
    MM_REQUIRE(delta <= 5, "Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS");
    MM_REQUIRE(delta >= 0 && delta_fit >= 0, "negative delta");
    MM_REQUIRE(raw_dtype == 0 || raw_dtype == 1, "raw_dtype must be 0 (float32) or 1 (uint16)");
    MM_REQUIRE(Z < 65536 && X < 65536 && Y < 65536, "dimensions must be < 65536");
    *count = 0;
    if ((long long)Z * X * Y == 0) return MM_OK;
    std::lock_guard<std::mutex> lock(c->mu);
    cudaStream_t st = (cudaStream_t)stream;
    Small *sm;
    int rc;
    if ((rc = small_get(c, &sm, st))) return rc;
    for (int attempt = 0; attempt < 2; ++attempt) {
        size_t cap = c->ws_bytes[WS_CAND] / sizeof(uint2);
        if (cap < 65536) cap = 65536;
        void *cand;
        if ((rc = ws_get(c, WS_CAND, cap * sizeof(uint2), &cand, st))) return rc;
        cap = c->ws_bytes[WS_CAND] / sizeof(uint2);
        MaximaArgs a = {};
        a.img = image; a.isz = isz; a.isx = isx; a.ivol = 0;
        a.Z = Z; a.X = X; a.Y = Y; a.nvol = 1;
        a.tiles = nullptr;
        a.raw_kind = raw_dtype; a.raw = raw; a.rsz = rsz; a.rsx = rsx; a.rvol = 0;
        a.th = threshold; a.delta = delta; a.delta_fit = delta_fit;
        a.sigmaZ = sigmaZ; a.sigmaXY = sigmaXY;
        a.div = norm_div; a.divp = nullptr; a.neg = negate; a.keep_filter = 0;
        if ((rc = mm_launch_maxima_fit(a, (uint2 *)cand, (unsigned)cap, &sm->cand, out, out_cap, nullptr, 0, st)))
            return rc;
        MM_CUDA_TRY(cudaMemcpyAsync(c->h_counters, &sm->cand, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        MM_CUDA_TRY(cudaStreamSynchronize(st));
        unsigned n = c->h_counters[0];
        if (n <= cap) {
            *count = n;
            return n > out_cap ? MM_EOVERFLOW : MM_OK;
        }
        if ((rc = ws_get(c, WS_CAND, (size_t)n * sizeof(uint2), &cand, st))) return rc;
    }
    mm_set_error("candidate list did not converge");
    return MM_EDEVICE;
}

}  // extern "C"

// The tile batches of one colour into out / sm->rows (candidates through
// cand[0, cap), overflow noted in sm->overflow): the body of mm_hyb_spots and
// mm_hyb_spots_async.
static int hyb_pass(mm_ctx *c, const TileGeom &g, int batch, const uint16_t *image, const float *flat,
                    const void *W, const void *zop, int blur_radius, float threshold, int delta, int delta_fit,
                    float sigmaZ, float sigmaXY, float *out, uint32_t out_cap, void *cand, size_t cap, Small *sm,
                    cudaStream_t st) {
    int rc;
    const int nt = ntiles_of(g);
    MM_CUDA_TRY(cudaMemsetAsync(&sm->overflow, 0, sizeof(unsigned), st));
    for (int t0 = 0; t0 < nt; t0 += batch) {
        TileGeom gb = g;
        gb.t0 = t0;
        gb.nt = (t0 + batch <= nt) ? batch : nt - t0;
        const int reach = delta_fit + (delta > delta_fit ? delta : delta_fit);
        const bool fold = fold_allowed(c, gb, blur_radius, (const float2 *)zop, true, reach);
        // the maxima scan covers the keep band (delta_fit + 1 past the kept
        // region, maxima.cu scan_range) and reads max(delta, delta_fit) around it
        const int win = delta_fit + 1 + (delta > delta_fit ? delta : delta_fit);
        if ((rc = run_tiles(c, gb, image, MM_DTYPE_U16, flat, (const float2 *)W, (const float2 *)zop, blur_radius,
                            nullptr, nullptr, nullptr, 0, 0, st, fold, win)))
            return rc;
        MaximaArgs a = {};
        a.img = (const float *)c->ws[WS_RES];
        a.isz = (long long)g.P * g.P; a.isx = g.P; a.ivol = (long long)g.Z * g.P * g.P;
        a.Z = g.Z; a.X = 0; a.Y = 0; a.nvol = gb.nt;
        a.tiles = &gb;
        a.raw_kind = 2; a.chan = image; a.flat = flat;
        a.th = threshold; a.delta = delta; a.delta_fit = delta_fit;
        a.sigmaZ = sigmaZ; a.sigmaXY = sigmaXY;
        a.div = 0.f; a.divp = nullptr; a.neg = 0; a.keep_filter = 1;
        {
            double vb = 0;
            for (int t = gb.t0; t < gb.t0 + gb.nt; ++t) {
                TileDesc d = mm_tile_desc(gb, t);
                vb += 4.0 * g.Z * d.xend * d.yend;
            }
            StageTimer tm(c, ST_MAXIMA_FIT, vb, st);
            if ((rc = mm_launch_maxima_fit(a, (uint2 *)cand, (unsigned)cap, &sm->cand, out, out_cap, &sm->rows,
                                           t0 == 0, st)))
                return rc;
        }
        if ((rc = mm_launch_note_overflow(&sm->cand, (unsigned)cap, &sm->overflow, st))) return rc;
    }
    return MM_OK;
}

// the candidate list: at least 1 M entries, as large as any earlier call made it
static int cand_list(mm_ctx *c, void **cand, size_t *cap, cudaStream_t st) {
    size_t n = c->ws_bytes[WS_CAND] / sizeof(uint2);
    if (n < (1u << 20)) n = 1u << 20;
    int rc = ws_get(c, WS_CAND, n * sizeof(uint2), cand, st);
    if (rc) return rc;
    *cap = c->ws_bytes[WS_CAND] / sizeof(uint2);
    return MM_OK;
}

extern "C" {

int mm_hyb_spots(mm_ctx *c, const uint16_t *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                 const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size, int zpad,
                 int overlap, int blur_radius, float threshold, int delta, int delta_fit, float sigmaZ, float sigmaXY,
                 int batch, float *out, uint32_t out_cap, uint32_t *count, void *stream) {
    MM_REQUIRE(c && image && W && count, "null argument");
    MM_REQUIRE(delta <= 5, "Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS");
    MM_REQUIRE(delta >= 0 && delta_fit >= 0, "negative delta");
    TileGeom g;
    int rc = fill_geom(g, Z, X, Y, isz, isx, fsx, tile_size, zpad, overlap, npsf);
    if (rc) return rc;
    const int nt = ntiles_of(g);
    if (batch <= 0) batch = nt;
    std::lock_guard<std::mutex> lock(c->mu);
    cudaStream_t st = (cudaStream_t)stream;
    Small *sm;
    if ((rc = small_get(c, &sm, st))) return rc;
    *count = 0;
    for (int attempt = 0; attempt < 2; ++attempt) {
        void *cand;
        size_t cap;
        if ((rc = cand_list(c, &cand, &cap, st))) return rc;
        if ((rc = hyb_pass(c, g, batch, image, flat, W, zop, blur_radius, threshold, delta, delta_fit, sigmaZ,
                           sigmaXY, out, out_cap, cand, cap, sm, st)))
            return rc;
        // rows, rows2, overflow and err are consecutive in Small
        MM_CUDA_TRY(cudaMemcpyAsync(c->h_counters, &sm->rows, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        MM_CUDA_TRY(cudaStreamSynchronize(st));
        if ((rc = timeout_seen(sm, c->h_counters[3], st))) return rc;
        unsigned over = c->h_counters[2];
        if (over == 0) {
            *count = c->h_counters[0];
            return *count > out_cap ? MM_EOVERFLOW : MM_OK;
        }
        if ((rc = ws_get(c, WS_CAND, (size_t)over * sizeof(uint2), &cand, st))) return rc;
    }
    mm_set_error("candidate list did not converge");
    return MM_EDEVICE;
}

int mm_hyb_spots_async(mm_ctx *c, const uint16_t *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                       const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size,
                       int zpad, int overlap, int blur_radius, float threshold, int delta, int delta_fit,
                       float sigmaZ, float sigmaXY, int batch, float *out, uint32_t out_cap, uint32_t *count_dev,
                       uint32_t *overflow_dev, void *stream) {
    MM_REQUIRE(c && image && W && count_dev && overflow_dev, "null argument");
    MM_REQUIRE(delta <= 5, "Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS");
    MM_REQUIRE(delta >= 0 && delta_fit >= 0, "negative delta");
    TileGeom g;
    int rc = fill_geom(g, Z, X, Y, isz, isx, fsx, tile_size, zpad, overlap, npsf);
    if (rc) return rc;
    const int nt = ntiles_of(g);
    if (batch <= 0) batch = nt;
    std::lock_guard<std::mutex> lock(c->mu);
    cudaStream_t st = (cudaStream_t)stream;
    Small *sm;
    if ((rc = small_get(c, &sm, st))) return rc;
    void *cand;
    size_t cap;
    if ((rc = cand_list(c, &cand, &cap, st))) return rc;
    if ((rc = hyb_pass(c, g, batch, image, flat, W, zop, blur_radius, threshold, delta, delta_fit, sigmaZ, sigmaXY,
                       out, out_cap, cand, cap, sm, st)))
        return rc;
    // a timed-out wait makes the result incomplete, like a candidate overflow
    if ((rc = mm_launch_note_overflow(&sm->err, 0, &sm->overflow, st))) return rc;
    MM_CUDA_TRY(cudaMemcpyAsync(count_dev, &sm->rows, sizeof(unsigned), cudaMemcpyDeviceToDevice, st));
    MM_CUDA_TRY(cudaMemcpyAsync(overflow_dev, &sm->overflow, sizeof(unsigned), cudaMemcpyDeviceToDevice, st));
    return MM_OK;
}

}  // extern "C"

// The DAPI block into out_plus / sm->rows and out_minus / sm->rows2 (stitched
// deconvolution into buffer, the RMS divisor in sm->div, both signs' maxima
// through the two halves of cand[0, cap), overflow noted in sm->overflow): the
// body of mm_dapi_spots and mm_dapi_spots_async.
static int dapi_pass(mm_ctx *c, const TileGeom &g, int batch, const uint16_t *image, int64_t isz, int64_t isx,
                     const float *flat, const void *W, const void *zop, int blur_radius, float threshold, int delta,
                     int delta_fit, float sigmaZ, float sigmaXY, float *buffer, float *out_plus, uint32_t cap_plus,
                     float *out_minus, uint32_t cap_minus, void *cand, size_t cap, Small *sm, cudaStream_t st) {
    int rc;
    const int nt = ntiles_of(g);
    const int Z = g.Z, X = g.X, Y = g.Y;
    const long long N = (long long)Z * X * Y;
    MM_CUDA_TRY(cudaMemsetAsync(buffer, 0, sizeof(float) * N, st));
    for (int t0 = 0; t0 < nt; t0 += batch) {
        TileGeom gb = g;
        gb.t0 = t0;
        gb.nt = (t0 + batch <= nt) ? batch : nt - t0;
        const bool fold = fold_allowed(c, gb, blur_radius, (const float2 *)zop, true, 0);
        if ((rc = run_tiles(c, gb, image, MM_DTYPE_U16, flat, (const float2 *)W, (const float2 *)zop, blur_radius,
                            nullptr, nullptr, buffer, (long long)X * Y, Y, st, fold, -1)))
            return rc;
    }
    {
        StageTimer tm(c, ST_SUMSQ, 4.0 * N, st);
        if ((rc = mm_launch_sumsq(buffer, N, sm->parts, &sm->sumsq, st))) return rc;
    }
    if ((rc = mm_launch_rms_div(&sm->sumsq, N, &sm->div, st))) return rc;
    MM_CUDA_TRY(cudaMemsetAsync(&sm->overflow, 0, sizeof(unsigned), st));
    // v / rms and -v / rms in one maxima pass: the candidates of each sign in
    // one half of the list, counted in rows / rows2
    MaximaArgs a = {};
    a.img = buffer; a.isz = (long long)X * Y; a.isx = Y; a.ivol = 0;
    a.Z = Z; a.X = X; a.Y = Y; a.nvol = 1;
    a.tiles = nullptr;
    a.raw_kind = 1; a.raw = image; a.rsz = isz; a.rsx = isx; a.rvol = 0;
    a.th = threshold; a.delta = delta; a.delta_fit = delta_fit;
    a.sigmaZ = sigmaZ; a.sigmaXY = sigmaXY;
    a.div = 0.f; a.divp = &sm->div; a.neg = 0; a.keep_filter = 0;
    const unsigned half = (unsigned)(cap / 2);
    {
        StageTimer tm(c, ST_MAXIMA_FIT, 4.0 * N, st);
        if ((rc = mm_launch_maxima_fit_pm(a, (uint2 *)cand, half, &sm->rows, &sm->rows2, out_plus, cap_plus,
                                          out_minus, cap_minus, st)))
            return rc;
    }
    if ((rc = mm_launch_note_overflow(&sm->rows, half, &sm->overflow, st))) return rc;
    if ((rc = mm_launch_note_overflow(&sm->rows2, half, &sm->overflow, st))) return rc;
    return MM_OK;
}

extern "C" {

int mm_dapi_spots(mm_ctx *c, const uint16_t *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                  const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size, int zpad,
                  int overlap, int blur_radius, float threshold, int delta, int delta_fit, float sigmaZ, float sigmaXY,
                  int batch, float *buffer, float *out_plus, uint32_t cap_plus, uint32_t *count_plus,
                  float *out_minus, uint32_t cap_minus, uint32_t *count_minus, float *rms, void *stream) {
    MM_REQUIRE(c && image && W && buffer && count_plus && count_minus, "null argument");
    MM_REQUIRE(delta <= 5, "Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS");
    MM_REQUIRE(delta >= 0 && delta_fit >= 0, "negative delta");
    MM_REQUIRE(overlap >= 1, "stitching needs overlap >= 1");
    TileGeom g;
    int rc = fill_geom(g, Z, X, Y, isz, isx, fsx, tile_size, zpad, overlap, npsf);
    if (rc) return rc;
    const int nt = ntiles_of(g);
    if (batch <= 0) batch = nt;
    std::lock_guard<std::mutex> lock(c->mu);
    cudaStream_t st = (cudaStream_t)stream;
    Small *sm;
    if ((rc = small_get(c, &sm, st))) return rc;
    for (int attempt = 0; attempt < 2; ++attempt) {
        void *cand;
        size_t cap;
        if ((rc = cand_list(c, &cand, &cap, st))) return rc;
        if ((rc = dapi_pass(c, g, batch, image, isz, isx, flat, W, zop, blur_radius, threshold, delta, delta_fit,
                            sigmaZ, sigmaXY, buffer, out_plus, cap_plus, out_minus, cap_minus, cand, cap, sm, st)))
            return rc;
        MM_CUDA_TRY(cudaMemcpyAsync(c->h_counters, &sm->rows, 4 * sizeof(unsigned), cudaMemcpyDeviceToHost, st));
        float hdiv = 0.f;
        MM_CUDA_TRY(cudaMemcpyAsync(c->h_counters + 4, &sm->div, sizeof(float), cudaMemcpyDeviceToHost, st));
        MM_CUDA_TRY(cudaStreamSynchronize(st));
        if ((rc = timeout_seen(sm, c->h_counters[3], st))) return rc;
        memcpy(&hdiv, c->h_counters + 4, sizeof(float));
        if (rms) *rms = hdiv;
        if (c->h_counters[2] == 0) {
            *count_plus = c->h_counters[0];
            *count_minus = c->h_counters[1];
            return (*count_plus > cap_plus || *count_minus > cap_minus) ? MM_EOVERFLOW : MM_OK;
        }
        if ((rc = ws_get(c, WS_CAND, 2 * (size_t)c->h_counters[2] * sizeof(uint2), &cand, st))) return rc;
    }
    mm_set_error("candidate list did not converge");
    return MM_EDEVICE;
}

int mm_dapi_spots_async(mm_ctx *c, const uint16_t *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                        const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size,
                        int zpad, int overlap, int blur_radius, float threshold, int delta, int delta_fit,
                        float sigmaZ, float sigmaXY, int batch, float *buffer, float *out_plus, uint32_t cap_plus,
                        float *out_minus, uint32_t cap_minus, uint32_t *counts_dev, float *rms_dev, void *stream) {
    MM_REQUIRE(c && image && W && buffer && counts_dev, "null argument");
    MM_REQUIRE(delta <= 5, "Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS");
    MM_REQUIRE(delta >= 0 && delta_fit >= 0, "negative delta");
    MM_REQUIRE(overlap >= 1, "stitching needs overlap >= 1");
    TileGeom g;
    int rc = fill_geom(g, Z, X, Y, isz, isx, fsx, tile_size, zpad, overlap, npsf);
    if (rc) return rc;
    const int nt = ntiles_of(g);
    if (batch <= 0) batch = nt;
    std::lock_guard<std::mutex> lock(c->mu);
    cudaStream_t st = (cudaStream_t)stream;
    Small *sm;
    if ((rc = small_get(c, &sm, st))) return rc;
    void *cand;
    size_t cap;
    if ((rc = cand_list(c, &cand, &cap, st))) return rc;
    if ((rc = dapi_pass(c, g, batch, image, isz, isx, flat, W, zop, blur_radius, threshold, delta, delta_fit, sigmaZ,
                        sigmaXY, buffer, out_plus, cap_plus, out_minus, cap_minus, cand, cap, sm, st)))
        return rc;
    if ((rc = mm_launch_note_overflow(&sm->err, 0, &sm->overflow, st))) return rc;
    // rows, rows2 and overflow are consecutive in Small
    MM_CUDA_TRY(cudaMemcpyAsync(counts_dev, &sm->rows, 3 * sizeof(unsigned), cudaMemcpyDeviceToDevice, st));
    if (rms_dev) MM_CUDA_TRY(cudaMemcpyAsync(rms_dev, &sm->div, sizeof(float), cudaMemcpyDeviceToDevice, st));
    return MM_OK;
}

}  // extern "C"

extern "C" int mm_ctx_set_option(mm_ctx *c, int option, int value) {
    MM_REQUIRE(c, "null context");
    MM_REQUIRE(option == MM_OPT_BLUR_MODE || option == MM_OPT_ZFORM, "unknown option %d", option);
    std::lock_guard<std::mutex> lock(c->mu);
    if (option == MM_OPT_BLUR_MODE) {
        MM_REQUIRE(value == MM_BLUR_AUTO || value == MM_BLUR_EXACT || value == MM_BLUR_SPECTRAL,
                   "unknown blur mode %d", value);
        c->blur_mode = value;
    } else {
        MM_REQUIRE(value >= MM_ZFORM_AUTO && value <= MM_ZFORM_TENSOR, "unknown z form %d", value);
        c->zform = value;
    }
    return MM_OK;
}

extern "C" int mm_tile_geometry(int Z, int X, int Y, int tile_size, int zpad, int overlap, int npsf, int tile,
                                int32_t *desc, int32_t *map_z, int32_t *map_x, int32_t *map_y) {
    TileGeom g;
    int rc = fill_geom(g, Z, X, Y, 0, 0, 0, tile_size, zpad, overlap, npsf);
    if (rc) return rc;
    const int nt = ntiles_of(g);
    if (tile < 0) return nt;  // query: number of tiles
    MM_REQUIRE(tile < nt, "tile %d outside the %d tiles of the channel", tile, nt);
    TileDesc d = mm_tile_desc(g, tile);
    if (desc) {
        int32_t v[13] = {d.x, d.y, d.x0, d.y0, d.xd, d.yd, d.xs, d.ys, d.xend, d.yend, d.psf, g.P, g.Zp};
        memcpy(desc, v, sizeof(v));
    }
    if (map_z)
        for (int j = 0; j < g.Zp; ++j) map_z[j] = mm_map_z(j, g.Z, g.zpad, g.Zp);
    if (map_x)
        for (int j = 0; j < g.P; ++j) map_x[j] = mm_map_xy(j, d.x == 0, d.xd, g.P, g.ov);
    if (map_y)
        for (int j = 0; j < g.P; ++j) map_y[j] = mm_map_xy(j, d.y == 0, d.yd, g.P, g.ov);
    return MM_OK;
}

extern "C" int mm_fft_c2c(void *data, int n, int nlines, int inverse, void *stream) {
    MM_REQUIRE(data && n >= 1 && nlines >= 1, "bad FFT arguments");
    return mm_launch_cols((float2 *)data, n, nlines, nlines, 0, 1, inverse != 0, (cudaStream_t)stream);
}

extern "C" int mm_profile_enable(mm_ctx *c, int on) {
    MM_REQUIRE(c, "null context");
    std::lock_guard<std::mutex> lock(c->mu);
    Prof &p = c->prof;
    if (on && !p.created) {
        for (int i = 0; i < kMaxRec; ++i) {
            MM_CUDA_TRY(cudaEventCreate(&p.ev0[i]));
            MM_CUDA_TRY(cudaEventCreate(&p.ev1[i]));
        }
        p.created = true;
    }
    if (p.n) {
        int rc = prof_collect(c);
        if (rc) return rc;
    }
    for (int i = 0; i < ST_N; ++i) {
        p.ms[i] = 0;
        p.tot_bytes[i] = 0;
        p.launches[i] = 0;
    }
    p.on = on != 0;
    return MM_OK;
}

extern "C" int mm_profile_read(mm_ctx *c, int nmax, double *ms, double *bytes, int64_t *launches) {
    MM_REQUIRE(c, "null context");
    std::lock_guard<std::mutex> lock(c->mu);
    int rc = prof_collect(c);
    if (rc) return rc;
    const int n = nmax < ST_N ? nmax : ST_N;
    for (int i = 0; i < n; ++i) {
        if (ms) ms[i] = c->prof.ms[i];
        if (bytes) bytes[i] = c->prof.tot_bytes[i];
        if (launches) launches[i] = c->prof.launches[i];
    }
    return ST_N;
}

extern "C" const char *mm_stage_name(int i) { return (i >= 0 && i < ST_N) ? kStageNames[i] : ""; }

extern "C" uint64_t mm_launch_count(void) { return mm_launch_counter_get(); }

int mm_median_impl(const float *x, long long n, unsigned *scratch, float *med_dev, float *out, cudaStream_t st);

extern "C" int mm_median_f32(mm_ctx *c, const float *x, int64_t n, float *median, float *out, void *stream) {
    MM_REQUIRE(c && x && median, "null argument");
    MM_REQUIRE(n > 0, "median of an empty array");
    std::lock_guard<std::mutex> lock(c->mu);
    cudaStream_t st = (cudaStream_t)stream;
    void *scr;
    int rc;
    if ((rc = ws_get(c, WS_SELECT, sizeof(unsigned) * 272, &scr, st))) return rc;
    float *med_dev = reinterpret_cast<float *>(static_cast<unsigned *>(scr) + 264);
    if ((rc = mm_median_impl(x, n, static_cast<unsigned *>(scr), med_dev, out, st))) return rc;
    MM_CUDA_TRY(cudaMemcpyAsync(c->h_counters + 8, med_dev, sizeof(float), cudaMemcpyDeviceToHost, st));
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    memcpy(median, c->h_counters + 8, sizeof(float));
    return MM_OK;
}
