// Tile geometry shared by the deconvolution kernels and their host launchers.
#pragma once
#include "fft.cuh"

// One launch works on tiles [t0, t0 + nt) of a channel's tile grid
// (deconvolver.py:186-206: origins x-major, step tile_size).
struct TileGeom {
    int Z, X, Y;          // channel shape (deconvolver.py:178)
    long long isz, isx;   // u16 image strides in elements (y stride 1)
    long long fsx;        // flat-field row stride (y stride 1)
    int ts, ov, zpad;     // tile_size, overlap, zpad
    int P, H, Zp;         // padded tile edge, half spectrum length, padded depth
    int ny;               // tiles along y
    int t0, nt;           // first tile and tile count of this launch
    int npsf;             // number of Wiener spectra (1 = shared)
    int ntot;             // tiles the whole call processes (zip-truncated when npsf > 1)
};

struct TileDesc {
    int x, y;        // tile origin
    int x0, y0;      // first input row / column (max(x - ov, 0))
    int xd, yd;      // input extent
    int xs, ys;      // placement offset inside the padded tile (ov on the first row/col)
    int xend, yend;  // yielded extent (deconvolver.py:120-144), at most P
    int psf;         // spectrum index
};

__device__ __host__ inline TileDesc mm_tile_desc(const TileGeom &g, int ti) {
    TileDesc d;
    int ix = ti / g.ny, iy = ti % g.ny;
    d.x = ix * g.ts;
    d.y = iy * g.ts;
    d.x0 = d.x - g.ov > 0 ? d.x - g.ov : 0;
    d.y0 = d.y - g.ov > 0 ? d.y - g.ov : 0;
    int x1 = d.x + g.ts + g.ov < g.X ? d.x + g.ts + g.ov : g.X;
    int y1 = d.y + g.ts + g.ov < g.Y ? d.y + g.ts + g.ov : g.Y;
    d.xd = x1 - d.x0;
    d.yd = y1 - d.y0;
    d.xs = d.x == 0 ? g.ov : 0;
    d.ys = d.y == 0 ? g.ov : 0;
    // the yielded view tile_res[:, :xend, :yend] of a P x P tile: slicing
    // clips xend = xd + ov at P when xd > P - ov (deconvolver.py:133-144, 170)
    d.xend = d.xd + ((d.x == 0 || d.xd < g.P) ? g.ov : 0);
    d.yend = d.yd + ((d.y == 0 || d.yd < g.P) ? g.ov : 0);
    if (d.xend > g.P) d.xend = g.P;
    if (d.yend > g.P) d.yend = g.P;
    d.psf = g.npsf == 1 ? 0 : ti;
    return d;
}

// Deconvolver.apply (deconvolver.py:179-183) writes tile centres in x-major
// order, each over [x, x + xend - 2 ov) x [y, y + yend - 2 ov).  A truncated
// second-to-last tile reaches past its own span into the last tile's, which
// overwrites it later.  So the value that survives at an output pixel is the
// one of the last tile (in order) whose span covers it: the tile (ox / ts,
// oy / ts) when that tile is processed, else the latest covering predecessor
// (only the tile just before the owner along an axis can reach past its span).
__device__ __host__ inline int mm_stitch_owner(const TileGeom &g, int ox, int oy) {
    const int ix = ox / g.ts, iy = oy / g.ts;
    const int own = ix * g.ny + iy;
    if (own < g.ntot) return own;
    int best = -1;
    for (int cx = ix; cx >= ix - 1 && cx >= 0; --cx)
        for (int cy = iy; cy >= iy - 1 && cy >= 0; --cy) {
            const int t = cx * g.ny + cy;
            if (t >= g.ntot || t <= best) continue;
            const TileDesc d = mm_tile_desc(g, t);
            if (ox >= d.x && ox < d.x + d.xend - 2 * g.ov && oy >= d.y && oy < d.y + d.yend - 2 * g.ov) best = t;
        }
    return best;
}

// Padded index -> source index inside the tile, or -1 for a zero.  Restates
// the placement and the reflect calls of deconvolver.py:123-148 (fill.py
// mirror semantics) as a per-axis gather: every mirror copies whole
// hyperplanes, so the padded tile is tile[mz[z], mx[x], my[y]] (zero where any
// index is -1).
__device__ __host__ inline int mm_map_xy(int j, bool first, int d, int P, int ov) {
    if (first) {  // placed at ov, reflect 'in' about ov (deconvolver.py:132-134)
        int q = j;
        if (j < ov) {
            int src = 2 * ov - j;
            if (src < P) q = src;
        }
        return (q >= ov && q < ov + d) ? q - ov : -1;
    }
    if (d < P) {  // placed at 0, reflect 'out' about d-1 (deconvolver.py:135-137)
        if (j < d) return j;
        int src = 2 * (d - 1) - j;
        return src >= 0 ? src : -1;
    }
    return j;
}

__device__ __host__ inline int mm_map_z0(int q, int Z, int zpad) {
    return (q >= zpad && q < zpad + Z) ? q - zpad : -1;
}

// z: placed at zpad; reflect 'in' about zpad, then 'out' about zpad+Z-1
// (deconvolver.py:145-148).
__device__ __host__ inline int mm_map_z(int j, int Z, int zpad, int Zp) {
    int i2 = zpad + Z - 1;
    int q = j;
    if (j > i2) {
        int src = 2 * i2 - j;
        if (src >= 0) q = src;
    }
    if (q < zpad) {
        int src = 2 * zpad - q;
        if (src < Zp) return mm_map_z0(src, Z, zpad);
    }
    return mm_map_z0(q, Z, zpad);
}

// host launchers (deconv.cu)
int mm_launch_rows_fwd_img(const TileGeom &g, const void *img, int dtype, const float *flat, float2 *S,
                           cudaStream_t st);
int mm_launch_rows_fwd_f32(const float *vol, int nrows, int P, float2 *S, cudaStream_t st);
int mm_launch_cols(float2 *S, int n, long long se, int nlines, long long plane_stride, int nplanes,
                   bool inv, cudaStream_t st);
int mm_launch_zpass(const TileGeom &g, float2 *S, const float2 *W, long long wstride, cudaStream_t st);

// z pass from the z kernel w (Zp, P, P/2+1) per spectrum, the inverse DFT of
// W along z (zop.cu): as a matrix per frequency over a batch that shares one
// spectrum (mm_launch_zop_apply), or as the direct sum per tile
// (mm_launch_zconv).
// The matrix form's CTAs shrink with the batch (threads = 4 frequencies x
// ceil(Z / 5) row groups x ceil(nt / 5) tile groups), so a launch costs nearly
// as much for 10 tiles as for 25 (3.5 against 3.9 ms at Z = 50, P = 678);
// batches of fewer tiles than this take the direct sum.
#define MM_ZOP_MIN_TILES 10
#define MM_ZOP_MAX_Z 64
#define MM_ZOP_MAX_ZP 400
#define MM_ZOP_MAX_COPIES 4
int mm_zop_supported(int Z, int zpad);
int mm_zker_build_impl(const float2 *W, int Zp, long long plane, float2 *w, cudaStream_t st);
// fresp: NULL, or a per-frequency factor (plane entries) applied to the
// result, the blur subtraction folded into the z step (mm_blur_response_get)
int mm_launch_zop_apply(float2 *S, const float2 *w, int Z, int zpad, int Zp, long long plane, int nt,
                        const float *fresp, cudaStream_t st);
int mm_zconv_supported(int Z, int zpad);
int mm_launch_zconv(float2 *S, const float2 *w, long long wstride, int Z, int zpad, int Zp, long long plane, int t0,
                    int nt, int npsf, const float *fresp, cudaStream_t st);
// The z operator with the matrix of each frequency formed in registers from
// the z kernel (Toeplitz plus two masked Hankel parts, 1 <= zpad <= Z - 1,
// Z a multiple of 5) and its operands staged by TMA (zop_tma.cu).  A CTA that
// gives up waiting for its copies sets *err.  mm_zth_supported returns the
// number of tile chunks a batch of nt tiles is split into (0: not supported).
int mm_zth_supported(int Z, int zpad, int nt, long long plane);
// The same z step on the tensor cores (zop_mma.cu): tcgen05 MMAs with the
// matrix in tensor memory, TF32 operands split into two parts; Z <= 56,
// 1 <= zpad <= Z - 1, nt <= 32, plane a multiple of 4.  A CTA that gives up
// waiting sets *err.
int mm_zmma_supported(int Z, int zpad, int nt, long long plane);
int mm_launch_zmma_apply(float2 *S, const float2 *w, int Z, int zpad, int Zp, long long plane, int nt,
                         const float *fresp, unsigned *err, cudaStream_t st);
int mm_launch_zth_apply(float2 *S, const float2 *w, int Z, int zpad, int Zp, long long plane, int nt,
                        const float *fresp, unsigned *err, cudaStream_t st);
// The register form with a z kernel per tile (zop_pt.cu): tile t of the
// launch, spectrum index t0 + t, takes the kernel w + (t0 + t) * wstride when
// npsf > 1, else w.  Z a multiple of 5 up to 80, 1 <= zpad <= Z - 1, an even
// plane.  A CTA that gives up waiting for its copies sets *err.
int mm_zpt_supported(int Z, int zpad, int nt, long long plane);
int mm_launch_zpt_apply(float2 *S, const float2 *w, long long wstride, int Z, int zpad, int Zp, long long plane,
                        int t0, int nt, int npsf, const float *fresp, unsigned *err, cudaStream_t st);
// 1 - D(kx) D(ky) per half-spectrum frequency of a P x P plane, D the
// frequency response of the box mean of width 2 delta + 1 (zop.cu)
int mm_blur_response_get(int P, int delta, const float **out);
int mm_launch_zfwd(float2 *S, int Zp, int plane, cudaStream_t st);
int mm_launch_rows_inv(const float2 *S, int nrows, int P, int H, float *out, float *blur, int delta,
                       cudaStream_t st);
// the inverse y pass (no blur) over the rows and columns of each tile that the
// caller reads: reach >= 0, the band [ov - reach, extent - ov + reach) of the
// hyb keep filter; reach < 0, the stitched centre [ov, extent - ov)
// (reach < 0 with `stitch` given: the centre goes straight into the stitched
// FOV buffer, strides osz, osx, in Deconvolver.apply's overwrite order)
int mm_launch_rows_inv_win(const float2 *S, const TileGeom &g, int reach, float *out, float *stitch, long long osz,
                           long long osx, cudaStream_t st);
int mm_launch_blur_x_sub(const TileGeom &g, const float *res, const float *tmp, int delta,
                         float *res_out, float *stitch, long long osz, long long osx, cudaStream_t st);
int mm_launch_make_raw(const TileGeom &g, const void *img, int dtype, const float *flat, float *raw,
                       cudaStream_t st);

// maxima + fit (maxima.cu)
struct MaximaArgs {
    const float *img;
    long long isz, isx, ivol;   // image strides (y stride 1), per-volume stride
    int Z, X, Y, nvol;          // dense dims (X, Y ignored in tile mode)
    const TileGeom *tiles;      // tile mode: dims and raw view from the tile geometry
    int raw_kind;               // 0 f32 array, 1 u16 array, 2 tile raw view (u16 chan), 3 (f32 chan)
    const void *raw;
    long long rsz, rsx, rvol;
    const void *chan;
    const float *flat;
    float th;
    int delta, delta_fit;
    float sigmaZ, sigmaXY;
    float div;                  // 0: none, else v -> v / div
    const float *divp;          // device divisor, overrides div when set
    int neg;                    // v -> -v after the division
    int keep_filter;            // tile mode: keep-filter + origin offset, rows appended
};
int mm_maxima_ensure_init(cudaStream_t st);
int mm_launch_maxima_fit(const MaximaArgs &a, uint2 *cand, unsigned cand_cap, unsigned *ncand, float *out,
                         unsigned out_cap, unsigned *out_count, int zero_out_count, cudaStream_t st);
int mm_launch_maxima_fit_pm(const MaximaArgs &a, uint2 *cand, unsigned cap, unsigned *ncand_plus,
                            unsigned *ncand_minus, float *out_plus, unsigned cap_plus, float *out_minus,
                            unsigned cap_minus, cudaStream_t st);
int mm_launch_note_overflow(const unsigned *ncand, unsigned cap, unsigned *overflow, cudaStream_t st);
// largest number of per-block partial sums (grid cap of the elementwise kernels)
#define MM_SUM_PARTS 4864
int mm_launch_sumsq(const float *x, long long n, double *parts, double *out, cudaStream_t st);
int mm_launch_sum_parts(const double *parts, int nparts, double *out, cudaStream_t st);
int mm_launch_rms_div(const double *sumsq, long long n, float *div, cudaStream_t st);
int mm_wiener_build_impl(const float *psf, int pz, int px, int py, int tile_height, int tile_size, int zpad,
                         int overlap, float beta, float2 *W, float *vol, float2 *S, double *dsum, double *parts,
                         cudaStream_t st);
