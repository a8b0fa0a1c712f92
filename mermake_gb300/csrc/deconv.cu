// Tiled Wiener deconvolution kernels (restating deconvolver.py:98-170).
//
// Spectrum layout per tile: S[t][z][x][ky], complex64, z over the Z real
// planes only, x over P, ky over H = P/2 + 1 (the last axis is real-to-half).
// The padded depth Zp exists only inside the z pass, because every padded
// plane is a copy of a real plane (or zero) and the 2-D transform is linear
// per plane.
//
//   rows_fwd_img  y: gather u16 (or f32) tile rows through the pad maps, divide by the
//                 flat, pack two real rows per complex line, FFT, unpack to
//                 two half spectra.                       (deconvolver.py:123-148, 155)
//   (the x and z passes are in fft_cols.cu and fft_z.cu)
//   rows_inv      y: two half spectra -> one complex line -> IFFT -> two real
//                 rows, and their box mean along y (sliding window)
//   blur_x_sub    box mean along x of that, subtracted from the result
//                 (blur.cu:1-52 semantics), optionally stitching the centre
//                 into the FOV output
//                                                         (deconvolver.py:160-163, 183)
//   make_raw      the raw view handed to the spot fit     (deconvolver.py:165-170)
#include "deconv.cuh"

namespace {

constexpr int kThreads = kFftThreads;  // k_rows_fwd_f32
constexpr int kSmemLimit = kFftSmemLimit;
constexpr FftCfg kRowsFwdCfg = kFftPair;
constexpr FftCfg kRowsInvCfg = kFftPair;
constexpr int kBlurThreads = 512;  // k_blur_x_sub, k_make_raw

template <typename K>
int set_smem(K *kernel, size_t bytes) {
    return mm_set_smem((const void *)kernel, bytes);
}

// ---------------------------------------------------------------------------
// y pass, forward, tile source (u16 or f32) through the pad maps.  A CTA takes
// 2 nl padded rows in x-major, z-minor order, so its rows share few flat-field
// rows.  uint16 tiles: the CTA first stages its raw rows (4-byte cp.async
// words) and their flat rows into the idle ping-pong buffer, all in flight at
// once, then builds the lines from shared memory through the y map (divided by
// the flat), so the gathers do not stall on global latency row by row.
// float32 tiles gather straight from global memory.
// ---------------------------------------------------------------------------
template <typename T, int LMAX, int NF, int NLF>
__device__ __forceinline__ void rows_fwd_group(const TileGeom &g, const T *__restrict__ img,
                                               const float *__restrict__ flat, float2 *__restrict__ S,
                                               const FftPlan &P, int nl, const FftSmem &L, int bx, int by) {
    if constexpr (NF > 0) nl = NLF;
    const int n = NF > 0 ? NF : P.n;
    const int ti = g.t0 + by;
    const TileDesc d = mm_tile_desc(g, ti);
    const long long nrows = (long long)g.Z * g.P;
    const long long row0 = (long long)bx * 2 * nl;  // in (x, z) order
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    {
        // a group whose padded rows are all zero (x beyond the reflected data
        // of a thin tile, deconvolver.py:135-137) transforms to zero: write it
        const long long rl = min(row0 + 2 * nl, nrows) - 1;
        bool zero = true;
        for (int xp = (int)(row0 / g.Z); xp <= (int)(rl / g.Z); ++xp) zero &= mm_map_xy(xp, d.x == 0, d.xd, g.P, g.ov) < 0;
        if (zero) {
            const int H = NF > 0 ? NF / 2 + 1 : g.H;
            float2 *Sb = S + (long long)by * nrows * H;
            const int nr = (int)(rl - row0 + 1);
            for (int it = threadIdx.x; it < nr * H; it += blockDim.x) {
                const int q = it / H, k = it - q * H;
                const long long r = row0 + q;
                const int xp = (int)(r / g.Z);
                Sb[((r - (long long)xp * g.Z) * g.P + xp) * H + k] = make_float2(0.f, 0.f);
            }
            return;
        }
    }
    float *Af = reinterpret_cast<float *>(L.A);
    // the y map of the tile (same for every row), after the scratch
    int *ymap = reinterpret_cast<int *>(L.scr + fft_scr_f4(P, nl, nw));
    for (int e = threadIdx.x; e < n; e += blockDim.x) ymap[e] = mm_map_xy(e, d.y == 0, d.yd, g.P, g.ov);

    if constexpr (sizeof(T) == 2) {
        const int rs = (d.yd + 3) & ~1;  // staged row length (even, room for one leading element)
        uint16_t *Bu = reinterpret_cast<uint16_t *>(L.B);
        float *Bfl = reinterpret_cast<float *>(Bu + 2 * nl * rs);
        const long long rlast = min(row0 + 2 * nl, nrows) - 1;
        const int xpa = (int)(row0 / g.Z), xpb = (int)(rlast / g.Z);
        const int nfx = xpb - xpa + 1;
        const bool fstage = flat && (size_t)2 * nl * rs * sizeof(uint16_t) + (size_t)nfx * d.yd * sizeof(float) <=
                                        (size_t)n * nl * sizeof(float2);
        for (int q = warp; q < 2 * nl; q += nw) {
            const long long r = row0 + q;
            if (r >= nrows) continue;
            const int xp = (int)(r / g.Z), z = (int)(r - (long long)xp * g.Z);
            const int sx = mm_map_xy(xp, d.x == 0, d.xd, g.P, g.ov);
            if (sx < 0) continue;
            const uint16_t *src = reinterpret_cast<const uint16_t *>(img) + z * g.isz +
                                  (long long)(d.x0 + sx) * g.isx + d.y0;
            // a row starting 2 bytes past a word boundary is copied from the
            // element before it (inside the same allocation, which is aligned)
            const int off = (int)((reinterpret_cast<uintptr_t>(src) >> 1) & 1);
            const uint16_t *a = src - off;
            uint16_t *dst = Bu + q * rs;
            const int nwords = (d.yd + off) >> 1;
            for (int w = lane; w < nwords; w += 32) cp_async4(dst + 2 * w, a + 2 * w);
            if (((d.yd + off) & 1) && lane == 0) dst[d.yd - 1 + off] = src[d.yd - 1];
        }
        if (fstage)
            for (int it = threadIdx.x; it < nfx * d.yd; it += blockDim.x) {
                const int fx = it / d.yd, y = it - fx * d.yd;
                const int sx = mm_map_xy(xpa + fx, d.x == 0, d.xd, g.P, g.ov);
                if (sx >= 0) cp_async4(&Bfl[it], &flat[(long long)(d.x0 + sx) * g.fsx + d.y0 + y]);
            }
        cp_async_wait_all();
        __syncthreads();
        for (int q = warp; q < 2 * nl; q += nw) {
            const long long r = row0 + q;
            const int l = q >> 1, comp = q & 1;
            int sx = -1, off = 0;
            const float *frow = nullptr;
            if (r < nrows) {
                const int xp = (int)(r / g.Z), z = (int)(r - (long long)xp * g.Z);
                sx = mm_map_xy(xp, d.x == 0, d.xd, g.P, g.ov);
                if (sx >= 0) {
                    const uint16_t *src = reinterpret_cast<const uint16_t *>(img) + z * g.isz +
                                          (long long)(d.x0 + sx) * g.isx + d.y0;
                    off = (int)((reinterpret_cast<uintptr_t>(src) >> 1) & 1);
                    if (flat)
                        frow = fstage ? Bfl + (xp - xpa) * d.yd : flat + (long long)(d.x0 + sx) * g.fsx + d.y0;
                }
            }
            const uint16_t *rowp = Bu + q * rs + off;
            for (int e = lane; e < n; e += 32) {
                float v = 0.f;
                const int sy = ymap[e];
                if (sx >= 0 && sy >= 0) {
                    // the fast division is within 2 ulp; the raw view (k_make_raw)
                    // keeps the reference's IEEE quotient
                    v = (float)rowp[sy];
                    if (frow) v = __fdividef(v, frow[sy]);
                }
                Af[2 * sidx(e, l, nl) + comp] = v;
            }
        }
    } else {
        __syncthreads();
        for (int q = warp; q < 2 * nl; q += nw) {
            const long long r = row0 + q;
            const int l = q >> 1, comp = q & 1;
            const T *src = nullptr;
            const float *fsrc = nullptr;
            if (r < nrows) {
                const int xp = (int)(r / g.Z), z = (int)(r - (long long)xp * g.Z);
                const int sx = mm_map_xy(xp, d.x == 0, d.xd, g.P, g.ov);
                if (sx >= 0) {
                    src = img + z * g.isz + (long long)(d.x0 + sx) * g.isx + d.y0;
                    if (flat) fsrc = flat + (long long)(d.x0 + sx) * g.fsx + d.y0;
                }
            }
            constexpr int U = 24;  // a whole padded row (up to 768) in flight per warp
            for (int e0 = lane; e0 < n; e0 += 32 * U) {
                float v[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int e = e0 + 32 * u;
                    v[u] = 0.f;
                    if (src && e < n) {
                        const int sy = ymap[e];
                        if (sy >= 0) {
                            v[u] = (float)src[sy];
                            if (fsrc) v[u] = __fdividef(v[u], fsrc[sy]);
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int e = e0 + 32 * u;
                    if (e < n) Af[2 * sidx(e, l, nl) + comp] = v[u];
                }
            }
        }
    }
    __syncthreads();
    float2 *R = fft_run<false, LMAX, NF, NLF>(L.A, L.B, nl, P, L.tw, L.tab, L.scr);

    // unpack the two real rows of each line into their spectrum rows z P + x;
    // the spectrum row of each of the 2 nl rows goes in the (now idle) y map
    const int H = NF > 0 ? NF / 2 + 1 : g.H;
    const float invH = 1.0f / (float)H;
    float2 *Sb = S + (long long)by * nrows * H;
    int *drow = ymap;
    if (threadIdx.x < 2 * nl) {
        const long long r = row0 + threadIdx.x;
        const int xp = (int)(r / g.Z);
        drow[threadIdx.x] = r < nrows ? (int)(r - (long long)xp * g.Z) * g.P + xp : -1;
    }
    __syncthreads();
    for (int it = threadIdx.x; it < nl * H; it += blockDim.x) {
        const int l = fdiv_i(it, H, invH), k = it - l * H;
        const float2 ck = R[sidx(k, l, nl)];
        const float2 cn = R[sidx(k == 0 ? 0 : n - k, l, nl)];
        const int d0 = drow[2 * l], d1 = drow[2 * l + 1];
        if (d0 >= 0) Sb[(long long)d0 * H + k] = make_float2(0.5f * (ck.x + cn.x), 0.5f * (ck.y - cn.y));
        if (d1 >= 0) Sb[(long long)d1 * H + k] = make_float2(0.5f * (ck.y + cn.y), -0.5f * (ck.x - cn.x));
    }
}

// persistent: the CTAs walk the groups (tables loaded once); NF > 0: the
// engine specialised for length NF at NLF lines per CTA
template <typename T, int LMAX, int NF = 0, int NLF = 0>
__global__ void __launch_bounds__(kRowsFwdCfg.threads, kRowsFwdCfg.ctas)
k_rows_fwd_img(TileGeom g, const T *__restrict__ img, const float *__restrict__ flat,
               float2 *__restrict__ S, FftPlan P, int nl, int gx, int ngroups) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const FftSmem L = fft_smem_layout(smem_raw, P, nl);
    fft_load_tables(P, L.tw, L.tab);
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const int by = grp / gx;
        rows_fwd_group<T, LMAX, NF, NLF>(g, img, flat, S, P, nl, L, grp - by * gx, by);
        __syncthreads();
    }
}

// y pass, forward, dense f32 source (the padded PSF volume)
template <int LMAX>
__global__ void __launch_bounds__(kThreads)
k_rows_fwd_f32(const float *__restrict__ vol, long long nrows, float2 *__restrict__ S, FftPlan P, int nl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = P.n, H = n / 2 + 1;
    const float invH = 1.0f / (float)H, invn = 1.0f / (float)n;
    const FftSmem L = fft_smem_layout(smem_raw, P, nl);
    fft_load_tables(P, L.tw, L.tab);
    const long long row0 = (long long)blockIdx.x * 2 * nl;
    float *Af = reinterpret_cast<float *>(L.A);
    for (int it = threadIdx.x; it < 2 * nl * n; it += blockDim.x) {
        const int q = fdiv_i(it, n, invn), e = it - q * n;
        const long long row = row0 + q;
        Af[2 * sidx(e, q >> 1, nl) + (q & 1)] = row < nrows ? vol[row * n + e] : 0.f;
    }
    __syncthreads();
    float2 *R = fft_lines<false, LMAX>(L.A, L.B, nl, P, L.tw, L.tab, L.scr);
    for (int it = threadIdx.x; it < nl * H; it += blockDim.x) {
        const int l = fdiv_i(it, H, invH), k = it - l * H;
        const long long r0 = row0 + 2 * l;
        const float2 ck = R[sidx(k, l, nl)];
        const float2 cn = R[sidx(k == 0 ? 0 : n - k, l, nl)];
        if (r0 < nrows) S[r0 * H + k] = make_float2(0.5f * (ck.x + cn.x), 0.5f * (ck.y - cn.y));
        if (r0 + 1 < nrows) S[(r0 + 1) * H + k] = make_float2(0.5f * (ck.y + cn.y), -0.5f * (ck.x - cn.x));
    }
}

// ---------------------------------------------------------------------------
// y pass, inverse: rows 2l and 2l+1 of H-long half spectra -> one complex line
// -> IFFT -> two real rows.  With delta >= 0 the row's box mean along y
// (blur.cu:1-52 semantics: window [c-delta, c+delta] clipped, divided by the
// in-range count) is written to `blur` as well: each lane slides a window
// over a contiguous segment of the row held in shared memory.
// ---------------------------------------------------------------------------
// The stitched destination of a group's rows (Deconvolver.apply,
// deconvolver.py:179-183): rows of plane z of tile ti starting at batch row
// `base`; a voxel (x, y) of the window [ov, xend - ov) x [ov, yend - ov) goes to
// the FOV voxel (d.x + x - ov, d.y + y - ov) when this tile is that voxel's
// last writer in the reference's order (mm_stitch_owner).
struct StitchMap {
    float *out;
    long long osz, osx;
    long long base;
    int z, ti, xlo;
    TileDesc d;
    const TileGeom *g;
};

template <int LMAX, int NF, int NLF>
__device__ __forceinline__ void rows_inv_group(const float2 *__restrict__ S, long long nrows, int H,
                                               float *__restrict__ out, float *__restrict__ blur, int delta,
                                               const FftPlan &P, int nl, const FftSmem &L, long long row0,
                                               int ylo = 0, int yhi = 1 << 30, const StitchMap *smap = nullptr) {
    // rows [row0, nrows) of the group exist (nrows: the end of the group's
    // window, or of the batch); only columns [ylo, yhi) are stored, into `out`
    // (row-major, n per row) or the stitched FOV buffer (smap)
    if constexpr (NF > 0) {
        nl = NLF;
        H = NF / 2 + 1;
    }
    const int n = NF > 0 ? NF : P.n;
    const bool even = (n % 2) == 0;
    const float invH = 1.0f / (float)H, invn = 1.0f / (float)n;
    constexpr int U = 4;
    for (int base = threadIdx.x; base < nl * H; base += U * blockDim.x) {
        float2 x1[U], x2[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int it = base + u * blockDim.x;
            x1[u] = x2[u] = make_float2(0.f, 0.f);
            if (it < nl * H) {
                const int l = fdiv_i(it, H, invH), k = it - l * H;
                const long long r0 = row0 + 2 * l;
                if (r0 < nrows) x1[u] = S[r0 * H + k];
                if (r0 + 1 < nrows) x2[u] = S[(r0 + 1) * H + k];
            }
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int it = base + u * blockDim.x;
            if (it >= nl * H) break;
            const int l = fdiv_i(it, H, invH), k = it - l * H;
            if (k == 0 || (even && k == n / 2)) {
                L.A[sidx(k, l, nl)] = make_float2(x1[u].x, x2[u].x);
            } else {
                L.A[sidx(k, l, nl)] = make_float2(x1[u].x - x2[u].y, x1[u].y + x2[u].x);
                L.A[sidx(n - k, l, nl)] = make_float2(x1[u].x + x2[u].y, x2[u].x - x1[u].y);
            }
        }
    }
    __syncthreads();
    float2 *R = fft_run<true, LMAX, NF, NLF>(L.A, L.B, nl, P, L.tw, L.tab, L.scr);
    const float *Rf = reinterpret_cast<const float *>(R);
    for (int it = threadIdx.x; it < 2 * nl * n; it += blockDim.x) {
        const int q = fdiv_i(it, n, invn), e = it - q * n;
        const long long row = row0 + q;
        if (row >= nrows || e < ylo || e >= yhi) continue;
        const float v = Rf[2 * sidx(e, q >> 1, nl) + (q & 1)];
        if (!smap) {
            out[row * n + e] = v;
            continue;
        }
        const long long xr = row - smap->base;
        if (xr < smap->xlo) continue;  // the row paired in from before the window
        const TileGeom &g = *smap->g;
        const int ox = smap->d.x + (int)xr - g.ov, oy = smap->d.y + e - g.ov;
        // inside its own span a tile is the final writer; past it, ask who is
        const bool own = ox < smap->d.x + g.ts && oy < smap->d.y + g.ts;
        if (ox < g.X && oy < g.Y && (own || mm_stitch_owner(g, ox, oy) == smap->ti))
            smap->out[smap->z * smap->osz + (long long)ox * smap->osx + oy] = v;
    }
    if (delta < 0) return;
    // y blur: the free ping-pong buffer holds 2 nl rows of n floats
    float *Bf = reinterpret_cast<float *>(R == L.A ? L.B : L.A);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    // odd segment length: the 32 lanes' strided reads fall in distinct banks
    const int seg = ((n + 31) / 32) | 1;
    // mean = sum x (1 / count), the reciprocals of the window counts from a
    // table in the (now idle) scratch
    float *rtab = reinterpret_cast<float *>(L.scr);
    for (int c = threadIdx.x; c <= 2 * delta + 1; c += blockDim.x) rtab[c] = c ? 1.0f / (float)c : 0.f;
    __syncthreads();
    // a warp per line: both real rows of the line at once (float2 reads, all banks)
    for (int l = warp; l < nl; l += nw) {
        const int s0 = lane * seg, s1 = min(s0 + seg, n);
        if (s0 < n) {
            int lo = max(s0 - delta, 0), hi = min(s0 + delta, n - 1);
            float2 sum = make_float2(0.f, 0.f);
            for (int i = lo; i <= hi; ++i) sum = cadd(sum, R[sidx(i, l, nl)]);
            for (int e = s0; e < s1; ++e) {
                if (e > s0) {
                    const int add = e + delta, drop = e - delta - 1;
                    if (add <= n - 1) sum = cadd(sum, R[sidx(add, l, nl)]);
                    if (drop >= 0) sum = csub(sum, R[sidx(drop, l, nl)]);
                }
                const float rc = rtab[min(e + delta, n - 1) - max(e - delta, 0) + 1];
                Bf[(2 * l) * n + e] = sum.x * rc;
                Bf[(2 * l + 1) * n + e] = sum.y * rc;
            }
        }
        __syncwarp();
        for (int c = 0; c < 2; ++c) {
            const long long row = row0 + 2 * l + c;
            if (row < nrows)
                for (int e = lane; e < n; e += 32) blur[row * n + e] = Bf[(2 * l + c) * n + e];
        }
    }
}

// persistent: the CTAs walk the row groups (tables loaded once); NF > 0 as
// for k_rows_fwd_img
template <int LMAX, int NF = 0, int NLF = 0>
__global__ void __launch_bounds__(kRowsInvCfg.threads, kRowsInvCfg.ctas)
k_rows_inv(const float2 *__restrict__ S, long long nrows, int H, float *__restrict__ out,
           float *__restrict__ blur, int delta, FftPlan P, int nl, int ngroups) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const FftSmem L = fft_smem_layout(smem_raw, P, nl);
    fft_load_tables(P, L.tw, L.tab);
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        rows_inv_group<LMAX, NF, NLF>(S, nrows, H, out, blur, delta, P, nl, L, (long long)grp * 2 * nl);
        __syncthreads();
    }
}

// The rows and columns of tile t (of the batch) that the caller reads: the
// window [lo, hi) of padded indices along x and y, from the tile's yielded
// extent.  reach >= 0: the hyb keep band, [ov - reach, extent - ov + reach);
// reach < 0: the stitched centre, [ov, extent - ov).
__device__ __forceinline__ void read_window(const TileGeom &g, int t, int reach, int &xlo, int &xhi, int &ylo,
                                            int &yhi) {
    const TileDesc d = mm_tile_desc(g, g.t0 + t);
    const int r = reach < 0 ? 0 : reach;
    xlo = max(0, g.ov - r);
    ylo = max(0, g.ov - r);
    xhi = min(d.xend, d.xend - g.ov + r);
    yhi = min(d.yend, d.yend - g.ov + r);
    if (xhi < xlo) xhi = xlo;
    if (yhi < ylo) yhi = ylo;
}

// The inverse y pass over the read windows only: per tile, the rows x in
// [xlo, xhi) of every plane, in groups of 2 nl rows (a plane's last group is
// cut at xhi), stores limited to the columns [ylo, yhi).  Rows and columns
// outside are not written.  The CTAs first tabulate the groups per tile
// (tiles <= kMaxWinTiles), then walk the groups as k_rows_inv does.
constexpr int kMaxWinTiles = 256;
template <int LMAX, int NF = 0, int NLF = 0>
__global__ void __launch_bounds__(kRowsInvCfg.threads, kRowsInvCfg.ctas)
k_rows_inv_win(const float2 *__restrict__ S, TileGeom g, int reach, float *__restrict__ out, FftPlan P, int nl,
               int cum_off, float *__restrict__ stitch, long long osz, long long osx) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    int *cum = reinterpret_cast<int *>(smem_raw + cum_off);  // groups before tile t (nt + 1 entries)
    const FftSmem L = fft_smem_layout(smem_raw, P, nl);
    fft_load_tables(P, L.tw, L.tab);
    if constexpr (NF > 0) nl = NLF;
    const int gr = 2 * nl;
    if (threadIdx.x == 0) {
        int acc = 0;
        for (int t = 0; t < g.nt; ++t) {
            cum[t] = acc;
            int xlo, xhi, ylo, yhi;
            read_window(g, t, reach, xlo, xhi, ylo, yhi);
            acc += g.Z * ((xhi - xlo + 1 + gr - 1) / gr);
        }
        cum[g.nt] = acc;
    }
    __syncthreads();
    const int ngroups = cum[g.nt];
    const long long plane = (long long)g.P;
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        int t = 0;
        while (cum[t + 1] <= grp) ++t;
        int xlo, xhi, ylo, yhi;
        read_window(g, t, reach, xlo, xhi, ylo, yhi);
        const int per_plane = (xhi - xlo + 1 + gr - 1) / gr;
        const int k = grp - cum[t];
        const int z = k / per_plane, c = k - z * per_plane;
        const long long base = ((long long)t * g.Z + z) * plane;
        // pairs of rows share a transform line, and a row's rounding depends
        // on its partner: start on an even row of the batch, so that the pairs
        // are those of the whole-tile pass (rows 2l and 2l + 1); the row
        // before the window that this may add is computed exactly as there
        const long long row0 = ((base + xlo) & ~1LL) + (long long)c * gr;
        if (stitch) {
            StitchMap sm;
            sm.out = stitch; sm.osz = osz; sm.osx = osx;
            sm.base = base; sm.z = z; sm.ti = g.t0 + t; sm.xlo = xlo;
            sm.d = mm_tile_desc(g, g.t0 + t);
            sm.g = &g;
            rows_inv_group<LMAX, NF, NLF>(S, base + xhi, g.H, out, nullptr, -1, P, nl, L, row0, ylo, yhi, &sm);
        } else {
            rows_inv_group<LMAX, NF, NLF>(S, base + xhi, g.H, out, nullptr, -1, P, nl, L, row0, ylo, yhi);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// x blur (box mean along x, blur.cu:1-52 semantics) of `tmp`, subtracted from
// res; writes the tile result in place and/or the stitched centre
// (deconvolver.py:160-163, 183).  One CTA = one z plane of one tile and 32
// consecutive y columns held in shared memory; each warp slides the window
// down a segment of rows.  delta < 0: no blur (res copied).
// ---------------------------------------------------------------------------
template <bool STITCH>
__global__ void __launch_bounds__(kBlurThreads)
k_blur_x_sub(TileGeom g, const float *__restrict__ res, const float *__restrict__ tmp, int delta,
             float *res_out, float *__restrict__ stitch, long long osz, long long osx) {
    extern __shared__ __align__(16) float colbuf[];  // P x 32, then the reciprocal table
    const int P = g.P;
    const int ti = g.t0 + blockIdx.z;
    const TileDesc d = mm_tile_desc(g, ti);
    const int z = blockIdx.y;
    const int y0 = blockIdx.x * 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int y = y0 + lane;
    const long long pbase = ((long long)blockIdx.z * g.Z + z) * P * P;
    float *rtab = colbuf + P * 32;  // 1 / count for counts 0..2 delta + 1
    if (delta >= 0) {
        // two rows of 32 columns per warp instruction, 8 bytes a lane when P is
        // even (every row then starts 8-byte aligned: P * 4 and y0 * 4 are
        // multiples of 8), else element by element
        const int hr = lane >> 4, c2 = (lane & 15) * 2;
        const bool even = (P & 1) == 0;
        for (int x = 2 * warp + hr; x < P; x += 2 * nw) {
            const int yy = y0 + c2;
            float *dst = &colbuf[x * 32 + c2];
            if (even && yy + 1 < P) {
                cp_async8(dst, &tmp[pbase + (long long)x * P + yy]);
            } else if (yy + 1 < P) {
                cp_async4(dst, &tmp[pbase + (long long)x * P + yy]);
                cp_async4(dst + 1, &tmp[pbase + (long long)x * P + yy + 1]);
            } else {
                dst[0] = yy < P ? tmp[pbase + (long long)x * P + yy] : 0.f;
                dst[1] = 0.f;
            }
        }
        for (int c = threadIdx.x; c <= 2 * delta + 1; c += blockDim.x) rtab[c] = c ? 1.0f / (float)c : 0.f;
        cp_async_wait_all();
        __syncthreads();
    }
    const int seg = (P + nw - 1) / nw;
    const int x0 = warp * seg, x1 = min(x0 + seg, P);
    float sum = 0.f;
    if (delta >= 0 && x0 < P) {
        const int lo = max(x0 - delta, 0), hi = min(x0 + delta, P - 1);
        for (int i = lo; i <= hi; ++i) sum += colbuf[i * 32 + lane];
    }
    const bool yok = y < P;
    constexpr int U = 16;  // rows of res loaded ahead of the in-place stores
    for (int xb = x0; xb < x1; xb += U) {
        float v[U];
#pragma unroll
        for (int u = 0; u < U; ++u)
            v[u] = (yok && xb + u < x1) ? res[pbase + (long long)(xb + u) * P + y] : 0.f;
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int x = xb + u;
            if (x >= x1) break;
            float val = v[u];
            if (delta >= 0) {
                // x is the same for the whole warp: the branches do not diverge
                if (x > x0) {
                    const int add = x + delta, drop = x - delta - 1;
                    if (add <= P - 1) sum += colbuf[add * 32 + lane];
                    if (drop >= 0) sum -= colbuf[drop * 32 + lane];
                }
                val -= sum * rtab[min(x + delta, P - 1) - max(x - delta, 0) + 1];
            }
            if (!yok) continue;
            if (res_out) res_out[pbase + (long long)x * P + y] = val;
            if (STITCH && x >= g.ov && x < d.xend - g.ov && y >= g.ov && y < d.yend - g.ov) {
                const int ox = d.x + x - g.ov, oy = d.y + y - g.ov;
                // inside its own span a tile is the final writer; past it, ask who is
                const bool own = ox < d.x + g.ts && oy < d.y + g.ts;
                if (ox < g.X && oy < g.Y && (own || mm_stitch_owner(g, ox, oy) == ti))
                    stitch[z * osz + (long long)ox * osx + oy] = val;
            }
        }
    }
}

// raw view: tile_pad[zpad:-zpad] after the flat is multiplied back inside the
// placed region (deconvolver.py:165-170); reflected pads keep the divided value.
template <typename T>
__global__ void k_make_raw(TileGeom g, const T *__restrict__ img, const float *__restrict__ flat,
                           float *__restrict__ raw) {
    const int ti = g.t0 + blockIdx.z;
    const TileDesc d = mm_tile_desc(g, ti);
    const int P = g.P;
    const long long plane = (long long)P * P;
    float *rt = raw + (long long)blockIdx.z * g.Z * plane;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)g.Z * plane;
         i += (long long)gridDim.x * blockDim.x) {
        int z = (int)(i / plane);
        int x = (int)((i / P) % P), y = (int)(i % P);
        int sx = mm_map_xy(x, d.x == 0, d.xd, P, g.ov);
        int sy = mm_map_xy(y, d.y == 0, d.yd, P, g.ov);
        float v = 0.f;
        if (sx >= 0 && sy >= 0) {
            int gx = d.x0 + sx, gy = d.y0 + sy;
            v = (float)img[z * g.isz + gx * g.isx + gy];
            if (flat) {
                float f = flat[gx * g.fsx + gy];
                v = __fdiv_rn(v, f);
                bool placed = x >= d.xs && x < d.xs + d.xd && y >= d.ys && y < d.ys + d.yd;
                if (placed) v = __fmul_rn(v, f);
            }
        }
        rt[i] = v;
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
int mm_launch_rows_fwd_img(const TileGeom &g, const void *img, int dtype, const float *flat, float2 *S,
                           cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(g.P, &P);
    if (rc) return rc;
    // lines per CTA, with room after the scratch for the y map (P ints), which
    // later holds the spectrum rows of the CTA's 2 nl <= 32 rows
    const size_t mapb = sizeof(int) * (size_t)(P.n > 32 ? P.n : 32);
    int nl = 16;
    while (nl > 1 && fft_smem(P, nl, kRowsFwdCfg) + mapb > (size_t)fft_smem_limit(kRowsFwdCfg)) nl >>= 1;
    size_t sm = fft_smem(P, nl, kRowsFwdCfg) + mapb;
    int gx = mm_cdiv((long)g.Z * g.P, 2 * nl);
    int ngroups = gx * g.nt;
    dim3 grid(fft_grid(ngroups, kRowsFwdCfg));
    TileGeom ga = g;
    const void *imga = img;
    const float *fa = flat;
    void *args[] = {&ga, &imga, &fa, &S, &P, &nl, &gx, &ngroups};
    const void *fn = dtype == MM_DTYPE_U16 ? MM_FFT_KERNEL(P, nl, 8, k_rows_fwd_img, uint16_t,)
                                          : MM_FFT_KERNEL(P, nl, 8, k_rows_fwd_img, float,);
    return launch_fft_kernel(fn, grid, sm, st, args, kRowsFwdCfg.threads);
}

int mm_launch_rows_fwd_f32(const float *vol, int nrows, int Pn, float2 *S, cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(Pn, &P);
    if (rc) return rc;
    int nl = pick_nl(P, 16);
    size_t sm = fft_smem(P, nl);
    long long nr = nrows;
    void *args[] = {&vol, &nr, &S, &P, &nl};
    return launch_fft_kernel(MM_BY_CLASS(P, k_rows_fwd_f32, ), dim3(mm_cdiv(nrows, 2 * nl)), sm, st, args);
}

int mm_launch_rows_inv(const float2 *S, int nrows, int Pn, int H, float *out, float *blur, int delta,
                       cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(Pn, &P);
    if (rc) return rc;
    // the y blur's reciprocal table goes in the scratch: room for 2 delta + 2 floats
    auto bytes = [&](int l) {
        const size_t scr = sizeof(float4) * fft_scr_f4(P, l, kRowsInvCfg.threads / 32);
        const size_t rt = delta >= 0 ? sizeof(float) * (2 * (size_t)delta + 2) : 0;
        return fft_smem(P, l, kRowsInvCfg) + (rt > scr ? ((rt - scr + 15) & ~(size_t)15) : 0);
    };
    const size_t lim = (size_t)fft_smem_limit(kRowsInvCfg);
    int nl = 16;
    while (nl > 1 && bytes(nl) > lim) nl >>= 1;
    MM_REQUIRE(bytes(nl) <= lim, "blur radius %d too large for the tile", delta);
    size_t sm = bytes(nl);
    long long nr = nrows;
    int ngroups = mm_cdiv(nrows, 2 * nl);
    void *args[] = {&S, &nr, &H, &out, &blur, &delta, &P, &nl, &ngroups};
    return launch_fft_kernel(MM_FFT_KERNEL(P, nl, 8, k_rows_inv, ), dim3(fft_grid(ngroups, kRowsInvCfg)), sm, st, args,
                             kRowsInvCfg.threads);
}

int mm_launch_rows_inv_win(const float2 *S, const TileGeom &g, int reach, float *out, float *stitch, long long osz,
                           long long osx, cudaStream_t st) {
    MM_REQUIRE(!stitch || reach < 0, "stitching stores the centre window only");
    FftPlan P;
    int rc = mm_fft_plan_get(g.P, &P);
    if (rc) return rc;
    MM_REQUIRE(g.nt <= kMaxWinTiles, "windowed inverse pass takes at most %d tiles per batch", kMaxWinTiles);
    const size_t lim = (size_t)fft_smem_limit(kRowsInvCfg);
    const size_t cumb = sizeof(int) * ((size_t)g.nt + 1);
    auto bytes = [&](int l) { return ((fft_smem(P, l, kRowsInvCfg) + 15) & ~(size_t)15) + cumb; };
    int nl = 16;
    while (nl > 1 && bytes(nl) > lim) nl >>= 1;
    MM_REQUIRE(bytes(nl) <= lim, "windowed inverse pass does not fit shared memory");
    const size_t sm = bytes(nl);
    int cum_off = (int)(sm - cumb);
    // an upper bound of the groups (the kernel counts the exact number)
    const long long ngroups = (long long)g.nt * g.Z * mm_cdiv(g.P, 2 * nl);
    TileGeom ga = g;
    void *args[] = {&S, &ga, &reach, &out, &P, &nl, &cum_off, &stitch, &osz, &osx};
    return launch_fft_kernel(MM_FFT_KERNEL(P, nl, 8, k_rows_inv_win, ), dim3(fft_grid(ngroups, kRowsInvCfg)), sm, st,
                             args, kRowsInvCfg.threads);
}

int mm_launch_blur_x_sub(const TileGeom &g, const float *res, const float *tmp, int delta, float *res_out,
                         float *stitch, long long osz, long long osx, cudaStream_t st) {
    size_t sm = delta >= 0 ? ((size_t)g.P * 32 + 2 * delta + 2) * sizeof(float) : 0;
    MM_REQUIRE(sm <= (size_t)kSmemLimit, "blur radius %d too large for the tile", delta);
    int rc;
    dim3 grid(mm_cdiv(g.P, 32), g.Z, g.nt);
    if (stitch) {
        if ((rc = set_smem(k_blur_x_sub<true>, sm > 0 ? sm : 1))) return rc;
        k_blur_x_sub<true><<<grid, kBlurThreads, sm, st>>>(g, res, tmp, delta, res_out, stitch, osz, osx);
    } else {
        if ((rc = set_smem(k_blur_x_sub<false>, sm > 0 ? sm : 1))) return rc;
        k_blur_x_sub<false><<<grid, kBlurThreads, sm, st>>>(g, res, tmp, delta, res_out, stitch, osz, osx);
    }
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_make_raw(const TileGeom &g, const void *img, int dtype, const float *flat, float *raw,
                       cudaStream_t st) {
    dim3 grid(304, 1, g.nt);
    if (dtype == MM_DTYPE_U16)
        k_make_raw<uint16_t><<<grid, kBlurThreads, 0, st>>>(g, (const uint16_t *)img, flat, raw);
    else
        k_make_raw<float><<<grid, kBlurThreads, 0, st>>>(g, (const float *)img, flat, raw);
    MM_CHECK_LAUNCH();
    return MM_OK;
}
