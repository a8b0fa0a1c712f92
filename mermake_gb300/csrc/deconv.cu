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
//   cols          x: in-place complex FFT along a strided axis (fwd / inv)
//   zpass         z: gather mapped planes, FFT(Zp), multiply by the
//                 pre-scaled Wiener spectrum, IFFT(Zp), keep [zpad, zpad+Z)
//                                                         (deconvolver.py:155-157)
//   rows_inv      y: two half spectra -> one complex line -> IFFT -> two real rows
//   blur_y, blur_x_sub   box blur (blur.cu:1-52 semantics) and subtraction,
//                 optionally stitching the centre into the FOV output
//                                                         (deconvolver.py:160-163, 183)
//   make_raw      the raw view handed to the spot fit     (deconvolver.py:165-170)
#include "deconv.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kSmemLimit = 200 * 1024;

// Lines per CTA for a length-n transform: the largest power of two (<= maxnl)
// whose ping-pong buffers plus tables fit the shared-memory budget.
int pick_nl(const FftPlan &P, int maxnl) {
    int nl = maxnl;
    while (nl > 1) {
        size_t b = (size_t)2 * P.n * (nl + 1) * sizeof(float2) + (size_t)(P.n + P.ntab) * sizeof(float2);
        if (b <= (size_t)kSmemLimit) break;
        nl >>= 1;
    }
    return nl;
}

size_t fft_smem(const FftPlan &P, int nl) {
    return (size_t)2 * P.n * (nl + 1) * sizeof(float2) + (size_t)(P.n + P.ntab) * sizeof(float2);
}

template <typename K>
int set_smem(K kernel, size_t bytes) {
    MM_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes));
    return MM_OK;
}

// ---------------------------------------------------------------------------
// y pass, forward, u16 tile source
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(kThreads)
k_rows_fwd_img(TileGeom g, const T *__restrict__ img, const float *__restrict__ flat,
               float2 *__restrict__ S, FftPlan P, int nl) {
    extern __shared__ float2 smem[];
    const int n = P.n, ld = nl + 1;
    float2 *A = smem, *B = A + n * ld, *tw = B + n * ld, *tab = tw + n;
    fft_load_tables(P, tw, tab);

    const int ti = g.t0 + blockIdx.y;
    const TileDesc d = mm_tile_desc(g, ti);
    const long long nrows = (long long)g.Z * g.P;
    const long long row0 = (long long)blockIdx.x * 2 * nl;

    for (int it = threadIdx.x; it < 2 * nl * n; it += blockDim.x) {
        int q = it / n, e = it % n;
        long long row = row0 + q;
        float v = 0.f;
        if (row < nrows) {
            int z = (int)(row / g.P), xp = (int)(row % g.P);
            int sx = mm_map_xy(xp, d.x == 0, d.xd, g.P, g.ov);
            int sy = mm_map_xy(e, d.y == 0, d.yd, g.P, g.ov);
            if (sx >= 0 && sy >= 0) {
                int gx = d.x0 + sx, gy = d.y0 + sy;
                v = (float)img[z * g.isz + gx * g.isx + gy];
                if (flat) v = __fdiv_rn(v, flat[gx * g.fsx + gy]);
            }
        }
        float *s = reinterpret_cast<float *>(&A[e * ld + (q >> 1)]);
        s[q & 1] = v;
    }
    __syncthreads();
    float2 *R = fft_lines<false>(A, B, ld, nl, P, tw, tab);

    const int H = g.H;
    float2 *Sb = S + (long long)blockIdx.y * nrows * H;
    for (int it = threadIdx.x; it < nl * H; it += blockDim.x) {
        int l = it / H, k = it % H;
        long long r0 = row0 + 2 * l;
        float2 ck = R[k * ld + l];
        float2 cn = R[((n - k) % n) * ld + l];
        float2 x1 = make_float2(0.5f * (ck.x + cn.x), 0.5f * (ck.y - cn.y));
        float2 x2 = make_float2(0.5f * (ck.y + cn.y), -0.5f * (ck.x - cn.x));
        if (r0 < nrows) Sb[r0 * H + k] = x1;
        if (r0 + 1 < nrows) Sb[(r0 + 1) * H + k] = x2;
    }
}

// y pass, forward, dense f32 source (the padded PSF volume)
__global__ void __launch_bounds__(kThreads)
k_rows_fwd_f32(const float *__restrict__ vol, long long nrows, float2 *__restrict__ S, FftPlan P, int nl) {
    extern __shared__ float2 smem[];
    const int n = P.n, ld = nl + 1, H = n / 2 + 1;
    float2 *A = smem, *B = A + n * ld, *tw = B + n * ld, *tab = tw + n;
    fft_load_tables(P, tw, tab);
    const long long row0 = (long long)blockIdx.x * 2 * nl;
    for (int it = threadIdx.x; it < 2 * nl * n; it += blockDim.x) {
        int q = it / n, e = it % n;
        long long row = row0 + q;
        float v = row < nrows ? vol[row * n + e] : 0.f;
        float *s = reinterpret_cast<float *>(&A[e * ld + (q >> 1)]);
        s[q & 1] = v;
    }
    __syncthreads();
    float2 *R = fft_lines<false>(A, B, ld, nl, P, tw, tab);
    for (int it = threadIdx.x; it < nl * H; it += blockDim.x) {
        int l = it / H, k = it % H;
        long long r0 = row0 + 2 * l;
        float2 ck = R[k * ld + l];
        float2 cn = R[((n - k) % n) * ld + l];
        if (r0 < nrows) S[r0 * H + k] = make_float2(0.5f * (ck.x + cn.x), 0.5f * (ck.y - cn.y));
        if (r0 + 1 < nrows) S[(r0 + 1) * H + k] = make_float2(0.5f * (ck.y + cn.y), -0.5f * (ck.x - cn.x));
    }
}

// ---------------------------------------------------------------------------
// strided complex FFT, in place: line l of plane p starts at S + p*plane_stride + l,
// element e at + e*se.  Lines are contiguous, so a CTA's loads are runs of nl.
// ---------------------------------------------------------------------------
template <bool INV>
__global__ void __launch_bounds__(kThreads)
k_cols(float2 *__restrict__ S, long long se, int nlines, long long plane_stride, FftPlan P, int nl) {
    extern __shared__ float2 smem[];
    const int n = P.n, ld = nl + 1;
    float2 *A = smem, *B = A + n * ld, *tw = B + n * ld, *tab = tw + n;
    fft_load_tables(P, tw, tab);
    float2 *base = S + (long long)blockIdx.y * plane_stride;
    const int l0 = blockIdx.x * nl;
    for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
        int l = it % nl, e = it / nl;
        A[e * ld + l] = (l0 + l < nlines) ? base[e * se + l0 + l] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *R = fft_lines<INV>(A, B, ld, nl, P, tw, tab);
    for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
        int l = it % nl, e = it / nl;
        if (l0 + l < nlines) base[e * se + l0 + l] = R[e * ld + l];
    }
}

// ---------------------------------------------------------------------------
// z pass of the deconvolution: forward FFT over the padded depth, Wiener
// multiply, inverse FFT, keep the real planes.  W is (Zp, P, H) per spectrum,
// already scaled by 1 / (Zp * P * P).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_zpass(TileGeom g, float2 *__restrict__ S, const float2 *__restrict__ W, long long wstride, FftPlan P,
        int nl) {
    extern __shared__ float2 smem[];
    const int n = P.n, ld = nl + 1;
    float2 *A = smem, *B = A + n * ld, *tw = B + n * ld, *tab = tw + n;
    fft_load_tables(P, tw, tab);
    const int ti = g.t0 + blockIdx.y;
    const TileDesc d = mm_tile_desc(g, ti);
    const long long plane = (long long)g.P * g.H;
    float2 *St = S + (long long)blockIdx.y * g.Z * plane;
    const float2 *Wt = W + (long long)d.psf * wstride;
    const long long q0 = (long long)blockIdx.x * nl;
    for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
        int l = it % nl, e = it / nl;
        int src = mm_map_z(e, g.Z, g.zpad, g.Zp);
        float2 v = make_float2(0.f, 0.f);
        if (src >= 0 && q0 + l < plane) v = St[src * plane + q0 + l];
        A[e * ld + l] = v;
    }
    __syncthreads();
    float2 *R = fft_lines<false>(A, B, ld, nl, P, tw, tab);
    float2 *O = (R == A) ? B : A;
    for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
        int l = it % nl, e = it / nl;
        float2 w = (q0 + l < plane) ? Wt[e * plane + q0 + l] : make_float2(0.f, 0.f);
        O[e * ld + l] = cmul(R[e * ld + l], w);
    }
    __syncthreads();
    float2 *R2 = fft_lines<true>(O, R, ld, nl, P, tw, tab);
    for (int it = threadIdx.x; it < nl * g.Z; it += blockDim.x) {
        int l = it % nl, z = it / nl;
        if (q0 + l < plane) St[z * plane + q0 + l] = R2[(g.zpad + z) * ld + l];
    }
}

// z pass, forward only, all planes (the PSF transform)
__global__ void __launch_bounds__(kThreads)
k_zfwd(float2 *__restrict__ S, long long plane, FftPlan P, int nl) {
    extern __shared__ float2 smem[];
    const int n = P.n, ld = nl + 1;
    float2 *A = smem, *B = A + n * ld, *tw = B + n * ld, *tab = tw + n;
    fft_load_tables(P, tw, tab);
    const long long q0 = (long long)blockIdx.x * nl;
    for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
        int l = it % nl, e = it / nl;
        A[e * ld + l] = (q0 + l < plane) ? S[e * plane + q0 + l] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    float2 *R = fft_lines<false>(A, B, ld, nl, P, tw, tab);
    for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
        int l = it % nl, e = it / nl;
        if (q0 + l < plane) S[e * plane + q0 + l] = R[e * ld + l];
    }
}

// ---------------------------------------------------------------------------
// y pass, inverse: rows 2l and 2l+1 of H-long half spectra -> real rows of P.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_rows_inv(const float2 *__restrict__ S, long long nrows, int H, float *__restrict__ out, FftPlan P, int nl) {
    extern __shared__ float2 smem[];
    const int n = P.n, ld = nl + 1;
    float2 *A = smem, *B = A + n * ld, *tw = B + n * ld, *tab = tw + n;
    fft_load_tables(P, tw, tab);
    const long long row0 = (long long)blockIdx.x * 2 * nl;
    const bool even = (n % 2) == 0;
    for (int it = threadIdx.x; it < nl * H; it += blockDim.x) {
        int l = it / H, k = it % H;
        long long r0 = row0 + 2 * l;
        float2 x1 = r0 < nrows ? S[r0 * H + k] : make_float2(0.f, 0.f);
        float2 x2 = r0 + 1 < nrows ? S[(r0 + 1) * H + k] : make_float2(0.f, 0.f);
        if (k == 0 || (even && k == n / 2)) {
            A[k * ld + l] = make_float2(x1.x, x2.x);
        } else {
            A[k * ld + l] = make_float2(x1.x - x2.y, x1.y + x2.x);
            A[(n - k) * ld + l] = make_float2(x1.x + x2.y, x2.x - x1.y);
        }
    }
    __syncthreads();
    float2 *R = fft_lines<true>(A, B, ld, nl, P, tw, tab);
    for (int it = threadIdx.x; it < 2 * nl * n; it += blockDim.x) {
        int q = it / n, e = it % n;
        long long row = row0 + q;
        if (row < nrows) {
            float2 c = R[e * ld + (q >> 1)];
            out[row * n + e] = (q & 1) ? c.y : c.x;
        }
    }
}

// ---------------------------------------------------------------------------
// box blur, blur.cu:1-52 semantics: mean over [c-delta, c+delta] clipped to the
// axis, divided by the in-range count.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
k_blur_y(const float *__restrict__ in, float *__restrict__ out, long long nrows, int P, int delta) {
    extern __shared__ float rowbuf[];
    const int rows_per = blockDim.x / 32;
    const long long row = (long long)blockIdx.x * rows_per + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    float *r = rowbuf + (threadIdx.x / 32) * P;
    if (row < nrows)
        for (int e = lane; e < P; e += 32) r[e] = in[row * P + e];
    __syncwarp();
    if (row >= nrows) return;
    for (int e = lane; e < P; e += 32) {
        int s = e - delta < 0 ? 0 : e - delta;
        int t = e + delta > P - 1 ? P - 1 : e + delta;
        float sum = 0.f;
        for (int i = s; i <= t; ++i) sum += r[i];
        out[row * P + e] = sum / (float)(t - s + 1);
    }
}

// x blur of tmp, subtracted from res; writes the tile result in place and/or
// the stitched centre (deconvolver.py:183).  One CTA = one z plane of one tile
// and 32 consecutive y columns.  delta < 0: no blur (res copied).
__global__ void __launch_bounds__(kThreads)
k_blur_x_sub(TileGeom g, const float *__restrict__ res, const float *__restrict__ tmp, int delta,
             float *__restrict__ res_out, float *__restrict__ stitch, long long osz, long long osx) {
    extern __shared__ float colbuf[];  // P x 33
    const int P = g.P;
    const int ti = g.t0 + blockIdx.z;
    const TileDesc d = mm_tile_desc(g, ti);
    const int z = blockIdx.y;
    const int y0 = blockIdx.x * 32;
    const long long pbase = ((long long)blockIdx.z * g.Z + z) * P * P;
    if (delta >= 0) {
        for (int it = threadIdx.x; it < P * 32; it += blockDim.x) {
            int x = it / 32, c = it % 32;
            colbuf[x * 33 + c] = (y0 + c < P) ? tmp[pbase + (long long)x * P + y0 + c] : 0.f;
        }
        __syncthreads();
    }
    for (int it = threadIdx.x; it < P * 32; it += blockDim.x) {
        int x = it / 32, c = it % 32;
        int y = y0 + c;
        if (y >= P) continue;
        float v = res[pbase + (long long)x * P + y];
        if (delta >= 0) {
            int s = x - delta < 0 ? 0 : x - delta;
            int t = x + delta > P - 1 ? P - 1 : x + delta;
            float sum = 0.f;
            for (int i = s; i <= t; ++i) sum += colbuf[i * 33 + c];
            v = v - sum / (float)(t - s + 1);
        }
        if (res_out) res_out[pbase + (long long)x * P + y] = v;
        if (stitch && x >= g.ov && x < d.xend - g.ov && y >= g.ov && y < d.yend - g.ov) {
            long long ox = d.x + x - g.ov, oy = d.y + y - g.ov;
            if (ox < g.X && oy < g.Y) stitch[z * osz + ox * osx + oy] = v;
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
    int nl = pick_nl(P, 16);
    size_t sm = fft_smem(P, nl);
    dim3 grid(mm_cdiv((long)g.Z * g.P, 2 * nl), g.nt);
    if (dtype == MM_DTYPE_U16) {
        if ((rc = set_smem(k_rows_fwd_img<uint16_t>, sm))) return rc;
        k_rows_fwd_img<uint16_t><<<grid, kThreads, sm, st>>>(g, (const uint16_t *)img, flat, S, P, nl);
    } else {
        if ((rc = set_smem(k_rows_fwd_img<float>, sm))) return rc;
        k_rows_fwd_img<float><<<grid, kThreads, sm, st>>>(g, (const float *)img, flat, S, P, nl);
    }
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_rows_fwd_f32(const float *vol, int nrows, int Pn, float2 *S, cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(Pn, &P);
    if (rc) return rc;
    int nl = pick_nl(P, 16);
    size_t sm = fft_smem(P, nl);
    if ((rc = set_smem(k_rows_fwd_f32, sm))) return rc;
    k_rows_fwd_f32<<<mm_cdiv(nrows, 2 * nl), kThreads, sm, st>>>(vol, nrows, S, P, nl);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_cols(float2 *S, int n, long long se, int nlines, long long plane_stride, int nplanes, bool inv,
                   cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(n, &P);
    if (rc) return rc;
    int nl = pick_nl(P, 16);
    size_t sm = fft_smem(P, nl);
    dim3 grid(mm_cdiv(nlines, nl), nplanes);
    if (inv) {
        if ((rc = set_smem(k_cols<true>, sm))) return rc;
        k_cols<true><<<grid, kThreads, sm, st>>>(S, se, nlines, plane_stride, P, nl);
    } else {
        if ((rc = set_smem(k_cols<false>, sm))) return rc;
        k_cols<false><<<grid, kThreads, sm, st>>>(S, se, nlines, plane_stride, P, nl);
    }
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_zpass(const TileGeom &g, float2 *S, const float2 *W, long long wstride, cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(g.Zp, &P);
    if (rc) return rc;
    int nl = pick_nl(P, 32);
    size_t sm = fft_smem(P, nl);
    if ((rc = set_smem(k_zpass, sm))) return rc;
    dim3 grid(mm_cdiv((long)g.P * g.H, nl), g.nt);
    k_zpass<<<grid, kThreads, sm, st>>>(g, S, W, wstride, P, nl);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_zfwd(float2 *S, int Zp, int plane, cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(Zp, &P);
    if (rc) return rc;
    int nl = pick_nl(P, 32);
    size_t sm = fft_smem(P, nl);
    if ((rc = set_smem(k_zfwd, sm))) return rc;
    k_zfwd<<<mm_cdiv(plane, nl), kThreads, sm, st>>>(S, plane, P, nl);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_rows_inv(const float2 *S, int nrows, int Pn, int H, float *out, cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(Pn, &P);
    if (rc) return rc;
    int nl = pick_nl(P, 16);
    size_t sm = fft_smem(P, nl);
    if ((rc = set_smem(k_rows_inv, sm))) return rc;
    k_rows_inv<<<mm_cdiv(nrows, 2 * nl), kThreads, sm, st>>>(S, nrows, H, out, P, nl);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_blur_y(const float *in, float *out, int nrows, int P, int delta, cudaStream_t st) {
    size_t sm = (size_t)(kThreads / 32) * P * sizeof(float);
    int rc;
    if ((rc = set_smem(k_blur_y, sm))) return rc;
    k_blur_y<<<mm_cdiv(nrows, kThreads / 32), kThreads, sm, st>>>(in, out, nrows, P, delta);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_blur_x_sub(const TileGeom &g, const float *res, const float *tmp, int delta, float *res_out,
                         float *stitch, long long osz, long long osx, cudaStream_t st) {
    size_t sm = delta >= 0 ? (size_t)g.P * 33 * sizeof(float) : 0;
    int rc;
    if ((rc = set_smem(k_blur_x_sub, sm > 0 ? sm : 1))) return rc;
    dim3 grid(mm_cdiv(g.P, 32), g.Z, g.nt);
    k_blur_x_sub<<<grid, kThreads, sm, st>>>(g, res, tmp, delta, res_out, stitch, osz, osx);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_make_raw(const TileGeom &g, const void *img, int dtype, const float *flat, float *raw,
                       cudaStream_t st) {
    dim3 grid(304, 1, g.nt);
    if (dtype == MM_DTYPE_U16)
        k_make_raw<uint16_t><<<grid, kThreads, 0, st>>>(g, (const uint16_t *)img, flat, raw);
    else
        k_make_raw<float><<<grid, kThreads, 0, st>>>(g, (const float *)img, flat, raw);
    MM_CHECK_LAUNCH();
    return MM_OK;
}
