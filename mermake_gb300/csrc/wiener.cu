// Wiener spectrum builder (restating deconvolver.py:24-36, 48-75, 238-270).
//
// The PSF is centred/cropped into (Z, ts, ts) (center_psf), zero padded by
// (zpad, ov, ov) and rolled by -shape//2, all by index arithmetic in one
// kernel; its sum is reduced in double precision and divided out after the
// transform (the transform is linear).  The real 3-D transform reuses the
// deconvolution passes.  The regulariser is the reference's 5-neighbour
// "Laplacian" (6 at the centre; -1 at axis-0 +-1, axis-1 +-1, axis-2 -1 only),
// whose power spectrum is evaluated in closed form:
//   |L|^2 = (6 - 2 cos t0 - 2 cos t1 - cos t2)^2 + sin^2 t2,  t_a = 2 pi k_a / n_a.
// Output: W = conj(H) / (|H|^2 + beta |L|^2) / (Zp * P * P), half spectrum
// (Zp, P, P/2+1); the 1/(Zp P P) is the inverse transform's normalisation.
#include "deconv.cuh"

namespace {

struct PsfGeom {
    int pz, px, py;       // PSF shape
    int tz, tx, ty;       // centre_psf target (Z, ts, ts)
    int padz, padxy;      // zpad, ov
    int nz, nx, ny;       // padded shape (Zp, P, P)
};

__device__ inline int centred_src(int c, int T, int S) {
    // deconvolver.py:256-265
    int s0 = (T - S) / 2 > 0 ? (T - S) / 2 : 0;
    int s1 = (S - T) / 2 > 0 ? (S - T) / 2 : 0;
    int len = T < S ? T : S;
    if (c < s0 || c >= s0 + len) return -1;
    return c - s0 + s1;
}

__device__ inline int unroll_pad(int i, int n, int pad, int T, int S) {
    // np.roll(a, -n//2)[i] = a[(i + ceil(n/2)) mod n]; then remove the pad
    int p = (i + (n + 1) / 2) % n;
    int c = p - pad;
    if (c < 0 || c >= T) return -1;
    return centred_src(c, T, S);
}

__global__ void k_psf_place(PsfGeom g, const float *__restrict__ psf, float *__restrict__ vol,
                            double *__restrict__ parts) {
    const long long total = (long long)g.nz * g.nx * g.ny;
    double acc = 0.0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        int z = (int)(i / ((long long)g.nx * g.ny));
        int x = (int)((i / g.ny) % g.nx);
        int y = (int)(i % g.ny);
        int sz = unroll_pad(z, g.nz, g.padz, g.tz, g.pz);
        int sx = unroll_pad(x, g.nx, g.padxy, g.tx, g.px);
        int sy = unroll_pad(y, g.ny, g.padxy, g.ty, g.py);
        float v = 0.f;
        if (sz >= 0 && sx >= 0 && sy >= 0) v = psf[((long long)sz * g.px + sx) * g.py + sy];
        vol[i] = v;
        acc += (double)v;
    }
    // the PSF sum in a fixed order (k_sum_parts adds the block partials)
    acc = mm_block_sum(acc);
    if (threadIdx.x == 0) parts[blockIdx.x] = acc;
}

__global__ void k_wiener(const float2 *__restrict__ Hs, int nz, int nx, int hy, int ny, float beta,
                         const double *__restrict__ sum, float2 *__restrict__ W) {
    const long long total = (long long)nz * nx * hy;
    const double inv_sum = 1.0 / sum[0];
    const double scale = 1.0 / ((double)nz * nx * ny);
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        int kz = (int)(i / ((long long)nx * hy));
        int kx = (int)((i / hy) % nx);
        int ky = (int)(i % hy);
        double c0 = cospi(2.0 * kz / nz), c1 = cospi(2.0 * kx / nx);
        double c2 = cospi(2.0 * ky / ny), s2 = sinpi(2.0 * ky / ny);
        double a = 6.0 - 2.0 * c0 - 2.0 * c1 - c2;
        double L2 = a * a + s2 * s2;
        float2 h = Hs[i];
        double hr = h.x * inv_sum, hi = h.y * inv_sum;
        double D = hr * hr + hi * hi + (double)beta * L2;
        W[i] = make_float2((float)(hr / D * scale), (float)(-hi / D * scale));
    }
}

}  // namespace

int mm_wiener_build_impl(const float *psf, int pz, int px, int py, int tile_height, int tile_size, int zpad,
                         int overlap, float beta, float2 *W, float *vol, float2 *S, double *dsum, double *parts,
                         cudaStream_t st) {
    PsfGeom g;
    g.pz = pz; g.px = px; g.py = py;
    g.tz = tile_height; g.tx = tile_size; g.ty = tile_size;
    g.padz = zpad; g.padxy = overlap;
    g.nz = tile_height + 2 * zpad;
    g.nx = tile_size + 2 * overlap;
    g.ny = g.nx;
    const int H = g.ny / 2 + 1;
    k_psf_place<<<608, 256, 0, st>>>(g, psf, vol, parts);
    MM_CHECK_LAUNCH();
    int rc;
    if ((rc = mm_launch_sum_parts(parts, 608, dsum, st))) return rc;
    if ((rc = mm_launch_rows_fwd_f32(vol, g.nz * g.nx, g.ny, S, st))) return rc;
    if ((rc = mm_launch_cols(S, g.nx, H, H, (long long)g.nx * H, g.nz, false, st))) return rc;
    if ((rc = mm_launch_zfwd(S, g.nz, g.nx * H, st))) return rc;
    k_wiener<<<608, 256, 0, st>>>(S, g.nz, g.nx, H, g.ny, beta, dsum, W);
    MM_CHECK_LAUNCH();
    return MM_OK;
}
