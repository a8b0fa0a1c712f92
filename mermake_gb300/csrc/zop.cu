// z pass of the tiled deconvolution as a matrix per frequency, for a single
// Wiener spectrum (mermake/deconvolver.py:139-157 with one PSF).
//
// After the x/y transforms, each (x, y) frequency p of a tile holds Z complex
// values, one per real plane.  The reference pads them to Zp planes (reflect
// at zpad and zpad+Z-1, mm_map_z), transforms over Zp, multiplies by W, and
// transforms back, then keeps planes [zpad, zpad+Z).  That is a linear map of
// the Z values, Y[i] = sum_j M_p[i][j] X[j], and because padding only copies
// planes, every entry is a sum of samples of one vector per frequency:
//
//   M_p[i][j] = sum_{z : map_z(z) = j} w_p[(zpad + i - z) mod Zp],
//   w_p[d]    = sum_kz W[kz][p] exp(+2 pi i kz d / Zp)
//
// (w_p is the unnormalised inverse DFT of W along z; W already holds the
// 1 / (Zp P P) normalisation).  At most four z map to one j.  The "z kernel" w
// (Zp, P, P/2+1) complex64, the size of W, is built once per spectrum
// (k_zker_build) and kept resident.  With one spectrum every tile of a batch
// uses the same M_p, so the z pass of nt tiles is, per p, a (Z x Z) by
// (Z x nt) complex product: regular FP32 FMA work with register blocking, in
// place of two transforms over the padded depth.
#include <math.h>

#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "deconv.cuh"

namespace {

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gsrc) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// w[d][p] = sum_kz W[kz][p] e^{+2 pi i kz d / Zp}: a CTA stages W for kBuildP
// consecutive p and the Zp roots of unity (double precision, rounded once);
// a warp per d, two p per lane.
constexpr int kBuildP = 64;
constexpr int kBuildThreads = 256;

__global__ void __launch_bounds__(kBuildThreads)
k_zker_build(const float2 *__restrict__ W, float2 *__restrict__ w, int Zp, long long plane) {
    extern __shared__ __align__(16) float2 Ws[];  // Zp x kBuildP, then Zp roots
    float2 *root = Ws + (size_t)Zp * kBuildP;
    const long long p0 = (long long)blockIdx.x * kBuildP;
    for (int it = threadIdx.x; it < Zp * kBuildP; it += blockDim.x) {
        const int kz = it / kBuildP, pp = it - kz * kBuildP;
        Ws[it] = p0 + pp < plane ? W[(long long)kz * plane + p0 + pp] : make_float2(0.f, 0.f);
    }
    for (int k = threadIdx.x; k < Zp; k += blockDim.x) {
        double s, c;
        sincospi(2.0 * (double)k / (double)Zp, &s, &c);
        root[k] = make_float2((float)c, (float)s);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int d = warp; d < Zp; d += nw) {
        float ax = 0.f, ay = 0.f, bx = 0.f, by = 0.f;
        int e = 0;
        for (int kz = 0; kz < Zp; ++kz) {
            const float2 c = root[e];
            const float2 w0 = Ws[kz * kBuildP + lane], w1 = Ws[kz * kBuildP + 32 + lane];
            ax = fmaf(c.x, w0.x, fmaf(-c.y, w0.y, ax));
            ay = fmaf(c.x, w0.y, fmaf(c.y, w0.x, ay));
            bx = fmaf(c.x, w1.x, fmaf(-c.y, w1.y, bx));
            by = fmaf(c.x, w1.y, fmaf(c.y, w1.x, by));
            e += d;
            if (e >= Zp) e -= Zp;
        }
        const long long base = (long long)d * plane + p0;
        if (p0 + lane < plane) w[base + lane] = make_float2(ax, ay);
        if (p0 + 32 + lane < plane) w[base + 32 + lane] = make_float2(bx, by);
    }
}

// ---------------------------------------------------------------------------
// Apply: Y[t][i][p] = sum_j M_p[i][j] X[t][j][p] in place on the batch
// spectrum S (nt, Z, plane).  A CTA owns kPB consecutive p.  It stages their
// z kernel and sums all of M (Z x Z x kPB) into shared memory once, with a
// thread per (j, p) walking i (the kernel index of each copy of plane j just
// advances by one per i).  Then it walks j in chunks of kJC with the chunk of
// X (TC tile rows) staged by cp.async into a ring of three buffers, so a
// single barrier per chunk both publishes chunk c and frees the buffer of
// chunk c - 1 for chunk c + 2.  Thread (p, ig, tg) keeps the TI x TT block of
// outputs i in [ig TI, ig TI + TI), t in [tg TT, tg TT + TT) in registers.
// Row strides (Z kPB + 4 for M, kJC kPB + 4 for X, in float2) put the i-groups
// a warp reads on bank windows that overlap at most twice, the minimum for
// 256 bytes.  With Z = 50 and 25 tiles a CTA has 200 threads and 110 KB, so
// two run on an SM and one's barrier waits overlap the other's FMAs.  Tiles go
// in chunks of TC = tgn TT; every read of a chunk's rows precedes its writes,
// and chunks touch disjoint rows, so the update is in place.
// ---------------------------------------------------------------------------
constexpr int kPB = 4;
constexpr int kJC = 10;
constexpr int kXS = kJC * kPB + 4;
constexpr int kTI = 5, kTT = 5;
constexpr int kNBuf = 3;
constexpr int kApplyMaxThreads = 256;

// for each real plane j: how many padded planes copy it, and the kernel index
// (zpad - z) mod Zp of each copy z (at most MM_ZOP_MAX_COPIES)
struct ZopTab {
    int n[MM_ZOP_MAX_Z];
    int off[MM_ZOP_MAX_Z][MM_ZOP_MAX_COPIES];
};

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
    c.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x));
    c.y = fmaf(a.x, b.y, fmaf(a.y, b.x, c.y));
    return c;
}

// ZC > 0: the tile height known at compile time (Z = 50, the depth of every
// channel of the benchmark FOV), so the chunk and row bounds fold; a multiple
// of kJC and kTI drops the tail checks.
template <bool V16, int ZC>
__global__ void __launch_bounds__(kApplyMaxThreads, 2)
k_zop_apply(float2 *__restrict__ S, const float2 *__restrict__ w, int Z, int Zp, long long plane, int nt, int ign,
            int tgn, const ZopTab tab, const float *__restrict__ fresp) {
    extern __shared__ __align__(16) float2 sm[];
    if constexpr (ZC > 0) {
        Z = ZC;
        ign = (ZC + kTI - 1) / kTI;
    }
    constexpr bool kFullChunks = ZC > 0 && ZC % kJC == 0 && ZC % kTI == 0;
    const int rowsM = ign * kTI, TC = tgn * kTT;
    const int msw = Z * kPB + 4;       // M row stride
    float2 *ws = sm;                   // Zp x kPB
    float2 *Ms = ws + Zp * kPB;        // rowsM x msw
    float2 *Xb = Ms + rowsM * msw;     // kNBuf x TC x kXS
    const int tid = threadIdx.x, nth = blockDim.x;
    const int p = tid % kPB;
    const int rest = tid / kPB;
    const int ig = rest % ign, tg = rest / ign;
    const long long p0 = (long long)blockIdx.x * kPB;
    const int nch = (Z + kJC - 1) / kJC;

    auto load_x = [&](int tc0, int c, int buf) {
        float2 *Xs = Xb + buf * TC * kXS;
        const int j0 = c * kJC;
        for (int u = tid; u < TC * kJC * (kPB / 2); u += nth) {
            const int pp = (u % (kPB / 2)) * 2;
            const int r = u / (kPB / 2);
            const int jj = r % kJC, row = r / kJC;
            const int j = j0 + jj;
            float2 *dst = Xs + row * kXS + jj * kPB + pp;
            const long long pg = p0 + pp;
            const bool ok = j < Z && tc0 + row < nt;
            const float2 *src = S + ((long long)(tc0 + row) * Z + j) * plane + pg;
            if (V16) {
                // plane is even here, so pg < plane implies pg + 1 < plane
                if (ok && pg < plane)
                    cp_async16(dst, src);
                else
                    *reinterpret_cast<float4 *>(dst) = make_float4(0.f, 0.f, 0.f, 0.f);
            } else {
                if (ok && pg < plane)
                    cp_async8(dst, src);
                else
                    dst[0] = make_float2(0.f, 0.f);
                if (ok && pg + 1 < plane)
                    cp_async8(dst + 1, src + 1);
                else
                    dst[1] = make_float2(0.f, 0.f);
            }
        }
        cp_async_commit();
    };

    // the z kernel of this CTA's p, and the first two X chunks
    for (int e = tid; e < Zp * kPB; e += nth) {
        const int d = e / kPB, pp = e - d * kPB;
        if (p0 + pp < plane)
            cp_async8(&ws[e], &w[(long long)d * plane + p0 + pp]);
        else
            ws[e] = make_float2(0.f, 0.f);
    }
    cp_async_commit();
    load_x(0, 0, 0);
    if (nch > 1) {
        load_x(0, 1, 1);
        cp_async_wait_group<2>();
    } else {
        cp_async_wait_group<1>();
    }
    __syncthreads();
    // M[i][j] = sum over the copies of plane j of ws[(i + off) mod Zp]: a thread
    // per (j, p) adds each copy's run of the kernel, ten rows i at a time (the
    // run wraps past Zp at most once, handled by the slow branch)
    for (int q = tid; q < Z * kPB; q += nth) {
        const int j = q / kPB, pp = q - j * kPB;
        const int n = tab.n[j];
        float2 *col = Ms + j * kPB + pp;
        for (int i0 = 0; i0 < Z; i0 += 10) {
            float2 acc[10];
#pragma unroll
            for (int ii = 0; ii < 10; ++ii) acc[ii] = make_float2(0.f, 0.f);
            for (int k = 0; k < n; ++k) {
                int d0 = tab.off[j][k] + i0;
                if (d0 >= Zp) d0 -= Zp;
                if (d0 + 10 <= Zp) {
                    const float2 *wp = ws + d0 * kPB + pp;
#pragma unroll
                    for (int ii = 0; ii < 10; ++ii) {
                        const float2 t = wp[ii * kPB];
                        acc[ii].x += t.x;
                        acc[ii].y += t.y;
                    }
                } else {
#pragma unroll
                    for (int ii = 0; ii < 10; ++ii) {
                        const int dd = (d0 + ii) % Zp;
                        const float2 t = ws[dd * kPB + pp];
                        acc[ii].x += t.x;
                        acc[ii].y += t.y;
                    }
                }
            }
#pragma unroll
            for (int ii = 0; ii < 10; ++ii)
                if (i0 + ii < Z) col[(i0 + ii) * msw] = acc[ii];
        }
    }

    for (int tc0 = 0; tc0 < nt; tc0 += TC) {
        if (tc0 > 0) {
            __syncthreads();  // every read of the previous tile chunk's buffers is done
            load_x(tc0, 0, 0);
            if (nch > 1) load_x(tc0, 1, 1);
        }
        float2 acc[kTI][kTT];
#pragma unroll
        for (int a = 0; a < kTI; ++a)
#pragma unroll
            for (int b = 0; b < kTT; ++b) acc[a][b] = make_float2(0.f, 0.f);

        for (int c = 0; c < nch; ++c) {
            if (c + 1 < nch)
                cp_async_wait_group<1>();
            else
                cp_async_wait_group<0>();
            __syncthreads();  // chunk c (and M) visible; chunk c - 1's buffer free
            if (c + 2 < nch) load_x(tc0, c + 2, (c + 2) % kNBuf);
            const int j0 = c * kJC;
            const int jn = kFullChunks ? kJC : (Z - j0 < kJC ? Z - j0 : kJC);
            const float2 *mr = Ms + (ig * kTI) * msw + j0 * kPB + p;
            const float2 *xr = Xb + (c % kNBuf) * TC * kXS + (tg * kTT) * kXS + p;
#pragma unroll
            for (int jj = 0; jj < kJC; ++jj) {
                if (!kFullChunks && jj >= jn) break;
                float2 m[kTI], x[kTT];
#pragma unroll
                for (int a = 0; a < kTI; ++a) m[a] = mr[a * msw + jj * kPB];
#pragma unroll
                for (int b = 0; b < kTT; ++b) x[b] = xr[b * kXS + jj * kPB];
#pragma unroll
                for (int a = 0; a < kTI; ++a)
#pragma unroll
                    for (int b = 0; b < kTT; ++b) acc[a][b] = cfma(m[a], x[b], acc[a][b]);
            }
        }
        if (p0 + p < plane) {
            // the blur subtraction as a factor of this frequency (1 when not folded)
            const float f = fresp ? fresp[p0 + p] : 1.f;
#pragma unroll
            for (int a = 0; a < kTI; ++a) {
                const int i = ig * kTI + a;
                if (!kFullChunks && i >= Z) break;
#pragma unroll
                for (int b = 0; b < kTT; ++b) {
                    const int t = tc0 + tg * kTT + b;
                    if (t < nt) S[((long long)t * Z + i) * plane + p0 + p] = cscale(acc[a][b], f);
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Direct z convolution, for batches whose tiles each have their own spectrum
// (a PSF grid) or are too few for the matrix form:
//   Y[t][i][p] = sum_{z < Zp} w_t[(zpad + i - z) mod Zp][p] X[t][map_z(z)][p]
// (map_z(z) < 0: a zero plane), with w_t the z kernel of tile t's spectrum.
// A CTA owns kCq consecutive p (a lane each) of one tile; warp g computes the
// outputs i in [g kCI, g kCI + kCI).  The CTA stages, for its p, the run of
// the periodic z kernel its windows read (wx[u] = w[(u + zpad + 1 - Tpad)
// mod Zp], so no index wraps) and the tile's Z planes plus a zero row, every
// copy in flight at once (cp.async).  The z loop runs in
// blocks of kCI planes: for a block the 2 kCI - 1 kernel values every output
// of the thread needs are one contiguous run of wx, held in registers, so a
// block costs kCI^2 complex FMAs for 3 kCI - 1 shared-memory loads.  Every
// read of the tile's planes precedes the barrier and the CTAs own disjoint
// (tile, p), so the update is in place.
// ---------------------------------------------------------------------------
constexpr int kCq = 32;
constexpr int kCI = 8;  // the plane map is read as int4 pairs below
constexpr int kConvMaxThreads = 512;  // 16 i-groups: Z <= 128

// kernel rows a CTA reads: the windows of all its warps and z blocks form one
// run of ceil(Z / kCI) kCI + Tpad - 1 consecutive rows of the periodic kernel
__device__ __host__ __forceinline__ int zconv_tpad(int Zp) { return (Zp + kCI - 1) / kCI * kCI; }
__device__ __host__ __forceinline__ int zconv_wx_rows(int Z, int Zp) {
    return (Z + kCI - 1) / kCI * kCI + zconv_tpad(Zp) - 1;
}

__global__ void __launch_bounds__(kConvMaxThreads)
k_zconv(float2 *__restrict__ S, const float2 *__restrict__ w, long long wstride, int Z, int zpad, int Zp,
        long long plane, int t0, int npsf, const float *__restrict__ fresp) {
    extern __shared__ __align__(16) float2 sm[];
    const int Lw = zconv_wx_rows(Z, Zp);
    const int Tpad = zconv_tpad(Zp);
    float2 *wx = sm;                                          // Lw x kCq
    float2 *xs = wx + (size_t)Lw * kCq;                       // (Z + 1) x kCq, row Z zero
    int *zm = reinterpret_cast<int *>(xs + (size_t)(Z + 1) * kCq);  // Tpad rows of xs
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int t = blockIdx.y;
    const long long p = (long long)blockIdx.x * kCq + lane;
    const bool pv = p < plane;
    const float2 *wp = w + (npsf == 1 ? 0 : (long long)(t0 + t)) * wstride;
    float2 *Sp = S + (long long)t * Z * plane;
    // all staging copies in flight at once (cp.async), then one wait
    for (int u = g; u < Lw; u += nw) {
        int d = (u + zpad + 1 - Tpad) % Zp;
        if (d < 0) d += Zp;
        if (pv)
            cp_async8(&wx[u * kCq + lane], &wp[(long long)d * plane + p]);
        else
            wx[u * kCq + lane] = make_float2(0.f, 0.f);
    }
    for (int j = g; j <= Z; j += nw) {
        if (j < Z && pv)
            cp_async8(&xs[j * kCq + lane], &Sp[(long long)j * plane + p]);
        else
            xs[j * kCq + lane] = make_float2(0.f, 0.f);
    }
    for (int z = threadIdx.x; z < Tpad; z += blockDim.x) {
        const int m = z < Zp ? mm_map_z(z, Z, zpad, Zp) : -1;
        zm[z] = m < 0 ? Z : m;
    }
    cp_async_commit();
    cp_async_wait_group<0>();
    __syncthreads();
    const int i0 = g * kCI;
    if (i0 >= Z) return;
    float2 acc[kCI];
#pragma unroll
    for (int a = 0; a < kCI; ++a) acc[a] = make_float2(0.f, 0.f);
    for (int zb = 0; zb < Tpad; zb += kCI) {
        // term (z = zb + s, i = i0 + a) uses w[(zpad + i - z) mod Zp] = wx[i0 - zb + Tpad - kCI + (kCI - 1 - s + a)]
        float2 x[kCI], wr[2 * kCI - 1];
        // the block's plane map as two 16-byte broadcasts (zb is a multiple of
        // kCI = 8 and zm starts on a 256-byte boundary)
        const int4 m0 = *reinterpret_cast<const int4 *>(zm + zb), m1 = *reinterpret_cast<const int4 *>(zm + zb + 4);
        const int mz[kCI] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
        for (int s = 0; s < kCI; ++s) x[s] = xs[mz[s] * kCq + lane];
        const float2 *wb = wx + (i0 - zb + Tpad - kCI) * kCq + lane;
#pragma unroll
        for (int r = 0; r < 2 * kCI - 1; ++r) wr[r] = wb[r * kCq];
#pragma unroll
        for (int s = 0; s < kCI; ++s)
#pragma unroll
            for (int a = 0; a < kCI; ++a) acc[a] = cfma(wr[kCI - 1 - s + a], x[s], acc[a]);
    }
    if (pv) {
        const float f = fresp ? fresp[p] : 1.f;
#pragma unroll
        for (int a = 0; a < kCI; ++a)
            if (i0 + a < Z) Sp[(long long)(i0 + a) * plane + p] = cscale(acc[a], f);
    }
}

}  // namespace

static size_t mm_zconv_smem(int Z, int Zp) {
    return sizeof(float2) * ((size_t)zconv_wx_rows(Z, Zp) + Z + 1) * kCq + sizeof(int) * (size_t)zconv_tpad(Zp);
}

int mm_zconv_supported(int Z, int zpad) {
    const int Zp = Z + 2 * zpad;
    return Z >= 1 && zpad >= 1 && (Z + kCI - 1) / kCI * 32 <= kConvMaxThreads && Zp <= MM_ZOP_MAX_ZP &&
           mm_zconv_smem(Z, Zp) <= 227 * 1024;
}

int mm_launch_zconv(float2 *S, const float2 *w, long long wstride, int Z, int zpad, int Zp, long long plane, int t0,
                    int nt, int npsf, const float *fresp, cudaStream_t st) {
    MM_REQUIRE(Zp == Z + 2 * zpad && mm_zconv_supported(Z, zpad),
               "z convolution needs Z <= %d and Zp <= %d (Z %d, zpad %d)", kConvMaxThreads / 32 * kCI, MM_ZOP_MAX_ZP,
               Z, zpad);
    if (nt <= 0) return MM_OK;
    const size_t sm = mm_zconv_smem(Z, Zp);
    if (int rc = mm_set_smem((const void *)k_zconv, sm)) return rc;
    const int threads = (Z + kCI - 1) / kCI * 32;
    dim3 grid((unsigned)((plane + kCq - 1) / kCq), (unsigned)nt);
    k_zconv<<<grid, threads, sm, st>>>(S, w, wstride, Z, zpad, Zp, plane, t0, npsf, fresp);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_zker_build_impl(const float2 *W, int Zp, long long plane, float2 *w, cudaStream_t st) {
    MM_REQUIRE(Zp >= 1 && Zp <= MM_ZOP_MAX_ZP, "z kernel needs 1 <= Zp <= %d (got %d)", MM_ZOP_MAX_ZP, Zp);
    const size_t sm = sizeof(float2) * (size_t)Zp * (kBuildP + 1);
    if (int rc = mm_set_smem((const void *)k_zker_build, sm)) return rc;
    k_zker_build<<<(unsigned)((plane + kBuildP - 1) / kBuildP), kBuildThreads, sm, st>>>(W, w, Zp, plane);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_zop_supported(int Z, int zpad) {
    const int Zp = Z + 2 * zpad;
    if (Z < 1 || Z > MM_ZOP_MAX_Z || zpad < 1 || Zp > MM_ZOP_MAX_ZP) return 0;
    for (int j = 0; j < Z; ++j) {
        int n = 0;
        for (int z = 0; z < Zp; ++z) n += mm_map_z(z, Z, zpad, Zp) == j;
        if (n > MM_ZOP_MAX_COPIES) return 0;
    }
    return 1;
}

int mm_launch_zop_apply(float2 *S, const float2 *w, int Z, int zpad, int Zp, long long plane, int nt,
                        const float *fresp, cudaStream_t st) {
    MM_REQUIRE(Zp == Z + 2 * zpad && mm_zop_supported(Z, zpad),
               "z operator needs Z <= %d, Zp <= %d and at most %d copies of a plane (Z %d, zpad %d)", MM_ZOP_MAX_Z,
               MM_ZOP_MAX_ZP, MM_ZOP_MAX_COPIES, Z, zpad);
    if (nt <= 0) return MM_OK;
    ZopTab tab = {};
    for (int j = 0; j < Z; ++j)
        for (int z = 0; z < Zp; ++z)
            if (mm_map_z(z, Z, zpad, Zp) == j) {
                const int o = ((zpad - z) % Zp + Zp) % Zp;
                tab.off[j][tab.n[j]++] = o;
            }
    int ign = (Z + kTI - 1) / kTI;
    const int tmax = kApplyMaxThreads / (kPB * ign);
    int tgn = (nt + kTT - 1) / kTT;
    if (tgn > tmax) tgn = tmax;
    const int threads = kPB * ign * tgn;
    const size_t sm = sizeof(float2) * ((size_t)Zp * kPB + (size_t)ign * kTI * (Z * kPB + 4) +
                                        (size_t)kNBuf * tgn * kTT * kXS);
    MM_REQUIRE(sm <= 227 * 1024, "z operator shared memory %zu bytes exceeds the limit", sm);
    const void *fn = Z == 50 ? ((plane % 2 == 0) ? (const void *)k_zop_apply<true, 50> : (const void *)k_zop_apply<false, 50>)
                             : ((plane % 2 == 0) ? (const void *)k_zop_apply<true, 0> : (const void *)k_zop_apply<false, 0>);
    if (int rc = mm_set_smem(fn, sm)) return rc;
    dim3 grid((unsigned)((plane + kPB - 1) / kPB));
    void *args[] = {&S, &w, &Z, &Zp, &plane, &nt, &ign, &tgn, &tab, &fresp};
    MM_CUDA_TRY(cudaLaunchKernel(fn, grid, dim3(threads), args, sm, st));
    mm_launch_counter_add();
    return MM_OK;
}

// ---------------------------------------------------------------------------
// The blur subtraction of tile_wise (deconvolver.py:160-163: res minus its box
// mean along x, then y, window 2 d + 1, blur.cu:1-52) as a frequency response.
// At a voxel at least d from every edge of the P x P plane the truncated box
// mean is the circular one, so there res - box_x(box_y(res)) is the inverse
// transform of the spectrum times
//   f(kx, ky) = 1 - D(kx) D(ky),   D(k) = (1 / (2d + 1)) sum_{e=-d..d} cos(2 pi k e / P)
// over the half spectrum (kx < P, ky < P/2 + 1).  The table (float, P x H) is
// computed in double on the host and cached per (device, P, d); the first
// request uploads it synchronously.
// ---------------------------------------------------------------------------
int mm_blur_response_get(int P, int delta, const float **out) {
    static std::mutex mu;
    static std::map<std::tuple<int, int, int>, float *> cache;
    MM_REQUIRE(P >= 1 && delta >= 0 && 2 * delta + 1 <= P, "blur window %d too wide for a plane of %d", 2 * delta + 1,
               P);
    int dev = 0;
    MM_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    auto key = std::make_tuple(dev, P, delta);
    auto it = cache.find(key);
    if (it != cache.end()) {
        *out = it->second;
        return MM_OK;
    }
    const int H = P / 2 + 1;
    std::vector<double> D(P);
    for (int k = 0; k < P; ++k) {
        double acc = 0.0;
        for (int e = -delta; e <= delta; ++e) acc += cos(2.0 * M_PI * (double)(((long long)k * e) % P) / (double)P);
        D[k] = acc / (double)(2 * delta + 1);
    }
    std::vector<float> f((size_t)P * H);
    for (int kx = 0; kx < P; ++kx)
        for (int ky = 0; ky < H; ++ky) f[(size_t)kx * H + ky] = (float)(1.0 - D[kx] * D[ky]);
    float *d = nullptr;
    MM_CUDA_TRY(cudaMalloc(&d, sizeof(float) * f.size()));
    MM_CUDA_TRY(cudaMemcpy(d, f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
    cache[key] = d;
    *out = d;
    return MM_OK;
}
