// z pass of the tiled deconvolution as a matrix per frequency, for a single
// Wiener spectrum (mermake/deconvolver.py:139-157 with one PSF).
//
// After the x/y transforms, each (x, y) frequency p of a tile holds Z complex
// values, one per real plane.  The reference pads them to Zp planes (reflect
// at zpad and zpad+Z-1, mm_map_z), transforms over Zp, multiplies by W, and
// transforms back, then keeps planes [zpad, zpad+Z).  That is a linear map of
// the Z values:
//
//   Y[i] = sum_j M_p[i][j] X[j],
//   M_p[i][j] = sum_kz E[i][j][kz] W[kz][p],
//   E[i][j][kz] = sum_{z : map_z(z) = j} exp(+2 pi i kz (zpad + i - z) / Zp)
//
// (W already holds the 1 / (Zp P P) normalisation of both inverse transforms).
// With one spectrum every tile of a batch uses the same M_p, so the z pass of
// nt tiles becomes, per p, a (Z x Z) by (Z x nt) complex product: regular FP32
// FMA work with register blocking, in place of two transforms over the padded
// depth.  M is built once per spectrum (k_zop_coef, k_zop_build) and kept
// resident, (Z, Z, P, P/2+1) complex64.
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

// E[i][j][kz] in double precision from exact integer phases, rounded once.
__global__ void k_zop_coef(float2 *__restrict__ E, int Z, int zpad, int Zp) {
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long total = (long long)Z * Z * Zp;
    if (idx >= total) return;
    const int kz = (int)(idx % Zp);
    const long long r = idx / Zp;
    const int j = (int)(r % Z), i = (int)(r / Z);
    double re = 0.0, im = 0.0;
    for (int z = 0; z < Zp; ++z) {
        if (mm_map_z(z, Z, zpad, Zp) != j) continue;
        long long e = ((long long)kz * (zpad + i - z)) % Zp;
        if (e < 0) e += Zp;
        double s, c;
        sincospi(2.0 * (double)e / (double)Zp, &s, &c);
        re += c;
        im += s;
    }
    E[idx] = make_float2((float)re, (float)im);
}

// M[i][j][p] = sum_kz E[i][j][kz] W[kz][p]: a CTA stages W for kBuildP
// consecutive p; a warp per (i, j) pair, two p per lane.
constexpr int kBuildP = 64;
constexpr int kBuildThreads = 256;

__global__ void __launch_bounds__(kBuildThreads)
k_zop_build(const float2 *__restrict__ W, const float2 *__restrict__ E, float2 *__restrict__ M, int Z, int Zp,
            long long plane) {
    extern __shared__ __align__(16) float2 Ws[];  // Zp x kBuildP
    const long long p0 = (long long)blockIdx.x * kBuildP;
    for (int it = threadIdx.x; it < Zp * kBuildP; it += blockDim.x) {
        const int kz = it / kBuildP, pp = it - kz * kBuildP;
        Ws[it] = p0 + pp < plane ? W[(long long)kz * plane + p0 + pp] : make_float2(0.f, 0.f);
    }
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int ij = warp; ij < Z * Z; ij += nw) {
        const float2 *e = E + (long long)ij * Zp;
        float ax = 0.f, ay = 0.f, bx = 0.f, by = 0.f;
        for (int kz = 0; kz < Zp; ++kz) {
            const float2 c = __ldg(e + kz);
            const float2 w0 = Ws[kz * kBuildP + lane], w1 = Ws[kz * kBuildP + 32 + lane];
            ax = fmaf(c.x, w0.x, fmaf(-c.y, w0.y, ax));
            ay = fmaf(c.x, w0.y, fmaf(c.y, w0.x, ay));
            bx = fmaf(c.x, w1.x, fmaf(-c.y, w1.y, bx));
            by = fmaf(c.x, w1.y, fmaf(c.y, w1.x, by));
        }
        const long long base = (long long)ij * plane + p0;
        if (p0 + lane < plane) M[base + lane] = make_float2(ax, ay);
        if (p0 + 32 + lane < plane) M[base + 32 + lane] = make_float2(bx, by);
    }
}

// ---------------------------------------------------------------------------
// Apply: Y[t][i][p] = sum_j M[i][j][p] X[t][j][p] in place on the batch
// spectrum S (nt, Z, plane).  A CTA owns kPB consecutive p and walks j in
// chunks of kJC, staging M (Z rows) and X (TC tile rows) of the chunk in
// shared memory with cp.async, double-buffered.  Thread (p, ig, tg) keeps the
// TI x TT block of outputs i in [ig TI, ig TI + TI), t in [tg TT, tg TT + TT)
// in registers.  Shared rows are kMS float2 apart (kJC * kPB + 4): the four
// i-groups a warp reads fall on different bank windows.  The tiles go in
// chunks of TC = tgn * TT; every read of a chunk's rows precedes its writes,
// and chunks touch disjoint rows, so the update is in place.
// ---------------------------------------------------------------------------
constexpr int kPB = 8;
constexpr int kJC = 10;
constexpr int kMS = kJC * kPB + 4;
constexpr int kTI = 5, kTT = 5;
constexpr int kApplyMaxThreads = 640;

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
    c.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x));
    c.y = fmaf(a.x, b.y, fmaf(a.y, b.x, c.y));
    return c;
}

template <bool V16>
__global__ void __launch_bounds__(kApplyMaxThreads, 1)
k_zop_apply(float2 *__restrict__ S, const float2 *__restrict__ M, int Z, long long plane, int nt, int ign,
            int tgn) {
    extern __shared__ __align__(16) float2 sm[];
    const int rowsM = ign * kTI, TC = tgn * kTT;
    const int stage = (rowsM + TC) * kMS;
    const int tid = threadIdx.x;
    const int p = tid & (kPB - 1);
    const int rest = tid >> 3;
    const int ig = rest % ign, tg = rest / ign;
    const long long p0 = (long long)blockIdx.x * kPB;
    const int nch = (Z + kJC - 1) / kJC;
    const int nM = Z * kJC * (kPB / 2);  // 16-byte units of a chunk's M rows
    const int nU = nM + TC * kJC * (kPB / 2);

    for (int tc0 = 0; tc0 < nt; tc0 += TC) {
        auto load = [&](int c, int buf) {
            float2 *Ms = sm + buf * stage, *Xs = Ms + rowsM * kMS;
            const int j0 = c * kJC;
            for (int u = tid; u < nU; u += blockDim.x) {
                const bool isM = u < nM;
                const int v = isM ? u : u - nM;
                const int pp = (v & (kPB / 2 - 1)) * 2;
                const int r = v / (kPB / 2);
                const int jj = r % kJC, row = r / kJC;
                const int j = j0 + jj;
                float2 *dst = (isM ? Ms : Xs) + row * kMS + jj * kPB + pp;
                const long long pg = p0 + pp;
                const bool ok = j < Z && (isM || tc0 + row < nt);
                const float2 *src = isM ? M + ((long long)row * Z + j) * plane + pg
                                        : S + ((long long)(tc0 + row) * Z + j) * plane + pg;
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

        float2 acc[kTI][kTT];
#pragma unroll
        for (int a = 0; a < kTI; ++a)
#pragma unroll
            for (int b = 0; b < kTT; ++b) acc[a][b] = make_float2(0.f, 0.f);

        load(0, 0);
        for (int c = 0; c < nch; ++c) {
            if (c + 1 < nch) {
                load(c + 1, (c + 1) & 1);
                cp_async_wait_group<1>();
            } else {
                cp_async_wait_group<0>();
            }
            __syncthreads();
            const float2 *Ms = sm + (c & 1) * stage, *Xs = Ms + rowsM * kMS;
            const float2 *mr = Ms + (ig * kTI) * kMS + p;
            const float2 *xr = Xs + (tg * kTT) * kMS + p;
#pragma unroll
            for (int jj = 0; jj < kJC; ++jj) {
                float2 m[kTI], x[kTT];
#pragma unroll
                for (int a = 0; a < kTI; ++a) m[a] = mr[a * kMS + jj * kPB];
#pragma unroll
                for (int b = 0; b < kTT; ++b) x[b] = xr[b * kMS + jj * kPB];
#pragma unroll
                for (int a = 0; a < kTI; ++a)
#pragma unroll
                    for (int b = 0; b < kTT; ++b) acc[a][b] = cfma(m[a], x[b], acc[a][b]);
            }
            __syncthreads();
        }
        if (p0 + p < plane) {
#pragma unroll
            for (int a = 0; a < kTI; ++a) {
                const int i = ig * kTI + a;
                if (i >= Z) break;
#pragma unroll
                for (int b = 0; b < kTT; ++b) {
                    const int t = tc0 + tg * kTT + b;
                    if (t < nt) S[((long long)t * Z + i) * plane + p0 + p] = acc[a][b];
                }
            }
        }
    }
}

}  // namespace

size_t mm_zop_coef_bytes(int Z, int Zp) { return sizeof(float2) * (size_t)Z * Z * Zp; }

int mm_zop_build_impl(const float2 *W, int Z, int zpad, int Zp, long long plane, float2 *E, float2 *M,
                      cudaStream_t st) {
    MM_REQUIRE(Z >= 1 && Z <= MM_ZOP_MAX_Z, "z operator needs 1 <= Z <= %d (got %d)", MM_ZOP_MAX_Z, Z);
    MM_REQUIRE(Zp <= MM_ZOP_MAX_ZP, "z operator needs Zp <= %d (got %d)", MM_ZOP_MAX_ZP, Zp);
    const long long ne = (long long)Z * Z * Zp;
    k_zop_coef<<<(unsigned)((ne + 255) / 256), 256, 0, st>>>(E, Z, zpad, Zp);
    MM_CHECK_LAUNCH();
    const size_t sm = sizeof(float2) * (size_t)Zp * kBuildP;
    MM_CUDA_TRY(cudaFuncSetAttribute(k_zop_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_zop_build<<<(unsigned)((plane + kBuildP - 1) / kBuildP), kBuildThreads, sm, st>>>(W, E, M, Z, Zp, plane);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_zop_apply(float2 *S, const float2 *M, int Z, long long plane, int nt, cudaStream_t st) {
    MM_REQUIRE(Z >= 1 && Z <= MM_ZOP_MAX_Z, "z operator needs 1 <= Z <= %d (got %d)", MM_ZOP_MAX_Z, Z);
    if (nt <= 0) return MM_OK;
    int ign = (Z + kTI - 1) / kTI;
    const int tmax = kApplyMaxThreads / (kPB * ign);
    int tgn = (nt + kTT - 1) / kTT;
    if (tgn > tmax) tgn = tmax;
    const int threads = kPB * ign * tgn;
    const size_t sm = sizeof(float2) * 2 * (size_t)(ign * kTI + tgn * kTT) * kMS;
    const void *fn = (plane % 2 == 0) ? (const void *)k_zop_apply<true> : (const void *)k_zop_apply<false>;
    MM_CUDA_TRY(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    dim3 grid((unsigned)((plane + kPB - 1) / kPB));
    void *args[] = {&S, &M, &Z, &plane, &nt, &ign, &tgn};
    MM_CUDA_TRY(cudaLaunchKernel(fn, grid, dim3(threads), args, sm, st));
    mm_launch_counter_add();
    return MM_OK;
}
