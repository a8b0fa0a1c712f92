// z pass of the tiled deconvolution (deconvolver.py:155-157): gather the mapped
// planes, FFT over the padded depth, multiply by the pre-scaled Wiener spectrum,
// inverse FFT, keep the planes [zpad, zpad+Z); and the forward-only z pass of
// the PSF transform.
#include "deconv.cuh"

namespace {
constexpr int kThreads = kFftThreads;
constexpr int kSmemLimit = kFftSmemLimit;

// ---------------------------------------------------------------------------
// z pass of the deconvolution: forward FFT over the padded depth, Wiener
// multiply, inverse FFT, keep the real planes.  W is (Zp, P, H) per spectrum,
// already scaled by 1 / (Zp * P * P).  A CTA holds nl = NQ * TG lines: NQ
// consecutive plane positions of TG tiles at a time (line l = tile-in-group
// (l / NQ) and position (l % NQ)), so that every thread has a butterfly in the
// radix stages and the tiles of a group read the same Wiener values (through
// L1) when they share a spectrum.  The CTA walks the batch group by group.
// ---------------------------------------------------------------------------
constexpr int kZThreads = 256;
constexpr int kZq = 16;  // plane positions per CTA

template <int LMAX>
__global__ void __launch_bounds__(kZThreads, 1)
k_zpass(TileGeom g, float2 *__restrict__ S, const float2 *__restrict__ W, long long wstride, FftPlan P, int nl,
        int tg) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = P.n, lnl = log2_pow2(nl);
    const int lnq = log2_pow2(kZq);
    const FftSmem L = fft_smem_layout(smem_raw, P, nl);
    // the Wiener chunk of the CTA's kZq positions (Zp x kZq), then the z map
    float2 *Ws = reinterpret_cast<float2 *>(L.scr + fft_scr_f4(P, nl, kZThreads / 32));
    int *zmap = reinterpret_cast<int *>(Ws + (size_t)n * kZq);
    fft_load_tables(P, L.tw, L.tab);
    for (int e = threadIdx.x; e < n; e += blockDim.x) zmap[e] = mm_map_z(e, g.Z, g.zpad, g.Zp);
    __syncthreads();
    const long long plane = (long long)g.P * g.H;
    const long long q0 = (long long)blockIdx.x * kZq;
    int wpsf = -1;
    for (int t0 = 0; t0 < g.nt; t0 += tg) {
        // with several spectra a group is one tile (tg == 1); with one spectrum
        // the chunk is staged once and reused by every group
        const int psf = g.npsf == 1 ? 0 : g.t0 + t0;
        if (psf != wpsf) {
            for (int it = threadIdx.x; it < kZq * n; it += blockDim.x) {
                const int qo = it & (kZq - 1), e = it >> lnq;
                if (q0 + qo < plane)
                    cp_async8(&Ws[e * kZq + qo], &W[(long long)psf * wstride + e * plane + q0 + qo]);
                else
                    Ws[e * kZq + qo] = make_float2(0.f, 0.f);
            }
            wpsf = psf;
        }
        for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
            const int l = it & (nl - 1), e = it >> lnl;
            const int t = t0 + (l >> lnq);
            const long long q = q0 + (l & (kZq - 1));
            const int src = zmap[e];
            if (src >= 0 && t < g.nt && q < plane)
                cp_async8(&L.A[sidx(e, l, nl)], &S[((long long)t * g.Z + src) * plane + q]);
            else
                L.A[sidx(e, l, nl)] = make_float2(0.f, 0.f);
        }
        cp_async_wait_all();
        __syncthreads();
        float2 *R = fft_lines<false, LMAX>(L.A, L.B, nl, P, L.tw, L.tab, L.scr);
        for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
            const int l = it & (nl - 1), e = it >> lnl;
            R[sidx(e, l, nl)] = cmul(R[sidx(e, l, nl)], Ws[e * kZq + (l & (kZq - 1))]);
        }
        __syncthreads();
        float2 *R2 = fft_lines<true, LMAX>(R, R == L.A ? L.B : L.A, nl, P, L.tw, L.tab, L.scr);
        for (int it = threadIdx.x; it < nl * g.Z; it += blockDim.x) {
            const int l = it & (nl - 1), z = it >> lnl;
            const int t = t0 + (l >> lnq);
            const long long q = q0 + (l & (kZq - 1));
            if (t < g.nt && q < plane) S[((long long)t * g.Z + z) * plane + q] = R2[sidx(g.zpad + z, l, nl)];
        }
        __syncthreads();
    }
}

// z pass, forward only, all planes (the PSF transform)
template <int LMAX>
__global__ void __launch_bounds__(kThreads, 1)
k_zfwd(float2 *__restrict__ S, long long plane, FftPlan P, int nl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = P.n, lnl = log2_pow2(nl);
    const FftSmem L = fft_smem_layout(smem_raw, P, nl);
    fft_load_tables(P, L.tw, L.tab);
    const long long q0 = (long long)blockIdx.x * nl;
    for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
        const int l = it & (nl - 1), e = it >> lnl;
        if (q0 + l < plane)
            cp_async8(&L.A[sidx(e, l, nl)], &S[e * plane + q0 + l]);
        else
            L.A[sidx(e, l, nl)] = make_float2(0.f, 0.f);
    }
    cp_async_wait_all();
    __syncthreads();
    float2 *R = fft_lines<false, LMAX>(L.A, L.B, nl, P, L.tw, L.tab, L.scr);
    for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
        const int l = it & (nl - 1), e = it >> lnl;
        if (q0 + l < plane) S[e * plane + q0 + l] = R[sidx(e, l, nl)];
    }
}

}  // namespace

int mm_launch_zpass(const TileGeom &g, float2 *S, const float2 *W, long long wstride, cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(g.Zp, &P);
    if (rc) return rc;
    // lines per CTA: kZq positions of tg tiles (tg up to 4, one tile when each
    // tile has its own spectrum), fewer positions' worth of tiles if too large
    auto bytes = [&](int l) {
        return fft_smem_bytes(P, l, kZThreads / 32) + sizeof(float2) * (size_t)P.n * kZq +
               sizeof(int) * (size_t)P.n;
    };
    int tg = 1;
    if (g.npsf == 1)
        while (tg < 4 && tg * 2 <= g.nt && bytes(kZq * tg * 2) <= (size_t)kSmemLimit) tg *= 2;
    int nl = kZq * tg;
    MM_REQUIRE(bytes(nl) <= (size_t)kSmemLimit, "padded depth %d too large for the z pass", g.Zp);
    size_t sm = bytes(nl);
    dim3 grid(mm_cdiv((long)g.P * g.H, kZq));
    TileGeom ga = g;
    void *args[] = {&ga, &S, &W, &wstride, &P, &nl, &tg};
    const void *fn = MM_BY_CLASS(P, k_zpass, );
    if ((rc = mm_set_smem(fn, sm))) return rc;
    MM_CUDA_TRY(cudaLaunchKernel(fn, grid, dim3(kZThreads), args, sm, st));
    mm_launch_counter_add();
    return MM_OK;
}

int mm_launch_zfwd(float2 *S, int Zp, int plane, cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(Zp, &P);
    if (rc) return rc;
    int nl = pick_nl(P, 16);
    size_t sm = fft_smem(P, nl);
    long long pl = plane;
    void *args[] = {&S, &pl, &P, &nl};
    return launch_fft_kernel(MM_BY_CLASS(P, k_zfwd, ), dim3(mm_cdiv(plane, nl)), sm, st, args);
}

