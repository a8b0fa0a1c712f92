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
// already scaled by 1 / (Zp * P * P).  One CTA owns nl plane positions for
// every tile of the batch: with a single spectrum its chunk of W is staged in
// shared memory once and reused by all tiles.
// ---------------------------------------------------------------------------
template <int LMAX>
__global__ void __launch_bounds__(kThreads, 2)
k_zpass(TileGeom g, float2 *__restrict__ S, const float2 *__restrict__ W, long long wstride, FftPlan P, int nl) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int n = P.n, lnl = log2_pow2(nl);
    const FftSmem L = fft_smem_layout(smem_raw, P, nl);
    float2 *Ws = reinterpret_cast<float2 *>(reinterpret_cast<unsigned char *>(L.scr) +
                                            sizeof(float4) * MM_FFT_SCR_PER_WARP * (kThreads / 32));
    int *zmap = reinterpret_cast<int *>(Ws + (size_t)n * nl);
    fft_load_tables(P, L.tw, L.tab);
    for (int e = threadIdx.x; e < n; e += blockDim.x) zmap[e] = mm_map_z(e, g.Z, g.zpad, g.Zp);
    __syncthreads();
    const long long plane = (long long)g.P * g.H;
    const long long q0 = (long long)blockIdx.x * nl;
    int wloaded = -1;
    for (int tb = 0; tb < g.nt; ++tb) {
        const int ti = g.t0 + tb;
        const TileDesc d = mm_tile_desc(g, ti);
        float2 *St = S + (long long)tb * g.Z * plane;
        if (d.psf != wloaded) {
            const float2 *Wt = W + (long long)d.psf * wstride;
            for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
                const int l = it & (nl - 1), e = it >> lnl;
                if (q0 + l < plane)
                    cp_async8(&Ws[sidx(e, l, nl)], &Wt[e * plane + q0 + l]);
                else
                    Ws[sidx(e, l, nl)] = make_float2(0.f, 0.f);
            }
            wloaded = d.psf;
        }
        for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
            const int l = it & (nl - 1), e = it >> lnl;
            const int src = zmap[e];
            if (src >= 0 && q0 + l < plane)
                cp_async8(&L.A[sidx(e, l, nl)], &St[src * plane + q0 + l]);
            else
                L.A[sidx(e, l, nl)] = make_float2(0.f, 0.f);
        }
        cp_async_wait_all();
        __syncthreads();
        float2 *R = fft_lines<false, LMAX>(L.A, L.B, nl, P, L.tw, L.tab, L.scr);
        float2 *O = (R == L.A) ? L.B : L.A;
        for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
            const int l = it & (nl - 1), e = it >> lnl;
            O[sidx(e, l, nl)] = cmul(R[sidx(e, l, nl)], Ws[sidx(e, l, nl)]);
        }
        __syncthreads();
        float2 *R2 = fft_lines<true, LMAX>(O, R, nl, P, L.tw, L.tab, L.scr);
        for (int it = threadIdx.x; it < nl * g.Z; it += blockDim.x) {
            const int l = it & (nl - 1), z = it >> lnl;
            if (q0 + l < plane) St[z * plane + q0 + l] = R2[sidx(g.zpad + z, l, nl)];
        }
        __syncthreads();
    }
}

// z pass, forward only, all planes (the PSF transform)
template <int LMAX>
__global__ void __launch_bounds__(kThreads, 2)
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
    // room for the staged Wiener chunk (one more n*nl buffer) and the z map
    int nl = 16;
    auto bytes = [&](int l) { return fft_smem(P, l) + sizeof(float2) * (size_t)P.n * l + sizeof(int) * P.n; };
    while (nl > 1 && bytes(nl) > (size_t)kSmemLimit) nl >>= 1;
    size_t sm = bytes(nl);
    dim3 grid(mm_cdiv((long)g.P * g.H, nl));
    TileGeom ga = g;
    void *args[] = {&ga, &S, &W, &wstride, &P, &nl};
    return launch_fft_kernel(MM_BY_CLASS(P, k_zpass, ), grid, sm, st, args);
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

