// x pass of the tiled deconvolution, and the engine's general strided
// transform: in-place complex FFT along a strided axis (forward or inverse).
#include "deconv.cuh"

namespace {
constexpr FftCfg kColsCfg = kFftPair;

// ---------------------------------------------------------------------------
// strided complex FFT, in place: line l of plane p starts at S + p*plane_stride + l,
// element e at + e*se.  Lines are contiguous, so a CTA's loads are runs of nl,
// staged into shared memory with cp.async.
// ---------------------------------------------------------------------------
// NF > 0: the engine specialised for length NF at NLF lines per CTA
template <bool INV, int LMAX, int NF = 0, int NLF = 0>
__global__ void __launch_bounds__(kColsCfg.threads, kColsCfg.ctas)
k_cols(float2 *__restrict__ S, long long se, int nlines, long long plane_stride, FftPlan P, int nl, int gx,
       int ngroups) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    if constexpr (NF > 0) nl = NLF;
    const int n = NF > 0 ? NF : P.n, lnl = NF > 0 ? ilog2c(NLF) : log2_pow2(nl);
    const FftSmem L = fft_smem_layout(smem_raw, P, nl);
    fft_load_tables(P, L.tw, L.tab);
    // persistent: the CTAs walk the groups of nl lines (tables loaded once)
    for (int grp = blockIdx.x; grp < ngroups; grp += gridDim.x) {
        const int by = grp / gx, bx = grp - by * gx;
        float2 *base = S + (long long)by * plane_stride;
        const int l0 = bx * nl;
        for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
            const int l = it & (nl - 1), e = it >> lnl;
            if (l0 + l < nlines)
                cp_async8(&L.A[sidx(e, l, nl)], &base[e * se + l0 + l]);
            else
                L.A[sidx(e, l, nl)] = make_float2(0.f, 0.f);
        }
        cp_async_wait_all();
        __syncthreads();
        float2 *R = fft_run<INV, LMAX, NF, NLF>(L.A, L.B, nl, P, L.tw, L.tab, L.scr);
        for (int it = threadIdx.x; it < nl * n; it += blockDim.x) {
            const int l = it & (nl - 1), e = it >> lnl;
            if (l0 + l < nlines) base[e * se + l0 + l] = R[sidx(e, l, nl)];
        }
        __syncthreads();  // the next group's loads overwrite the line buffers
    }
}

}  // namespace

int mm_launch_cols(float2 *S, int n, long long se, int nlines, long long plane_stride, int nplanes, bool inv,
                   cudaStream_t st) {
    FftPlan P;
    int rc = mm_fft_plan_get(n, &P);
    if (rc) return rc;
    int nl = pick_nl(P, 16, kColsCfg);
    size_t sm = fft_smem(P, nl, kColsCfg);
    int gx = mm_cdiv(nlines, nl);
    int ngroups = gx * nplanes;
    // persistent: kColsCfg.ctas CTAs per SM (their line buffers fill its shared memory)
    dim3 grid(fft_grid(ngroups, kColsCfg));
    void *args[] = {&S, &se, &nlines, &plane_stride, &P, &nl, &gx, &ngroups};
    const void *fn = inv ? MM_FFT_KERNEL(P, nl, 8, k_cols, true,) : MM_FFT_KERNEL(P, nl, 8, k_cols, false,);
    return launch_fft_kernel(fn, grid, sm, st, args, kColsCfg.threads);
}

