// Batched mixed-radix Stockham FFT on lines held in shared memory.
//
// The deconvolution needs transforms at the exact padded tile lengths of the
// reference (deconvolver.py:86-90, 155-157), which carry large prime factors
// (678 = 2*3*113, 478 = 2*239, 148 = 4*37, 118 = 2*59, ...).  A length is
// factored into radix-2/3/4/5/7 stages, computed in registers, and "generic"
// odd-prime stages, computed as a direct DFT that pairs x[r] with x[R-r] (half
// the multiplies of a plain DFT).  The generic stages run first, where the
// Stockham twiddles are all 1.
//
// Layout: a CTA holds `nl` lines; element e of line l is at s[e*ld + l]
// ("column" layout, ld = nl + 1 to break bank conflicts on row loads).  Each
// stage reads one buffer and writes the other (ping-pong), so a kernel gives
// two buffers of n*ld float2 each.  Twiddles exp(-2*pi*i*m/n) are computed on
// the host in double precision and rounded once to float.
#pragma once
#include "mm_common.cuh"

#define MM_FFT_MAXST 16
#define MM_FFT_MAXN 4096

struct FftPlan {
    int n;
    int nst;
    int rad[MM_FFT_MAXST];
    int ns[MM_FFT_MAXST];     // product of the radices of the earlier stages
    int ptab[MM_FFT_MAXST];   // generic stage: offset of its cos/sin table in `tab`
    int ntab;                 // float2 entries in `tab`
    const float2 *tw;         // device, n entries: exp(-2 pi i m / n)
    const float2 *tab;        // device, per generic stage R entries: exp(-2 pi i m / R)
};

// ---- small radices, all values in registers ------------------------------
template <bool INV>
__device__ __forceinline__ float2 mul_i(float2 a) {
    // forward transforms use exp(-i...), so "-i*a"; the inverse uses "+i*a"
    return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

template <int R, bool INV>
__device__ __forceinline__ void dft_small(float2 *v);

template <>
__device__ __forceinline__ void dft_small<2, false>(float2 *v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
}
template <>
__device__ __forceinline__ void dft_small<2, true>(float2 *v) { dft_small<2, false>(v); }

template <bool INV>
__device__ __forceinline__ void dft4(float2 *v) {
    float2 s02 = cadd(v[0], v[2]), d02 = csub(v[0], v[2]);
    float2 s13 = cadd(v[1], v[3]), d13 = mul_i<INV>(csub(v[1], v[3]));
    v[0] = cadd(s02, s13);
    v[2] = csub(s02, s13);
    v[1] = cadd(d02, d13);
    v[3] = csub(d02, d13);
}
template <>
__device__ __forceinline__ void dft_small<4, false>(float2 *v) { dft4<false>(v); }
template <>
__device__ __forceinline__ void dft_small<4, true>(float2 *v) { dft4<true>(v); }

// Odd radix R in registers: out[k] = x0 + sum_r a_r cos(2 pi r k/R) -/+ i b_r sin(...)
// with a_r = x_r + x_{R-r}, b_r = x_r - x_{R-r}.
template <int R>
struct OddTab;
template <>
struct OddTab<3> {
    __device__ static float c(int m) { return m == 0 ? 1.0f : -0.5f; }
    __device__ static float s(int m) { return m == 0 ? 0.0f : 0.86602540378443864676f; }
};
template <>
struct OddTab<5> {
    __device__ static float c(int m) {
        return m == 0 ? 1.0f : (m == 1 ? 0.30901699437494742410f : -0.80901699437494742410f);
    }
    __device__ static float s(int m) {
        return m == 0 ? 0.0f : (m == 1 ? 0.95105651629515357212f : 0.58778525229247312917f);
    }
};
template <>
struct OddTab<7> {
    __device__ static float c(int m) {
        return m == 0 ? 1.0f
                      : (m == 1 ? 0.62348980185873353053f
                                : (m == 2 ? -0.22252093395631440429f : -0.90096886790241912624f));
    }
    __device__ static float s(int m) {
        return m == 0 ? 0.0f
                      : (m == 1 ? 0.78183148246802980871f
                                : (m == 2 ? 0.97492791218182360702f : 0.43388373911755812048f));
    }
};

template <int R, bool INV>
__device__ __forceinline__ void dft_odd(float2 *v) {
    constexpr int H = (R - 1) / 2;
    float2 a[H], b[H];
#pragma unroll
    for (int r = 1; r <= H; ++r) {
        a[r - 1] = cadd(v[r], v[R - r]);
        b[r - 1] = csub(v[r], v[R - r]);
    }
    float2 x0 = v[0];
    float2 s0 = x0;
#pragma unroll
    for (int r = 0; r < H; ++r) s0 = cadd(s0, a[r]);
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        float ax = x0.x, ay = x0.y, bx = 0.f, by = 0.f;
#pragma unroll
        for (int r = 1; r <= H; ++r) {
            int m = (r * k) % R;
            float c = m <= H ? OddTab<R>::c(m) : OddTab<R>::c(R - m);
            float s = m <= H ? OddTab<R>::s(m) : -OddTab<R>::s(R - m);
            ax += a[r - 1].x * c;
            ay += a[r - 1].y * c;
            bx += b[r - 1].x * s;
            by += b[r - 1].y * s;
        }
        // forward: out[k] = A - i B  -> (ax + by, ay - bx); out[R-k] = A + i B
        if (!INV) {
            v[k] = make_float2(ax + by, ay - bx);
            v[R - k] = make_float2(ax - by, ay + bx);
        } else {
            v[k] = make_float2(ax - by, ay + bx);
            v[R - k] = make_float2(ax + by, ay - bx);
        }
    }
    v[0] = s0;
}
template <>
__device__ __forceinline__ void dft_small<3, false>(float2 *v) { dft_odd<3, false>(v); }
template <>
__device__ __forceinline__ void dft_small<3, true>(float2 *v) { dft_odd<3, true>(v); }
template <>
__device__ __forceinline__ void dft_small<5, false>(float2 *v) { dft_odd<5, false>(v); }
template <>
__device__ __forceinline__ void dft_small<5, true>(float2 *v) { dft_odd<5, true>(v); }
template <>
__device__ __forceinline__ void dft_small<7, false>(float2 *v) { dft_odd<7, false>(v); }
template <>
__device__ __forceinline__ void dft_small<7, true>(float2 *v) { dft_odd<7, true>(v); }

template <int R, bool INV>
__device__ __forceinline__ void stage_small(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                            int n, int ld, int nl, int Ns, const float2 *tw) {
    const int m = n / R;
    const int tstep = n / (Ns * R);
    const int items = m * nl;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        int l = it % nl;
        int j = it / nl;
        int k = j % Ns;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[(j + r * m) * ld + l];
        if (Ns > 1) {
#pragma unroll
            for (int r = 1; r < R; ++r) {
                float2 w = tw[k * r * tstep];
                v[r] = INV ? cmulc(v[r], w) : cmul(v[r], w);
            }
        }
        dft_small<R, INV>(v);
        int d = (j - k) * R + k;
#pragma unroll
        for (int r = 0; r < R; ++r) dst[(d + r * Ns) * ld + l] = v[r];
    }
}

// Generic odd radix R (a prime >= 11): direct symmetric DFT.  Phase 1 applies
// the Stockham twiddles in place; phase 2 has one work item per (line,
// butterfly, output pair k / R-k) and loops over the R inputs.
template <bool INV>
__device__ void stage_generic(float2 *__restrict__ src, float2 *__restrict__ dst, int n, int ld,
                              int nl, int R, int Ns, const float2 *tw, const float2 *cs) {
    const int m = n / R;
    const int tstep = n / (Ns * R);
    if (Ns > 1) {
        for (int it = threadIdx.x; it < n * nl; it += blockDim.x) {
            int l = it % nl;
            int e = it / nl;
            int j = e % m, r = e / m;
            if (r == 0) continue;
            float2 w = tw[(j % Ns) * r * tstep];
            float2 x = src[e * ld + l];
            src[e * ld + l] = INV ? cmulc(x, w) : cmul(x, w);
        }
        __syncthreads();
    }
    const int H = (R - 1) / 2;
    const int items = m * nl * (H + 1);
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        int l = it % nl;
        int rest = it / nl;
        int k = rest % (H + 1);
        int j = rest / (H + 1);
        int kk = j % Ns;
        int d = (j - kk) * R + kk;
        const float2 *x = src + j * ld + l;
        const int xs = m * ld;
        float2 x0 = x[0];
        if (k == 0) {
            float sx = x0.x, sy = x0.y;
            for (int r = 1; r < R; ++r) {
                float2 t = x[r * xs];
                sx += t.x;
                sy += t.y;
            }
            dst[d * ld + l] = make_float2(sx, sy);
            continue;
        }
        float ax = x0.x, ay = x0.y, bx = 0.f, by = 0.f;
        int mi = 0;
        for (int r = 1; r <= H; ++r) {
            mi += k;
            if (mi >= R) mi -= R;
            float2 w = cs[mi];  // (cos, -sin) of 2 pi mi / R
            float2 u = x[r * xs], v = x[(R - r) * xs];
            ax += (u.x + v.x) * w.x;
            ay += (u.y + v.y) * w.x;
            bx += (u.x - v.x) * w.y;
            by += (u.y - v.y) * w.y;
        }
        // w.y = -sin: forward out[k] = A - iB with B = sum b sin  ->  (ax - by', ay + bx')
        float2 o1, o2;
        if (!INV) {
            o1 = make_float2(ax - by, ay + bx);
            o2 = make_float2(ax + by, ay - bx);
        } else {
            o1 = make_float2(ax + by, ay - bx);
            o2 = make_float2(ax - by, ay + bx);
        }
        dst[(d + k * Ns) * ld + l] = o1;
        dst[(d + (R - k) * Ns) * ld + l] = o2;
    }
}

// Runs the whole plan on nl lines.  Returns the buffer holding the result.
template <bool INV>
__device__ float2 *fft_lines(float2 *A, float2 *B, int ld, int nl, const FftPlan &P,
                             const float2 *tw_s, const float2 *tab_s) {
    float2 *src = A, *dst = B;
    for (int st = 0; st < P.nst; ++st) {
        const int R = P.rad[st], Ns = P.ns[st];
        switch (R) {
            case 2: stage_small<2, INV>(src, dst, P.n, ld, nl, Ns, tw_s); break;
            case 3: stage_small<3, INV>(src, dst, P.n, ld, nl, Ns, tw_s); break;
            case 4: stage_small<4, INV>(src, dst, P.n, ld, nl, Ns, tw_s); break;
            case 5: stage_small<5, INV>(src, dst, P.n, ld, nl, Ns, tw_s); break;
            case 7: stage_small<7, INV>(src, dst, P.n, ld, nl, Ns, tw_s); break;
            default: stage_generic<INV>(src, dst, P.n, ld, nl, R, Ns, tw_s, tab_s + P.ptab[st]); break;
        }
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    return src;
}

// Copies the plan tables into shared memory (call by all threads, then sync).
__device__ __forceinline__ void fft_load_tables(const FftPlan &P, float2 *tw_s, float2 *tab_s) {
    for (int i = threadIdx.x; i < P.n; i += blockDim.x) tw_s[i] = P.tw[i];
    for (int i = threadIdx.x; i < P.ntab; i += blockDim.x) tab_s[i] = P.tab[i];
}

// Host side: plan cache (fft_plan.cu).
int mm_fft_plan_get(int n, FftPlan *out);
