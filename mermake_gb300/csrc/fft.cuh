// Batched mixed-radix Stockham FFT on lines held in shared memory.
//
// The deconvolution needs transforms at the exact padded tile lengths of the
// reference (deconvolver.py:86-90, 155-157), which carry large prime factors
// (678 = 2*3*113, 478 = 2*239, 148 = 4*37, 118 = 2*59, ...).  A length is
// factored into stages of four kinds:
//   * radix 2/3/4/5/6/7 and the odd primes 11..37: one thread per butterfly,
//     values in registers;
//   * 113 (678 = 6*113) and 239 (478 = 2*239): Rader's algorithm, the prime
//     DFT as a cyclic convolution of length 112 = 16*7 or 238 = 14*17 done
//     with small register DFTs (stage_rader);
//   * primes 41..61, 79 and 89 ("lane" stage; 59, 79 and 89 are the primes of
//     the reference's padded depths such as 118 = 2*59): one warp per
//     butterfly and one lane per output pair (k, R-k); each lane keeps its
//     column of the DFT matrix in registers for the whole stage, and the warp
//     reads the paired inputs a_r = x_r + x_{R-r}, b_r = x_r - x_{R-r} as
//     shared-memory broadcasts (one 16-byte load per 4 FMAs);
//   * any other prime: a direct DFT with table look-ups ("generic" stage).
// The lane and generic stages pair x[r] with x[R-r], halving the multiplies of a
// plain DFT.  The large-prime stages run first, where the Stockham twiddles are
// all 1.
//
// Layout: a CTA holds `nl` lines (a power of two); element e of line l is at
// s[sidx(e, l, nl)] = s[e*nl + (l ^ (e & (nl-1)))]: lines are interleaved
// ("column" layout, so a half warp reads one element of 16 lines as 128
// contiguous bytes), and the XOR swizzle spreads the strided accesses of the
// row loads and of the lane stages over the banks.  Each stage reads one buffer
// and writes the other (ping-pong), so a kernel gives two buffers of n*nl
// float2 each.  Twiddles exp(-2*pi*i*m/n) are computed on
// the host in double precision and rounded once to float.
#pragma once
#include "mm_common.cuh"

#define MM_FFT_MAXST 16
#define MM_FFT_MAXN 4096

struct FftPlan {
    int n;
    int nst;
    int lclass;               // 0, 63 or 127: largest lane-stage prime class (fft_lines<., LMAX>)
    int rad[MM_FFT_MAXST];
    int ns[MM_FFT_MAXST];     // product of the radices of the earlier stages
    int ptab[MM_FFT_MAXST];   // generic stage: offset of its cos/sin table in `tab`
    int ntab;                 // float2 entries in `tab`
    const float2 *tw;         // device, n entries: exp(-2 pi i m / n)
    const float2 *tab;        // device, per generic stage R entries: exp(-2 pi i m / R)
};

// element e of line l in a CTA's line buffer (see the layout note above)
__device__ __forceinline__ int sidx(int e, int l, int nl) { return e * nl + (l ^ (e & (nl - 1))); }

// a / d for 0 <= a < 2^24 through the float reciprocal inv = 1/d, corrected to
// the exact quotient (integer division by a run-time divisor costs ~20
// instructions; this is 6)
__device__ __forceinline__ int fdiv_i(int a, int d, float inv) {
    int q = __float2int_rz(__int2float_rn(a) * inv);
    const int r = a - q * d;
    q += (r >= d) - (r < 0);
    return q;
}
__device__ __forceinline__ int log2_pow2(int nl) { return __ffs(nl) - 1; }
constexpr int ilog2c(int v) { return v <= 1 ? 0 : 1 + ilog2c(v / 2); }

// a / d for 0 <= a: by the constant C when the caller knows d at compile time
// (C > 0: a multiply and a shift), else through the reciprocal (fdiv_i)
template <int C>
__device__ __forceinline__ int divc(int a, int d, float inv) {
    if constexpr (C > 0)
        return (int)((unsigned)a / (unsigned)C);
    else
        return fdiv_i(a, d, inv);
}

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

// radix 6 = 2 x 3: X[k] = E[k mod 3] + w6^k O[k mod 3], E/O the 3-point DFTs of
// the even/odd samples (one pass instead of a radix-2 and a radix-3 stage)
template <bool INV>
__device__ __forceinline__ void dft6(float2 *v) {
    float2 e[3] = {v[0], v[2], v[4]}, o[3] = {v[1], v[3], v[5]};
    dft_odd<3, INV>(e);
    dft_odd<3, INV>(o);
    const float h = 0.5f, r = 0.86602540378443864676f;
    // w6 = (1/2, -+sqrt3/2), w6^2 = (-1/2, -+sqrt3/2)
    const float2 w1 = make_float2(h, INV ? r : -r), w2 = make_float2(-h, INV ? r : -r);
    const float2 o1 = cmul(o[1], w1), o2 = cmul(o[2], w2);
    v[0] = cadd(e[0], o[0]);
    v[3] = csub(e[0], o[0]);
    v[1] = cadd(e[1], o1);
    v[4] = csub(e[1], o1);
    v[2] = cadd(e[2], o2);
    v[5] = csub(e[2], o2);
}
template <>
__device__ __forceinline__ void dft_small<6, false>(float2 *v) { dft6<false>(v); }
template <>
__device__ __forceinline__ void dft_small<6, true>(float2 *v) { dft6<true>(v); }

// Odd radix 11..37 with one thread per butterfly: the paired inputs
// a_r = x_r + x_{R-r}, b_r = x_r - x_{R-r} and the stage's cos/sin values
// (loaded once per stage from the plan table) sit in registers; each output
// pair (k, R-k) is accumulated and written to shared memory at once, so no
// output array is held.
template <int R, bool INV>
__device__ __noinline__ void stage_odd_tab(const float2 *__restrict__ src, float2 *__restrict__ dst, int n,
                                           int nl, int Ns, const float2 *tw, const float2 *cs) {
    constexpr int H = (R - 1) / 2;
    float c[H], sn[H];
#pragma unroll
    for (int m = 1; m <= H; ++m) {
        c[m - 1] = cs[m].x;
        sn[m - 1] = -cs[m].y;  // table holds (cos, -sin)
    }
    const int m = n / R;
    const int tstep = n / (Ns * R);
    const int items = m * nl;
    const int lnl = log2_pow2(nl);
    const float invNs = 1.0f / (float)Ns;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int l = it & (nl - 1);
        const int j = it >> lnl;
        const int k = j - fdiv_i(j, Ns, invNs) * Ns;
        const float2 x0 = src[sidx(j, l, nl)];
        float2 a[H], b[H];
        float2 s0 = x0;
#pragma unroll
        for (int r = 1; r <= H; ++r) {
            float2 u = src[sidx(j + r * m, l, nl)], v = src[sidx(j + (R - r) * m, l, nl)];
            if (Ns > 1) {
                const float2 wu = tw[k * r * tstep], wv = tw[k * (R - r) * tstep];
                u = INV ? cmulc(u, wu) : cmul(u, wu);
                v = INV ? cmulc(v, wv) : cmul(v, wv);
            }
            a[r - 1] = cadd(u, v);
            b[r - 1] = csub(u, v);
            s0 = cadd(s0, a[r - 1]);
        }
        const int d = (j - k) * R + k;
        dst[sidx(d, l, nl)] = s0;
#pragma unroll
        for (int q = 1; q <= H; ++q) {
            float ax = x0.x, ay = x0.y, bx = 0.f, by = 0.f;
#pragma unroll
            for (int r = 1; r <= H; ++r) {
                const int mm = (r * q) % R;
                const float cc = mm <= H ? c[mm - 1] : c[R - mm - 1];
                const float ss = mm <= H ? sn[mm - 1] : -sn[R - mm - 1];
                ax += a[r - 1].x * cc;
                ay += a[r - 1].y * cc;
                bx += b[r - 1].x * ss;
                by += b[r - 1].y * ss;
            }
            float2 o1, o2;
            if (!INV) {
                o1 = make_float2(ax + by, ay - bx);
                o2 = make_float2(ax - by, ay + bx);
            } else {
                o1 = make_float2(ax - by, ay + bx);
                o2 = make_float2(ax + by, ay - bx);
            }
            dst[sidx(d + q * Ns, l, nl)] = o1;
            dst[sidx(d + (R - q) * Ns, l, nl)] = o2;
        }
    }
}

// Lane stage (primes 41..89, see top): warps per butterfly, lane per output
// pair.  For H = (R-1)/2 <= 32 one warp covers all pairs and keeps the whole
// DFT column (2H values) in registers.  For 32 < H <= 64 two k-groups of lanes
// are needed, and the r range is split in halves between two warps as well, so
// that each lane keeps at most 64 coefficients: four warps (2 k-groups x 2
// r-halves) form a stream, the r-half warps add their partial sums through
// shared memory between two named barriers.  Each stream takes two butterflies
// per iteration (eight independent FMA chains per warp).
// scr: MM_FFT_SCR_PER_WARP float4 of shared scratch per warp.
#define MM_FFT_SCR_PER_WARP 128
template <int R, bool INV>
__device__ __noinline__ void stage_lane(const float2 *__restrict__ src, float2 *__restrict__ dst, int n,
                                        int nl, int Ns, const float2 *__restrict__ tw,
                                        const float2 *__restrict__ cs, float4 *__restrict__ scr_all) {
    constexpr int H = (R - 1) / 2;
    constexpr int G = (H + 31) / 32;         // k-groups
    constexpr int RS = H > 32 ? 2 : 1;       // r-halves
    constexpr int HH = (H + RS - 1) / RS;    // r values per half
    constexpr int W = G * RS;                // warps per stream
    static_assert(HH <= 32 || RS == 1, "lane stage handles H <= 64");
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
    const int sub = warp % W, strm = warp / W, nstrm = nw / W;
    if (strm >= nstrm) return;
    const int g = sub / RS, h = sub % RS;
    const int r_lo = h * HH + 1;  // this warp's r range: [r_lo, r_lo + HH) within [1, H]
    float4 *scr = scr_all + warp * MM_FFT_SCR_PER_WARP;
    // exchange area: the r-half-1 warp of a k-group writes its partial sums into
    // its r-half-0 partner's scratch [64, 128)
    float4 *xch = scr_all + (strm * W + g * RS) * MM_FFT_SCR_PER_WARP + 64;
    const int k = g * 32 + lane + 1;
    const bool kv = k <= H;
    float cr[HH], sr[HH];
#pragma unroll
    for (int i = 0; i < HH; ++i) {
        const int r = r_lo + i;
        const float2 w = (kv && r <= H) ? cs[(r * k) % R] : make_float2(0.f, 0.f);  // (cos, -sin)
        cr[i] = w.x;
        sr[i] = w.y;
    }
    const int m = n / R;
    const int tstep = n / (Ns * R);
    const int nb = m * nl;
    const int lnl = log2_pow2(nl);
    const float invNs = 1.0f / (float)Ns;
    constexpr int SLOT = RS == 1 ? 64 : 32;  // a/b entries per butterfly in scr
    for (int b0 = strm; b0 < nb; b0 += 2 * nstrm) {
        const bool two = b0 + nstrm < nb;
        float2 x0[2];
        float sx[2], sy[2];
        int dd[2], ll[2];
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int bf = q ? (two ? b0 + nstrm : b0) : b0;
            const int l = bf & (nl - 1), j = bf >> lnl, kk = j - fdiv_i(j, Ns, invNs) * Ns;
            ll[q] = l;
            dd[q] = (j - kk) * R + kk;
            x0[q] = src[sidx(j, l, nl)];
            sx[q] = 0.f;
            sy[q] = 0.f;
            for (int i = lane; i < HH; i += 32) {
                const int r = r_lo + i;
                float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
                if (r <= H) {
                    float2 u = src[sidx(j + r * m, l, nl)], v = src[sidx(j + (R - r) * m, l, nl)];
                    if (Ns > 1) {
                        const float2 wu = tw[kk * r * tstep], wv = tw[kk * (R - r) * tstep];
                        u = INV ? cmulc(u, wu) : cmul(u, wu);
                        v = INV ? cmulc(v, wv) : cmul(v, wv);
                    }
                    t = make_float4(u.x + v.x, u.y + v.y, u.x - v.x, u.y - v.y);
                }
                scr[q * SLOT + i] = t;
                sx[q] += t.x;
                sy[q] += t.y;
            }
        }
        __syncwarp();
        float ax0 = 0.f, ay0 = 0.f, bx0 = 0.f, by0 = 0.f;
        float ax1 = 0.f, ay1 = 0.f, bx1 = 0.f, by1 = 0.f;
#pragma unroll
        for (int i = 0; i < HH; ++i) {
            const float4 t0 = scr[i], t1 = scr[SLOT + i];
            ax0 += t0.x * cr[i];
            ay0 += t0.y * cr[i];
            bx0 += t0.z * sr[i];
            by0 += t0.w * sr[i];
            ax1 += t1.x * cr[i];
            ay1 += t1.y * cr[i];
            bx1 += t1.z * sr[i];
            by1 += t1.w * sr[i];
        }
        // sums of a_r over this warp's r range (for X[0]), reduced in k-group 0
        if (g == 0) {
#pragma unroll
            for (int q = 0; q < 2; ++q)
                for (int o = 16; o > 0; o >>= 1) {
                    sx[q] += __shfl_xor_sync(0xffffffffu, sx[q], o);
                    sy[q] += __shfl_xor_sync(0xffffffffu, sy[q], o);
                }
        }
        if (RS == 2) {
            if (h == 1) {
                xch[lane] = make_float4(ax0, ay0, bx0, by0);
                xch[32 + lane] = make_float4(ax1, ay1, bx1, by1);
                if (g == 0 && lane == 0) {
                    // the two butterflies' sums go to this warp's own free scratch [64, 65)
                    *reinterpret_cast<float4 *>(scr + 64) = make_float4(sx[0], sy[0], sx[1], sy[1]);
                }
            }
            asm volatile("bar.sync %0, %1;" ::"r"(1 + strm), "r"(W * 32) : "memory");
            if (h == 0) {
                const float4 p0 = xch[lane], p1 = xch[32 + lane];
                ax0 += p0.x; ay0 += p0.y; bx0 += p0.z; by0 += p0.w;
                ax1 += p1.x; ay1 += p1.y; bx1 += p1.z; by1 += p1.w;
            }
        }
        if (h == 0) {
            float tx[2] = {sx[0], sx[1]}, ty[2] = {sy[0], sy[1]};
            if (RS == 2 && g == 0) {
                // sums of the partner r-half warp (warp g=0, h=1 of this stream)
                const float4 o = scr_all[(strm * W + 1) * MM_FFT_SCR_PER_WARP + 64];
                tx[0] += o.x; ty[0] += o.y;
                tx[1] += o.z; ty[1] += o.w;
            }
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                if (q == 1 && !two) break;
                const float ax = (q ? ax1 : ax0) + x0[q].x, ay = (q ? ay1 : ay0) + x0[q].y;
                const float bx = q ? bx1 : bx0, by = q ? by1 : by0;
                if (kv) {
                    float2 o1, o2;
                    if (!INV) {
                        o1 = make_float2(ax - by, ay + bx);
                        o2 = make_float2(ax + by, ay - bx);
                    } else {
                        o1 = make_float2(ax + by, ay - bx);
                        o2 = make_float2(ax - by, ay + bx);
                    }
                    dst[sidx(dd[q] + k * Ns, ll[q], nl)] = o1;
                    dst[sidx(dd[q] + (R - k) * Ns, ll[q], nl)] = o2;
                }
                if (g == 0 && lane == 0) dst[sidx(dd[q], ll[q], nl)] = make_float2(x0[q].x + tx[q], x0[q].y + ty[q]);
            }
        }
        if (RS == 2) asm volatile("bar.sync %0, %1;" ::"r"(1 + strm), "r"(W * 32) : "memory");
        __syncwarp();
    }
}

// 16-point DFT in registers (n = n1 + 4 n2, k = k1 + 4 k2: 4-point DFTs over
// n2, twiddles w16^(n1 k1), 4-point DFTs over n1), natural order in and out.
template <bool INV>
__device__ __forceinline__ void dft16(float2 *v) {
    const float c1 = 0.92387953251128675613f, s1 = 0.38268343236508977173f, r2 = 0.70710678118654752440f;
    // w16^e for e = 1, 2, 3, 4, 6, 9 (forward: exp(-2 pi i e / 16))
    const float sg = INV ? 1.f : -1.f;
    const float2 w1 = make_float2(c1, sg * s1), w2 = make_float2(r2, sg * r2), w3 = make_float2(s1, sg * c1);
    const float2 w6 = make_float2(-r2, sg * r2), w9 = make_float2(-c1, -sg * s1);
    float2 a[4][4];
#pragma unroll
    for (int n1 = 0; n1 < 4; ++n1) {
        float2 t[4] = {v[n1], v[n1 + 4], v[n1 + 8], v[n1 + 12]};
        dft4<INV>(t);
#pragma unroll
        for (int k1 = 0; k1 < 4; ++k1) a[n1][k1] = t[k1];
    }
    a[1][1] = cmul(a[1][1], w1);
    a[1][2] = cmul(a[1][2], w2);
    a[1][3] = cmul(a[1][3], w3);
    a[2][1] = cmul(a[2][1], w2);
    a[2][2] = mul_i<INV>(a[2][2]);  // w16^4 = -+i
    a[2][3] = cmul(a[2][3], w6);
    a[3][1] = cmul(a[3][1], w3);
    a[3][2] = cmul(a[3][2], w6);
    a[3][3] = cmul(a[3][3], w9);
#pragma unroll
    for (int k1 = 0; k1 < 4; ++k1) {
        float2 t[4] = {a[0][k1], a[1][k1], a[2][k1], a[3][k1]};
        dft4<INV>(t);
#pragma unroll
        for (int k2 = 0; k2 < 4; ++k2) v[k1 + 4 * k2] = t[k2];
    }
}

// radix 14 = 2 x 7: X[k] = E[k] + w14^k O[k], X[k+7] = E[k] - w14^k O[k]
// (k < 7), E/O the 7-point DFTs of the even/odd samples
template <bool INV>
__device__ __forceinline__ void dft14(float2 *v) {
    float2 e[7], o[7];
#pragma unroll
    for (int r = 0; r < 7; ++r) {
        e[r] = v[2 * r];
        o[r] = v[2 * r + 1];
    }
    dft_odd<7, INV>(e);
    dft_odd<7, INV>(o);
    // cos / sin of pi k / 7, k = 1..6
    const float c[6] = {0.90096886790241912624f, 0.62348980185873353053f, 0.22252093395631440429f,
                        -0.22252093395631440429f, -0.62348980185873353053f, -0.90096886790241912624f};
    const float sn[6] = {0.43388373911755812048f, 0.78183148246802980871f, 0.97492791218182360702f,
                         0.97492791218182360702f, 0.78183148246802980871f, 0.43388373911755812048f};
    v[0] = cadd(e[0], o[0]);
    v[7] = csub(e[0], o[0]);
#pragma unroll
    for (int k = 1; k < 7; ++k) {
        const float2 w = make_float2(c[k - 1], INV ? sn[k - 1] : -sn[k - 1]);
        const float2 t = cmul(o[k], w);
        v[k] = cadd(e[k], t);
        v[k + 7] = csub(e[k], t);
    }
}

// Odd radix R in registers with its cos/sin values passed in registers:
// c[m-1] = cos(2 pi m / R), sn[m-1] = sin(2 pi m / R), m = 1..(R-1)/2.
template <int R, bool INV>
__device__ __forceinline__ void dft_odd_t(float2 *v, const float *c, const float *sn) {
    constexpr int H = (R - 1) / 2;
    float2 a[H], b[H];
#pragma unroll
    for (int r = 1; r <= H; ++r) {
        a[r - 1] = cadd(v[r], v[R - r]);
        b[r - 1] = csub(v[r], v[R - r]);
    }
    const float2 x0 = v[0];
    float2 s0 = x0;
#pragma unroll
    for (int r = 0; r < H; ++r) s0 = cadd(s0, a[r]);
#pragma unroll
    for (int k = 1; k <= H; ++k) {
        float ax = x0.x, ay = x0.y, bx = 0.f, by = 0.f;
#pragma unroll
        for (int r = 1; r <= H; ++r) {
            const int m = (r * k) % R;
            const float cc = m <= H ? c[m - 1] : c[R - m - 1];
            const float ss = m <= H ? sn[m - 1] : -sn[R - m - 1];
            ax += a[r - 1].x * cc;
            ay += a[r - 1].y * cc;
            bx += b[r - 1].x * ss;
            by += b[r - 1].y * ss;
        }
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

// The register DFTs of the Rader stages: 7, 14 and 16 with constants, 17
// with the cos/sin values the stage loaded into c / sn.
template <int N, bool INV>
__device__ __forceinline__ void rader_dft(float2 *v, const float *c, const float *sn) {
    if constexpr (N == 7)
        dft_odd<7, INV>(v);
    else if constexpr (N == 14)
        dft14<INV>(v);
    else if constexpr (N == 16)
        dft16<INV>(v);
    else {
        static_assert(N == 17, "Rader sub-transform lengths are 7, 14, 16 and 17");
        dft_odd_t<17, INV>(v, c, sn);
    }
}

// A prime stage R by Rader's algorithm (113 = 1 + 16 x 7, 239 = 1 + 14 x 17).
// With g a primitive root mod R, X[g^m] = x_0 + sum_q u[q] h[(m - q) mod M],
// M = R - 1, u[q] = x[g^-q], h[s] = wR^(g^s), and X[0] = x_0 + sum u: a cyclic
// convolution of length M = N1 x N2, done as FFT-M, a product with the
// precomputed FFT of h (already divided by M), and an inverse FFT-M, in three
// passes over the CTA's m * nl butterflies held in dst as T[q1 * N2 + k2][b]:
//   1. gather u[q1 + N1 q2] (twiddled), N2-point DFT over q2, times wM^(q1 k2);
//   2. per (k2, b): N1-point DFT over q1, product with H[k2 + N2 k1], inverse
//      N1-point DFT over k1, times wM^-(q1 k2), all in registers;
//   3. inverse N2-point DFT over k2, then X[g^(q1 + N1 q2)] = x_0 + c into src.
// The stage's output is left in src; x_0 and sum u go through scr_all.
// tb: the stage's table (cos/sin of R, then the Rader tables of fft_plan.cu:
// FFT of h forward and inverse, wM, the (g^-q, g^q) index pairs, and for
// N2 = 17 the cos/sin of 17).
// NC, NLC, NSC > 0: the line length, lines per CTA and Ns known at compile
// time (the specialised engine, fft_lines_fixed), so the index arithmetic folds.
template <int R, int N1, int N2, bool INV, int NC = 0, int NLC = 0, int NSC = 0>
__device__ __noinline__ void stage_rader(float2 *__restrict__ src, float2 *__restrict__ dst, int n, int nl,
                                         int Ns, const float2 *__restrict__ tw, const float2 *__restrict__ tb,
                                         float4 *__restrict__ scr_all) {
    constexpr int M = R - 1;
    static_assert(N1 * N2 == M, "Rader split must cover R - 1");
    if constexpr (NC > 0) n = NC;
    if constexpr (NLC > 0) nl = NLC;
    if constexpr (NSC > 0) Ns = NSC;
    constexpr int NBC = (NC > 0 && NLC > 0) ? NC / R * NLC : 0;
    const int m = n / R, nb = m * nl;
    const int tstep = n / (Ns * R);
    const int lnl = NLC > 0 ? ilog2c(NLC) : log2_pow2(nl);
    const float invNs = 1.0f / (float)Ns, invnb = 1.0f / (float)nb;
    const float2 *Hh = tb + R + (INV ? M : 0);
    const float2 *wM = tb + R + 2 * M;
    const int2 *gq = reinterpret_cast<const int2 *>(tb + R + 3 * M);  // (g^-q, g^q)
    float c2[N2 == 17 ? 8 : 1], s2[N2 == 17 ? 8 : 1];
    if constexpr (N2 == 17) {
        const float2 *cs = tb + R + 4 * M;
#pragma unroll
        for (int k = 1; k <= 8; ++k) {
            c2[k - 1] = cs[k].x;
            s2[k - 1] = -cs[k].y;  // table holds (cos, -sin)
        }
    }
    float2 *x0s = reinterpret_cast<float2 *>(scr_all);
    float2 *s0s = x0s + nb;
    float2 *T = dst;

    for (int e = threadIdx.x; e < N1 * nb; e += blockDim.x) {
        const int q1 = divc<NBC>(e, nb, invnb), b = e - q1 * nb;
        const int l = b & (nl - 1), j = b >> lnl;
        const int kk = Ns > 1 ? j - divc<NSC>(j, Ns, invNs) * Ns : 0;
        float2 v[N2];
#pragma unroll
        for (int q2 = 0; q2 < N2; ++q2) {
            const int r = gq[q1 + N1 * q2].x;
            float2 x = src[sidx(j + r * m, l, nl)];
            if (Ns > 1) {
                const float2 w = tw[kk * r * tstep];
                x = INV ? cmulc(x, w) : cmul(x, w);
            }
            v[q2] = x;
        }
        if (q1 == 0) x0s[b] = src[sidx(j, l, nl)];
        rader_dft<N2, false>(v, c2, s2);
        T[(q1 * N2) * nb + b] = v[0];
#pragma unroll
        for (int k2 = 1; k2 < N2; ++k2) T[(q1 * N2 + k2) * nb + b] = cmul(v[k2], wM[q1 * k2]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < N2 * nb; e += blockDim.x) {
        const int k2 = divc<NBC>(e, nb, invnb), b = e - k2 * nb;
        float2 v[N1];
#pragma unroll
        for (int q1 = 0; q1 < N1; ++q1) v[q1] = T[(q1 * N2 + k2) * nb + b];
        rader_dft<N1, false>(v, c2, s2);
        if (k2 == 0) s0s[b] = v[0];
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[k1] = cmul(v[k1], Hh[k2 + N2 * k1]);
        rader_dft<N1, true>(v, c2, s2);
        T[k2 * nb + b] = v[0];
#pragma unroll
        for (int q1 = 1; q1 < N1; ++q1) T[(q1 * N2 + k2) * nb + b] = cmulc(v[q1], wM[q1 * k2]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < N1 * nb; e += blockDim.x) {
        const int q1 = divc<NBC>(e, nb, invnb), b = e - q1 * nb;
        const int l = b & (nl - 1), j = b >> lnl;
        const int kk = Ns > 1 ? j - divc<NSC>(j, Ns, invNs) * Ns : 0;
        const int d = (j - kk) * R + kk;
        float2 v[N2];
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) v[k2] = T[(q1 * N2 + k2) * nb + b];
        rader_dft<N2, true>(v, c2, s2);
        const float2 x0 = x0s[b];
#pragma unroll
        for (int q2 = 0; q2 < N2; ++q2) src[sidx(d + gq[q1 + N1 * q2].y * Ns, l, nl)] = cadd(x0, v[q2]);
        if (q1 == 0) src[sidx(d, l, nl)] = cadd(x0, s0s[b]);
    }
}

// 678 = 113 x 6 in two stages of one pass less: the Rader 113 stage (phases
// 1 and 2 of stage_rader, NL lines, Ns = 1), then its phase 3 fused with the
// radix-6 stage.  Sub-transform jb of a line (elements jb + 6 r) gives
// Y_jb[k], k < 113, and the radix-6 butterfly of output k combines the six
// Y_jb[k] (twiddled by w678^(k jb)) into X[k + 113 r'].  A pair of threads
// owns (q1, line): thread c runs phase 3 for the sub-transforms jb = c, c + 2,
// c + 4, which yields Y_jb[k] for the 7 outputs k = g^(q1 + 16 q2) (and k = 0
// when q1 = 0), so that the even (c = 0) and odd (c = 1) halves of each
// radix-6 butterfly (6 = 2 x 3, as dft6) are in the pair's registers: each
// thread does its 3-point DFT, the pair swaps three values by shuffle, and
// each writes three of the six outputs.  The result is left in A (the input,
// consumed by phase 1); T (phases 1-2) lives in B.  Needs 32 NL threads per
// work round (a pair per (q1, line), 16 values of q1) in whole warps.
template <bool INV, int NL>
__device__ __noinline__ void stage_rader113_x6(float2 *__restrict__ A, float2 *__restrict__ B,
                                               const float2 *__restrict__ tw, const float2 *__restrict__ tb,
                                               float4 *__restrict__ scr_all) {
    constexpr int R = 113, N1 = 16, N2 = 7, M = R - 1, n = 678, m = 6, nb = m * NL;
    constexpr int lnl = ilog2c(NL);
    const float2 *Hh = tb + R + (INV ? M : 0);
    const float2 *wM = tb + R + 2 * M;
    const int2 *gq = reinterpret_cast<const int2 *>(tb + R + 3 * M);  // (g^-q, g^q)
    float c2[1], s2[1];
    float2 *x0s = reinterpret_cast<float2 *>(scr_all);
    float2 *s0s = x0s + nb;
    float2 *T = B;
    for (int e = threadIdx.x; e < N1 * nb; e += blockDim.x) {
        const int q1 = e / nb, b = e - q1 * nb;
        const int l = b & (NL - 1), j = b >> lnl;
        float2 v[N2];
#pragma unroll
        for (int q2 = 0; q2 < N2; ++q2) v[q2] = A[sidx(j + gq[q1 + N1 * q2].x * m, l, NL)];
        if (q1 == 0) x0s[b] = A[sidx(j, l, NL)];
        rader_dft<N2, false>(v, c2, s2);
        T[(q1 * N2) * nb + b] = v[0];
#pragma unroll
        for (int k2 = 1; k2 < N2; ++k2) T[(q1 * N2 + k2) * nb + b] = cmul(v[k2], wM[q1 * k2]);
    }
    __syncthreads();
    for (int e = threadIdx.x; e < N2 * nb; e += blockDim.x) {
        const int k2 = e / nb, b = e - k2 * nb;
        float2 v[N1];
#pragma unroll
        for (int q1 = 0; q1 < N1; ++q1) v[q1] = T[(q1 * N2 + k2) * nb + b];
        rader_dft<N1, false>(v, c2, s2);
        if (k2 == 0) s0s[b] = v[0];
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[k1] = cmul(v[k1], Hh[k2 + N2 * k1]);
        rader_dft<N1, true>(v, c2, s2);
        T[k2 * nb + b] = v[0];
#pragma unroll
        for (int q1 = 1; q1 < N1; ++q1) T[(q1 * N2 + k2) * nb + b] = cmulc(v[q1], wM[q1 * k2]);
    }
    __syncthreads();
    const float h = 0.5f, rt = 0.86602540378443864676f;
    const float2 w61 = make_float2(h, INV ? rt : -rt), w62 = make_float2(-h, INV ? rt : -rt);
    for (int e = threadIdx.x; e < 2 * N1 * NL; e += blockDim.x) {
        const int c = e & 1, l = (e >> 1) & (NL - 1), q1 = e >> (1 + lnl);
        // phase 3 of sub-transforms jb = c + 2 i
        float2 y[3][N2], x0[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const int b = (c + 2 * i) * NL + l;
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) y[i][k2] = T[(q1 * N2 + k2) * nb + b];
            rader_dft<N2, true>(y[i], c2, s2);
            x0[i] = x0s[b];
        }
        // output k of the three sub-transforms, twiddled, 3-point DFT, swap
        // with the pair, three outputs X[k + 113 r]
        auto butterfly = [&](int k, float2 y0, float2 y1, float2 y2, unsigned mask) {
            float2 z[3] = {y0, y1, y2};
#pragma unroll
            for (int i = 1; i < 3; ++i) {
                const float2 w = tw[k * (c + 2 * i)];
                z[i] = INV ? cmulc(z[i], w) : cmul(z[i], w);
            }
            if (c) {
                const float2 w = tw[k];
                z[0] = INV ? cmulc(z[0], w) : cmul(z[0], w);
            }
            dft_odd<3, INV>(z);
            // c = 0 holds E (even jb), c = 1 the odd half O and sends w6^r O[r]
            if (c) {
                z[1] = cmul(z[1], w61);
                z[2] = cmul(z[2], w62);
            }
            float2 g[3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
                g[r] = make_float2(__shfl_xor_sync(mask, z[r].x, 1), __shfl_xor_sync(mask, z[r].y, 1));
#pragma unroll
            for (int r = 0; r < 3; ++r)
                A[sidx(k + R * (r + 3 * c), l, NL)] = c ? csub(g[r], z[r]) : cadd(z[r], g[r]);
        };
        // the lanes of a warp take the same rounds (32 NL work items in whole
        // warps), so the shuffles run with full warps; the q1 = 0 pairs (the
        // output k = 0 of the three sub-transforms) shuffle among themselves
#pragma unroll
        for (int q2 = 0; q2 < N2; ++q2)
            butterfly(gq[q1 + N1 * q2].y, cadd(x0[0], y[0][q2]), cadd(x0[1], y[1][q2]), cadd(x0[2], y[2][q2]),
                      0xffffffffu);
        const unsigned m0 = __ballot_sync(0xffffffffu, q1 == 0);
        if (q1 == 0) {
            float2 s0[3];
#pragma unroll
            for (int i = 0; i < 3; ++i) s0[i] = s0s[(c + 2 * i) * NL + l];
            butterfly(0, cadd(x0[0], s0[0]), cadd(x0[1], s0[1]), cadd(x0[2], s0[2]), m0);
        }
    }
    (void)n;
}

template <int R, bool INV, int NC = 0, int NLC = 0, int NSC = 0>
__device__ __forceinline__ void stage_small(const float2 *__restrict__ src, float2 *__restrict__ dst,
                                            int n, int nl, int Ns, const float2 *tw) {
    if constexpr (NC > 0) n = NC;
    if constexpr (NLC > 0) nl = NLC;
    if constexpr (NSC > 0) Ns = NSC;
    const int m = n / R;
    const int tstep = n / (Ns * R);
    const int items = m * nl;
    const int lnl = NLC > 0 ? ilog2c(NLC) : log2_pow2(nl);
    const float invNs = 1.0f / (float)Ns;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int l = it & (nl - 1);
        const int j = it >> lnl;
        const int k = j - divc<NSC>(j, Ns, invNs) * Ns;
        float2 v[R];
#pragma unroll
        for (int r = 0; r < R; ++r) v[r] = src[sidx(j + r * m, l, nl)];
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
        for (int r = 0; r < R; ++r) dst[sidx(d + r * Ns, l, nl)] = v[r];
    }
}

// Generic odd radix R (a prime >= 11): direct symmetric DFT.  Phase 1 applies
// the Stockham twiddles in place; phase 2 has one work item per (line,
// butterfly, output pair k / R-k) and loops over the R inputs.
template <bool INV>
__device__ void stage_generic(float2 *__restrict__ src, float2 *__restrict__ dst, int n,
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
            float2 x = src[sidx(e, l, nl)];
            src[sidx(e, l, nl)] = INV ? cmulc(x, w) : cmul(x, w);
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
        float2 x0 = src[sidx(j, l, nl)];
        if (k == 0) {
            float sx = x0.x, sy = x0.y;
            for (int r = 1; r < R; ++r) {
                float2 t = src[sidx(j + r * m, l, nl)];
                sx += t.x;
                sy += t.y;
            }
            dst[sidx(d, l, nl)] = make_float2(sx, sy);
            continue;
        }
        float ax = x0.x, ay = x0.y, bx = 0.f, by = 0.f;
        int mi = 0;
        for (int r = 1; r <= H; ++r) {
            mi += k;
            if (mi >= R) mi -= R;
            float2 w = cs[mi];  // (cos, -sin) of 2 pi mi / R
            float2 u = src[sidx(j + r * m, l, nl)], v = src[sidx(j + (R - r) * m, l, nl)];
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
        dst[sidx(d + k * Ns, l, nl)] = o1;
        dst[sidx(d + (R - k) * Ns, l, nl)] = o2;
    }
}

// Runs the whole plan on nl lines.  Returns the buffer holding the result.
#define MM_LANE_CASE(R)                                                                        \
    case R:                                                                                    \
        if constexpr (R <= LMAX)                                                               \
            stage_lane<R, INV>(src, dst, P.n, nl, Ns, tw_s, tab_s + P.ptab[st], scr);          \
        else                                                                                   \
            stage_generic<INV>(src, dst, P.n, nl, R, Ns, tw_s, tab_s + P.ptab[st]);            \
        break;
#define MM_ODD_CASE(R) \
    case R: stage_odd_tab<R, INV>(src, dst, P.n, nl, Ns, tw_s, tab_s + P.ptab[st]); break;

// LMAX: the largest prime given a lane (or, at 127, the Rader) stage in this
// instantiation (0, 63 or 127; the host picks the class of the plan), so that
// kernels whose lengths only need small lane stages keep fewer registers.
template <bool INV, int LMAX>
__device__ float2 *fft_lines(float2 *A, float2 *B, int nl, const FftPlan &P,
                             const float2 *tw_s, const float2 *tab_s, float4 *scr) {
    float2 *src = A, *dst = B;
    for (int st = 0; st < P.nst; ++st) {
        const int R = P.rad[st], Ns = P.ns[st];
        if constexpr (LMAX >= 113) {
            // 113 and 239 by Rader's algorithm (output left in src)
            if (R == 113 || R == 239) {
                if (R == 113)
                    stage_rader<113, 16, 7, INV>(src, dst, P.n, nl, Ns, tw_s, tab_s + P.ptab[st], scr);
                else
                    stage_rader<239, 14, 17, INV>(src, dst, P.n, nl, Ns, tw_s, tab_s + P.ptab[st], scr);
                __syncthreads();
                continue;
            }
        }
        switch (R) {
            case 2: stage_small<2, INV>(src, dst, P.n, nl, Ns, tw_s); break;
            case 3: stage_small<3, INV>(src, dst, P.n, nl, Ns, tw_s); break;
            case 4: stage_small<4, INV>(src, dst, P.n, nl, Ns, tw_s); break;
            case 5: stage_small<5, INV>(src, dst, P.n, nl, Ns, tw_s); break;
            case 6: stage_small<6, INV>(src, dst, P.n, nl, Ns, tw_s); break;
            case 7: stage_small<7, INV>(src, dst, P.n, nl, Ns, tw_s); break;
            MM_ODD_CASE(11) MM_ODD_CASE(13) MM_ODD_CASE(17) MM_ODD_CASE(19) MM_ODD_CASE(23)
            MM_ODD_CASE(29) MM_ODD_CASE(31) MM_ODD_CASE(37)
            MM_LANE_CASE(41) MM_LANE_CASE(43) MM_LANE_CASE(47) MM_LANE_CASE(53) MM_LANE_CASE(59)
            MM_LANE_CASE(61) MM_LANE_CASE(79) MM_LANE_CASE(89)
            default: stage_generic<INV>(src, dst, P.n, nl, R, Ns, tw_s, tab_s + P.ptab[st]); break;
        }
        __syncthreads();
        float2 *t = src;
        src = dst;
        dst = t;
    }
    return src;
}

// The engine specialised at compile time for the padded lengths of the
// benchmark tiles (678 = 113 x 6: tile 500, overlap 89; 478 = 239 x 2: tile
// 300), NL lines per CTA: the same stages as their plans (fft_plan.cu: the
// Rader stage first, at Ns = 1), with every size a constant.  Returns the
// buffer holding the result.
template <bool INV, int N, int NL>
__device__ float2 *fft_lines_fixed(float2 *A, float2 *B, const FftPlan &P, const float2 *tw_s,
                                   const float2 *tab_s, float4 *scr) {
    static_assert(N == 678 || N == 478, "specialised lengths: 678, 478");
    if constexpr (N == 678) {
        stage_rader113_x6<INV, NL>(A, B, tw_s, tab_s + P.ptab[0], scr);
        __syncthreads();
        return A;
    } else {
        stage_rader<239, 14, 17, INV, 478, NL, 1>(A, B, N, NL, 1, tw_s, tab_s + P.ptab[0], scr);
        __syncthreads();
        stage_small<2, INV, 478, NL, 239>(A, B, N, NL, 239, tw_s);
    }
    __syncthreads();
    return B;
}

// fft_lines, or the specialised engine when NF > 0 (NF = P.n, NLF = nl)
template <bool INV, int LMAX, int NF, int NLF>
__device__ __forceinline__ float2 *fft_run(float2 *A, float2 *B, int nl, const FftPlan &P, const float2 *tw_s,
                                           const float2 *tab_s, float4 *scr) {
    if constexpr (NF > 0)
        return fft_lines_fixed<INV, NF, NLF>(A, B, P, tw_s, tab_s, scr);
    else
        return fft_lines<INV, LMAX>(A, B, nl, P, tw_s, tab_s, scr);
}

// Shared-memory layout of an FFT kernel: ping-pong line buffers A and B
// (n * nl float2 each), the twiddle table (n), the radix tables (ntab),
// then MM_FFT_SCR_PER_WARP float4 of scratch per warp for the lane stages
// (16-byte aligned).
struct FftSmem {
    float2 *A, *B, *tw, *tab;
    float4 *scr;
};
// Scratch (float4 entries) the plan's stages use: MM_FFT_SCR_PER_WARP per warp
// for a lane stage, x_0 and sum u of every butterfly (one float4) for the
// 113- and 239-point stages, none for the others.
__device__ __host__ inline int fft_scr_f4(const FftPlan &P, int nl, int nwarps) {
    int f4 = 0;
    for (int s = 0; s < P.nst; ++s) {
        const int R = P.rad[s];
        int need = 0;
        if (R == 113 || R == 239)
            need = (P.n / R) * nl;
        else if (R == 41 || R == 43 || R == 47 || R == 53 || R == 59 || R == 61 || R == 79 || R == 89)
            need = MM_FFT_SCR_PER_WARP * nwarps;
        f4 = need > f4 ? need : f4;
    }
    return f4;
}
__device__ __host__ inline size_t fft_smem_bytes(const FftPlan &P, int nl, int nwarps) {
    size_t b = sizeof(float2) * ((size_t)2 * P.n * nl + P.n + P.ntab);
    b = (b + 15) & ~(size_t)15;
    return b + sizeof(float4) * fft_scr_f4(P, nl, nwarps);
}
__device__ inline FftSmem fft_smem_layout(void *base, const FftPlan &P, int nl) {
    FftSmem L;
    L.A = (float2 *)base;
    L.B = L.A + P.n * nl;
    L.tw = L.B + P.n * nl;
    L.tab = L.tw + P.n;
    size_t off = sizeof(float2) * ((size_t)2 * P.n * nl + P.n + P.ntab);
    off = (off + 15) & ~(size_t)15;
    L.scr = (float4 *)((char *)base + off);
    return L;
}

// Copies the plan tables into shared memory (call by all threads, then sync).
__device__ __forceinline__ void fft_load_tables(const FftPlan &P, float2 *tw_s, float2 *tab_s) {
    for (int i = threadIdx.x; i < P.n; i += blockDim.x) tw_s[i] = P.tw[i];
    for (int i = threadIdx.x; i < P.ntab; i += blockDim.x) tab_s[i] = P.tab[i];
}

// cp.async helpers: global -> shared copies without register staging, so a
// thread keeps many loads in flight.
__device__ __forceinline__ void cp_async8(void *smem_dst, const void *gsrc) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async4(void *smem_dst, const void *gsrc) {
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem_dst);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Host side: plan cache (fft_plan.cu).
int mm_fft_plan_get(int n, FftPlan *out);

// ---- launch helpers shared by the FFT kernel translation units -------------
// An FFT kernel runs `ctas` CTAs of `threads` threads per SM (228 KB of shared
// memory, 1 KB of it reserved per CTA): one CTA of 512 ("wide") or two of 256
// ("pair", so one CTA's barrier waits overlap the other's work).  The
// persistent passes launch that many CTAs per SM; each kernel's
// __launch_bounds__ names its layout.
struct FftCfg {
    int threads, ctas;
};
constexpr FftCfg kFftWide = {512, 1};
constexpr FftCfg kFftPair = {256, 2};
constexpr int kFftThreads = kFftWide.threads;  // the non-persistent FFT kernels
constexpr int kFftSmemLimit = 224 * 1024;
constexpr int fft_smem_limit(FftCfg c) { return (224 / c.ctas) * 1024; }

static inline size_t fft_smem(const FftPlan &P, int nl, FftCfg c = kFftWide) {
    return fft_smem_bytes(P, nl, c.threads / 32);
}
// Lines per CTA: the largest power of two <= maxnl whose buffers fit the budget.
static inline int pick_nl(const FftPlan &P, int maxnl, FftCfg c = kFftWide) {
    int nl = maxnl;
    while (nl > 1 && fft_smem(P, nl, c) > (size_t)fft_smem_limit(c)) nl >>= 1;
    return nl;
}
// Pointer to the kernel template instantiation of the plan's lane class.
#define MM_BY_CLASS(P, KERNEL_TMPL, ...)                                    \
    ((P).lclass == 0 ? (const void *)KERNEL_TMPL<__VA_ARGS__ 0>             \
     : (P).lclass == 63 ? (const void *)KERNEL_TMPL<__VA_ARGS__ 63>         \
                        : (const void *)KERNEL_TMPL<__VA_ARGS__ 127>)
// The kernel instantiation for plan P at nl lines per CTA: the specialised
// engine for 678 and 478 at NLF lines, else the run-time engine of the plan's
// lane class.
#define MM_FFT_KERNEL(P, nl, NLF, KERNEL_TMPL, ...)                                           \
    ((P).n == 678 && (nl) == NLF   ? (const void *)KERNEL_TMPL<__VA_ARGS__ 127, 678, NLF>    \
     : (P).n == 478 && (nl) == NLF ? (const void *)KERNEL_TMPL<__VA_ARGS__ 127, 478, NLF>    \
                                   : MM_BY_CLASS(P, KERNEL_TMPL, __VA_ARGS__))
// SMs of the current device (cached per device)
static inline int mm_sm_count() {
    static int cache[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) dev = 0;
    if (!cache[dev]) {
        int v = 0;
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev);
        cache[dev] = v > 0 ? v : 1;
    }
    return cache[dev];
}

// CTAs of a persistent pass over ngroups line groups
static inline unsigned fft_grid(long long ngroups, FftCfg c) {
    const long long cap = (long long)mm_sm_count() * c.ctas;
    return (unsigned)(ngroups < cap ? ngroups : cap);
}

static inline int launch_fft_kernel(const void *fn, dim3 grid, size_t sm, cudaStream_t st, void **args,
                                    int threads = kFftThreads) {
    if (int rc = mm_set_smem(fn, sm)) return rc;
    MM_CUDA_TRY(cudaLaunchKernel(fn, grid, dim3(threads), args, sm, st));
    mm_launch_counter_add();
    return MM_OK;
}
