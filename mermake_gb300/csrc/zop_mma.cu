// z operator of one Wiener spectrum over a tile batch on the tensor cores
// (tcgen05, TF32 inputs with FP32 accumulation, the operands split so that
// the products keep FP32 accuracy).
//
// Per frequency p the z step is a complex matrix product Y = M X with M the
// Z x Z matrix of the z kernel (Toeplitz plus two masked Hankel parts, the
// derivation is in zop.cu and zop_tma.cu) and X the Z x nt spectra of the
// batch's tiles.  In real form, with K index k = 2 j + c (plane j, c = 0 the
// real and 1 the imaginary part of X[j]):
//
//   row (i, 0): Yr[i] = sum_j  Mr[i][j] Xr[j] - Mi[i][j] Xi[j]
//   row (i, 1): Yi[i] = sum_j  Mi[i][j] Xr[j] + Mr[i][j] Xi[j]
//
// a (2Z x 2Z) . (2Z x nt) product, one 128-row tcgen05.mma tile for Z <= 56.
// Each operand is split into a TF32 high part and the remainder,
// a = a_hi + a_lo, and D = A_hi B_hi + A_hi B_lo + A_lo B_hi (the dropped
// A_lo B_lo is below FP32 rounding).
//
// Layout of a CTA (one per SM, persistent over groups of kPB = 4 consecutive
// frequencies, whose values are 32 contiguous bytes of every spectrum row):
//  - warps 0-7 form the operands and read the results.  Warp w owns TMEM
//    lanes 32 (w % 4) .. + 31 and half w / 4 of the columns.  Row pair i (the
//    rows (i, 0) and (i, 1)) sits in lanes 2s, 2s + 1 of quarter i / Pq,
//    s = i % Pq, Pq = ceil(Z / 4); the two lanes of a pair compute half of the
//    pair's M entries each and swap them with one shuffle per value.
//    A (M, split) goes to TMEM with tcgen05.st; B (X, split) to shared memory
//    in the K-major no-swizzle layout (8-row x 16-byte core matrices).  X of
//    the next group is loaded into registers while the current group is
//    formed.
//  - warp 8 (one lane) stages the z kernel rows of each group by TMA.
//  - warp 9 allocates the tensor memory; one lane issues the MMAs of each
//    frequency and commits them to an mbarrier.
// A and B are double buffered per frequency, so the MMAs of frequency f run
// while the compute warps read the results of f - 1 and form f + 1.  Results
// go through shared memory ([p][t][i], then [t][i][p] by a transpose) and
// leave by one TMA store per group.  Every wait is bounded: a thread that
// gives up records the failure in *err and the CTA winds down (the tensor
// memory is freed after the MMAs it issued have completed).
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "deconv.cuh"

namespace {

constexpr int kPB = 4;          // frequencies per group
constexpr int kCW = 8;          // compute warps
constexpr int kThreads = (kCW + 2) * 32;
constexpr int kTmemCols = 512;
constexpr unsigned kWaitPolls = 1u << 24;
constexpr int kXItems = 3;      // (tile, plane pair) items of X per compute thread

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
// true once the phase with this parity has completed; false after kWaitPolls polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    const unsigned a = smem_u32(bar);
    for (unsigned it = 0; it < kWaitPolls; ++it) {
        unsigned done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, const void *src, int c0, int c1, int c2) {
    asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.bulk_group [%0, {%2, %3, %4}], [%1];" ::"l"(map),
                 "r"(smem_u32(src)), "r"(c0), "r"(c1), "r"(c2)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// the shared-memory reads of every committed bulk store have completed
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// generic-proxy shared-memory writes before async-proxy (TMA, MMA) reads
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// tcgen05.mma, kind::tf32, A from tensor memory, B from shared memory
__device__ __forceinline__ void tc_mma_ts(unsigned d_tmem, unsigned a_tmem, uint64_t b_desc, unsigned idesc,
                                          unsigned accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// one arrive on *bar once every MMA this thread issued before has completed
__device__ __forceinline__ void tc_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 16 consecutive 32-bit columns of this thread's lane
__device__ __forceinline__ void tc_st16(unsigned taddr, const float *v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};" ::"r"(taddr),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]),
        "f"(v[9]), "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15])
        : "memory");
}
__device__ __forceinline__ void tc_st8(unsigned taddr, const float *v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
                 : "memory");
}
__device__ __forceinline__ void tc_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tc_ld16(unsigned taddr, float *v) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7]),
          "=f"(v[8]), "=f"(v[9]), "=f"(v[10]), "=f"(v[11]), "=f"(v[12]), "=f"(v[13]), "=f"(v[14]), "=f"(v[15])
        : "r"(taddr)
        : "memory");
}
__device__ __forceinline__ void tc_ld8(unsigned taddr, float *v) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
                 : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
                 : "r"(taddr)
                 : "memory");
}
__device__ __forceinline__ void tc_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// shared-memory matrix descriptor: K-major, no swizzle; lbo = byte step
// between core matrices along K, sbo = along the 8-row groups
__device__ __forceinline__ uint64_t smem_desc(unsigned addr, unsigned lbo, unsigned sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// x = hi + lo with hi holding the 10 explicit mantissa bits TF32 keeps
__device__ __forceinline__ void split_tf32(float x, float &hi, float &lo) {
    hi = __uint_as_float(__float_as_uint(x) & 0xFFFFE000u);
    lo = x - hi;
}

struct ZmmaArgs {
    int Z, Zp, nt;
    long long plane;
    int ngroups;      // plane / kPB
    int jin_hi;       // the reflection about zpad copies planes 1 .. jin_hi (= zpad)
    int jout_lo;      // the reflection about zpad + Z - 1 copies planes jout_lo .. Z - 2
    int kA;           // staged row of w[0]: 2Z - 2 rounded up to a multiple of 4
    int K;            // 2Z rounded up to a multiple of 8 (MMA K steps of 8)
    int Pq;           // row pairs per TMEM lane quarter
    int wrows;        // staged kernel rows: kA + 2Z - 1
    unsigned wbytesA, wbytesB;
    // shared-memory offsets (bytes)
    unsigned o_w, o_wt, o_b, o_i, o_o;
    unsigned wstride, wtstride, bstride, bhalf, sbo;
    const float *fresp;
    unsigned *err;
};

// N: MMA width (16 or 32 tiles)
template <int N>
__global__ void __launch_bounds__(kThreads, 1)
k_zmma_apply(float2 *__restrict__ S, const __grid_constant__ CUtensorMap wmapA,
             const __grid_constant__ CUtensorMap wmapB, const __grid_constant__ CUtensorMap omap, const ZmmaArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t wfull[2], wempty[2], bfull[2], mdone[2], cbar;
    __shared__ unsigned tmem_base_sh;
    __shared__ int give_up;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int Z = a.Z, K = a.K, Pq = a.Pq;
    const int kb = a.kA, ko = kb - (2 * Z - 2);
    const int hb = a.wrows;  // staged row of hB[0] (after the kernel rows)

    if (tid == 0) {
        give_up = 0;
        for (int b = 0; b < 2; ++b) {
            mbar_init(&wfull[b], 1);
            mbar_init(&wempty[b], kCW * 32);
            mbar_init(&bfull[b], kCW * 32);
            mbar_init(&mdone[b], 1);
        }
        mbar_init(&cbar, kCW * 32);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if ((smem_u32(smem) & 127u) != 0u) {
            atomicOr(a.err, 2u);
            give_up = 1;
        }
    }
    if (warp == kCW + 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const unsigned tmem = tmem_base_sh;
    // tensor-memory columns: A of slot s (hi, then lo), then D of slot s
    const unsigned colA = 0, colD = 4 * K;
    const int nitems = give_up ? 0 : (a.ngroups - (int)blockIdx.x + (int)gridDim.x - 1) / (int)gridDim.x;
    const int nfreq = nitems * kPB;

    if (warp == kCW) {
        // ---- producer: the z kernel rows of each group ----
        if (lane == 0) {
            int it = 0;
            for (; it < nitems; ++it) {
                const int buf = it & 1;
                if (it >= 2 && !mbar_wait(&wempty[buf], ((it - 2) >> 1) & 1)) {
                    atomicOr(a.err, 4u);
                    break;
                }
                fence_async_smem();
                unsigned char *w = smem + a.o_w + buf * a.wstride;
                const int p0 = ((int)blockIdx.x + it * (int)gridDim.x) * kPB;
                mbar_expect_tx(&wfull[buf], a.wbytesA + a.wbytesB);
                tma_load_2d(w, &wmapA, p0, a.Zp - kb, &wfull[buf]);
                tma_load_2d(w + a.wbytesA, &wmapB, p0, 0, &wfull[buf]);
            }
            // no copy may still be landing when the CTA exits
            for (int j = it - 2 < 0 ? 0 : it - 2; j < it; ++j)
                if (!mbar_wait(&wfull[j & 1], (j >> 1) & 1)) atomicOr(a.err, 4u);
        }
    } else if (warp == kCW + 1) {
        // ---- MMA issue ----
        if (lane == 0) {
            // kind::tf32, D F32, A and B TF32, both K-major, N columns, 128 rows
            const unsigned idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((unsigned)(N >> 3) << 17) | (8u << 24);
            int f = 0;
            for (; f < nfreq; ++f) {
                const int s = f & 1;
                if (!mbar_wait(&bfull[s], (f >> 1) & 1)) {
                    atomicOr(a.err, 8u);
                    break;
                }
                tc_fence_after();
                const unsigned d = tmem + colD + s * N;
                const unsigned a_hi = tmem + colA + s * 2 * K, a_lo = a_hi + K;
                const unsigned b_hi = smem_u32(smem + a.o_b + s * a.bstride), b_lo = b_hi + a.bhalf;
                for (int ks = 0; ks < K / 8; ++ks)
                    tc_mma_ts(d, a_hi + 8 * ks, smem_desc(b_hi + 256 * ks, 128, a.sbo), idesc, ks > 0);
                for (int ks = 0; ks < K / 8; ++ks)
                    tc_mma_ts(d, a_hi + 8 * ks, smem_desc(b_lo + 256 * ks, 128, a.sbo), idesc, 1);
                for (int ks = 0; ks < K / 8; ++ks)
                    tc_mma_ts(d, a_lo + 8 * ks, smem_desc(b_hi + 256 * ks, 128, a.sbo), idesc, 1);
                tc_commit(&mdone[s]);
            }
            // the tensor memory is freed only after the issued MMAs completed
            for (int j = f - 2 < 0 ? 0 : f - 2; j < f; ++j)
                if (!mbar_wait(&mdone[j & 1], (j >> 1) & 1)) atomicOr(a.err, 8u);
        }
    } else {
        // ---- compute warps ----
        const int q = warp & 3, h = warp >> 2;
        const int s_pair = lane >> 1, c = lane & 1;
        const int i = q * Pq + s_pair;  // row pair of this lane
        const bool row_ok = s_pair < Pq && i < Z;
        const unsigned lane_base = (unsigned)(32 * q) << 16;
        const int nchunk = (K + 15) / 16;
        const int nx = a.nt * (K / 4);  // X items (tile, plane pair) per frequency

        // X item e = tid + 256 r: tile n = e % nt, planes z = 2 (e / nt) and
        // z + 1, all kPB frequencies (2 x 32 bytes); its B core-matrix row
        // (n, kq = z / 2) holds (Xr[z], Xi[z], Xr[z+1], Xi[z+1])
        int xrow[kXItems], bofs[kXItems], xn[kXItems];
#pragma unroll
        for (int r = 0; r < kXItems; ++r) {
            const int e = tid + r * kCW * 32;
            const int n = e % a.nt, kq = e / a.nt;
            xrow[r] = e < nx ? n * Z + 2 * kq : -1;
            xn[r] = e < nx ? (2 * kq + 1 < Z ? 2 : (2 * kq < Z ? 1 : 0)) : 0;  // planes present
            bofs[r] = (n >> 3) * (int)a.sbo + kq * 128 + (n & 7) * 16;
        }
        // the group's X rows into L2 ahead of their use
        auto prefetch_x = [&](int it) {
            const long long p0 = ((long long)blockIdx.x + (long long)it * gridDim.x) * kPB;
#pragma unroll
            for (int r = 0; r < kXItems; ++r) {
                if (xn[r] >= 1)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(S + (long long)xrow[r] * a.plane + p0));
                if (xn[r] >= 2)
                    asm volatile("prefetch.global.L2 [%0];" ::"l"(S + ((long long)xrow[r] + 1) * a.plane + p0));
            }
        };
        // X of frequency pg of this thread's items (planes z, z + 1); the
        // first frequency of a group brings the 32-byte rows into L1
        auto load_x = [&](float2 (&x)[kXItems][2], long long pg) {
#pragma unroll
            for (int r = 0; r < kXItems; ++r) {
                x[r][0] = xn[r] >= 1 ? __ldg(S + (long long)xrow[r] * a.plane + pg) : make_float2(0.f, 0.f);
                x[r][1] = xn[r] >= 2 ? __ldg(S + ((long long)xrow[r] + 1) * a.plane + pg) : make_float2(0.f, 0.f);
            }
        };

        // B of one frequency, split
        auto form_b = [&](const float2 (&x)[kXItems][2], int slot) {
            unsigned char *bh = smem + a.o_b + slot * a.bstride, *bl = bh + a.bhalf;
#pragma unroll
            for (int r = 0; r < kXItems; ++r) {
                if (xrow[r] >= 0) {
                    float4 hi, lo;
                    split_tf32(x[r][0].x, hi.x, lo.x);
                    split_tf32(x[r][0].y, hi.y, lo.y);
                    split_tf32(x[r][1].x, hi.z, lo.z);
                    split_tf32(x[r][1].y, hi.w, lo.w);
                    *reinterpret_cast<float4 *>(bh + bofs[r]) = hi;
                    *reinterpret_cast<float4 *>(bl + bofs[r]) = lo;
                }
            }
        };

        // A of one frequency: this lane's row, column chunks h, h + 2, ...,
        // from the transposed kernel rows wt (kernel value w[s] at
        // wt[s + kb], the combined reflection hB[s] = w[s] + w[s - 2Z + 2] at
        // wt[s + hb])
        auto form_a = [&](const float2 *wt, int slot) {
            for (int ch = h; ch < nchunk; ch += 2) {
                const bool full16 = K - 16 * ch >= 16;
                // this lane computes positions jp0 + u (u < 4) of the chunk
                const int jp0 = 8 * ch + (full16 ? 4 * c : 0);
                float2 m[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const int j = jp0 + u;
                    float2 v = make_float2(0.f, 0.f);
                    if (row_ok && j < Z) {
                        const bool vin = (unsigned)(j - 1) < (unsigned)a.jin_hi;
                        const bool vout = j >= a.jout_lo && j <= Z - 2;
                        const int off = vin ? (vout ? hb : kb) : (vout ? ko : hb);
                        const float sc = (vin || vout) ? 1.f : 0.f;
                        const float2 t = wt[i - j + kb], hk = wt[i + j + off];
                        v = make_float2(fmaf(sc, hk.x, t.x), fmaf(sc, hk.y, t.y));
                    }
                    m[u] = v;
                }
                float2 mm[8];
                if (full16) {
                    // swap with the pair partner: lane c = 0 computed positions
                    // 0..3 of the chunk, c = 1 positions 4..7
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        const float ox = __shfl_xor_sync(0xffffffffu, m[u].x, 1);
                        const float oy = __shfl_xor_sync(0xffffffffu, m[u].y, 1);
                        mm[u] = c ? make_float2(ox, oy) : m[u];
                        mm[u + 4] = c ? m[u] : make_float2(ox, oy);
                    }
                } else {
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        mm[u] = m[u];
                        mm[u + 4] = make_float2(0.f, 0.f);
                    }
                }
                float hi[16], lo[16];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    // row (i, 0): (Mr, -Mi); row (i, 1): (Mi, Mr)
                    const float e0 = c ? mm[u].y : mm[u].x;
                    const float e1 = c ? mm[u].x : -mm[u].y;
                    split_tf32(e0, hi[2 * u], lo[2 * u]);
                    split_tf32(e1, hi[2 * u + 1], lo[2 * u + 1]);
                }
                const unsigned ta = tmem + lane_base + colA + slot * 2 * K + 16 * ch;
                if (full16) {
                    tc_st16(ta, hi);
                    tc_st16(ta + K, lo);
                } else {
                    tc_st8(ta, hi);
                    tc_st8(ta + K, lo);
                }
            }
        };

        // results of frequency fp of a group (slot), scaled by the blur
        // response, into the [p][t][i] buffer
        auto epilogue = [&](int fp, int slot, long long pg) {
            const float fr = a.fresp ? __ldg(a.fresp + pg) : 1.f;
            float v[16];
            const unsigned td = tmem + lane_base + colD + slot * N + (N / 2) * h;
            if (N == 32)
                tc_ld16(td, v);
            else
                tc_ld8(td, v);
            tc_wait_ld();
            float2 *ib = reinterpret_cast<float2 *>(smem + a.o_i) + (size_t)fp * a.nt * Z;
#pragma unroll
            for (int m2 = 0; m2 < N / 4; ++m2) {
                // tiles u = 2 m2 (lane c = 0) and 2 m2 + 1 (lane c = 1)
                const float give = c ? v[2 * m2] : v[2 * m2 + 1];
                const float got = __shfl_xor_sync(0xffffffffu, give, 1);
                const float yr = c ? got : v[2 * m2], yi = c ? v[2 * m2 + 1] : got;
                const int t = (N / 2) * h + 2 * m2 + c;
                if (row_ok && t < a.nt) ib[(size_t)t * Z + i] = make_float2(yr * fr, yi * fr);
            }
        };

        // barrier of the compute warps (bounded): every compute thread
        // arrives on cbar (its own writes released by its own arrive)
        unsigned cb_uses = 0;
        auto cbar_sync = [&]() -> bool {
            mbar_arrive(&cbar);
            const bool done = mbar_wait(&cbar, cb_uses & 1);
            ++cb_uses;
            return __all_sync(0xffffffffu, done);
        };
        auto wait_all = [&](uint64_t *bar, unsigned parity) -> bool {
            return __all_sync(0xffffffffu, mbar_wait(bar, parity));
        };

        // [p][t][i] -> [t][i][p] of a group, then one TMA store
        auto store_group = [&](int it) -> bool {
            if (tid == 0) bulk_wait_read0();
            if (!cbar_sync()) return false;
            const float2 *ib = reinterpret_cast<const float2 *>(smem + a.o_i);
            float4 *ob = reinterpret_cast<float4 *>(smem + a.o_o);
            const int nti = a.nt * Z;
            for (int e = tid; e < nti; e += kCW * 32) {
                const float2 y0 = ib[e], y1 = ib[nti + e], y2 = ib[2 * nti + e], y3 = ib[3 * nti + e];
                ob[2 * e] = make_float4(y0.x, y0.y, y1.x, y1.y);
                ob[2 * e + 1] = make_float4(y2.x, y2.y, y3.x, y3.y);
            }
            fence_async_smem();
            if (!cbar_sync()) return false;
            if (tid == 0) {
                tma_store_3d(&omap, smem + a.o_o, ((int)blockIdx.x + it * (int)gridDim.x) * kPB, 0, 0);
                bulk_commit();
            }
            return true;
        };

        // one group: its kernel rows transposed, then per frequency the
        // results of two frequencies back and the operands of this one
        auto group = [&](int it) -> bool {
            const int wbuf = it & 1;
            if (!wait_all(&wfull[wbuf], (it >> 1) & 1)) {
                if (lane == 0) atomicOr(a.err, 1u);
                return false;
            }
            {
                const float2 *w = reinterpret_cast<const float2 *>(smem + a.o_w + wbuf * a.wstride);
                float2 *wt = reinterpret_cast<float2 *>(smem + a.o_wt + wbuf * kPB * a.wtstride);
                const int rows = a.wrows + 2 * Z - 1;
                for (int e = tid; e < rows * kPB; e += kCW * 32) {
                    const int r = e >> 2, p = e & 3;
                    float2 v;
                    if (r < a.wrows) {
                        v = w[r * kPB + p];
                    } else {
                        const int sr = r - a.wrows;
                        v = cadd(w[(sr + kb) * kPB + p], w[(sr + ko) * kPB + p]);
                    }
                    wt[p * (a.wtstride / 8) + r] = v;
                }
            }
            if (!cbar_sync()) return false;
            // the staged rows are no longer read
            mbar_arrive(&wempty[wbuf]);
            if (it + 1 < nitems) prefetch_x(it + 1);
            const long long pbase = ((long long)blockIdx.x + (long long)it * gridDim.x) * kPB;
            const long long pprev = pbase - (long long)gridDim.x * kPB;
#pragma unroll
            for (int fp = 0; fp < kPB; ++fp) {
                const int f = it * kPB + fp, slot = f & 1;
                if (f >= 2) {
                    // results of f - 2 (of the previous group when fp < 2),
                    // which also frees slot `slot`
                    if (!wait_all(&mdone[slot], ((f - 2) >> 1) & 1)) {
                        if (lane == 0) atomicOr(a.err, 16u);
                        return false;
                    }
                    tc_fence_after();
                    const int pf = (fp + 2) & 3;
                    epilogue(pf, slot, (fp < 2 ? pprev : pbase) + pf);
                    if (fp == 1 && !store_group(it - 1)) return false;
                }
                const float2 *wt = reinterpret_cast<const float2 *>(smem + a.o_wt + wbuf * kPB * a.wtstride) +
                                   (size_t)fp * (a.wtstride / 8);
                float2 xv[kXItems][2];
                load_x(xv, pbase + fp);  // in flight while A is formed
                form_a(wt, slot);
                form_b(xv, slot);
                tc_wait_st();
                fence_async_smem();
                tc_fence_before();
                mbar_arrive(&bfull[slot]);
            }
            return true;
        };

        bool ok = true;
        if (nitems > 0) prefetch_x(0);
        for (int it = 0; it < nitems && ok; ++it) ok = group(it);
        // the last two frequencies and the last group
        if (ok && nfreq > 0) {
            for (int f = nfreq < 2 ? 0 : nfreq - 2; f < nfreq && ok; ++f) {
                const int slot = f & 1;
                if (!wait_all(&mdone[slot], (f >> 1) & 1)) {
                    if (lane == 0) atomicOr(a.err, 16u);
                    ok = false;
                    break;
                }
                tc_fence_after();
                const int fp = f & 3;
                epilogue(fp, slot, ((long long)blockIdx.x + (long long)(f / kPB) * gridDim.x) * kPB + fp);
            }
            if (ok) store_group(nitems - 1);
        }
        if (tid == 0) bulk_wait0();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kCW + 1)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// rows of float2 (8-byte elements), innermost dimension first
int make_map(CUtensorMap *m, const void *base, int rank, const cuuint64_t *dims, const cuuint64_t *strides_bytes,
             const cuuint32_t *box) {
    auto fn = encode_fn();
    MM_REQUIRE(fn != nullptr, "cuTensorMapEncodeTiled is not available");
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, (cuuint32_t)rank, const_cast<void *>(base), dims,
                    strides_bytes, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) {
        mm_set_error("cuTensorMapEncodeTiled failed (%d)", (int)r);
        return MM_EDEVICE;
    }
    return MM_OK;
}

constexpr unsigned align128(size_t x) { return (unsigned)((x + 127) & ~(size_t)127); }

// the shared-memory plan of a launch; false when it does not fit one CTA
bool zmma_plan(int Z, int nt, ZmmaArgs *a, size_t *smem_bytes) {
    const int N = nt <= 16 ? 16 : 32;
    a->Z = Z;
    a->nt = nt;
    a->kA = (2 * Z - 2 + 3) & ~3;
    a->K = (2 * Z + 7) & ~7;
    a->Pq = (Z + 3) / 4;
    a->wrows = a->kA + 2 * Z - 1;
    a->wbytesA = (unsigned)(kPB * a->kA * sizeof(float2));
    a->wbytesB = (unsigned)(kPB * (2 * Z - 1) * sizeof(float2));
    a->wstride = align128((size_t)kPB * a->wrows * sizeof(float2));
    // per frequency: the kernel rows, then hB (2Z - 1 rows)
    a->wtstride = (unsigned)(((a->wrows + 2 * Z - 1) * sizeof(float2) + 15) & ~(size_t)15);
    a->sbo = (unsigned)(a->K / 4) * 128;
    a->bhalf = align128((size_t)(N / 8) * a->sbo);
    a->bstride = 2 * a->bhalf;
    a->o_w = 0;
    a->o_wt = a->o_w + 2 * a->wstride;
    a->o_b = align128(a->o_wt + (size_t)2 * kPB * a->wtstride);
    a->o_i = a->o_b + 2 * a->bstride;
    a->o_o = align128(a->o_i + (size_t)kPB * nt * Z * sizeof(float2));
    *smem_bytes = a->o_o + align128((size_t)kPB * nt * Z * sizeof(float2));
    return *smem_bytes <= 200 * 1024;
}

}  // namespace

int mm_zmma_supported(int Z, int zpad, int nt, long long plane) {
    if (Z < 1 || Z > 56 || zpad < 1 || zpad > Z - 1 || nt < 1 || nt > 32 || plane % kPB != 0) return 0;
    // X items per compute thread, TMEM columns: A double buffered (hi, lo) and D double buffered
    const int K = (2 * Z + 7) & ~7, N = nt <= 16 ? 16 : 32;
    if (nt * (K / 4) > kXItems * kCW * 32 || 4 * K + 2 * N > kTmemCols) return 0;
    if (plane / kPB >= (1LL << 31)) return 0;
    ZmmaArgs a = {};
    size_t sm;
    return zmma_plan(Z, nt, &a, &sm) && encode_fn() != nullptr;
}

int mm_launch_zmma_apply(float2 *S, const float2 *w, int Z, int zpad, int Zp, long long plane, int nt,
                         const float *fresp, unsigned *err, cudaStream_t st) {
    MM_REQUIRE(Zp == Z + 2 * zpad && mm_zmma_supported(Z, zpad, nt, plane),
               "z operator (tensor form) does not take Z %d, zpad %d, %d tiles", Z, zpad, nt);
    MM_REQUIRE(((uintptr_t)S & 31) == 0 && ((uintptr_t)w & 15) == 0 && (plane * 8) % 32 == 0,
               "spectra must be 32-byte aligned with rows of whole 32-byte groups");
    ZmmaArgs a = {};
    size_t sm = 0;
    zmma_plan(Z, nt, &a, &sm);
    a.Zp = Zp;
    a.plane = plane;
    a.ngroups = (int)(plane / kPB);
    a.jin_hi = zpad;
    a.jout_lo = Z - 1 - zpad;
    a.fresp = fresp;
    a.err = err;
    MM_REQUIRE(a.o_w % 128 == 0 && a.wstride % 128 == 0 && a.wbytesA % 128 == 0 && a.o_b % 128 == 0 &&
                   a.bhalf % 128 == 0 && a.o_o % 128 == 0 && a.wtstride % 8 == 0,
               "shared-memory layout of the tensor z operator");
    CUtensorMap wA, wB, om;
    const cuuint32_t kA = (cuuint32_t)a.kA, kb1 = (cuuint32_t)(2 * Z - 1);
    {
        cuuint64_t dims[2] = {(cuuint64_t)plane, (cuuint64_t)Zp};
        cuuint64_t strides[1] = {(cuuint64_t)plane * 8};
        cuuint32_t boxA[2] = {kPB, kA}, boxB[2] = {kPB, kb1};
        if (int rc = make_map(&wA, w, 2, dims, strides, boxA)) return rc;
        if (int rc = make_map(&wB, w, 2, dims, strides, boxB)) return rc;
    }
    {
        cuuint64_t dims[3] = {(cuuint64_t)plane, (cuuint64_t)Z, (cuuint64_t)nt};
        cuuint64_t strides[2] = {(cuuint64_t)plane * 8, (cuuint64_t)plane * 8 * Z};
        cuuint32_t box[3] = {kPB, (cuuint32_t)Z, (cuuint32_t)nt};
        if (int rc = make_map(&om, S, 3, dims, strides, box)) return rc;
    }
    const void *fn = nt <= 16 ? (const void *)k_zmma_apply<16> : (const void *)k_zmma_apply<32>;
    if (int rc = mm_set_smem(fn, sm)) return rc;
    const int grid = a.ngroups < mm_sm_count() ? a.ngroups : mm_sm_count();
    void *args[] = {&S, &wA, &wB, &om, &a};
    MM_CUDA_TRY(cudaLaunchKernel(fn, dim3(grid), dim3(kThreads), args, sm, st));
    mm_launch_counter_add();
    return MM_OK;
}
