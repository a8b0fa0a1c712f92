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
//  - warps 0-11 form the operands and read the results, three per TMEM lane
//    quarter (warp w owns lanes 32 (w % 4) .. + 31).  Row pair i (the rows
//    (i, 0) and (i, 1)) sits in lanes 2s, 2s + 1 of quarter i / Pq, s = i % Pq,
//    Pq = ceil(Z / 4).  A (M, split) goes to TMEM with tcgen05.st, its
//    16-column chunks shared round robin by the quarter's warps; each entry
//    is the sum of two reads of a per-frequency table of the z kernel, kept
//    once as conj(w) for the (i, 0) rows and once as (Im w, Re w) for the
//    (i, 1) rows, so that the sum is already the lane's pair of A values.  B
//    (X, split) goes to shared memory in the K-major no-swizzle layout (8-row
//    x 16-byte core matrices).  Results leave TMEM in pairs of frequencies
//    (16 bytes per tile and row) into a [t][i][p] stage that one TMA store
//    per group writes back in place.
//  - warp 12 (one lane) stages the z kernel rows of each group and X of each
//    pair of its frequencies by TMA.
//  - warp 13 allocates the tensor memory; one lane issues the 3 x K/8 MMAs of
//    each frequency and commits them to an mbarrier.
// A and B are double buffered per frequency, so the MMAs of frequency f run
// while the compute warps read the results of f - 1 and form f + 1.  Every
// wait is bounded: a thread that gives up records the failure in *err and
// the CTA winds down (the tensor memory is freed after the MMAs it issued
// have completed).
//
// Throughput: a tensor copy moves one box row per ~5.3 SM cycles whatever
// its width from 16 to 64 bytes, and the batch spectrum's layout (frequency
// innermost) makes every box row short (16 bytes of X per plane and tile for
// a pair of frequencies, 32 bytes of output).  At 25 tiles of 678^2 and
// Z = 50 the copies alone take ~3.85 of the 4.06 ms a launch takes, against
// 3.3 ms for the register form (zop_tma.cu), which stays the default; this
// form is selected by MM_ZFORM_TENSOR.

#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "deconv.cuh"

namespace {

constexpr int kPB = 4;          // frequencies per group
constexpr int kCW = 12;         // compute warps: three per TMEM lane quarter
constexpr int kThreads = (kCW + 2) * 32;
constexpr int kTmemCols = 512;
constexpr unsigned kWaitPolls = 1u << 24;
constexpr int kXItems = 2;      // (tile, plane pair) items of X per compute thread
constexpr int kZeroRows = 64;   // zero rows after each table (a row index i + offset, i < 64)

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
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int c0, int c1, int c2,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
        "[%5];" ::"r"(smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
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

// 16 consecutive 32-bit columns of this thread's lane.  No memory clobber:
// the stores read only registers, and tcgen05.wait::st (volatile, with a
// clobber) orders them before anything that reads the tensor memory.
__device__ __forceinline__ void tc_st16(unsigned taddr, const float *v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16};" ::"r"(taddr),
        "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]), "f"(v[8]),
        "f"(v[9]), "f"(v[10]), "f"(v[11]), "f"(v[12]), "f"(v[13]), "f"(v[14]), "f"(v[15]));
}
__device__ __forceinline__ void tc_st8(unsigned taddr, const float *v) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1, %2, %3, %4, %5, %6, %7, %8};" ::"r"(taddr),
                 "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7]));
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
    unsigned wbytesA, wbytesB, xbytes;  // TMA boxes: kernel rows (two), X of two frequencies
    // shared-memory offsets (bytes)
    int trows;        // rows of a table: kernel rows, hB (2Z - 1), kZeroRows zeros
    unsigned o_w, o_x, o_wt, o_z, o_b, o_o;
    unsigned wstride, xstride, wtstride, bstride, bhalf, sbo;
    const float *fresp;
    unsigned *err;
};

// Geometry of depth Z (compile-time where Z is): K (2Z rounded up to 8),
// the staged row kb of w[0], and the table rows of the column positions j:
// the T value w[i - j] at row i + zm_toff(j), the H value (hB[i + j],
// w[i + j], w[i + j - 2Z + 2] or none, by the planes the reflections copy) at
// row i + zm_hoff(j); padding positions (j >= Z) and "none" read zero rows.
__host__ __device__ constexpr int zm_K(int Z) { return (2 * Z + 7) & ~7; }
__host__ __device__ constexpr int zm_kb(int Z) { return (2 * Z - 2 + 3) & ~3; }
__host__ __device__ constexpr int zm_wrows(int Z) { return zm_kb(Z) + 2 * Z - 1; }
__host__ __device__ constexpr int zm_zb(int Z) { return zm_wrows(Z) + 2 * Z - 1; }
__host__ __device__ constexpr int zm_toff(int Z, int j) { return j < Z ? zm_kb(Z) - j : zm_zb(Z); }
__host__ __device__ constexpr int zm_hoff(int Z, int zpad, int j) {
    return j >= Z ? zm_zb(Z)
                  : (j >= 1 && j <= zpad) ? ((j >= Z - 1 - zpad && j <= Z - 2) ? zm_wrows(Z) + j : zm_kb(Z) + j)
                  : (j >= Z - 1 - zpad && j <= Z - 2) ? zm_kb(Z) - (2 * Z - 2) + j
                                                      : zm_zb(Z);
}

// N: MMA width (16 or 32 tiles).  ZC > 0: depth and zpad (ZPC) known at
// compile time (the benchmark FOV's hyb and DAPI blocks), so that the table
// offsets of every column position fold into the loads.
template <int N, int ZC, int ZPC>
__global__ void __launch_bounds__(kThreads, 1)
k_zmma_apply(const __grid_constant__ CUtensorMap wmapA, const __grid_constant__ CUtensorMap wmapB,
             const __grid_constant__ CUtensorMap xmap, const __grid_constant__ CUtensorMap omap, const ZmmaArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t wfull[2], wempty[2], xfull[2], xempty[2], bfull[2], mdone[2], cbar;
    __shared__ unsigned tmem_base_sh;
    __shared__ int give_up;
    __shared__ int2 colt[64];  // per column position j: table rows of its T and H values, minus the row i
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr bool CT = ZC > 0;
    const int Z = CT ? ZC : a.Z, K = CT ? zm_K(ZC) : a.K, Pq = CT ? (ZC + 3) / 4 : a.Pq;
    const int kb = CT ? zm_kb(ZC) : a.kA, ko = kb - (2 * Z - 2);
    const int hb = CT ? zm_wrows(ZC) : a.wrows;  // table row of hB[0] (after the kernel rows)
    const int zb = hb + 2 * Z - 1;               // first zero row of a table

    if (tid == 0) {
        give_up = 0;
        for (int b = 0; b < 2; ++b) {
            mbar_init(&wfull[b], 1);
            mbar_init(&wempty[b], kCW * 32);
            mbar_init(&bfull[b], kCW * 32);
            mbar_init(&mdone[b], 1);
            mbar_init(&xfull[b], 1);
            mbar_init(&xempty[b], kCW * 32);
        }
        mbar_init(&cbar, kCW * 32);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if ((smem_u32(smem) & 127u) != 0u) {
            atomicOr(a.err, 2u);
            give_up = 1;
        }
    }
    if (tid < a.K / 2) {
        // T value w[i - j], H value (by the planes the reflections copy):
        // hB[i + j], w[i + j], w[i + j - 2Z + 2] or none; padding positions
        // (j >= Z) and "none" read the zero rows
        const int j = tid;
        const bool vin = j >= 1 && j <= a.jin_hi, vout = j >= a.jout_lo && j <= Z - 2;
        const int off = vin ? (vout ? hb : kb) : (vout ? ko : zb);
        colt[j] = j < Z ? make_int2(kb - j, off == zb ? zb : off + j) : make_int2(zb, zb);
    }
    {
        // the zero rows of every table (never rewritten), and the zero table of
        // the lanes without a row
        float2 *t0 = reinterpret_cast<float2 *>(smem + a.o_wt);
        const int ntab = 2 * 2 * kPB;  // buffers x row types x frequencies
        for (int e = tid; e < ntab * kZeroRows; e += kThreads)
            t0[(e / kZeroRows) * (a.wtstride / 8) + zb + e % kZeroRows] = make_float2(0.f, 0.f);
        float2 *z0 = reinterpret_cast<float2 *>(smem + a.o_z);
        for (int e = tid; e < a.trows; e += kThreads) z0[e] = make_float2(0.f, 0.f);
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
        // ---- producer: the z kernel rows of each group and X of each pair
        // of its frequencies, by TMA ----
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
                // X of frequencies 2x, 2x + 1 of the group into buffer x, once
                // the previous group's pair has been read
                bool stop = false;
                for (int x = 0; x < 2; ++x) {
                    if (it >= 1 && !mbar_wait(&xempty[x], (it - 1) & 1)) {
                        atomicOr(a.err, 4u);
                        stop = true;
                        break;
                    }
                    fence_async_smem();
                    mbar_expect_tx(&xfull[x], a.xbytes);
                    tma_load_3d(smem + a.o_x + x * a.xstride, &xmap, p0 + 2 * x, 0, 0, &xfull[x]);
                }
                if (stop) {
                    ++it;  // this group's copies were (partly) issued
                    break;
                }
            }
            // no copy may still be landing when the CTA exits
            for (int j = it - 2 < 0 ? 0 : it - 2; j < it; ++j)
                if (!mbar_wait(&wfull[j & 1], (j >> 1) & 1)) atomicOr(a.err, 4u);
            if (it >= 1)
                for (int x = 0; x < 2; ++x)
                    if (!mbar_wait(&xfull[x], (it - 1) & 1)) atomicOr(a.err, 4u);
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
        const int q = warp & 3, h = warp >> 2;  // h: 0..2 within the quarter
        const int s_pair = lane >> 1, c = lane & 1;
        const int i = q * Pq + s_pair;  // row pair of this lane
        const bool row_ok = s_pair < Pq && i < Z;
        const unsigned lane_base = (unsigned)(32 * q) << 16;
        const int nchunk = (K + 15) / 16;
        const int nx = a.nt * (K / 4);  // X items (tile, plane pair) per frequency

        // X item e = tid + 256 r: tile n = e % nt, planes z = 2 (e / nt) and
        // z + 1; its B core-matrix row (n, kq = z / 2) holds
        // (Xr[z], Xi[z], Xr[z+1], Xi[z+1]).  The staged X of two frequencies
        // is [t][z][2] complex.
        int xoff[kXItems], bofs[kXItems], xn[kXItems];
#pragma unroll
        for (int r = 0; r < kXItems; ++r) {
            const int e = tid + r * kCW * 32;
            const int n = e % a.nt, kq = e / a.nt;
            xoff[r] = (n * Z + 2 * kq) * 2;
            xn[r] = e < nx ? (2 * kq + 1 < Z ? 2 : (2 * kq < Z ? 1 : 0)) : -1;  // planes present, -1: no item
            bofs[r] = (n >> 3) * (int)a.sbo + kq * 128 + (n & 7) * 16;
        }

        // B of frequency fp of the group, split, from the staged X
        // ([t][z][2] complex: the pair of frequencies of its buffer)
        auto form_b = [&](int fp, int slot) {
            const float2 *xs = reinterpret_cast<const float2 *>(smem + a.o_x + (fp >> 1) * a.xstride) + (fp & 1);
            unsigned char *bh = smem + a.o_b + slot * a.bstride, *bl = bh + a.bhalf;
#pragma unroll
            for (int r = 0; r < kXItems; ++r) {
                if (xn[r] >= 0) {
                    const float2 x0 = xn[r] >= 1 ? xs[xoff[r]] : make_float2(0.f, 0.f);
                    const float2 x1 = xn[r] >= 2 ? xs[xoff[r] + 2] : make_float2(0.f, 0.f);
                    float4 hi, lo;
                    split_tf32(x0.x, hi.x, lo.x);
                    split_tf32(x0.y, hi.y, lo.y);
                    split_tf32(x1.x, hi.z, lo.z);
                    split_tf32(x1.y, hi.w, lo.w);
                    *reinterpret_cast<float4 *>(bh + bofs[r]) = hi;
                    *reinterpret_cast<float4 *>(bl + bofs[r]) = lo;
                }
            }
        };

        // A of one frequency: this lane's row, column chunks h, h + 2, ...
        // tb: the frequency's table for this lane's row type, offset by its
        // row i (the zero table for lanes without a row).  Row (i, 0) reads
        // conj(w), row (i, 1) reads (Im w, Re w), so that each entry of the
        // sum is already the lane's pair of A values: (Mr, -Mi) or (Mi, Mr).
        auto form_chunk = [&](int ch, const float2 *tb, int slot) {
            float hi[16], lo[16];
            const bool full16 = K - 16 * ch >= 16;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                if (u < 4 || full16) {
                    const int j = 8 * ch + u;
                    int to, ho;
                    if constexpr (CT) {
                        to = zm_toff(ZC, j);
                        ho = zm_hoff(ZC, ZPC, j);
                    } else {
                        const int2 cj = colt[j];
                        to = cj.x;
                        ho = cj.y;
                    }
                    const float2 t = tb[to], hk = tb[ho];
                    split_tf32(t.x + hk.x, hi[2 * u], lo[2 * u]);
                    split_tf32(t.y + hk.y, hi[2 * u + 1], lo[2 * u + 1]);
                }
            }
            const unsigned ta = tmem + lane_base + colA + slot * 2 * K + 16 * ch;
            if (full16) {
                tc_st16(ta, hi);
                tc_st16(ta + K, lo);
            } else {
                tc_st8(ta, hi);
                tc_st8(ta + K, lo);
            }
        };
        auto form_a = [&](const float2 *tb, int slot) {
            if constexpr (CT) {
                constexpr int nch = (zm_K(ZC) + 15) / 16;
#pragma unroll
                for (int ch = 0; ch < nch; ++ch)
                    if (ch % (kCW / 4) == h) form_chunk(ch, tb, slot);
            } else {
                for (int ch = h; ch < nchunk; ch += kCW / 4) form_chunk(ch, tb, slot);
            }
        };

        // results of one frequency (slot), scaled by its blur response: this
        // lane's (Yr, Yi) of tiles (N / 2) h + 2 m2 + c, m2 < N / 4 (warps
        // h = 0, 1 of each quarter)
        auto read_results = [&](int slot, long long pg, float2 (&y)[8]) {
            const float fr = a.fresp ? __ldg(a.fresp + pg) : 1.f;
            float v[16];
            const unsigned td = tmem + lane_base + colD + slot * N + (N / 2) * h;
            if (N == 32)
                tc_ld16(td, v);
            else
                tc_ld8(td, v);
            tc_wait_ld();
#pragma unroll
            for (int m2 = 0; m2 < N / 4; ++m2) {
                // lane c = 0 holds Yr and takes tile 2 m2, lane c = 1 holds Yi
                // and takes tile 2 m2 + 1
                const float give = c ? v[2 * m2] : v[2 * m2 + 1];
                const float got = __shfl_xor_sync(0xffffffffu, give, 1);
                y[m2] = make_float2((c ? got : v[2 * m2]) * fr, (c ? v[2 * m2 + 1] : got) * fr);
            }
        };
        // two frequencies' results (p0, p0 + 1 of the group) into the
        // [t][i][p] stage, 16 bytes per tile and row
        auto write_results = [&](const float2 (&y0)[8], const float2 (&y1)[8], int p0) {
            float4 *ob = reinterpret_cast<float4 *>(smem + a.o_o);
#pragma unroll
            for (int m2 = 0; m2 < N / 4; ++m2) {
                const int t = (N / 2) * h + 2 * m2 + c;
                if (row_ok && t < a.nt)
                    ob[(((size_t)t * Z + i) * kPB + p0) >> 1] = make_float4(y0[m2].x, y0[m2].y, y1[m2].x, y1[m2].y);
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

        // the stage of a group, once every compute thread has written its part
        auto store_group = [&](int it) -> bool {
            fence_async_smem();
            if (!cbar_sync()) return false;
            if (tid == 0) {
                tma_store_3d(&omap, smem + a.o_o, ((int)blockIdx.x + it * (int)gridDim.x) * kPB, 0, 0);
                bulk_commit();
            }
            return true;
        };
        // before the first write of a group: the previous group's store has
        // read the stage
        auto stage_free = [&]() -> bool {
            if (tid == 0) bulk_wait_read0();
            return cbar_sync();
        };

        float2 yhold[8];  // results of the even frequency of a pair
        // one group: its kernel rows transposed, then per frequency the
        // results of two frequencies back and the operands of this one
        auto group = [&](int it) -> bool {
            const int wbuf = it & 1;
            if (!wait_all(&wfull[wbuf], (it >> 1) & 1)) {
                if (lane == 0) atomicOr(a.err, 1u);
                return false;
            }
            {
                // the group's kernel rows and hB, per frequency and row type
                const float2 *w = reinterpret_cast<const float2 *>(smem + a.o_w + wbuf * a.wstride);
                float2 *tab = reinterpret_cast<float2 *>(smem + a.o_wt);
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
                    float2 *t0 = tab + (size_t)((wbuf * kPB + p) * 2) * (a.wtstride / 8);
                    t0[r] = make_float2(v.x, -v.y);
                    t0[a.wtstride / 8 + r] = make_float2(v.y, v.x);
                }
            }
            if (!cbar_sync()) return false;
            // the staged rows are no longer read
            mbar_arrive(&wempty[wbuf]);
            const long long pbase = ((long long)blockIdx.x + (long long)it * gridDim.x) * kPB;
            const long long pprev = pbase - (long long)gridDim.x * kPB;
#pragma unroll
            for (int fp = 0; fp < kPB; ++fp) {
                const int f = it * kPB + fp, slot = f & 1;
                if (f >= 2) {
                    // results of f - 2 (of the previous group when fp < 2),
                    // which also frees slot `slot`; written in pairs of
                    // frequencies, the group stored after its fourth
                    if (!wait_all(&mdone[slot], ((f - 2) >> 1) & 1)) {
                        if (lane == 0) atomicOr(a.err, 16u);
                        return false;
                    }
                    tc_fence_after();
                    const int pe = (fp + 2) & 3;
                    if (pe == 0 || pe == 2) {
                        if (h < 2) read_results(slot, (fp < 2 ? pprev : pbase) + pe, yhold);
                    } else {
                        float2 y[8];
                        if (h < 2) read_results(slot, (fp < 2 ? pprev : pbase) + pe, y);
                        if (pe == 1 && !stage_free()) return false;
                        if (h < 2) write_results(yhold, y, pe - 1);
                        if (pe == 3 && !store_group(it - 1)) return false;
                    }
                }
                const float2 *tb =
                    row_ok ? reinterpret_cast<const float2 *>(smem + a.o_wt) +
                                 (size_t)((wbuf * kPB + fp) * 2 + c) * (a.wtstride / 8) + i
                           : reinterpret_cast<const float2 *>(smem + a.o_z);
                form_a(tb, slot);
                if ((fp & 1) == 0 && !wait_all(&xfull[fp >> 1], it & 1)) {
                    if (lane == 0) atomicOr(a.err, 1u);
                    return false;
                }
                form_b(fp, slot);
                if (fp & 1) mbar_arrive(&xempty[fp >> 1]);
                tc_wait_st();
                fence_async_smem();
                tc_fence_before();
                mbar_arrive(&bfull[slot]);
            }
            return true;
        };

        bool ok = true;
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
                const int fp = f & 3;  // 2, then 3
                const long long pg = ((long long)blockIdx.x + (long long)(f / kPB) * gridDim.x) * kPB + fp;
                if (h < 2) {
                    if (fp == 2) {
                        read_results(slot, pg, yhold);
                    } else {
                        float2 y[8];
                        read_results(slot, pg, y);
                        write_results(yhold, y, 2);
                    }
                }
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
    // a table per buffer, frequency and row type: the kernel rows, hB (2Z - 1
    // rows), then kZeroRows zero rows
    a->trows = a->wrows + 2 * Z - 1 + kZeroRows;
    a->wtstride = (unsigned)((a->trows * sizeof(float2) + 15) & ~(size_t)15);
    a->sbo = (unsigned)(a->K / 4) * 128;
    a->bhalf = align128((size_t)(N / 8) * a->sbo);
    a->bstride = 2 * a->bhalf;
    a->o_w = 0;
    a->xbytes = (unsigned)(2 * Z * nt * sizeof(float2));
    a->xstride = align128(a->xbytes);
    a->o_x = a->o_w + 2 * a->wstride;
    a->o_wt = a->o_x + 2 * a->xstride;
    a->o_z = align128(a->o_wt + (size_t)2 * 2 * kPB * a->wtstride);
    a->o_b = align128(a->o_z + (size_t)a->trows * sizeof(float2));
    a->o_o = a->o_b + 2 * a->bstride;
    *smem_bytes = a->o_o + align128((size_t)kPB * nt * Z * sizeof(float2));
    return *smem_bytes <= 220 * 1024;
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
    MM_REQUIRE(a.o_x % 128 == 0 && a.xstride % 128 == 0 && a.o_w % 128 == 0 && a.wstride % 128 == 0 && a.wbytesA % 128 == 0 && a.o_b % 128 == 0 &&
                   a.bhalf % 128 == 0 && a.o_o % 128 == 0 && a.wtstride % 8 == 0,
               "shared-memory layout of the tensor z operator");
    CUtensorMap wA, wB, om, xm;
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
        cuuint32_t xbox[3] = {2, (cuuint32_t)Z, (cuuint32_t)nt};
        if (int rc = make_map(&xm, S, 3, dims, strides, xbox)) return rc;
    }
    const void *fn;
    if (Z == 50 && zpad == 49)
        fn = nt <= 16 ? (const void *)k_zmma_apply<16, 50, 49> : (const void *)k_zmma_apply<32, 50, 49>;
    else if (Z == 50 && zpad == 24)
        fn = nt <= 16 ? (const void *)k_zmma_apply<16, 50, 24> : (const void *)k_zmma_apply<32, 50, 24>;
    else
        fn = nt <= 16 ? (const void *)k_zmma_apply<16, 0, 0> : (const void *)k_zmma_apply<32, 0, 0>;
    if (int rc = mm_set_smem(fn, sm)) return rc;
    const int grid = a.ngroups < mm_sm_count() ? a.ngroups : mm_sm_count();
    void *args[] = {&wA, &wB, &xm, &om, &a};
    MM_CUDA_TRY(cudaLaunchKernel(fn, dim3(grid), dim3(kThreads), args, sm, st));
    mm_launch_counter_add();
    return MM_OK;
}
