// z operator of one Wiener spectrum over a tile batch, with the matrix of each
// frequency formed in registers and the operands staged asynchronously (the
// kernel rows by TMA, the spectra by cp.async).
//
// Y[t][i][p] = sum_j M_p[i][j] X[t][j][p] (zop.cu has the derivation).  When
// 1 <= zpad <= Z - 1 every real plane j has at most three padded copies
// (mermake/deconvolver.py:145-148: itself, its reflection about zpad for
// 1 <= j <= zpad, and its reflection about zpad + Z - 1 for
// Z - 1 - zpad <= j <= Z - 2), so with w the z kernel (indices mod Zp)
//
//   M[i][j] = w[i - j] + [1 <= j <= zpad] w[i + j] + [Z-1-zpad <= j <= Z-2] w[i + j - 2Z + 2]:
//
// a Toeplitz matrix plus two masked Hankel matrices.  A thread owns rows
// i0 .. i0 + 4 of kTT tiles; along j each family's five values slide by one
// place, so the thread keeps them in three register rings of five and loads
// one new value of each per column (the slots are compile-time constants with
// j unrolled by five).  No matrix is stored: shared memory holds only the
// operands, X (nt x Z x kPB: 32-byte rows, copied by cp.async) and the kernel
// rows w[-kA .. 2Z-2] (two TMA boxes of the (Zp, plane) kernel, the negative
// rows from its top; kA is 2Z - 2 rounded up to a multiple of four, so that
// both boxes land on 128-byte boundaries as tiled TMA requires), double
// buffered.  The persistent CTAs take groups of kPB consecutive frequencies.
// A producer warp issues each group's copies once the buffer is free; the
// compute warps take the group's work in warp-sized units from a shared
// counter, wait only for their buffer to fill (its "full" mbarrier completes
// with the copies: 32 cp.async arrivals and the TMA bytes) and release it with
// one arrive per unit on its "empty" mbarrier, so no CTA barrier separates the
// groups.  Every wait is bounded: a thread that gives up
// records the failure in *err and returns.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <mutex>

#include "deconv.cuh"

namespace {

constexpr int kPB = 4;      // frequencies per group (32 bytes of a plane row)
constexpr int kLPR = kPB / 2;  // 16-byte pieces of a row (copying lanes per row)
constexpr int kTI = 5;      // rows of a thread, and the unroll of the column loop
constexpr int kTT = 5;      // tiles of a thread
constexpr int kThreadsMax = 256;
constexpr unsigned kWaitPolls = 1u << 24;

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
// true once the barrier's phase with this parity has completed; false after
// kWaitPolls polls
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
// 16 bytes global -> shared through L2, completion tracked per thread
__device__ __forceinline__ void cp_async16(void *dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
// one arrive on *bar (counted in its initial count) once this thread's
// earlier cp.async copies have landed
__device__ __forceinline__ void cp_async_arrive(uint64_t *bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int c0, int c1, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
    c.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x));
    c.y = fmaf(a.x, b.y, fmaf(a.y, b.x, c.y));
    return c;
}

struct ZthArgs {
    int Z, Zp, nt;
    int ntc;           // tiles of a chunk (the X box's height)
    int ntg;           // tile groups of kTT a CTA computes (ceil(ntc / kTT))
    int nchunks;       // chunks the batch's tiles are split into
    long long plane;
    int nitems;        // frequency groups (ceil(plane / kPB)) x chunks
    int kA;            // staged row of w[0]: 2Z - 2 rounded up to a multiple of 4
    unsigned xbytes;   // X bytes of an item (kPB x Z x ntc float2)
    unsigned wbytesA;  // kernel rows -kA .. -1 (kA x 32 bytes, a multiple of 128)
    unsigned wbytesB;  // kernel rows 0 .. 2Z-2
    unsigned bufstride, woff;  // bytes per buffer, offset of the kernel rows in it
    unsigned zoff;     // bytes: the zero rows (2Z + 3 of them) after the two buffers
    // the columns j in segments of one reflection class: segment k covers
    // [segj[k], segj[k + 1]) (segj[nseg] = Z) with class segc[k]: 0 only the
    // reflection about zpad (w[i + j]), 1 only the one about zpad + Z - 1
    // (w[i + j - 2Z + 2]), 2 both (hB[i + j]), 3 neither
    int nseg, segj[6], segc[6];
    const float *fresp;
    unsigned *err;
};

// Work item -> frequency group and the first tile of its chunk.  Chunk c
// owns tiles [c * ntc, min((c + 1) * ntc, nt)); its box starts at
// min(c * ntc, nt - ntc) so that every box lies inside the batch (the last
// chunk's box may reach back into the previous chunk, whose tiles it computes
// again but does not store).
__device__ __forceinline__ void zth_item(const ZthArgs &a, int item, int &grp, int &own0, int &box0) {
    grp = item / a.nchunks;
    const int c = item - grp * a.nchunks;
    own0 = c * a.ntc;
    box0 = min(own0, a.nt - a.ntc);
}

// ZC > 0: Z known at compile time (50, the depth of every channel of the
// benchmark FOV); otherwise any multiple of kTI.  CH: the batch is split
// into several tile chunks (otherwise item == frequency group, one box of
// all nt tiles).
template <int ZC, bool CH>
__global__ void __launch_bounds__(kThreadsMax, 2)
k_zth_apply(float2 *__restrict__ S, const __grid_constant__ CUtensorMap wmapA, const __grid_constant__ CUtensorMap wmapB, const ZthArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t full[2], empty[2], wfull[2];
    __shared__ int3 item_of[2];  // (group, first owned tile, box start) of each buffer's item
    __shared__ unsigned unit_next;  // the next (item, warp unit) a compute warp takes
    const int Z = ZC > 0 ? ZC : a.Z;
    const int nig = Z / kTI;
    const int tid = threadIdx.x;
    const int kb = a.kA;              // row of w[0] in the staged kernel rows
    const int ko = kb - (2 * Z - 2);  // row of w[-(2Z-2)], the lowest index the rings read

    // every TMA destination (buffer starts, kernel rows, their second box) is
    // 128-byte aligned given an aligned base: check the base, and give up
    // (recording the failure) rather than issue a misaligned copy
    if ((smem_u32(smem) & 127u) != 0u) {
        if (tid == 0) atomicOr(a.err, 2u);
        return;
    }
    const int lane = tid & 31, warp = tid >> 5;
    const int ncw = (kPB * nig * a.ntg + 31) / 32;  // compute warps; warp ncw produces
    if (tid == 0) {
        for (int b = 0; b < 2; ++b) {
            // the producer warp's 32 copy arrivals and its 32 arrivals once
            // hB is written
            mbar_init(&full[b], 64);
            mbar_init(&empty[b], ncw);
            mbar_init(&wfull[b], 1);
        }
        unit_next = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    {
        float2 *zr = reinterpret_cast<float2 *>(smem + a.zoff);
        for (int e = tid; e < (2 * Z + 3) * kPB; e += blockDim.x) zr[e] = make_float2(0.f, 0.f);
    }
    __syncthreads();

    if (warp == ncw) {
        // producer warp: the copies of item `it` go to buffer it & 1 once the
        // compute warps have released its previous use (item it - 2).  X (the
        // box's nt x Z rows of 32 bytes) by cp.async from all 32 lanes: a
        // tensor copy moves a box row per ~5 SM cycles, which rows this short
        // would make the bound; the kernel rows (2Z - 1 + kA rows) by TMA.
        int grp, own0, box0;
        for (int item = blockIdx.x, it = 0; item < a.nitems; item += gridDim.x, ++it) {
            const int buf = it & 1;
            const bool ok = it < 2 || mbar_wait(&empty[buf], ((it - 2) >> 1) & 1);
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) atomicOr(a.err, 4u);
                break;
            }
            // order the compute warps' reads of the buffer before the copies
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            unsigned char *b = smem + (size_t)buf * a.bufstride;
            zth_item(a, item, grp, own0, box0);
            if (lane == 0) item_of[buf] = make_int3(grp, own0, box0);  // published by the arrives below
            const int p0 = grp * kPB;
            const int nchunk = kLPR * Z * a.ntc;  // 16-byte pieces of the box's rows
            // a piece past the plane (the last group of a plane of 2 mod 4
            // frequencies) is not copied: its results are not stored
            const long long pc = p0 + 2 * (lane % kLPR);
            if (pc < a.plane) {
                for (int k = lane; k < nchunk; k += 32) {
                    const int row = k / kLPR;  // (tile - box0) * Z + plane
                    cp_async16(b + (size_t)k * 16, S + ((long long)box0 * Z + row) * a.plane + pc);
                }
            }
            cp_async_arrive(&full[buf]);
            if (lane == 0) {
                mbar_expect_tx(&wfull[buf], a.wbytesA + a.wbytesB);
                tma_load_2d(b + a.woff, &wmapA, p0, a.Zp - kb, &wfull[buf]);
                tma_load_2d(b + a.woff + a.wbytesA, &wmapB, p0, 0, &wfull[buf]);
            }
            // hB[s] = w[s] + w[s - 2Z + 2], s < 2Z - 1, after the kernel rows
            if (!__all_sync(0xffffffffu, mbar_wait(&wfull[buf], (it >> 1) & 1))) {
                if (lane == 0) atomicOr(a.err, 4u);
                break;
            }
            {
                const float2 *w = reinterpret_cast<const float2 *>(b + a.woff);
                float2 *hbr = reinterpret_cast<float2 *>(b + a.woff + a.wbytesA + a.wbytesB);
                for (int e = lane; e < (2 * Z - 1) * kPB; e += 32) {
                    const int sr = e / kPB, pp = e - sr * kPB;
                    hbr[e] = cadd(w[(sr + kb) * kPB + pp], w[(sr + ko) * kPB + pp]);
                }
            }
            mbar_arrive(&full[buf]);
        }
        // no copy may still be landing when the CTA exits
        asm volatile("cp.async.wait_all;" ::: "memory");
        return;
    }

    // An item's threads (kPB x Z/kTI x ntg) come in ncw warp units: unit u
    // is threads 32u .. 32u + 31 of the item.  The compute warps take the
    // units in order from a shared counter, so a warp on a less loaded SM
    // sub-partition takes more of them (ncw warps of two CTAs do not divide
    // evenly over four sub-partitions).  The parity wait below passes on this
    // item's own phase: to pass on item it - 2's, a warp would have to take a
    // unit of item it while that item's buffer is unfilled.  The producer
    // fills in order, so no unit of items it - 2 and it - 1 could have
    // finished, and their 2 ncw units would occupy more warps than the CTA's
    // ncw.
    for (;;) {
        unsigned sq = 0;
        if (lane == 0) sq = atomicAdd(&unit_next, 1u);
        sq = __shfl_sync(0xffffffffu, sq, 0);
        const int it = (int)(sq / (unsigned)ncw), unit = (int)(sq - (unsigned)it * (unsigned)ncw);
        const long long item_ll = blockIdx.x + (long long)it * gridDim.x;
        if (item_ll >= a.nitems) break;
        const int item = (int)item_ll;
        const int buf = it & 1;
        if (!mbar_wait(&full[buf], (it >> 1) & 1)) {
            atomicOr(a.err, 1u);
            return;
        }
        const int vt = unit * 32 + lane;
        const int p = vt % kPB;
        const int r = vt / kPB;
        const int ig = r % nig, tg = r / nig;
        const int i0 = ig * kTI, tl0 = tg * kTT;  // first row, first tile of the chunk's box
        const float2 *X = reinterpret_cast<const float2 *>(smem + (size_t)buf * a.bufstride);
        const float2 *W = reinterpret_cast<const float2 *>(smem + (size_t)buf * a.bufstride + a.woff);
        if (tg < a.ntg) {
            float2 acc[kTI][kTT];
#pragma unroll
            for (int u = 0; u < kTI; ++u)
#pragma unroll
                for (int b = 0; b < kTT; ++b) acc[u][b] = make_float2(0.f, 0.f);
            // rings: the direct value of position q (= row - column) in slot
            // q mod 5; the reflected value of position q (= row + column), from
            // the source of the column's class, in slot q mod 5 (i0 and the
            // column blocks are multiples of 5).  A column that starts a
            // segment of another class reloads the reflected ring.
            const int wrows = a.kA + 2 * Z - 1;
            const int zrow = (int)((a.zoff - (unsigned)buf * a.bufstride - a.woff) / (kPB * sizeof(float2)));
            auto seg_row = [&](int k) {
                const int cls = a.segc[k];
                return cls == 0 ? kb : cls == 1 ? ko : cls == 2 ? wrows : zrow;
            };
            int sk = 0, hrow = seg_row(0), jnext = a.nseg > 1 ? a.segj[1] : Z;
            float2 rT[kTI], rH[kTI];
#pragma unroll
            for (int q = 1; q < kTI; ++q) rT[q] = W[(i0 + q + kb) * kPB + p];
#pragma unroll
            for (int q = 0; q < kTI - 1; ++q) rH[q] = W[(i0 + q + hrow) * kPB + p];
            rT[0] = rH[kTI - 1] = make_float2(0.f, 0.f);
            // the box's tiles past ntc read stale buffer contents; their
            // results are not stored
            const float2 *xr = X + ((size_t)tl0 * Z) * kPB + p;
            for (int j0 = 0; j0 < Z; j0 += kTI) {
#pragma unroll
                for (int u = 0; u < kTI; ++u) {
                    const int j = j0 + u;
                    rT[(kTI - u) % kTI] = W[(i0 - j + kb) * kPB + p];
                    if (j == jnext) {
                        ++sk;
                        hrow = seg_row(sk);
                        jnext = sk + 1 < a.nseg ? a.segj[sk + 1] : Z;
#pragma unroll
                        for (int q = 0; q < kTI - 1; ++q) rH[(q + u) % kTI] = W[(i0 + j + q + hrow) * kPB + p];
                    }
                    rH[(u + kTI - 1) % kTI] = W[(i0 + j + kTI - 1 + hrow) * kPB + p];
                    float2 m[kTI];
#pragma unroll
                    for (int q = 0; q < kTI; ++q) m[q] = cadd(rT[(q - u + kTI) % kTI], rH[(q + u) % kTI]);
                    float2 x[kTT];
#pragma unroll
                    for (int b = 0; b < kTT; ++b) x[b] = xr[((size_t)b * Z + j) * kPB];
#pragma unroll
                    for (int q = 0; q < kTI; ++q)
#pragma unroll
                        for (int b = 0; b < kTT; ++b) acc[q][b] = cfma(m[q], x[b], acc[q][b]);
                }
            }
            // the operands are in registers: release the buffer before the stores
            const int3 ii = CH ? item_of[buf] : make_int3(item, 0, 0);
            const int own0 = ii.y, box0 = ii.z;
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[buf]);
            const long long pg = (long long)ii.x * kPB + p;
            if (pg < a.plane) {
                const float f = a.fresp ? a.fresp[pg] : 1.f;
                // box0 + ntc >= t_end: the condition keeps t inside the box
                const int t_end = CH ? min(own0 + a.ntc, a.nt) : a.nt;
#pragma unroll
                for (int b = 0; b < kTT; ++b) {
                    const int t = CH ? box0 + tl0 + b : tl0 + b;
                    if ((!CH || t >= own0) && t < t_end) {
#pragma unroll
                        for (int q = 0; q < kTI; ++q)
                            S[((long long)t * Z + i0 + q) * a.plane + pg] = cscale(acc[q][b], f);
                    }
                }
            }
        } else {
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[buf]);
        }
    }
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

// the compute warps (threads kPB x Z/kTI x ntg, rounded up to whole warps)
// and the producer warp
int zth_threads(int Z, int ntg) { return ((kPB * (Z / kTI) * ntg + 31) / 32 + 1) * 32; }

// staged row of w[0]: the rows -(2Z-2) .. -1 rounded up to a multiple of four,
// so that the second kernel box starts on a 128-byte boundary
int zth_ka(int Z) { return (2 * Z - 2 + 3) & ~3; }

// bytes per buffer: X for ntg whole tile groups (the last group's threads
// read tiles past the box, whose results are not stored), then the kernel
// rows -kA .. 2Z - 2 and hB[0 .. 2Z - 2]; both parts start on 128-byte
// boundaries
size_t zth_bufstride(int Z, int ntg, unsigned *woff) {
    const size_t xb = (size_t)kPB * Z * ntg * kTT * sizeof(float2);
    const size_t wb = (size_t)kPB * (zth_ka(Z) + 2 * Z - 1 + 2 * Z - 1) * sizeof(float2);
    const size_t xo = (xb + 127) & ~(size_t)127;
    if (woff) *woff = (unsigned)xo;
    return (xo + wb + 127) & ~(size_t)127;
}

// shared memory of one CTA, two CTAs per SM
constexpr size_t kSmemMax = 112 * 1024;

// the zero rows after the two buffers
size_t zth_zero_bytes(int Z) { return ((size_t)(2 * Z + 3) * kPB * sizeof(float2) + 127) & ~(size_t)127; }

// How a batch of nt tiles is split: the fewest chunks whose tile groups fit
// one CTA (threads and shared memory), then the tiles spread evenly over them.
struct ZthPlan {
    int nchunks, ntc, ntg;
};
bool zth_plan(int Z, int nt, ZthPlan *pl) {
    const int ntg_all = (nt + kTT - 1) / kTT;
    int ntg_max = ntg_all;
    while (ntg_max > 0 && (zth_threads(Z, ntg_max) > kThreadsMax ||
                           2 * zth_bufstride(Z, ntg_max, nullptr) + zth_zero_bytes(Z) > kSmemMax))
        --ntg_max;
    if (ntg_max == 0) return false;
    pl->nchunks = (ntg_all + ntg_max - 1) / ntg_max;
    pl->ntc = (nt + pl->nchunks - 1) / pl->nchunks;
    pl->ntg = (pl->ntc + kTT - 1) / kTT;
    return true;
}

}  // namespace

int mm_zth_supported(int Z, int zpad, int nt, long long plane) {
    if (Z < kTI || Z % kTI != 0 || zpad < 1 || zpad > Z - 1 || nt < 1 || plane % 2 != 0) return 0;
    if (2 * Z - 1 > 256 || zth_ka(Z) > 256) return 0;  // TMA box height
    ZthPlan pl;
    return zth_plan(Z, nt, &pl) && encode_fn() != nullptr ? pl.nchunks : 0;
}

int mm_launch_zth_apply(float2 *S, const float2 *w, int Z, int zpad, int Zp, long long plane, int nt,
                        const float *fresp, unsigned *err, cudaStream_t st) {
    MM_REQUIRE(Zp == Z + 2 * zpad && mm_zth_supported(Z, zpad, nt, plane),
               "z operator (TMA form) does not take Z %d, zpad %d, %d tiles", Z, zpad, nt);
    MM_REQUIRE(((uintptr_t)S & 15) == 0 && ((uintptr_t)w & 15) == 0, "spectra must be 16-byte aligned");
    ZthPlan pl;
    zth_plan(Z, nt, &pl);
    CUtensorMap wA, wB;
    const cuuint32_t kb = (cuuint32_t)(2 * Z - 2), kA = (cuuint32_t)zth_ka(Z);
    {
        cuuint64_t dims[2] = {(cuuint64_t)plane, (cuuint64_t)Zp};
        cuuint64_t strides[1] = {(cuuint64_t)plane * 8};
        cuuint32_t boxA[2] = {kPB, kA}, boxB[2] = {kPB, kb + 1};
        if (int rc = make_map(&wA, w, 2, dims, strides, boxA)) return rc;
        if (int rc = make_map(&wB, w, 2, dims, strides, boxB)) return rc;
    }
    ZthArgs a = {};
    a.Z = Z;
    a.Zp = Zp;
    a.nt = nt;
    a.ntc = pl.ntc;
    a.ntg = pl.ntg;
    a.nchunks = pl.nchunks;
    a.plane = plane;
    const long long nitems = ((plane + kPB - 1) / kPB) * pl.nchunks;
    MM_REQUIRE(nitems < (1LL << 31), "z operator: too many frequency groups");
    a.nitems = (int)nitems;
    // the column segments of one reflection class
    a.nseg = 0;
    for (int j = 0, prev = -1; j < Z; ++j) {
        const bool vin = j >= 1 && j <= zpad, vout = j >= Z - 1 - zpad && j <= Z - 2;
        const int cls = vin ? (vout ? 2 : 0) : (vout ? 1 : 3);
        if (cls != prev) {
            MM_REQUIRE(a.nseg < 6, "z operator: more than six column segments");
            a.segj[a.nseg] = j;
            a.segc[a.nseg] = cls;
            ++a.nseg;
            prev = cls;
        }
    }
    a.kA = (int)kA;
    a.xbytes = (unsigned)(kPB * Z * pl.ntc * sizeof(float2));
    a.wbytesA = (unsigned)(kPB * kA * sizeof(float2));
    a.wbytesB = (unsigned)(kPB * (kb + 1) * sizeof(float2));
    a.bufstride = (unsigned)zth_bufstride(Z, pl.ntg, &a.woff);
    a.zoff = 2 * a.bufstride;
    MM_REQUIRE(a.bufstride % 128 == 0 && a.woff % 128 == 0 && a.wbytesA % 128 == 0,
               "TMA destinations of the z operator must be 128-byte aligned");
    MM_REQUIRE(a.xbytes <= a.woff, "z operator: the X box overruns its buffer");
    a.fresp = fresp;
    a.err = err;
    const size_t sm = 2 * (size_t)a.bufstride + zth_zero_bytes(Z);
    const int threads = zth_threads(Z, a.ntg);
    const void *fn = pl.nchunks > 1 ? (const void *)k_zth_apply<0, true>
                     : Z == 50     ? (const void *)k_zth_apply<50, false>
                                   : (const void *)k_zth_apply<0, false>;
    if (int rc = mm_set_smem(fn, sm)) return rc;
    int per_sm = 0;
    MM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, sm));
    if (per_sm < 1) per_sm = 1;
    const long long cap = (long long)mm_sm_count() * per_sm;
    const unsigned grid = (unsigned)(a.nitems < cap ? a.nitems : cap);
    void *args[] = {&S, &wA, &wB, &a};
    MM_CUDA_TRY(cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, sm, st));
    mm_launch_counter_add();
    return MM_OK;
}
