// z operator with a z kernel per tile (a PSF per tile, the multi-PSF grid),
// the matrix of each (tile, frequency) formed in registers.  S holds the
// launch's nt tiles from its own tile 0; tile t takes the kernel of spectrum
// t0 + t (kernel 0 for all when npsf == 1).
//
// The map of the z step (zop.cu) is Y[i] = sum_j M[i][j] X[j] with, for
// 1 <= zpad <= Z - 1,
//
//   M[i][j] = w[i - j] + [1 <= j <= zpad] w[i + j] + [Z-1-zpad <= j <= Z-2] w[i + j - 2Z + 2]
//
// (the planes the reflection padding copies, mermake/deconvolver.py:145-148),
// w the tile's own z kernel.  The direct sum over the padded planes (k_zconv)
// does Zp products per output; the matrix does Z.  Here no matrix is shared
// between tiles, so a thread owns five rows of one tile and forms them from
// two register rings of five along j (zop_tma.cu has the scheme): the direct
// value w[i - j] and the reflected value of the column's class (w[i + j],
// w[i + j - 2Z + 2], their sum, or zero), one complex add per entry.
//
// A persistent CTA takes items of pb frequencies (pb = 16 or 8: rows of 128
// or 64 bytes) x a chunk of tiles, the items of a chunk in frequency order
// (neighbouring CTAs read neighbouring pieces of the same rows).  Two
// producer warps copy, with cp.async from all lanes, the chunk's X rows and
// each tile's kernel rows w[-kA .. 2Z-2] (rows outside the padded depth are
// zero rows written once) into one of two buffers, whose "full" mbarrier
// completes as they land; the compute warps release it on its "empty"
// mbarrier.  Every wait is bounded.
//
// Two variants.  For zpad = Z - 1 (FULL) the column classes are fixed
// (column 0, columns 1 .. Z - 2, column Z - 1) and the middle columns' sum
// is formed as the ring is loaded (two rows per value): no hB rows, no zero
// rows and no barrier between the compute warps, one tile per item, so a
// CTA is small (51 KB at Z = 40) and four share an SM.  The generic variant
// checks the class per column and reads the sum from hB rows that its compute
// warps write per item into one of two regions, meeting on an mbarrier.
#include <cuda.h>

#include "deconv.cuh"

namespace {

constexpr int kTI = 5;     // rows of a thread, the unroll of the column loop
constexpr int kTiles = 5;  // tiles per item at most
constexpr int kBufs = 2;   // operand buffers (double buffered)
constexpr size_t kSmemMax = 112 * 1024;
constexpr int kFullTiles = 1;  // tiles per item of the zpad = Z - 1 variant
constexpr unsigned kWaitPolls = 1u << 24;

__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
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
__device__ __forceinline__ void copy16s(unsigned dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

__device__ __forceinline__ float2 cfma(float2 a, float2 b, float2 c) {
    c.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, c.x));
    c.y = fmaf(a.x, b.y, fmaf(a.y, b.x, c.y));
    return c;
}

struct ZptArgs {
    int Z, Zp, nt, t0, npsf;
    long long plane, wstride;
    int ntpi;              // tiles per item (chunk), at most kTiles
    int ngroups, nitems;   // frequency groups of pb; items = tile chunks x groups, chunk-major
    int kA;                // staged row of w[0]: 2Z - 2 rounded up to a multiple of 4
    int wrows;             // kernel rows per tile: kA + 2Z - 1
    unsigned xbytes;       // X bytes of a buffer (ntpi x Z x pb float2); the tiles' kernel rows follow
    unsigned bufstride;    // bytes per buffer
    unsigned hoff, hbytes; // two regions of hB rows (ntpi x (2Z - 1)) after the buffers
    unsigned zoff;         // the zero rows (2Z + 3) after them
    int nseg, segj[6], segc[6];  // column segments of one reflection class (zop_tma.cu)
    const float *fresp;
    unsigned *err;
};

constexpr int kMaxZ = 80;
constexpr int kProd = 2;  // producer warps
constexpr int kMaxCompute = 256;  // compute threads per CTA at most
constexpr int zpt_block(int Z, int ntpi, int pb) { return (pb * (Z / kTI) * ntpi + 31) / 32 * 32 + 32 * kProd; }

// A thread's five rows of one tile: the direct ring rT (slot q mod 5 holds
// w[i0 + q - j] as j advances), the reflected ring rH (slot q mod 5 holds the
// reflected value at i0 + q + j), and the accumulators.  W points at the
// thread's frequency of the tile's staged kernel rows (row kb = w[0]); hrow is
// the row offset of the reflected source of the current column's class.
struct Rings {
    float2 rT[kTI], rH[kTI], acc[kTI];
};
template <int PB>
__device__ __forceinline__ void ring_start(Rings &R, const float2 *W, int i0, int kb, int hrow) {
#pragma unroll
    for (int q = 1; q < kTI; ++q) R.rT[q] = W[(i0 + q + kb) * PB];
#pragma unroll
    for (int q = 0; q < kTI - 1; ++q) R.rH[q] = W[(i0 + q + hrow) * PB];
    R.rT[0] = R.rH[kTI - 1] = make_float2(0.f, 0.f);
}
// column j, u = j mod 5
template <int PB>
__device__ __forceinline__ void col_u(Rings &R, const float2 *W, const float2 *xr, int i0, int j, int kb, int hrow,
                                      int u) {
    R.rT[(kTI - u) % kTI] = W[(i0 - j + kb) * PB];
    R.rH[(u + kTI - 1) % kTI] = W[(i0 + j + kTI - 1 + hrow) * PB];
    const float2 x = xr[(size_t)j * PB];
#pragma unroll
    for (int q = 0; q < kTI; ++q) R.acc[q] = cfma(cadd(R.rT[(q - u + kTI) % kTI], R.rH[(q + u) % kTI]), x, R.acc[q]);
}
template <int PB, int U>
__device__ __forceinline__ void col(Rings &R, const float2 *W, const float2 *xr, int i0, int j, int kb, int hrow) {
    col_u<PB>(R, W, xr, i0, j, kb, hrow, U);
}
// a column that starts a class: the reflected ring from its source
template <int PB, int U>
__device__ __forceinline__ void reload(Rings &R, const float2 *W, int i0, int j, int hrow) {
#pragma unroll
    for (int q = 0; q < kTI - 1; ++q) R.rH[(q + U) % kTI] = W[(i0 + j + q + hrow) * PB];
}

// a column of the class with both reflections, its reflected value summed
// from the two kernel rows (kb: w[0], ko: w[-(2Z-2)])
template <int PB, int U>
__device__ __forceinline__ void col2(Rings &R, const float2 *W, const float2 *xr, int i0, int j, int kb, int ko) {
    R.rT[(kTI - U) % kTI] = W[(i0 - j + kb) * PB];
    const int h = i0 + j + kTI - 1;
    R.rH[(U + kTI - 1) % kTI] = cadd(W[(h + kb) * PB], W[(h + ko) * PB]);
    const float2 x = xr[(size_t)j * PB];
#pragma unroll
    for (int q = 0; q < kTI; ++q) R.acc[q] = cfma(cadd(R.rT[(q - U + kTI) % kTI], R.rH[(q + U) % kTI]), x, R.acc[q]);
}
template <int PB, int U>
__device__ __forceinline__ void reload2(Rings &R, const float2 *W, int i0, int j, int kb, int ko) {
#pragma unroll
    for (int q = 0; q < kTI - 1; ++q) R.rH[(q + U) % kTI] = cadd(W[(i0 + j + q + kb) * PB], W[(i0 + j + q + ko) * PB]);
}

template <int ZC, bool FULL, int PB>
__global__ void __launch_bounds__(kMaxCompute + 32 * kProd, 2)
k_zpt_apply(float2 *__restrict__ S, const float2 *__restrict__ w, const ZptArgs a) {
    constexpr int kPB = PB;          // frequencies per item
    constexpr int kRowB = kPB * 8;   // bytes of a staged row
    constexpr int kLPR = kPB / 2;    // copying lanes per row (16 bytes each)
    constexpr int kRPS = 32 / kLPR;  // rows a warp's copy instruction covers
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ __align__(8) uint64_t full[kBufs], empty[kBufs], hdone[2];
    const int Z = ZC > 0 ? ZC : a.Z;
    const int nig = Z / kTI;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ncw = (kPB * nig * a.ntpi + 31) / 32;  // compute warps; the warps after them copy
    const int kb = a.kA, ko = kb - (2 * Z - 2);
    if (tid == 0) {
        for (int b = 0; b < kBufs; ++b) {
            mbar_init(&full[b], 32 * kProd);
            mbar_init(&empty[b], ncw);
        }
        for (int b = 0; b < 2; ++b) mbar_init(&hdone[b], ncw);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    {
        // the zero rows, and the staged kernel rows that lie outside the
        // padded depth (as a TMA box of the (Zp, plane) kernel would fill
        // them): the same rows of every item, written once
        if (!FULL) {
            float2 *zr = reinterpret_cast<float2 *>(smem + a.zoff);
            for (int e = tid; e < (2 * Z + 3) * kPB; e += blockDim.x) zr[e] = make_float2(0.f, 0.f);
        }
        for (int e = tid; e < kBufs * a.ntpi * a.wrows * kPB; e += blockDim.x) {
            const int r = (e / kPB) % a.wrows, s = r - kb;
            if (s < -a.Zp || s >= a.Zp) {
                const int tb = e / (kPB * a.wrows);  // buffer * ntpi + tile
                const int b = tb / a.ntpi, tl = tb - b * a.ntpi;
                reinterpret_cast<float2 *>(smem + (size_t)b * a.bufstride + a.xbytes)[((size_t)tl * a.wrows + r) * kPB +
                                                                                      e % kPB] = make_float2(0.f, 0.f);
            }
        }
    }
    __syncthreads();

    if (warp >= ncw) {
        // ---- producer warps (kProd): 16-byte copies from all lanes, warp pw
        // copying tiles pw, pw + kProd, ...; the buffer's "full" barrier
        // completes when every lane's copies have landed ----
        const int pw = warp - ncw;
        const int rlo = max(kb - a.Zp, 0), rhi = min(a.wrows, kb + a.Zp);  // staged rows inside the padded depth
        int buf = 0, ph = 0;
        for (int item = blockIdx.x, it = 0; item < a.nitems; item += gridDim.x, ++it) {
            const bool ok = it < kBufs || mbar_wait(&empty[buf], ph ^ 1);
            if (!__all_sync(0xffffffffu, ok)) {
                if (lane == 0) atomicOr(a.err, 4u);
                break;
            }
            const int c = item / a.ngroups, grp = item - c * a.ngroups;
            const int tb0 = c * a.ntpi, ntl = min(a.ntpi, a.nt - tb0);
            const long long pc = (long long)grp * kPB + 2 * (lane % kLPR);  // this lane's 16 bytes of the row
            if (pc < a.plane) {
                // lane: row lane / kLPR (+ kRPS per step), piece lane % kLPR
                const long long step = kRPS * a.plane;
                const unsigned xb = smem_u32(smem + (size_t)buf * a.bufstride) + lane * 16;
                const unsigned wbase = xb + a.xbytes;
                for (int tl = pw; tl < ntl; tl += kProd) {
                    // X: rows (tile, plane) of kRowB bytes
                    const float2 *xs = S + ((long long)(tb0 + tl) * Z + lane / kLPR) * a.plane + pc;
                    unsigned xd = xb + tl * Z * kRowB;
                    for (int r = lane / kLPR; r < Z; r += kRPS, xs += step, xd += 512) copy16s(xd, xs);
                    // the tile's kernel rows: staged row r is w[r - kA + Zp] below
                    // kA and w[r - kA] from there
                    const float2 *wt = w + (long long)(a.npsf == 1 ? 0 : a.t0 + tb0 + tl) * a.wstride + pc;
                    const unsigned wd = wbase + tl * a.wrows * kRowB;
                    int r = rlo + lane / kLPR;
                    const float2 *src = wt + (long long)(r - kb + a.Zp) * a.plane;
                    unsigned dst = wd + rlo * kRowB;
                    for (; r < kb; r += kRPS, src += step, dst += 512) copy16s(dst, src);
                    r = kb + lane / kLPR;
                    src = wt + (long long)(lane / kLPR) * a.plane;
                    dst = wd + kb * kRowB;
                    for (; r < rhi; r += kRPS, src += step, dst += 512) copy16s(dst, src);
                }
            }
            asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(&full[buf])) : "memory");
            if (++buf == kBufs) buf = 0, ph ^= 1;
        }
        // no copy may still be landing when the CTA exits
        asm volatile("cp.async.wait_all;" ::: "memory");
        return;
    }

    const int p = tid % kPB, rr = tid / kPB;
    const int ig = rr % nig, tl = rr / nig;
    const int i0 = ig * kTI;
    int buf = 0, ph = 0;
    for (int item = blockIdx.x, it = 0; item < a.nitems; item += gridDim.x, ++it) {
        if (!mbar_wait(&full[buf], ph)) {
            atomicOr(a.err, 1u);
            return;
        }
        const int c = item / a.ngroups, grp = item - c * a.ngroups;
        const int tb0 = c * a.ntpi, ntl = min(a.ntpi, a.nt - tb0);
        const unsigned char *b = smem + (size_t)buf * a.bufstride;
        // hB[s] = w[s] + w[s - 2Z + 2], s < 2Z - 1, of each tile, into region
        // it & 1.  Every warp has left item it - 2 (the region's last user)
        // once all have met on hdone for item it - 1.
        float2 *hb = reinterpret_cast<float2 *>(smem + a.hoff + (it & 1) * a.hbytes);
        if (!FULL) {
            const float2 *wb = reinterpret_cast<const float2 *>(b + a.xbytes);
            for (int t2 = 0; t2 < ntl; ++t2) {
                const float2 *wt = wb + (size_t)t2 * a.wrows * kPB;
                float2 *ht = hb + (size_t)t2 * (2 * Z - 1) * kPB;
                for (int e = tid; e < (2 * Z - 1) * kPB; e += ncw * 32) ht[e] = cadd(wt[kb * kPB + e], wt[ko * kPB + e]);
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&hdone[it & 1]);
            if (!mbar_wait(&hdone[it & 1], (it >> 1) & 1)) {
                atomicOr(a.err, 2u);
                return;
            }
        }
        const bool mine = tl < ntl;
        float2 acc[kTI];
#pragma unroll
        for (int q = 0; q < kTI; ++q) acc[q] = make_float2(0.f, 0.f);
        if (mine) {
            const float2 *W = reinterpret_cast<const float2 *>(b + a.xbytes) + (size_t)tl * a.wrows * kPB;
            const float2 *xr = reinterpret_cast<const float2 *>(b) + (size_t)tl * Z * kPB + p;
            // the reflected ring's row offset per class: the hB rows and the
            // zero rows are addressed from this tile's kernel rows
            const int wpos = (int)((const unsigned char *)W - smem);
            const int rowb = (int)(kPB * sizeof(float2));
            const int hrowB = ((int)((const unsigned char *)(hb + (size_t)tl * (2 * Z - 1) * kPB) - smem) - wpos) / rowb;
            const int zrow = ((int)a.zoff - wpos) / rowb;
            Rings R;
#pragma unroll
            for (int q = 0; q < kTI; ++q) R.acc[q] = make_float2(0.f, 0.f);
            const float2 *Wp = W + p;
            if (FULL) {
                // zpad = Z - 1: column 0 takes w[i + j - 2Z + 2], columns
                // 1 .. Z - 2 the sum w[i + j] + w[i + j - 2Z + 2] (two loads
                // and an add per column), column Z - 1 w[i + j]
                ring_start<PB>(R, Wp, i0, kb, ko);
                col<PB, 0>(R, Wp, xr, i0, 0, kb, ko);
                reload2<PB, 1>(R, Wp, i0, 1, kb, ko);
                col2<PB, 1>(R, Wp, xr, i0, 1, kb, ko);
                col2<PB, 2>(R, Wp, xr, i0, 2, kb, ko);
                col2<PB, 3>(R, Wp, xr, i0, 3, kb, ko);
                col2<PB, 4>(R, Wp, xr, i0, 4, kb, ko);
                for (int j0 = kTI; j0 < Z - kTI; j0 += kTI) {
                    col2<PB, 0>(R, Wp, xr, i0, j0, kb, ko);
                    col2<PB, 1>(R, Wp, xr, i0, j0 + 1, kb, ko);
                    col2<PB, 2>(R, Wp, xr, i0, j0 + 2, kb, ko);
                    col2<PB, 3>(R, Wp, xr, i0, j0 + 3, kb, ko);
                    col2<PB, 4>(R, Wp, xr, i0, j0 + 4, kb, ko);
                }
                const int j0 = Z - kTI;
                col2<PB, 0>(R, Wp, xr, i0, j0, kb, ko);
                col2<PB, 1>(R, Wp, xr, i0, j0 + 1, kb, ko);
                col2<PB, 2>(R, Wp, xr, i0, j0 + 2, kb, ko);
                col2<PB, 3>(R, Wp, xr, i0, j0 + 3, kb, ko);
                reload<PB, 4>(R, Wp, i0, j0 + 4, kb);
                col<PB, 4>(R, Wp, xr, i0, j0 + 4, kb, kb);
            } else {
                auto seg_row = [&](int k) {
                    const int cls = a.segc[k];
                    return cls == 0 ? kb : cls == 1 ? ko : cls == 2 ? hrowB : zrow;
                };
                int sk = 0, hrow = seg_row(0), jnext = a.nseg > 1 ? a.segj[1] : Z;
                ring_start<PB>(R, Wp, i0, kb, hrow);
                for (int j0 = 0; j0 < Z; j0 += kTI) {
#pragma unroll
                    for (int u = 0; u < kTI; ++u) {
                        const int j = j0 + u;
                        if (j == jnext) {
                            ++sk;
                            hrow = seg_row(sk);
                            jnext = sk + 1 < a.nseg ? a.segj[sk + 1] : Z;
#pragma unroll
                            for (int q = 0; q < kTI - 1; ++q) R.rH[(q + u) % kTI] = Wp[(i0 + j + q + hrow) * kPB];
                        }
                        col_u<PB>(R, Wp, xr, i0, j, kb, hrow, u);
                    }
                }
            }
#pragma unroll
            for (int q = 0; q < kTI; ++q) acc[q] = R.acc[q];
        }
        // the operands are in registers: release the buffer before the stores
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[buf]);
        const long long pg = (long long)grp * kPB + p;
        if (mine && pg < a.plane) {
            const float f = a.fresp ? a.fresp[pg] : 1.f;
            const long long t = tb0 + tl;
#pragma unroll
            for (int q = 0; q < kTI; ++q) S[(t * Z + i0 + q) * a.plane + pg] = cscale(acc[q], f);
        }
        if (++buf == kBufs) buf = 0, ph ^= 1;
    }
}

int zpt_ka(int Z) { return (2 * Z - 2 + 3) & ~3; }
size_t zpt_zero_bytes(int Z, int pb) { return ((size_t)(2 * Z + 3) * pb * sizeof(float2) + 127) & ~(size_t)127; }
size_t zpt_bufstride(int Z, int ntpi, int pb, unsigned *xbytes) {
    const size_t xb = ((size_t)ntpi * Z * pb * sizeof(float2) + 127) & ~(size_t)127;
    const size_t wb = (size_t)ntpi * (zpt_ka(Z) + 2 * Z - 1) * pb * sizeof(float2);
    if (xbytes) *xbytes = (unsigned)xb;
    return (xb + wb + 127) & ~(size_t)127;
}
size_t zpt_hbytes(int Z, int ntpi, int pb) {
    return ((size_t)ntpi * (2 * Z - 1) * pb * sizeof(float2) + 127) & ~(size_t)127;
}
// shared memory of a CTA: the buffers, and for the generic variant the two hB
// regions and the zero rows (the variant for zpad = Z - 1 sums the two
// reflections as it reads them and has no column without one)
size_t zpt_smem(int Z, int ntpi, int pb, bool full) {
    const size_t bufs = kBufs * zpt_bufstride(Z, ntpi, pb, nullptr);
    return full ? bufs : bufs + 2 * zpt_hbytes(Z, ntpi, pb) + zpt_zero_bytes(Z, pb);
}
// zpad = Z - 1 (Z >= 10): the column classes at compile time
bool zpt_full(int Z, int zpad) { return zpad == Z - 1 && Z >= 2 * kTI; }
// Frequencies per item (pb), tiles per item and buffers, for two CTAs per SM
// (0 tiles: none fit).  The operands are rows of pb x 8 bytes at the
// spectrum's plane stride, and wider rows read DRAM faster: on 100 tiles of
// Z = 40, P = 478 (a PSF per tile) the z step took 8.0 ms with rows of 32
// bytes (five tiles per item), 7.1 ms with 64 (three) and 6.68 ms with 128
// (one); the copies alone took 6.2 ms at 32 bytes.  So pb is 16 where one
// tile fits two buffers, else 8.  The variant for zpad = Z - 1 then takes one
// tile per item and two buffers: small CTAs, four per SM at Z = 40, 5.39 ms
// on that workload, against 5.81 ms with four buffers (two CTAs per SM) and
// 6.68 ms for the generic variant's hB rows and per-item barrier.  The
// generic variant takes two buffers of as many tiles as fit.
int zpt_config(int Z, bool full, int *pb) {
    for (int w = 16; w >= 8; w /= 2) {
        if (full) {
            if (zpt_smem(Z, kFullTiles, w, true) <= kSmemMax && w * (Z / kTI) * kFullTiles <= kMaxCompute) {
                *pb = w;
                return kFullTiles;
            }
            continue;
        }
        for (int n = kTiles; n >= 1; --n)
            if (zpt_smem(Z, n, w, false) <= kSmemMax && w * (Z / kTI) * n <= kMaxCompute) {
                *pb = w;
                return n;
            }
    }
    return 0;
}

}  // namespace

int mm_zpt_supported(int Z, int zpad, int nt, long long plane) {
    if (Z < kTI || Z % kTI != 0 || Z > kMaxZ || zpad < 1 || zpad > Z - 1 || nt < 1 || plane % 2 != 0) return 0;
    int pb;
    return zpt_config(Z, zpt_full(Z, zpad), &pb) > 0;
}

int mm_launch_zpt_apply(float2 *S, const float2 *w, long long wstride, int Z, int zpad, int Zp, long long plane,
                        int t0, int nt, int npsf, const float *fresp, unsigned *err, cudaStream_t st) {
    MM_REQUIRE(Zp == Z + 2 * zpad && mm_zpt_supported(Z, zpad, nt, plane),
               "z operator (kernel per tile) does not take Z %d, zpad %d", Z, zpad);
    MM_REQUIRE(((uintptr_t)S & 15) == 0 && ((uintptr_t)w & 15) == 0, "spectra must be 16-byte aligned");
    ZptArgs a = {};
    a.Z = Z;
    a.Zp = Zp;
    a.nt = nt;
    a.t0 = t0;
    a.npsf = npsf;
    a.plane = plane;
    a.wstride = wstride;
    const bool full = zpt_full(Z, zpad);
    int pb = 0;
    a.ntpi = zpt_config(Z, full, &pb);
    a.ngroups = (int)((plane + pb - 1) / pb);
    const long long nitems = (long long)a.ngroups * ((nt + a.ntpi - 1) / a.ntpi);
    MM_REQUIRE(nitems < (1LL << 31), "z operator: too many items");
    a.nitems = (int)nitems;
    a.kA = zpt_ka(Z);
    a.wrows = a.kA + 2 * Z - 1;
    a.bufstride = (unsigned)zpt_bufstride(Z, a.ntpi, pb, &a.xbytes);
    a.hoff = kBufs * a.bufstride;
    a.hbytes = (unsigned)zpt_hbytes(Z, a.ntpi, pb);
    a.zoff = a.hoff + 2 * a.hbytes;
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
    a.fresp = fresp;
    a.err = err;
    const size_t sm = zpt_smem(Z, a.ntpi, pb, full);
    const int threads = zpt_block(Z, a.ntpi, pb);
    const void *fn;
    if (pb == 16)
        fn = !full     ? (const void *)k_zpt_apply<0, false, 16>
             : Z == 40 ? (const void *)k_zpt_apply<40, true, 16>
             : Z == 50 ? (const void *)k_zpt_apply<50, true, 16>
                       : (const void *)k_zpt_apply<0, true, 16>;
    else
        fn = full ? (const void *)k_zpt_apply<0, true, 8> : (const void *)k_zpt_apply<0, false, 8>;
    if (int rc = mm_set_smem(fn, sm)) return rc;
    int per_sm = 0;
    MM_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, threads, sm));
    if (per_sm < 1) per_sm = 1;
    const long long cap = (long long)mm_sm_count() * per_sm;
    const unsigned grid = (unsigned)(a.nitems < cap ? a.nitems : cap);
    void *args[] = {&S, &w, &a};
    MM_CUDA_TRY(cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, sm, st));
    mm_launch_counter_add();
    return MM_OK;
}
