// 3-D local maxima and per-spot fit (restating mermake/maxima.cu and
// mermake/maxima.py:17-98, plus the hyb keep-filter of mermake/__main__.py:254-261).
//
// k_maxima   one thread per voxel: v > threshold (strict) and no neighbour in
//            the sphere 0 < |d|^2 <= delta^2 is larger (ties keep both);
//            neighbours reflect once about the first/last sample
//            (maxima.cu:19, 25-62).  A neighbour that is still outside after
//            the reflection (a dimension shorter than delta) is skipped; the
//            reference kernel reads out of bounds there.  Maxima are compacted
//            with one atomic per warp (ballot + popc) into a candidate list;
//            the count/collect double pass of the reference becomes one pass.
//            The image may be read through v -> v / div (IEEE, round to nearest)
//            -> -v, which reproduces the DAPI normalisation (v / rms, then
//            negated for minima, __main__.py:219-225) bit for bit without
//            writing the normalised volume.
// k_fit      one warp per spot: gathers the sphere |d|^2 <= delta_fit^2 in the
//            reference's (dz, dx, dy) order (first 600 in-range samples,
//            maxima.cu:148, 190-232) and forms every output of
//            delta_fit_cross_corr from moment sums (float32 on centre-shifted
//            values; the variances and covariances in double, the rest in float):
//              bg = min v;  centroid = sum (c+d)(v-bg) / sum (v-bg)  (fallback c);
//              hn = cov(v, G) / (std'(v) std(G));  a = cov(raw, G) / (std'(raw) std(G))
//            with std' = std, or 1 where std == 0 (maxima.cu:233-341).  std(G) == 0
//            (delta_fit = 0) gives NaN for hn and a, as in the reference.
//            In tile mode the row is kept only if overlap <= xc < xend-overlap and
//            the same for yc, then shifted by the tile origin (__main__.py:256-260).
#include <atomic>
#include <mutex>

#include "deconv.cuh"

namespace {

constexpr int kMaxDelta = 5;
constexpr int kSphereCap = 515;
__device__ char4 g_sphere[kMaxDelta + 1][kSphereCap];  // neighbour offsets, nearest first
__device__ int g_sphere_n[kMaxDelta + 1];
// fit samples: the sphere |d|^2 <= df^2 incl. the centre, in the reference's
// (dz, dx, dy) loop order (maxima.cu:190-193)
__device__ char4 g_fit_sphere[kMaxDelta + 1][kSphereCap];
__device__ int g_fit_sphere_n[kMaxDelta + 1];

// Host-side construction of the two tables (the same on every device).
struct SphereTables {
    char4 fit[kMaxDelta + 1][kSphereCap];
    int fit_n[kMaxDelta + 1];
    char4 nb[kMaxDelta + 1][kSphereCap];
    int nb_n[kMaxDelta + 1];
};

void build_sphere_tables(SphereTables &t) {
    for (int d = 0; d <= kMaxDelta; ++d) {
        int n = 0;
        for (int dz = -d; dz <= d; ++dz)
            for (int dx = -d; dx <= d; ++dx)
                for (int dy = -d; dy <= d; ++dy)
                    if (dz * dz + dx * dx + dy * dy <= d * d) t.fit[d][n++] = make_char4(dz, dx, dy, 0);
        t.fit_n[d] = n;
    }
    for (int d = 0; d <= kMaxDelta; ++d) {
        int n = 0;
        for (int r2 = 1; r2 <= d * d; ++r2)
            for (int dz = -d; dz <= d; ++dz)
                for (int dx = -d; dx <= d; ++dx)
                    for (int dy = -d; dy <= d; ++dy)
                        if (dz * dz + dx * dx + dy * dy == r2) t.nb[d][n++] = make_char4(dz, dx, dy, 0);
        t.nb_n[d] = n;
    }
}

struct Xform {
    float div;           // 0: none
    int neg;
    const float *divp;   // device divisor (overrides div when set)
};
__device__ __forceinline__ Xform xf_resolve(Xform t) {
    if (t.divp) t.div = *t.divp;
    return t;
}
__device__ __forceinline__ float xf(float v, Xform t) {
    if (t.div != 0.f) v = __fdiv_rn(v, t.div);
    return t.neg ? -v : v;
}

__device__ __forceinline__ int refl(int i, int n) { return i < 0 ? -i : (i >= n ? 2 * n - i - 2 : i); }

// A set of volumes: either one dense volume, or the yielded views of a tile batch.
struct Vols {
    const float *img;
    long long isz, isx, ivol;  // strides (y stride 1) and per-volume stride
    int Z, X, Y;               // single-volume dims
    int tiles;                 // 1: dims and raw from the tile geometry
    TileGeom g;
    int raw_kind;              // 0: f32 array, 1: u16 array, 2/3: tile raw view of a u16/f32 channel
    const void *raw;
    long long rsz, rsx, rvol;
    const void *chan;
    const float *flat;
    int band;                  // >= 0 (keep mode): only maxima within `band` of the kept region are sought
};

// The voxels of volume (tile) vi whose maxima are sought: the whole view, or
// in keep mode (mermake/__main__.py:254-256: ov <= xc, yc < extent - ov on the
// fitted centroid) the band the kept rows can come from.  A centroid is a
// weighted mean of the maximum's position plus offsets |d| <= delta_fit with
// non-negative weights (v - min v), or the position itself, so a maximum
// farther than delta_fit outside the kept region cannot be kept; `band`
// (delta_fit + 1) leaves a pixel for the rounding of the centroid.  The
// maxima tests and fits still read the whole view.
__device__ __forceinline__ void scan_range(const Vols &V, int X, int Y, int &xlo, int &xhi, int &ylo, int &yhi) {
    xlo = 0; xhi = X; ylo = 0; yhi = Y;
    if (V.band >= 0) {
        const int ov = V.g.ov;
        xlo = max(0, ov - V.band);
        ylo = max(0, ov - V.band);
        xhi = min(X, X - ov + V.band);
        yhi = min(Y, Y - ov + V.band);
        if (xhi < xlo) xhi = xlo;
        if (yhi < ylo) yhi = ylo;
    }
}

__device__ __forceinline__ void vol_dims(const Vols &V, int vi, int &X, int &Y, TileDesc &d) {
    if (V.tiles) {
        d = mm_tile_desc(V.g, V.g.t0 + vi);
        X = d.xend;
        Y = d.yend;
    } else {
        X = V.X;
        Y = V.Y;
    }
}

__device__ __forceinline__ float raw_at(const Vols &V, int vi, const TileDesc &d, int z, int x, int y) {
    if (V.raw_kind == 0)
        return static_cast<const float *>(V.raw)[vi * V.rvol + z * V.rsz + x * V.rsx + y];
    if (V.raw_kind == 1)
        return (float)static_cast<const uint16_t *>(V.raw)[vi * V.rvol + z * V.rsz + x * V.rsx + y];
    // tile_pad[zpad + z, x, y] after the flat is multiplied back (deconvolver.py:165-170)
    const TileGeom &g = V.g;
    int sx = mm_map_xy(x, d.x == 0, d.xd, g.P, g.ov);
    int sy = mm_map_xy(y, d.y == 0, d.yd, g.P, g.ov);
    if (sx < 0 || sy < 0) return 0.f;
    int gx = d.x0 + sx, gy = d.y0 + sy;
    const long long ci = z * g.isz + gx * g.isx + gy;
    float v = V.raw_kind == 2 ? (float)static_cast<const uint16_t *>(V.chan)[ci] : static_cast<const float *>(V.chan)[ci];
    if (V.flat) {
        float f = V.flat[gx * g.fsx + gy];
        // the reference's IEEE quotient: the batched fit reads the same raw
        // values as a fit on the materialised raw view
        v = __fdiv_rn(v, f);
        if (x >= d.xs && x < d.xs + d.xd && y >= d.ys && y < d.ys + d.yd) v = __fmul_rn(v, f);
    }
    return v;
}

// A warp per (z, x) row, lanes along y: every row index is split once, loads
// are coalesced, and each lane keeps kMaxY values of the row in flight.  The
// voxels above the threshold (a few percent) are queued per warp in shared
// memory across rows; whenever 32 are queued, their neighbourhoods are tested
// one voxel per lane (and the last partial round at the end), so the test
// runs with full warps.  Each voxel's neighbours are loaded kNbBatch at a
// time before they are compared, so a test waits for one load latency per
// batch instead of one per neighbour.
constexpr int kMaxWarps = 8;
// values in flight per lane: 8 for one sign, 4 for both (the queue holds < 32
// left over + one chunk of 32 values per lane and sign: 288 entries either way)
constexpr int kMaxY1 = 8, kMaxY2 = 4;
constexpr int kQueue = 32 * kMaxY1 + 32;
static_assert(2 * 32 * kMaxY2 + 32 <= kQueue, "queue too small for the two-sign pass");
constexpr int kNbBatch = 8;
constexpr int kFitU = 2;  // fit sample rounds whose loads are in flight together (4 costs occupancy)

// 1 when the voxel (raw value vr) is not below any in-range neighbour of
// (z, x, y) in the sphere of radius delta, compared as transformed values.
// The transform x -> x / div (div > 0, round to nearest) is monotone, so a
// neighbour whose raw value is not above the voxel's (not below, for the
// negated volume) cannot be above it after the transform either; only the
// others are transformed and compared exactly.  An interior voxel (delta
// from every face) reads its neighbours at fixed offsets, with no reflection.
__device__ __forceinline__ bool max_test(const float *__restrict__ img, const Vols &V, Xform t, int Z, int X,
                                         int Y, int z, int x, int y, float vr, const char4 *sph, int nn,
                                         int delta) {
    const float vt = xf(vr, t);
    const bool mono = t.div >= 0.f;
    const bool inner = z >= delta && z < Z - delta && x >= delta && x < X - delta && y >= delta && y < Y - delta;
    const float *c = img + z * V.isz + x * V.isx + y;
    for (int q0 = 0; q0 < nn; q0 += kNbBatch) {
        float nb[kNbBatch];
#pragma unroll
        for (int u = 0; u < kNbBatch; ++u) {
            nb[u] = NAN;  // no neighbour: never above
            const int q = q0 + u;
            if (q < nn) {
                const char4 o = sph[q];
                if (inner) {
                    nb[u] = c[o.x * V.isz + o.y * V.isx + o.z];
                } else {
                    const int nz = refl(z + o.x, Z), nx = refl(x + o.y, X), ny = refl(y + o.z, Y);
                    if (nz >= 0 && nz < Z && nx >= 0 && nx < X && ny >= 0 && ny < Y)
                        nb[u] = img[nz * V.isz + nx * V.isx + ny];
                }
            }
        }
        bool below = false;
#pragma unroll
        for (int u = 0; u < kNbBatch; ++u) {
            const bool may = t.neg ? nb[u] < vr : nb[u] > vr;
            if (!mono || may) below |= vt < xf(nb[u], t);
        }
        if (below) return false;
    }
    return true;
}

// appends the lanes with `hit` to cand (warp-aggregated atomic on count)
__device__ __forceinline__ void append_cand(bool hit, unsigned key, int y, int vi, unsigned lane,
                                            uint2 *__restrict__ cand, unsigned cap, unsigned *__restrict__ count) {
    const unsigned m = __ballot_sync(0xffffffffu, hit);
    if (m) {
        unsigned slot = 0;
        const int leader = __ffs(m) - 1;
        if ((int)lane == leader) slot = atomicAdd(count, __popc(m));
        slot = __shfl_sync(0xffffffffu, slot, leader) + __popc(m & ((1u << lane) - 1));
        if (hit && slot < cap) cand[slot] = make_uint2(key, (unsigned)y | ((unsigned)vi << 16));
    }
}

// tests the queue entries (k, y, v)[0, cnt), cnt <= 32, one per lane, and
// appends the maxima to cand, or to cand2 for the entries of the negated
// volume (bit 30 of y, queued by the two-sign pass)
__device__ __forceinline__ void test_round(const float *__restrict__ img, const Vols &V, Xform t, int Z, int X,
                                           int Y, const char4 *sph, int nn, int delta, const unsigned *k, const int *yq,
                                           const float *vq, int cnt, unsigned lane, int vi, uint2 *__restrict__ cand,
                                           unsigned cap, unsigned *__restrict__ count, uint2 *__restrict__ cand2,
                                           unsigned *__restrict__ count2, bool both) {
    bool is_max = false, neg = false;
    unsigned key = 0;
    int y = 0;
    if ((int)lane < cnt) {
        key = k[lane];
        const int e = yq[lane];
        neg = (e >> 30) & 1;
        y = e & 0x3fffffff;
        Xform ts = t;
        if (neg) ts.neg = !ts.neg;
        is_max = max_test(img, V, ts, Z, X, Y, (int)(key & 0xffffu), (int)(key >> 16), y, vq[lane], sph, nn, delta);
    }
    append_cand(is_max && !neg, key, y, vi, lane, cand, cap, count);
    if (both) append_cand(is_max && neg, key, y, vi, lane, cand2, cap, count2);
}

// BOTH: the maxima of the volume and of its negation in one pass (the DAPI
// block's two signs), into cand / count and cand2 / count2
template <bool BOTH>
__global__ void __launch_bounds__(32 * kMaxWarps)
k_maxima(Vols V, float th, int delta, Xform t, uint2 *__restrict__ cand, unsigned cap,
         unsigned *__restrict__ count, uint2 *__restrict__ cand2, unsigned *__restrict__ count2) {
    constexpr int kMaxY = BOTH ? kMaxY2 : kMaxY1;
    constexpr bool both = BOTH;
    __shared__ unsigned qk[kMaxWarps][kQueue];  // z | x << 16
    __shared__ int qy[kMaxWarps][kQueue];
    __shared__ float qv[kMaxWarps][kQueue];
    t = xf_resolve(t);
    const int vi = blockIdx.y;
    int X, Y;
    TileDesc d;
    vol_dims(V, vi, X, Y, d);
    const int Z = V.Z;
    int xlo, xhi, ylo, yhi;
    scan_range(V, X, Y, xlo, xhi, ylo, yhi);
    const int nx = xhi - xlo;
    const int rows = Z * nx;
    const float *img = V.img + vi * V.ivol;
    const int nn = g_sphere_n[delta];
    const char4 *sph = g_sphere[delta];
    const unsigned lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    // a raw value with |x| <= lo is below the threshold after x -> x / div
    // (either sign): its quotient is not computed
    const bool skip_small = t.div > 0.f && th > 0.f;
    // the two-sign pass with th >= 0 (not NaN): one queue round per voxel
    const bool excl = both && th >= 0.f;
    const float lo = skip_small ? th * t.div * (1.f - 0x1p-18f) : 0.f;
    unsigned *my_k = qk[warp];
    int *my_y = qy[warp];
    float *my_v = qv[warp];

    int qn = 0;
    for (int row = blockIdx.x * wpb + warp; row < rows; row += gridDim.x * wpb) {
        const int z = row / nx, x = xlo + (row - z * nx);
        const unsigned key = (unsigned)z | ((unsigned)x << 16);
        const float *rp = img + z * V.isz + x * V.isx;
        for (int y0 = ylo; y0 < yhi; y0 += 32 * kMaxY) {
            float vals[kMaxY];
#pragma unroll
            for (int k = 0; k < kMaxY; ++k) {
                const int y = y0 + 32 * k + (int)lane;
                vals[k] = y < yhi ? rp[y] : 0.f;
            }
            // queue the voxels above the threshold (maxima.cu:19; a NaN
            // threshold admits every voxel) whose y neighbours held by the
            // adjacent lanes are not larger: a larger neighbour in the sphere
            // fails the test anyway, so only the others need it
#pragma unroll
            for (int k = 0; k < kMaxY; ++k) {
                const int y = y0 + 32 * k + (int)lane;
                // a value below the threshold enters only as a y neighbour,
                // which it cannot be above, so 0 stands for it there
                const float v = skip_small && fabsf(vals[k]) <= lo ? 0.f : xf(vals[k], t);
                const float vl = __shfl_up_sync(0xffffffffu, v, 1), vr = __shfl_down_sync(0xffffffffu, v, 1);
                const bool hasl = delta > 0 && lane > 0 && y - 1 < yhi, hasr = delta > 0 && lane < 31 && y + 1 < yhi;
                if (excl) {
                    // both signs in one queue round: with th >= 0 a voxel
                    // other than NaN is above the threshold in one sign at
                    // most (a round with a lane above it in both takes the
                    // two-round path below)
                    const bool lo0 = (hasl && v < vl) || (hasr && v < vr);
                    const bool lo1 = (hasl && -v < -vl) || (hasr && -v < -vr);
                    const bool up0 = y < yhi && !(v <= th) && !lo0;
                    const bool up1 = y < yhi && !(-v <= th) && !lo1;
                    if (!__any_sync(0xffffffffu, up0 && up1)) {
                        const bool up = up0 || up1;
                        const unsigned m = __ballot_sync(0xffffffffu, up);
                        if (up) {
                            const int at = qn + __popc(m & ((1u << lane) - 1));
                            my_k[at] = key;
                            my_y[at] = y | ((int)up1 << 30);
                            my_v[at] = vals[k];
                        }
                        qn += __popc(m);
                        continue;
                    }
                }
                for (int sgn = 0; sgn < (both ? 2 : 1); ++sgn) {
                    const float sv = sgn ? -v : v;
                    const bool lower = (hasl && sv < (sgn ? -vl : vl)) || (hasr && sv < (sgn ? -vr : vr));
                    const bool up = y < yhi && !(sv <= th) && !lower;
                    const unsigned m = __ballot_sync(0xffffffffu, up);
                    if (up) {
                        const int at = qn + __popc(m & ((1u << lane) - 1));
                        my_k[at] = key;
                        my_y[at] = y | (sgn << 30);
                        my_v[at] = vals[k];  // raw: max_test transforms it
                    }
                    qn += __popc(m);
                }
            }
            __syncwarp();
            if (qn >= 32) {
                const int full = qn & ~31;
                for (int q0 = 0; q0 < full; q0 += 32)
                    test_round(img, V, t, Z, X, Y, sph, nn, delta, my_k + q0, my_y + q0, my_v + q0, 32, lane, vi, cand, cap,
                               count, cand2, count2, both);
                const int rem = qn - full;
                __syncwarp();
                // the remainder (< 32 entries from index full >= 32) to the front
                if ((int)lane < rem) {
                    my_k[lane] = my_k[full + lane];
                    my_y[lane] = my_y[full + lane];
                    my_v[lane] = my_v[full + lane];
                }
                __syncwarp();
                qn = rem;
            }
        }
    }
    if (qn > 0)
        test_round(img, V, t, Z, X, Y, sph, nn, delta, my_k, my_y, my_v, qn, lane, vi, cand, cap, count, cand2, count2,
                   both);
}

// Sums 16 per-lane values over the warp with a reduce-scatter (16 + 15
// shuffles instead of 16 x 5): afterwards lane 0 holds all 16 totals.
__device__ __forceinline__ void warp_sum16(float (&v)[16], unsigned lane) {
#pragma unroll
    for (int w = 8, off = 16; w >= 1; w >>= 1, off >>= 1) {
        const bool up = lane & off;
#pragma unroll
        for (int j = 0; j < w; ++j) {
            const float send = up ? v[j] : v[j + w];
            const float keep = up ? v[j + w] : v[j];
            v[j] = keep + __shfl_xor_sync(0xffffffffu, send, off);
        }
    }
    // lane L now holds in v[0] the sum over lanes sharing bit 0 of value
    // index idx(L) = bits 4..1 of L read as (b4 b3 b2 b1) -> 8*b4 + 4*b3 + 2*b2 + b1
    v[0] += __shfl_xor_sync(0xffffffffu, v[0], 1);
    const float mine = v[0];
#pragma unroll
    for (int i = 0; i < 16; ++i) {
        const int src = ((i >> 3) & 1) << 4 | ((i >> 2) & 1) << 3 | ((i >> 1) & 1) << 2 | (i & 1) << 1;
        v[i] = __shfl_sync(0xffffffffu, mine, src);
    }
}

// Per-spot fit.  Each lane sums its samples in float32 after shifting the
// image and raw values by the centre voxel's (every moment used below is
// shift-invariant, so the shift removes the cancellation); the warp adds the
// lanes' sums and lane 0 forms the statistics (the cancelling terms in double
// precision, the quotients and roots in float, as the reference).  The
// Gaussian weights depend only on the offset and the sigmas, so a block
// tabulates them once.
__global__ void __launch_bounds__(256, 4)
k_fit(Vols V, const uint2 *__restrict__ cand, const unsigned *__restrict__ ncand, unsigned cap, int delta_fit,
      float sigmaZ, float sigmaXY, Xform t, float *__restrict__ out, unsigned out_cap,
      unsigned *__restrict__ out_count, int keep_filter) {
    __shared__ float gtab[kSphereCap];
    __shared__ char4 otab[kSphereCap];
    t = xf_resolve(t);
    const unsigned lane = threadIdx.x & 31;
    const unsigned nc = min(*ncand, cap);
    const bool table = delta_fit <= kMaxDelta;
    const int side = 2 * delta_fit + 1;
    const int nsamp = table ? g_fit_sphere_n[delta_fit] : side * side * side;
    const int df2 = delta_fit * delta_fit;
    const float gz = 2 * sigmaZ * sigmaZ, gxy = 2 * sigmaXY * sigmaXY;
    if (table)
        for (int i = threadIdx.x; i < nsamp; i += blockDim.x) {
            const char4 o = g_fit_sphere[delta_fit][i];
            otab[i] = o;
            gtab[i] = expf(-(o.x * o.x / gz + o.y * o.y / gxy + o.z * o.z / gxy));
        }
    __syncthreads();
    for (unsigned s = (blockIdx.x * blockDim.x + threadIdx.x) / 32; s < nc; s += gridDim.x * blockDim.x / 32) {
        uint2 c = cand[s];
        const int z0 = c.x & 0xffff, x0 = c.x >> 16, y0 = c.y & 0xffff, vi = c.y >> 16;
        int X, Y;
        TileDesc d;
        vol_dims(V, vi, X, Y, d);
        const int Z = V.Z;
        const float *img = V.img + vi * V.ivol;
        const float cv = xf(img[z0 * V.isz + x0 * V.isx + y0], t);
        const float crw = raw_at(V, vi, d, z0, x0, y0);
        // n, sv, svv, sg, sgg, svg, sr, srr, srg, sdz, sdx, sdy, svdz, svdx, svdy, (unused)
        float acc[16];
#pragma unroll
        for (int i = 0; i < 16; ++i) acc[i] = 0.f;
        float vmin = 1e20f;
        auto add = [&](float v, float r, float g, int dz, int dx, int dy) {
            const float dv = v - cv, dr = r - crw;
            acc[0] += 1.f;
            acc[1] += dv; acc[2] += dv * dv;
            acc[3] += g; acc[4] += g * g; acc[5] += dv * g;
            acc[6] += dr; acc[7] += dr * dr; acc[8] += dr * g;
            acc[9] += (float)dz; acc[10] += (float)dx; acc[11] += (float)dy;
            acc[12] += dv * dz; acc[13] += dv * dx; acc[14] += dv * dy;
            vmin = fminf(vmin, v);
        };
        if (table) {
            // at most 515 samples, so the reference's cap of 600 (maxima.cu:194)
            // never binds: kFitU rounds of loads in flight, then their sums in
            // the same per-lane order as one round at a time.  A spot
            // delta_fit or more from every face samples without reflection.
            const bool inner = z0 >= delta_fit && z0 < Z - delta_fit && x0 >= delta_fit && x0 < X - delta_fit &&
                               y0 >= delta_fit && y0 < Y - delta_fit;
            for (int c0 = 0; c0 < nsamp; c0 += 32 * kFitU) {
                float vv[kFitU], rr[kFitU], gg[kFitU];
                char4 oo[kFitU];
                bool okk[kFitU];
#pragma unroll
                for (int u = 0; u < kFitU; ++u) {
                    const int ci = c0 + 32 * u + (int)lane;
                    okk[u] = false;
                    vv[u] = rr[u] = gg[u] = 0.f;
                    oo[u] = make_char4(0, 0, 0, 0);
                    if (ci < nsamp) {
                        const char4 o = otab[ci];
                        int zz = z0 + o.x, xx = x0 + o.y, yy = y0 + o.z;
                        if (!inner) {
                            zz = refl(zz, Z);
                            xx = refl(xx, X);
                            yy = refl(yy, Y);
                        }
                        if (inner || (zz >= 0 && zz < Z && xx >= 0 && xx < X && yy >= 0 && yy < Y)) {
                            okk[u] = true;
                            oo[u] = o;
                            vv[u] = xf(img[zz * V.isz + xx * V.isx + yy], t);
                            rr[u] = raw_at(V, vi, d, zz, xx, yy);
                            gg[u] = gtab[ci];
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < kFitU; ++u)
                    if (okk[u]) add(vv[u], rr[u], gg[u], oo[u].x, oo[u].y, oo[u].z);
            }
        }
        int taken = 0;  // in-range samples before this chunk (cap 600, maxima.cu:194)
        for (int c0 = 0; !table && c0 < nsamp && taken < 600; c0 += 32) {
            const int ci = c0 + (int)lane;
            int dz = 0, dx = 0, dy = 0;
            bool ok = false;
            int zz = 0, xx = 0, yy = 0;
            if (ci < nsamp) {
                dz = ci / (side * side) - delta_fit;
                dx = (ci / side) % side - delta_fit;
                dy = ci % side - delta_fit;
                const bool in = dz * dz + dx * dx + dy * dy <= df2;
                if (in) {
                    zz = refl(z0 + dz, Z);
                    xx = refl(x0 + dx, X);
                    yy = refl(y0 + dy, Y);
                    ok = zz >= 0 && zz < Z && xx >= 0 && xx < X && yy >= 0 && yy < Y;
                }
            }
            const unsigned m = __ballot_sync(0xffffffffu, ok);
            const int rank = taken + __popc(m & ((1u << lane) - 1));
            taken += __popc(m);
            if (ok && rank < 600) {
                const float v = xf(img[zz * V.isz + xx * V.isx + yy], t);
                const float r = raw_at(V, vi, d, zz, xx, yy);
                add(v, r, expf(-(dz * dz / gz + dx * dx / gxy + dy * dy / gxy)), dz, dx, dy);
            }
        }
        warp_sum16(acc, lane);
        for (int o = 16; o > 0; o >>= 1) vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
        if (lane != 0 || acc[0] == 0.f) continue;
        // Only the variances and covariances cancel (mean square minus squared
        // mean of the shifted values): they are formed in double precision; the
        // quotients, roots and the centroid in float, as the reference does.
        const double N = acc[0], invN = 1.0 / N;
        const double mg = acc[3] * invN, mv = acc[1] * invN, mr = acc[6] * invN;
        const float varg = (float)fmax(acc[4] * invN - mg * mg, 0.0);
        const float varv = (float)fmax(acc[2] * invN - mv * mv, 0.0);
        const float varr = (float)fmax(acc[7] * invN - mr * mr, 0.0);
        const float covg_v = (float)(acc[5] * invN - mv * mg);
        const float covg_r = (float)(acc[8] * invN - mr * mg);
        const float stdg = sqrtf(varg);
        float stdv = sqrtf(varv), stdr = sqrtf(varr);
        if (!(stdv > 0.f)) stdv = 1.f;
        if (!(stdr > 0.f)) stdr = 1.f;
        const float hn = covg_v / (stdv * stdg);
        const float a = covg_r / (stdr * stdg);
        // sum (c + d)(v - bg) / sum (v - bg), with v - bg = dv + (cv - bg)
        const float shift = cv - vmin;
        const float sw = acc[1] + acc[0] * shift;
        float zc, xc, yc;
        if (sw > 0.f) {
            zc = z0 + (acc[12] + shift * acc[9]) / sw;
            xc = x0 + (acc[13] + shift * acc[10]) / sw;
            yc = y0 + (acc[14] + shift * acc[11]) / sw;
        } else {
            zc = z0; xc = x0; yc = y0;
        }
        float row[8];
        row[0] = zc; row[1] = xc; row[2] = yc; row[3] = vmin;
        row[4] = a;
        row[5] = crw;
        row[6] = hn;
        row[7] = cv;
        unsigned o;
        if (keep_filter) {
            const int ov = V.g.ov;
            if (!(row[1] >= ov && row[2] >= ov && row[1] < (float)(X - ov) && row[2] < (float)(Y - ov))) continue;
            row[1] += (float)(d.x - ov);
            row[2] += (float)(d.y - ov);
            o = atomicAdd(out_count, 1u);
        } else {
            o = s;
        }
        if (o < out_cap)
            for (int k = 0; k < 8; ++k) out[(long long)o * 8 + k] = row[k];
    }
}

__global__ void k_note_overflow(const unsigned *__restrict__ ncand, unsigned cap, unsigned *__restrict__ overflow) {
    unsigned n = *ncand;
    if (n > cap) atomicMax(overflow, n);
}

}  // namespace

int mm_launch_note_overflow(const unsigned *ncand, unsigned cap, unsigned *overflow, cudaStream_t st) {
    k_note_overflow<<<1, 1, 0, st>>>(ncand, cap, overflow);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

// Uploads the neighbour and fit tables to the current device once.  Callers on
// several host threads may race here for a new device: the per-device flag is
// atomic and the upload runs under a lock, so exactly one of them uploads and
// the others wait for it.
int mm_maxima_ensure_init(cudaStream_t st) {
    static std::atomic<int> done_dev[64];
    static std::mutex mu;
    int dev = 0;
    MM_CUDA_TRY(cudaGetDevice(&dev));
    MM_REQUIRE(dev >= 0 && dev < 64, "device index %d out of range", dev);
    if (done_dev[dev].load(std::memory_order_acquire)) return MM_OK;
    std::lock_guard<std::mutex> lock(mu);
    if (done_dev[dev].load(std::memory_order_relaxed)) return MM_OK;
    static SphereTables tab;
    static bool built = false;
    if (!built) {
        build_sphere_tables(tab);
        built = true;
    }
    MM_CUDA_TRY(cudaMemcpyToSymbolAsync(g_fit_sphere, tab.fit, sizeof(tab.fit), 0, cudaMemcpyHostToDevice, st));
    MM_CUDA_TRY(cudaMemcpyToSymbolAsync(g_fit_sphere_n, tab.fit_n, sizeof(tab.fit_n), 0, cudaMemcpyHostToDevice, st));
    MM_CUDA_TRY(cudaMemcpyToSymbolAsync(g_sphere, tab.nb, sizeof(tab.nb), 0, cudaMemcpyHostToDevice, st));
    MM_CUDA_TRY(cudaMemcpyToSymbolAsync(g_sphere_n, tab.nb_n, sizeof(tab.nb_n), 0, cudaMemcpyHostToDevice, st));
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    done_dev[dev].store(1, std::memory_order_release);
    return MM_OK;
}



static Vols make_vols(const MaximaArgs &a) {
    Vols V = {};
    V.img = a.img; V.isz = a.isz; V.isx = a.isx; V.ivol = a.ivol;
    V.Z = a.Z; V.X = a.X; V.Y = a.Y;
    V.tiles = a.tiles != nullptr;
    if (a.tiles) V.g = *a.tiles;
    V.raw_kind = a.raw_kind; V.raw = a.raw; V.rsz = a.rsz; V.rsx = a.rsx; V.rvol = a.rvol;
    V.chan = a.chan; V.flat = a.flat;
    V.band = (a.tiles && a.keep_filter) ? a.delta_fit + 1 : -1;
    return V;
}

static dim3 maxima_grid(const MaximaArgs &a) {
    // a warp per (z, x) row, 8 rows per CTA, the CTAs of all volumes together
    // about four rounds of the SMs' resident CTAs (four per SM), so that each
    // warp's queue of candidates persists over many rows (measured on fov3c:
    // 4, 8, 16 CTAs per SM gave 50.10, 49.38, 49.25 ms per FOV)
    long long rows = (long long)a.Z * (a.tiles ? (long long)a.tiles->P : (long long)a.X);
    long long gx = (rows + 7) / 8;
    const long long cap = (long long)mm_sm_count() * 16 / (a.nvol > 0 ? a.nvol : 1);
    if (gx > cap) gx = cap;
    if (gx < 1) gx = 1;
    return dim3((unsigned)gx, a.nvol);
}

// Launches maxima + fit.  cand/ncand: scratch list and its device counter;
// out/out_count: rows and their device counter (keep mode) -- counters are
// zeroed here.
int mm_launch_maxima_fit(const MaximaArgs &a, uint2 *cand, unsigned cand_cap, unsigned *ncand, float *out,
                         unsigned out_cap, unsigned *out_count, int zero_out_count, cudaStream_t st) {
    const Vols V = make_vols(a);
    Xform t = {a.div, a.neg, a.divp};
    MM_CUDA_TRY(cudaMemsetAsync(ncand, 0, sizeof(unsigned), st));
    if (out_count && zero_out_count) MM_CUDA_TRY(cudaMemsetAsync(out_count, 0, sizeof(unsigned), st));
    k_maxima<false><<<maxima_grid(a), 32 * kMaxWarps, 0, st>>>(V, a.th, a.delta, t, cand, cand_cap, ncand, nullptr,
                                                                nullptr);
    MM_CHECK_LAUNCH();
    k_fit<<<mm_sm_count() * 8, 256, 0, st>>>(V, cand, ncand, cand_cap, a.delta_fit, a.sigmaZ, a.sigmaXY, t, out, out_cap,
                                   out_count, a.keep_filter);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

// Maxima + fit of the volume (a.neg is the plus sign) and of its negation, the
// maxima in one pass: candidates of the plus sign in cand[0, cap), of the minus
// sign in cand[cap, 2 cap), counted in ncand_plus / ncand_minus (zeroed here);
// fit rows i of each sign into out_plus / out_minus (no keep filter).
int mm_launch_maxima_fit_pm(const MaximaArgs &a, uint2 *cand, unsigned cap, unsigned *ncand_plus,
                            unsigned *ncand_minus, float *out_plus, unsigned cap_plus, float *out_minus,
                            unsigned cap_minus, cudaStream_t st) {
    const Vols V = make_vols(a);
    Xform tp = {a.div, a.neg, a.divp}, tm = {a.div, !a.neg, a.divp};
    MM_CUDA_TRY(cudaMemsetAsync(ncand_plus, 0, sizeof(unsigned), st));
    MM_CUDA_TRY(cudaMemsetAsync(ncand_minus, 0, sizeof(unsigned), st));
    k_maxima<true><<<maxima_grid(a), 32 * kMaxWarps, 0, st>>>(V, a.th, a.delta, tp, cand, cap, ncand_plus, cand + cap,
                                                               ncand_minus);
    MM_CHECK_LAUNCH();
    k_fit<<<mm_sm_count() * 8, 256, 0, st>>>(V, cand, ncand_plus, cap, a.delta_fit, a.sigmaZ, a.sigmaXY, tp, out_plus, cap_plus,
                                   nullptr, 0);
    MM_CHECK_LAUNCH();
    k_fit<<<mm_sm_count() * 8, 256, 0, st>>>(V, cand + cap, ncand_minus, cap, a.delta_fit, a.sigmaZ, a.sigmaXY, tm, out_minus,
                                   cap_minus, nullptr, 0);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

// ---------------------------------------------------------------------------
// find_local_maxima without allocation (mm_find_local_maxima_noalloc).
//
// Some callers cannot allocate device memory while they run: code executing
// inside another framework's memory pool or under a fixed device-memory
// budget, and real-time loops that must not take cudaMalloc's implicit device
// synchronisation.  For them the candidate list and its counter live in this
// file-scope array, which every GPU that loads it keeps until the process
// exits.  The CUDA runtime loads a module lazily by default (at the first use
// of one of its kernels or symbols on a device), so the device memory of the
// array is reserved, and the neighbour tables uploaded, by the first call on
// each device (or by the first use of any maxima kernel there): that first
// call allocates and synchronises the device.  Make it at start-up, before any
// stream capture and before the code that must not allocate.  Host code may
// not use the array's name as a device address, so that first call fetches
// the address with cudaGetSymbolAddress, with its device current.  Every call
// shares the array: calls whose work overlaps on the GPU (other streams, other
// host threads) race on it and must be serialised by the caller.
// ---------------------------------------------------------------------------
#define MM_NOALLOC_MAX_VOXELS (1u << 21)  // 2,097,152 voxels -> 16 MiB of candidates
#define MM_NOALLOC_HEAD 256               // counter block before the candidate list
static __device__ __align__(256) unsigned char g_noalloc_scratch[MM_NOALLOC_HEAD +
                                                                 sizeof(uint2) * MM_NOALLOC_MAX_VOXELS];

namespace {
std::mutex g_noalloc_mu;
void *g_noalloc_ptr[64] = {};
}  // namespace

extern "C" int mm_find_local_maxima_noalloc(const float *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                                            const void *raw, int raw_dtype, int64_t rsz, int64_t rsx,
                                            float threshold, int delta, int delta_fit, float sigmaZ, float sigmaXY,
                                            float norm_div, int negate, float *out, uint32_t out_cap,
                                            uint32_t *count, void *stream) {
    MM_REQUIRE(image && raw && count, "null argument");
    MM_REQUIRE(delta <= 5, "Delta must be an less than or equal to 5 due to MAX_KERNEL_POINTS");
    MM_REQUIRE(delta >= 0 && delta_fit >= 0, "negative delta");
    MM_REQUIRE(raw_dtype == 0 || raw_dtype == 1, "raw_dtype must be 0 (float32) or 1 (uint16)");
    MM_REQUIRE(Z >= 0 && X >= 0 && Y >= 0 && Z < 65536 && X < 65536 && Y < 65536, "dimensions must be in [0, 65536)");
    const unsigned long long nvox = (unsigned long long)Z * X * Y;
    MM_REQUIRE(nvox <= MM_NOALLOC_MAX_VOXELS,
               "volume of %llu voxels exceeds the %u-voxel limit of mm_find_local_maxima_noalloc "
               "(its candidate list is a fixed static array); use mm_find_local_maxima",
               nvox, MM_NOALLOC_MAX_VOXELS);
    *count = 0;
    if (nvox == 0) return MM_OK;
    cudaStream_t st = (cudaStream_t)stream;
    int dev = 0;
    MM_CUDA_TRY(cudaGetDevice(&dev));
    MM_REQUIRE(dev >= 0 && dev < 64, "device index %d out of range", dev);
    void *base = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_noalloc_mu);
        if (!g_noalloc_ptr[dev]) {
            void *p = nullptr;
            MM_CUDA_TRY(cudaGetSymbolAddress(&p, g_noalloc_scratch));
            int rc = mm_maxima_ensure_init(st);  // neighbour-offset table, launched once per device
            if (rc) return rc;
            g_noalloc_ptr[dev] = p;
        }
        base = g_noalloc_ptr[dev];
    }
    unsigned *ncand = static_cast<unsigned *>(base);
    uint2 *cand = reinterpret_cast<uint2 *>(static_cast<unsigned char *>(base) + MM_NOALLOC_HEAD);
    MaximaArgs a = {};
    a.img = image; a.isz = isz; a.isx = isx; a.ivol = 0;
    a.Z = Z; a.X = X; a.Y = Y; a.nvol = 1;
    a.tiles = nullptr;
    a.raw_kind = raw_dtype; a.raw = raw; a.rsz = rsz; a.rsx = rsx; a.rvol = 0;
    a.th = threshold; a.delta = delta; a.delta_fit = delta_fit;
    a.sigmaZ = sigmaZ; a.sigmaXY = sigmaXY;
    a.div = norm_div; a.divp = nullptr; a.neg = negate; a.keep_filter = 0;
    // the launcher clears the candidate counter (the array keeps the last call's contents)
    int rc = mm_launch_maxima_fit(a, cand, MM_NOALLOC_MAX_VOXELS, ncand, out, out_cap, nullptr, 0, st);
    if (rc) return rc;
    MM_CUDA_TRY(cudaMemcpyAsync(count, ncand, sizeof(unsigned), cudaMemcpyDeviceToHost, st));
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    return *count > out_cap ? MM_EOVERFLOW : MM_OK;
}
