// Drift alignment of maxima point sets (restating mermake/align.py:12-129 and
// mermake/utils.py:10-36).
//
// Aligner(X_ref, resc, trim, th): rows whose last column exceeds th are kept
// (align.py:121-129), the first three columns are the points.  The reference
// image is the set of voxels round(X/resc) after trimming `trim` voxels from
// the x and y extremes (align.py:37-59); get_best_translation_points splats the
// moving set the same way, takes the argmax of the full linear correlation of
// the two 0/1 images (utils.fftconvolve, align.py:107-111), and refines it with
// five nearest-neighbour rounds at radii linspace(resc, target, 5)
// (align.py:61-77).
//
// The correlation of two 0/1 images at shift s is the number of voxel pairs
// (i in moving, j in reference) with i - j = s, so it is computed exactly as a
// histogram of pair differences instead of an FFT (whose float result rounds
// to the same integers); the argmax takes the first maximal index in C order,
// as argmax does.  Nearest neighbours are brute force in double precision,
// ties to the lowest reference index.
#include <limits.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "deconv.cuh"

// per-aligner scratch for the moving sets, grown on demand
struct MmDriftWork {
    float *pts = nullptr;
    int *iv = nullptr, *keep = nullptr, *small = nullptr, *vox = nullptr;
    size_t cap = 0;
    unsigned char *grid = nullptr;
    size_t grid_bytes = 0;
    int *hist = nullptr;
    size_t hist_bytes = 0;
    int *h_small = nullptr;
};

// Uniform cell grid of the reference points for the nearest-neighbour
// refinement: cells of edge cs >= the largest match radius, so every point
// within the radius of a query lies in the query's cell or its neighbours.
struct MmCellGrid {
    int dims[3] = {0, 0, 0};
    float lo[3] = {0, 0, 0};
    float cs = 0;
    int *start = nullptr;     // device, cells + 1: first sorted point of each cell
    float *pts = nullptr;     // device, n x 3: points sorted by cell (index order within a cell)
    int *idx = nullptr;       // device, n: original index of each sorted point
    double *state = nullptr;  // device: shift (3), integer-shift flag, matched count
    double *parts = nullptr;  // device: per-block partial sums of a refinement round
};

struct mm_aligner {
    int n;            // reference points kept by the threshold
    float *pts;       // device, n x 3
    int nvox;         // unique reference voxels
    int *vox;         // device, nvox x 3 (z, x, y)
    int shape[3];     // reference image shape
    int resc, trim;
    float th;         // NaN: no threshold
    MmDriftWork w;
    MmCellGrid cg;
};

namespace {

// stable compaction of the rows whose last column exceeds th (all rows when th is NaN)
__global__ void k_compact_rows(const float *__restrict__ X, int n, int cols, long long ld, float th,
                               float *__restrict__ out, int *__restrict__ nout) {
    __shared__ int warp_tot[32];
    __shared__ int base;
    if (threadIdx.x == 0) base = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int r0 = 0; r0 < n; r0 += blockDim.x) {
        const int r = r0 + threadIdx.x;
        bool keep = false;
        if (r < n) {
            const float last = X[r * ld + cols - 1];
            keep = isnan(th) ? true : (last > th);
        }
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) warp_tot[warp] = __popc(m);
        __syncthreads();
        int before = 0;
        for (int w = 0; w < warp; ++w) before += warp_tot[w];
        const int pos = base + before + __popc(m & ((1u << lane) - 1));
        if (keep)
            for (int c = 0; c < 3; ++c) out[pos * 3 + c] = X[r * ld + c];
        __syncthreads();
        if (threadIdx.x == 0) {
            int t = 0;
            for (int w = 0; w < nw; ++w) t += warp_tot[w];
            base += t;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) *nout = base;
}

// round(X / resc) half to even (np.round of a float32 quotient), min/max per axis
__global__ void k_round_minmax(const float *__restrict__ pts, const int *__restrict__ n_p, int resc,
                               int *__restrict__ iv, int *__restrict__ mm) {
    const int n = *n_p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int c = 0; c < 3; ++c) {
            const int v = (int)rintf(__fdiv_rn(pts[i * 3 + c], (float)resc));
            iv[i * 3 + c] = v;
            atomicMin(&mm[c], v);
            atomicMax(&mm[3 + c], v);
        }
}

// keep = all(Xm + n <= X <= XM - n) with n = (0, trim, trim); max over kept
__global__ void k_trim_max(const int *__restrict__ iv, const int *__restrict__ n_p, const int *__restrict__ mm,
                           int trim, int *__restrict__ keep, int *__restrict__ kmax) {
    const int n = *n_p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        bool k = true;
        for (int c = 0; c < 3; ++c) {
            const int t = c == 0 ? 0 : trim;
            const int v = iv[i * 3 + c];
            k = k && v <= mm[3 + c] - t && v >= mm[c] + t;
        }
        keep[i] = k;
        if (k)
            for (int c = 0; c < 3; ++c) atomicMax(&kmax[c], iv[i * 3 + c]);
    }
}

// imf[tuple(X.T)] = 1: mark the voxels (negative indices wrap, as NumPy's do)
__global__ void k_mark(const int *__restrict__ iv, const int *__restrict__ keep, const int *__restrict__ n_p,
                       const int *__restrict__ shape, unsigned char *__restrict__ grid) {
    const int n = *n_p;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (!keep[i]) continue;
        long long lin = 0;
        bool ok = true;
        for (int c = 0; c < 3; ++c) {
            int v = iv[i * 3 + c];
            if (v < 0) v += shape[c];
            ok = ok && v >= 0 && v < shape[c];
            lin = lin * shape[c] + v;
        }
        if (ok) grid[lin] = 1;
    }
}

// unique voxels of the grid, any order
__global__ void k_grid_list(const unsigned char *__restrict__ grid, long long total, int s1, int s2,
                            int *__restrict__ vox, int *__restrict__ nvox) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        if (!grid[i]) continue;
        const int p = atomicAdd(nvox, 1);
        vox[p * 3 + 0] = (int)(i / ((long long)s1 * s2));
        vox[p * 3 + 1] = (int)((i / s2) % s1);
        vox[p * 3 + 2] = (int)(i % s2);
    }
}

// correlation as a histogram of pair differences: output index i - j + (sb - 1)
__global__ void k_pair_hist(const int *__restrict__ a, const int *__restrict__ na, const int *__restrict__ b,
                            int nb, int c0, int c1, int c2, int o1, int o2, int *__restrict__ hist) {
    const long long total = (long long)(*na) * nb;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < total;
         p += (long long)gridDim.x * blockDim.x) {
        const int i = (int)(p / nb), j = (int)(p % nb);
        const int z = a[i * 3 + 0] - b[j * 3 + 0] + c0;
        const int x = a[i * 3 + 1] - b[j * 3 + 1] + c1;
        const int y = a[i * 3 + 2] - b[j * 3 + 2] + c2;
        atomicAdd(&hist[((long long)z * o1 + x) * o2 + y], 1);
    }
}

// first index of the maximum: max of (count << 32 | ~index)
__global__ void k_argmax(const int *__restrict__ hist, long long total, unsigned long long *__restrict__ best) {
    unsigned long long b = 0;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const unsigned long long key = ((unsigned long long)(unsigned)hist[i] << 32) | (unsigned)(~(unsigned)i);
        b = key > b ? key : b;
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long t = __shfl_xor_sync(0xffffffffu, b, o);
        b = t > b ? t : b;
    }
    if ((threadIdx.x & 31) == 0) atomicMax(best, b);
}

// five nearest-neighbour refinements in one CTA (align.py:61-77).  t0: the
// coarse shift (integer, times resc).  out: tzxy (3 floats) and the count of
// the last round.
// Nearest-neighbour refinement (align.py:55-76, five rounds with radii
// np.linspace(resc, target, 5)), one round per launch over many CTAs.  Each
// moving point X - shift looks for its nearest reference point among the
// cells around it (distance in double, ties to the lower reference index:
// the point a brute-force search over all references would pick); if it lies
// within the round's radius, X - R (float32) is added in double.  Blocks
// write partial sums that k_refine_update adds in a fixed order.
constexpr int kRefineThreads = 256;
constexpr int kRefineMaxBlocks = 304;

__global__ void k_refine_init(const unsigned long long *__restrict__ best, int o1, int o2, int sb0, int sb1,
                              int sb2, int resc, double *__restrict__ state) {
    const unsigned long long b = *best;
    const long long idx = (long long)(~(unsigned)(b & 0xffffffffu));
    const long long z = idx / ((long long)o1 * o2), x = (idx / o2) % o1, y = idx % o2;
    state[0] = (double)((z - sb0 + 1) * resc);
    state[1] = (double)((x - sb1 + 1) * resc);
    state[2] = (double)((y - sb2 + 1) * resc);
    state[3] = 1.0;  // the shift is still the integer coarse one
    state[4] = 0.0;
}

__global__ void __launch_bounds__(kRefineThreads)
k_refine_round(const float *__restrict__ X, const int *__restrict__ n_p, const float *__restrict__ gp,
               const int *__restrict__ gidx, const int *__restrict__ gstart, int gd0, int gd1, int gd2, float lo0,
               float lo1, float lo2, float cs, int reach, double dist_th, const double *__restrict__ state,
               double *__restrict__ parts) {
    const int n = *n_p;
    const bool tint = state[3] != 0.0;
    const double tz0 = state[0], tz1 = state[1], tz2 = state[2];
    const float t0 = (float)tz0, t1 = (float)tz1, t2 = (float)tz2;
    double sz = 0, sx = 0, sy = 0, cnt = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        // XT = X - tzxy: float64 against the integer coarse shift, float32 after
        double q0, q1, q2;
        if (tint) {
            q0 = (double)X[i * 3] - tz0;
            q1 = (double)X[i * 3 + 1] - tz1;
            q2 = (double)X[i * 3 + 2] - tz2;
        } else {
            q0 = (double)(X[i * 3] - t0);
            q1 = (double)(X[i * 3 + 1] - t1);
            q2 = (double)(X[i * 3 + 2] - t2);
        }
        const int c0 = (int)floor((q0 - lo0) / cs), c1 = (int)floor((q1 - lo1) / cs), c2 = (int)floor((q2 - lo2) / cs);
        double bd = 1e300;
        int bj = 0x7fffffff, bk = -1;
        for (int a = max(c0 - reach, 0); a <= min(c0 + reach, gd0 - 1); ++a)
            for (int b = max(c1 - reach, 0); b <= min(c1 + reach, gd1 - 1); ++b) {
                const int lc = max(c2 - reach, 0), hc = min(c2 + reach, gd2 - 1);
                if (lc > hc) continue;
                const long long row = ((long long)a * gd1 + b) * gd2;
                const int e0 = gstart[row + lc], e1 = gstart[row + hc + 1];
                for (int k = e0; k < e1; ++k) {
                    const double d0 = q0 - gp[k * 3], d1 = q1 - gp[k * 3 + 1], d2 = q2 - gp[k * 3 + 2];
                    const double d = d0 * d0 + d1 * d1 + d2 * d2;
                    const int j = gidx[k];
                    if (d < bd || (d == bd && j < bj)) {
                        bd = d;
                        bj = j;
                        bk = k;
                    }
                }
            }
        if (bk >= 0 && sqrt(bd) < dist_th) {
            // X_ - X_ref_ in float32, summed in double
            sz += (double)(X[i * 3] - gp[bk * 3]);
            sx += (double)(X[i * 3 + 1] - gp[bk * 3 + 1]);
            sy += (double)(X[i * 3 + 2] - gp[bk * 3 + 2]);
            cnt += 1;
        }
    }
    sz = mm_block_sum(sz);
    __syncthreads();
    sx = mm_block_sum(sx);
    __syncthreads();
    sy = mm_block_sum(sy);
    __syncthreads();
    cnt = mm_block_sum(cnt);
    if (threadIdx.x == 0) {
        parts[blockIdx.x * 4 + 0] = sz;
        parts[blockIdx.x * 4 + 1] = sx;
        parts[blockIdx.x * 4 + 2] = sy;
        parts[blockIdx.x * 4 + 3] = cnt;
    }
}

__global__ void k_refine_update(const double *__restrict__ parts, int nblocks, double *__restrict__ state,
                                int last, float *__restrict__ out, int *__restrict__ npts) {
    if (threadIdx.x != 0) return;
    double s[4] = {0, 0, 0, 0};
    for (int b = 0; b < nblocks; ++b)
        for (int k = 0; k < 4; ++k) s[k] += parts[b * 4 + k];
    state[4] = s[3];
    if (s[3] > 0) {  // else: no point kept, the shift stays (align.py:72-74)
        for (int k = 0; k < 3; ++k) state[k] = (double)(float)(s[k] / s[3]);
        state[3] = 0.0;
    }
    if (last) {
        for (int k = 0; k < 3; ++k) out[k] = (float)state[k];
        npts[0] = (int)state[4];
        npts[1] = (int)state[3];
    }
}

struct Splat {
    int shape[3];
    int nvox;
};

// threshold + splat of a point set; fills vox (device, capacity n) and returns shape/nvox on the host
int splat(const float *pts_dev, const int *n_dev, int n_host, int resc, int trim, int *iv, int *keep, int *mm,
          int *kmax, unsigned char **grid_buf, size_t *grid_bytes, int *vox, int *nvox_dev, int *h_small,
          Splat *out, cudaStream_t st) {
    const int init[9] = {INT_MAX, INT_MAX, INT_MAX, INT_MIN, INT_MIN, INT_MIN, INT_MIN, INT_MIN, INT_MIN};
    MM_CUDA_TRY(cudaMemcpyAsync(mm, init, sizeof(int) * 6, cudaMemcpyHostToDevice, st));
    MM_CUDA_TRY(cudaMemcpyAsync(kmax, init + 6, sizeof(int) * 3, cudaMemcpyHostToDevice, st));
    const int g = n_host > 0 ? mm_cdiv(n_host, 256) : 1;
    k_round_minmax<<<g, 256, 0, st>>>(pts_dev, n_dev, resc, iv, mm);
    MM_CHECK_LAUNCH();
    k_trim_max<<<g, 256, 0, st>>>(iv, n_dev, mm, trim, keep, kmax);
    MM_CHECK_LAUNCH();
    MM_CUDA_TRY(cudaMemcpyAsync(h_small, kmax, sizeof(int) * 3, cudaMemcpyDeviceToHost, st));
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    if (h_small[0] == INT_MIN) {  // nothing survives the trim: a (1,1,1) zero image (align.py:51-53)
        out->shape[0] = out->shape[1] = out->shape[2] = 1;
        out->nvox = 0;
        return MM_OK;
    }
    for (int c = 0; c < 3; ++c) out->shape[c] = h_small[c] + 1;
    MM_REQUIRE(out->shape[0] > 0 && out->shape[1] > 0 && out->shape[2] > 0, "negative splat extent");
    const size_t total = (size_t)out->shape[0] * out->shape[1] * out->shape[2];
    if (*grid_bytes < total) {
        if (*grid_buf) cudaFree(*grid_buf);
        *grid_buf = nullptr;
        *grid_bytes = 0;
        MM_CUDA_TRY(cudaMalloc(grid_buf, total));
        *grid_bytes = total;
    }
    MM_CUDA_TRY(cudaMemsetAsync(*grid_buf, 0, total, st));
    MM_CUDA_TRY(cudaMemcpyAsync(mm, out->shape, sizeof(int) * 3, cudaMemcpyHostToDevice, st));
    k_mark<<<g, 256, 0, st>>>(iv, keep, n_dev, mm, *grid_buf);
    MM_CHECK_LAUNCH();
    MM_CUDA_TRY(cudaMemsetAsync(nvox_dev, 0, sizeof(int), st));
    const int gg = (int)((total + 255) / 256 < 152 * 16 ? (total + 255) / 256 : 152 * 16);
    k_grid_list<<<gg, 256, 0, st>>>(*grid_buf, (long long)total, out->shape[1], out->shape[2], vox, nvox_dev);
    MM_CHECK_LAUNCH();
    MM_CUDA_TRY(cudaMemcpyAsync(h_small, nvox_dev, sizeof(int), cudaMemcpyDeviceToHost, st));
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    out->nvox = h_small[0];
    return MM_OK;
}

int work_reserve(MmDriftWork &w, size_t n) {
    if (!w.h_small) MM_CUDA_TRY(cudaMallocHost(&w.h_small, 64 * sizeof(int)));
    if (!w.small) MM_CUDA_TRY(cudaMalloc(&w.small, 64 * sizeof(int)));
    if (n < 16) n = 16;
    if (w.cap >= n) return MM_OK;
    cudaFree(w.pts);
    cudaFree(w.iv);
    cudaFree(w.keep);
    cudaFree(w.vox);
    w.pts = nullptr; w.iv = w.keep = w.vox = nullptr;
    w.cap = 0;
    MM_CUDA_TRY(cudaMalloc(&w.pts, n * 3 * sizeof(float)));
    MM_CUDA_TRY(cudaMalloc(&w.iv, n * 3 * sizeof(int)));
    MM_CUDA_TRY(cudaMalloc(&w.keep, n * sizeof(int)));
    MM_CUDA_TRY(cudaMalloc(&w.vox, n * 3 * sizeof(int)));
    w.cap = n;
    return MM_OK;
}

void work_free(MmDriftWork &w) {
    cudaFree(w.pts); cudaFree(w.iv); cudaFree(w.keep); cudaFree(w.vox); cudaFree(w.small);
    cudaFree(w.grid); cudaFree(w.hist);
    if (w.h_small) cudaFreeHost(w.h_small);
    w = MmDriftWork();
}

// small-buffer slots (ints) inside Work::small
enum { SM_N = 0, SM_MM = 1, SM_KMAX = 8, SM_NVOX = 12, SM_NPTS = 14, SM_BEST = 16, SM_OUT = 20 };

// The cell grid of the reference points (host-side counting sort, points in
// index order within a cell), and the refinement's small device state.
int cell_grid_build(MmCellGrid &g, const float *pts_dev, int n, float cs_min, cudaStream_t st) {
    std::vector<float> p((size_t)n * 3);
    MM_CUDA_TRY(cudaMemcpyAsync(p.data(), pts_dev, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, st));
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    float lo[3], hi[3];
    for (int c = 0; c < 3; ++c) lo[c] = hi[c] = p[c];
    for (int i = 0; i < n; ++i)
        for (int c = 0; c < 3; ++c) {
            lo[c] = std::min(lo[c], p[i * 3 + c]);
            hi[c] = std::max(hi[c], p[i * 3 + c]);
        }
    // cells of edge >= cs_min, coarser if the box would need more than 2^24 cells
    double cs = cs_min;
    for (;;) {
        double cells = 1;
        for (int c = 0; c < 3; ++c) cells *= std::floor((hi[c] - lo[c]) / cs) + 1;
        if (cells <= (double)(1 << 24)) break;
        cs *= 1.5;
    }
    g.cs = (float)cs;
    for (int c = 0; c < 3; ++c) {
        g.lo[c] = lo[c];
        g.dims[c] = (int)std::floor((hi[c] - lo[c]) / g.cs) + 1;
    }
    const long long ncell = (long long)g.dims[0] * g.dims[1] * g.dims[2];
    std::vector<int> cell(n), start(ncell + 1, 0), idx(n);
    for (int i = 0; i < n; ++i) {
        int k[3];
        for (int c = 0; c < 3; ++c)
            k[c] = std::min(g.dims[c] - 1, std::max(0, (int)std::floor(((double)p[i * 3 + c] - g.lo[c]) / g.cs)));
        cell[i] = (int)(((long long)k[0] * g.dims[1] + k[1]) * g.dims[2] + k[2]);
        start[cell[i] + 1]++;
    }
    for (long long c = 0; c < ncell; ++c) start[c + 1] += start[c];
    std::vector<int> fill(start.begin(), start.end() - 1);
    std::vector<float> sp((size_t)n * 3);
    for (int i = 0; i < n; ++i) {
        const int at = fill[cell[i]]++;
        idx[at] = i;
        for (int c = 0; c < 3; ++c) sp[at * 3 + c] = p[i * 3 + c];
    }
    MM_CUDA_TRY(cudaMalloc(&g.start, sizeof(int) * (ncell + 1)));
    MM_CUDA_TRY(cudaMalloc(&g.pts, sizeof(float) * 3 * n));
    MM_CUDA_TRY(cudaMalloc(&g.idx, sizeof(int) * n));
    MM_CUDA_TRY(cudaMalloc(&g.state, sizeof(double) * 8));
    MM_CUDA_TRY(cudaMalloc(&g.parts, sizeof(double) * 4 * kRefineMaxBlocks));
    MM_CUDA_TRY(cudaMemcpyAsync(g.start, start.data(), sizeof(int) * (ncell + 1), cudaMemcpyHostToDevice, st));
    MM_CUDA_TRY(cudaMemcpyAsync(g.pts, sp.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice, st));
    MM_CUDA_TRY(cudaMemcpyAsync(g.idx, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, st));
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    return MM_OK;
}

void cell_grid_free(MmCellGrid &g) {
    cudaFree(g.start); cudaFree(g.pts); cudaFree(g.idx); cudaFree(g.state); cudaFree(g.parts);
    g = MmCellGrid();
}

}  // namespace

extern "C" int mm_aligner_create(const float *X_ref, int n, int cols, int64_t ld, float th, int resc, int trim,
                                 mm_aligner **out, void *stream) {
    MM_REQUIRE(out && (X_ref || n == 0), "null argument");
    MM_REQUIRE(n >= 0 && cols >= 3 && ld >= cols, "point rows need at least 3 columns");
    MM_REQUIRE(resc >= 1 && trim >= 0, "resc must be >= 1 and trim >= 0");
    cudaStream_t st = (cudaStream_t)stream;
    mm_aligner *S = new mm_aligner();
    S->pts = nullptr;
    S->vox = nullptr;
    S->resc = resc;
    S->trim = trim;
    S->th = th;
    MmDriftWork &w = S->w;
    int rc = work_reserve(w, (size_t)n);
    if (rc) { work_free(w); delete S; return rc; }
    int nkeep = 0;
    if (n > 0) {
        k_compact_rows<<<1, 1024, 0, st>>>(X_ref, n, cols, ld, th, w.pts, w.small + SM_N);
        if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(w.h_small, w.small + SM_N, sizeof(int),
                                                                 cudaMemcpyDeviceToHost, st) != cudaSuccess ||
            cudaStreamSynchronize(st) != cudaSuccess) {
            work_free(w); delete S;
            mm_set_error("aligner: compaction failed");
            return MM_EDEVICE;
        }
        mm_launch_counter_add();
        nkeep = w.h_small[0];
    }
    if (nkeep == 0) {
        work_free(w); delete S;
        mm_set_error("No points left after thresholding; cannot build KDTree. Check your data and/or threshold value.");
        return MM_EINVAL;
    }
    S->n = nkeep;
    Splat sp;
    rc = splat(w.pts, w.small + SM_N, nkeep, resc, trim, w.iv, w.keep, w.small + SM_MM, w.small + SM_KMAX, &w.grid,
               &w.grid_bytes, w.vox, w.small + SM_NVOX, w.h_small, &sp, st);
    if (rc) { work_free(w); delete S; return rc; }
    for (int c = 0; c < 3; ++c) S->shape[c] = sp.shape[c];
    S->nvox = sp.nvox;
    // keep the reference points and voxels in buffers of their own
    S->pts = nullptr;
    S->vox = nullptr;
    if (cudaMalloc(&S->pts, sizeof(float) * 3 * nkeep) != cudaSuccess ||
        cudaMalloc(&S->vox, sizeof(int) * 3 * (sp.nvox > 0 ? sp.nvox : 1)) != cudaSuccess) {
        cudaGetLastError();
        cudaFree(S->pts); cudaFree(S->vox); work_free(w); delete S;
        mm_set_error("aligner: out of device memory");
        return MM_ENOMEM;
    }
    cudaMemcpyAsync(S->pts, w.pts, sizeof(float) * 3 * nkeep, cudaMemcpyDeviceToDevice, st);
    if (sp.nvox) cudaMemcpyAsync(S->vox, w.vox, sizeof(int) * 3 * sp.nvox, cudaMemcpyDeviceToDevice, st);
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    if ((rc = cell_grid_build(S->cg, S->pts, nkeep, (float)resc, st))) {
        cell_grid_free(S->cg); cudaFree(S->pts); cudaFree(S->vox); work_free(w); delete S;
        return rc;
    }
    *out = S;
    return MM_OK;
}

extern "C" int mm_aligner_destroy(mm_aligner *S) {
    if (!S) return MM_OK;
    cudaDeviceSynchronize();
    cudaFree(S->pts);
    cudaFree(S->vox);
    work_free(S->w);
    cell_grid_free(S->cg);
    delete S;
    return MM_OK;
}

extern "C" int mm_aligner_info(const mm_aligner *S, int *n_points, int *n_voxels, int *shape3) {
    MM_REQUIRE(S, "null aligner");
    if (n_points) *n_points = S->n;
    if (n_voxels) *n_voxels = S->nvox;
    if (shape3)
        for (int c = 0; c < 3; ++c) shape3[c] = S->shape[c];
    return MM_OK;
}

extern "C" int mm_aligner_translation(mm_aligner *S, const float *X, int n, int cols, int64_t ld, float target,
                                      float *tzxy, int *npts, void *stream) {
    MM_REQUIRE(S && tzxy && npts && (X || n == 0), "null argument");
    MM_REQUIRE(n >= 0 && cols >= 3 && ld >= cols, "point rows need at least 3 columns");
    const mm_aligner &A = *S;
    MmDriftWork &w = S->w;
    cudaStream_t st = (cudaStream_t)stream;
    int rc = work_reserve(w, (size_t)(n > A.nvox ? n : A.nvox));
    if (rc) return rc;
    // get_best_translation_points: threshold on the last column (align.py:97-101)
    int nm = 0;
    if (n > 0) {
        k_compact_rows<<<1, 1024, 0, st>>>(X, n, cols, ld, A.th, w.pts, w.small + SM_N);
        MM_CHECK_LAUNCH();
        MM_CUDA_TRY(cudaMemcpyAsync(w.h_small, w.small + SM_N, sizeof(int), cudaMemcpyDeviceToHost, st));
        MM_CUDA_TRY(cudaStreamSynchronize(st));
        nm = w.h_small[0];
    } else {
        MM_CUDA_TRY(cudaMemsetAsync(w.small + SM_N, 0, sizeof(int), st));
    }
    Splat sp = {{1, 1, 1}, 0};
    if (nm > 0) {
        rc = splat(w.pts, w.small + SM_N, nm, A.resc, A.trim, w.iv, w.keep, w.small + SM_MM, w.small + SM_KMAX,
                   &w.grid, &w.grid_bytes, w.vox, w.small + SM_NVOX, w.h_small, &sp, st);
        if (rc) return rc;
    }
    // full correlation shape sa + sb - 1
    const int o0 = sp.shape[0] + A.shape[0] - 1, o1 = sp.shape[1] + A.shape[1] - 1, o2 = sp.shape[2] + A.shape[2] - 1;
    const size_t total = (size_t)o0 * o1 * o2;
    if (w.hist_bytes < total * sizeof(int)) {
        cudaFree(w.hist);
        w.hist = nullptr;
        w.hist_bytes = 0;
        MM_CUDA_TRY(cudaMalloc(&w.hist, total * sizeof(int)));
        w.hist_bytes = total * sizeof(int);
    }
    MM_CUDA_TRY(cudaMemsetAsync(w.hist, 0, total * sizeof(int), st));
    MM_CUDA_TRY(cudaMemcpyAsync(w.small + SM_NVOX, &sp.nvox, sizeof(int), cudaMemcpyHostToDevice, st));
    const long long pairs = (long long)sp.nvox * A.nvox;
    if (pairs > 0) {
        const int g = (int)((pairs + 255) / 256 < 152 * 32 ? (pairs + 255) / 256 : 152 * 32);
        k_pair_hist<<<g, 256, 0, st>>>(w.vox, w.small + SM_NVOX, A.vox, A.nvox, A.shape[0] - 1, A.shape[1] - 1,
                                       A.shape[2] - 1, o1, o2, w.hist);
        MM_CHECK_LAUNCH();
    }
    unsigned long long *best = reinterpret_cast<unsigned long long *>(w.small + SM_BEST);
    MM_CUDA_TRY(cudaMemsetAsync(best, 0, sizeof(unsigned long long), st));
    const int ga = (int)((total + 255) / 256 < 152 * 16 ? (total + 255) / 256 : 152 * 16);
    k_argmax<<<ga, 256, 0, st>>>(w.hist, (long long)total, best);
    MM_CHECK_LAUNCH();
    float *outp = reinterpret_cast<float *>(w.small + SM_OUT);
    const MmCellGrid &G = A.cg;
    k_refine_init<<<1, 1, 0, st>>>(best, o1, o2, A.shape[0], A.shape[1], A.shape[2], A.resc, G.state);
    MM_CHECK_LAUNCH();
    // radius in cells: the largest match radius over the rounds
    const double rmax = std::max((double)A.resc, (double)target);
    const int reach = (int)std::ceil(rmax / G.cs);
    int nb = (nm + kRefineThreads - 1) / kRefineThreads;
    nb = std::max(1, std::min(nb, kRefineMaxBlocks));
    for (int it = 0; it < 5; ++it) {
        // np.linspace(resc, target, 5)
        const double dist_th = (double)A.resc + (double)it * (((double)target - (double)A.resc) / 4.0);
        k_refine_round<<<nb, kRefineThreads, 0, st>>>(w.pts, w.small + SM_N, G.pts, G.idx, G.start, G.dims[0],
                                                      G.dims[1], G.dims[2], G.lo[0], G.lo[1], G.lo[2], G.cs, reach,
                                                      dist_th, G.state, G.parts);
        MM_CHECK_LAUNCH();
        k_refine_update<<<1, 32, 0, st>>>(G.parts, nb, G.state, it == 4, outp, w.small + SM_NPTS);
        MM_CHECK_LAUNCH();
    }
    MM_CUDA_TRY(cudaMemcpyAsync(w.h_small, outp, sizeof(float) * 3, cudaMemcpyDeviceToHost, st));
    MM_CUDA_TRY(cudaMemcpyAsync(w.h_small + 4, w.small + SM_NPTS, sizeof(int) * 2, cudaMemcpyDeviceToHost, st));
    MM_CUDA_TRY(cudaStreamSynchronize(st));
    memcpy(tzxy, w.h_small, sizeof(float) * 3);
    npts[0] = w.h_small[4];
    return MM_OK;
}
