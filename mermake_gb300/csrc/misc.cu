// Small kernels behind the library's general entry points:
//   mirror       fill.py:6-52       in-place reflect about index i along one axis
//   box_1d       blur.cu:1-52       truncated-window mean along one axis (any layout)
//   subtract     math.py:4-33       uint16 saturating / reflecting subtraction
//   sumsq        __main__.py:221    sum of squares for the DAPI RMS (double accumulation)
#include <stdint.h>
#include "deconv.cuh"

namespace {

struct NdShape {
    int ndim;
    long long shape[8];
    long long stride[8];  // elements
};

__global__ void k_mirror(float *arr, NdShape s, long long size, int axis, int i, int mode) {
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < size;
         idx += (long long)gridDim.x * blockDim.x) {
        long long tmp = idx, off = 0, j = 0;
        for (int d = s.ndim - 1; d >= 0; --d) {
            long long c = tmp % s.shape[d];
            tmp /= s.shape[d];
            off += c * s.stride[d];
            if (d == axis) j = c;
        }
        long long n = s.shape[axis], dist = j - i, src;
        if (mode == 0 && dist > 0) {
            src = i - dist;
            if (src < 0) continue;
        } else if (mode == 1 && dist < 0) {
            src = i - dist;
            if (src >= n) continue;
        } else {
            continue;
        }
        arr[off] = arr[off + (src - j) * s.stride[axis]];
    }
}

// One thread per output voxel; the window is read along `axis` (strides in elements).
__global__ void k_box_1d(const float *__restrict__ in, float *__restrict__ out, int sz, int sx, int sy,
                         long long isz, long long isx, long long isy, long long osz, long long osx, long long osy,
                         int delta, int axis) {
    const long long total = (long long)sz * sx * sy;
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        int z = (int)(idx / ((long long)sx * sy));
        int x = (int)((idx / sy) % sx);
        int y = (int)(idx % sy);
        int c = axis == 0 ? z : (axis == 1 ? x : y);
        int n = axis == 0 ? sz : (axis == 1 ? sx : sy);
        long long st = axis == 0 ? isz : (axis == 1 ? isx : isy);
        long long b = z * isz + x * isx + y * isy - c * st;
        int s = c - delta < 0 ? 0 : c - delta;
        int e = c + delta > n - 1 ? n - 1 : c + delta;
        float sum = 0.f;
        for (int i = s; i <= e; ++i) sum += in[b + i * st];
        out[z * osz + x * osx + y * osy] = e >= s ? sum / (float)(e - s + 1) : 0.f;
    }
}

__global__ void k_subtract_u16(const uint16_t *__restrict__ x, const uint16_t *__restrict__ y,
                               uint16_t *__restrict__ z, NdShape sx, NdShape sy, NdShape sz, long long size,
                               int mode) {
    for (long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x; idx < size;
         idx += (long long)gridDim.x * blockDim.x) {
        long long tmp = idx, ox = 0, oy = 0, oz = 0;
        for (int d = sx.ndim - 1; d >= 0; --d) {
            long long c = tmp % sx.shape[d];
            tmp /= sx.shape[d];
            ox += c * sx.stride[d];
            oy += c * sy.stride[d];
            oz += c * sz.stride[d];
        }
        uint16_t a = x[ox], b = y[oy];
        // mode 0: subtract_clamp (math.py:4-11); mode 1: subtract_reflect (math.py:20-27)
        z[oz] = mode == 0 ? (uint16_t)(a > b ? a - b : 0) : (uint16_t)(a >= b ? a - b : b - a);
    }
}

// Sums of squares in a fixed order (the result does not depend on block
// timing): each block writes its partial sum, k_sum_parts adds the partials.
// Four squares are added in float (one 16-byte load) and the group goes into
// the double accumulator, so the FP64 pipe (a small fraction of the FP32 rate
// on this part) sees one add per four elements; the relative error of a
// group is below 3e-7 and the groups add in double.
__global__ void k_sumsq(const float *__restrict__ x, long long n, double *__restrict__ parts) {
    double acc = 0.0;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x, nth = (long long)gridDim.x * blockDim.x;
    long long done = 0;
    if ((reinterpret_cast<uintptr_t>(x) & 15) == 0) {
        const float4 *x4 = reinterpret_cast<const float4 *>(x);
        const long long n4 = n / 4;
        for (long long i = tid; i < n4; i += nth) {
            const float4 v = x4[i];
            acc += (double)fmaf(v.w, v.w, fmaf(v.z, v.z, fmaf(v.y, v.y, v.x * v.x)));
        }
        done = n4 * 4;
    }
    for (long long i = done + tid; i < n; i += nth) {
        const double v = x[i];
        acc += v * v;
    }
    acc = mm_block_sum(acc);
    if (threadIdx.x == 0) parts[blockIdx.x] = acc;
}

__global__ void k_sum_parts(const double *__restrict__ parts, int nparts, double *__restrict__ out) {
    double acc = 0.0;
    for (int i = threadIdx.x; i < nparts; i += blockDim.x) acc += parts[i];
    acc = mm_block_sum(acc);
    if (threadIdx.x == 0) out[0] = acc;
}

// DAPI divisor (__main__.py:221-222): norm = sqrt of the sum of squares rounded
// to float (cp.linalg.norm of a float32 vector), divided in double by sqrt(N)
// (cp.sqrt of the Python int size), then rounded to float when used as the
// divisor of a float32 array.  The sum itself is accumulated in double.
__global__ void k_rms_div(const double *__restrict__ sumsq, long long n, float *__restrict__ div) {
    float norm = sqrtf((float)sumsq[0]);
    div[0] = (float)((double)norm / sqrt((double)n));
}

int grid_for(long long n) {
    long long g = (n + 255) / 256;
    if (g > 152 * 32) g = 152 * 32;
    return g < 1 ? 1 : (int)g;
}

int fill_shape(NdShape &s, int ndim, const int64_t *shape, const int64_t *strides) {
    if (ndim < 1 || ndim > 8) {
        mm_set_error("ndim %d outside [1, 8]", ndim);
        return MM_EINVAL;
    }
    s.ndim = ndim;
    for (int d = 0; d < ndim; ++d) {
        s.shape[d] = shape[d];
        s.stride[d] = strides[d];
    }
    return MM_OK;
}

}  // namespace

extern "C" int mm_reflect_f32(float *arr, int ndim, const int64_t *shape, const int64_t *strides, int axis, int i,
                              int mode, void *stream) {
    NdShape s;
    int rc = fill_shape(s, ndim, shape, strides);
    if (rc) return rc;
    MM_REQUIRE(axis >= 0 && axis < ndim, "axis %d is out of bounds for array of dimension %d", axis, ndim);
    MM_REQUIRE(i >= 0 && i < shape[axis], "index %d is out of bounds for axis %d with size %lld", i, axis,
               (long long)shape[axis]);
    MM_REQUIRE(mode == 0 || mode == 1, "mode must be 'out' (0) or 'in' (1)");
    long long size = 1;
    for (int d = 0; d < ndim; ++d) size *= shape[d];
    if (size == 0) return MM_OK;
    k_mirror<<<grid_for(size), 256, 0, (cudaStream_t)stream>>>(arr, s, size, axis, i, mode);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

extern "C" int mm_box_1d_f32(const float *in, const int64_t *in_strides, float *out, const int64_t *out_strides,
                             int size_z, int size_x, int size_y, int delta, int axis, void *stream) {
    MM_REQUIRE(axis >= 0 && axis <= 2, "axis %d out of range for a (z, x, y) volume", axis);
    MM_REQUIRE(delta >= 0, "negative blur half-width %d", delta);
    long long total = (long long)size_z * size_x * size_y;
    if (total == 0) return MM_OK;
    k_box_1d<<<grid_for(total), 256, 0, (cudaStream_t)stream>>>(
        in, out, size_z, size_x, size_y, in_strides[0], in_strides[1], in_strides[2], out_strides[0],
        out_strides[1], out_strides[2], delta, axis);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

extern "C" int mm_subtract_u16(const uint16_t *x, const int64_t *xs, const uint16_t *y, const int64_t *ys,
                               uint16_t *z, const int64_t *zs, int ndim, const int64_t *shape, int mode,
                               void *stream) {
    NdShape a, b, c;
    int rc;
    if ((rc = fill_shape(a, ndim, shape, xs)) || (rc = fill_shape(b, ndim, shape, ys)) ||
        (rc = fill_shape(c, ndim, shape, zs)))
        return rc;
    MM_REQUIRE(mode == 0 || mode == 1, "mode must be clamp (0) or reflect (1)");
    long long size = 1;
    for (int d = 0; d < ndim; ++d) size *= shape[d];
    if (size == 0) return MM_OK;
    k_subtract_u16<<<grid_for(size), 256, 0, (cudaStream_t)stream>>>(x, y, z, a, b, c, size, mode);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_sum_parts(const double *parts, int nparts, double *out, cudaStream_t st) {
    k_sum_parts<<<1, 256, 0, st>>>(parts, nparts, out);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

int mm_launch_sumsq(const float *x, long long n, double *parts, double *out, cudaStream_t st) {
    if (n == 0) {
        MM_CUDA_TRY(cudaMemsetAsync(out, 0, sizeof(double), st));
        return MM_OK;
    }
    const int g = grid_for(n);
    k_sumsq<<<g, 256, 0, st>>>(x, n, parts);
    MM_CHECK_LAUNCH();
    return mm_launch_sum_parts(parts, g, out, st);
}

int mm_launch_rms_div(const double *sumsq, long long n, float *div, cudaStream_t st) {
    k_rms_div<<<1, 1, 0, st>>>(sumsq, n, div);
    MM_CHECK_LAUNCH();
    return MM_OK;
}

// ---------------------------------------------------------------------------
// Median of a float32 array (cp.median in mermake/io.py:52): the k-th smallest
// value by radix selection over the order-preserving bit pattern of the floats,
// four 8-bit digits, one histogram per digit; an even count averages the two
// middle values in float32 ((a + b) / 2), as the reference's mean does.
// ---------------------------------------------------------------------------
namespace {

__device__ __forceinline__ unsigned f2key(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float key2f(unsigned k) {
    const unsigned u = (k & 0x80000000u) ? (k & 0x7fffffffu) : ~k;
    return __uint_as_float(u);
}

// state: [0] prefix, [1] mask, [2] rank still to skip inside the prefix
__global__ void k_select_hist(const float *__restrict__ x, long long n, const unsigned *__restrict__ state,
                              int shift, unsigned *__restrict__ hist) {
    __shared__ unsigned h[256];
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const unsigned prefix = state[0], mask = state[1];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const unsigned k = f2key(x[i]);
        if ((k & mask) == prefix) atomicAdd(&h[(k >> shift) & 255u], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

__global__ void k_select_pick(unsigned *__restrict__ state, unsigned *__restrict__ hist, int shift) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    unsigned r = state[2];
    int b = 0;
    for (; b < 255; ++b) {
        if (r < hist[b]) break;
        r -= hist[b];
    }
    state[0] |= (unsigned)b << shift;
    state[1] |= 255u << shift;
    state[2] = r;
    for (int i = 0; i < 256; ++i) hist[i] = 0;
}

__global__ void k_select_init(unsigned *__restrict__ state, unsigned long long rank, unsigned *__restrict__ hist) {
    state[0] = 0;
    state[1] = 0;
    state[2] = (unsigned)rank;
    for (int i = 0; i < 256; ++i) hist[i] = 0;
}

__global__ void k_median_finish(const unsigned *__restrict__ s_lo, const unsigned *__restrict__ s_hi, int even,
                                float *__restrict__ med) {
    const float a = key2f(s_lo[0]);
    med[0] = even ? (a + key2f(s_hi[0])) / 2.0f : a;
}

__global__ void k_divide(const float *__restrict__ x, long long n, const float *__restrict__ d, float *__restrict__ out) {
    const float dv = d[0];
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = __fdiv_rn(x[i], dv);
}

int select_kth(const float *x, long long n, unsigned long long k, unsigned *state, unsigned *hist, cudaStream_t st) {
    k_select_init<<<1, 1, 0, st>>>(state, k, hist);
    MM_CHECK_LAUNCH();
    for (int shift = 24; shift >= 0; shift -= 8) {
        k_select_hist<<<grid_for(n), 256, 0, st>>>(x, n, state, shift, hist);
        MM_CHECK_LAUNCH();
        k_select_pick<<<1, 1, 0, st>>>(state, hist, shift);
        MM_CHECK_LAUNCH();
    }
    return MM_OK;
}

}  // namespace

int mm_median_impl(const float *x, long long n, unsigned *scratch, float *med_dev, float *out, cudaStream_t st) {
    // scratch: 2 x 4 state words + 256 histogram words
    unsigned *s_lo = scratch, *s_hi = scratch + 4, *hist = scratch + 8;
    int rc;
    const int even = (n % 2) == 0;
    if ((rc = select_kth(x, n, even ? n / 2 - 1 : n / 2, s_lo, hist, st))) return rc;
    if (even && (rc = select_kth(x, n, n / 2, s_hi, hist, st))) return rc;
    k_median_finish<<<1, 1, 0, st>>>(s_lo, s_hi, even, med_dev);
    MM_CHECK_LAUNCH();
    if (out) {
        k_divide<<<grid_for(n), 256, 0, st>>>(x, n, med_dev, out);
        MM_CHECK_LAUNCH();
    }
    return MM_OK;
}
