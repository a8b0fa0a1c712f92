/*
 * Plain-C restatement of the reference's NVRTC kernels -- TEST ORACLE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this file's shared library; the product path never does.
 *
 *   orc_box_1d        mermake/blur.cu:1-52          (kernel box_1d)
 *   orc_mirror        mermake/fill.py:6-52          (kernel mirror)
 *   orc_local_maxima  mermake/maxima.cu:1-68,72-145 (count + collect)
 *   orc_delta_fit     mermake/maxima.cu:147-341     (delta_fit_cross_corr)
 *   orc_box_mean_f64  blur.cu semantics in double precision
 *
 * Arithmetic is float32 in the reference's own order, so that these functions
 * reproduce the reference's rounding.  One deliberate difference: when a
 * reflected neighbour index is still outside the volume (a dimension shorter
 * than the neighbourhood radius, e.g. size 1), the reference kernel reads out
 * of bounds; here such a neighbour is skipped.  The GPU kernels do the same.
 *
 * OpenMP (when compiled with -fopenmp) parallelises over z planes; results
 * do not depend on the thread count (maxima are returned in raster order).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static inline int reflect_idx(int i, int n) {
    /* maxima.cu:44-52: one reflection about the first/last sample */
    if (i < 0) return -i;
    if (i >= n) return 2 * n - i - 2;
    return i;
}

void orc_box_1d(const float *in, float *out, int size_z, int size_x, int size_y,
                int delta, int axis) {
    long total = (long)size_z * size_x * size_y;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < total; ++idx) {
        int z = (int)(idx / ((long)size_x * size_y));
        long tmp = idx % ((long)size_x * size_y);
        int x = (int)(tmp / size_y);
        int y = (int)(tmp % size_y);
        float sum = 0.0f;
        int num = 0, start, end, i;
        if (axis == 0) {
            start = z - delta < 0 ? 0 : z - delta;
            end = z + delta > size_z - 1 ? size_z - 1 : z + delta;
            for (i = start; i <= end; ++i) { sum += in[((long)i * size_x + x) * size_y + y]; num++; }
        } else if (axis == 1) {
            start = x - delta < 0 ? 0 : x - delta;
            end = x + delta > size_x - 1 ? size_x - 1 : x + delta;
            for (i = start; i <= end; ++i) { sum += in[((long)z * size_x + i) * size_y + y]; num++; }
        } else {
            start = y - delta < 0 ? 0 : y - delta;
            end = y + delta > size_y - 1 ? size_y - 1 : y + delta;
            for (i = start; i <= end; ++i) { sum += in[((long)z * size_x + x) * size_y + i]; num++; }
        }
        out[idx] = num > 0 ? sum / (float)num : 0.0f;
    }
}

void orc_box_mean_f64(const double *in, double *out, int size_z, int size_x, int size_y,
                      int delta, int axis) {
    long total = (long)size_z * size_x * size_y;
#pragma omp parallel for schedule(static)
    for (long idx = 0; idx < total; ++idx) {
        int z = (int)(idx / ((long)size_x * size_y));
        long tmp = idx % ((long)size_x * size_y);
        int x = (int)(tmp / size_y);
        int y = (int)(tmp % size_y);
        int c = axis == 0 ? z : (axis == 1 ? x : y);
        int n = axis == 0 ? size_z : (axis == 1 ? size_x : size_y);
        long st = axis == 0 ? (long)size_x * size_y : (axis == 1 ? size_y : 1);
        long base = idx - (long)c * st;
        int s = c - delta < 0 ? 0 : c - delta, e = c + delta > n - 1 ? n - 1 : c + delta;
        double sum = 0.0;
        for (int i = s; i <= e; ++i) sum += in[base + (long)i * st];
        out[idx] = sum / (double)(e - s + 1);
    }
}

/* fill.py:6-52: in-place mirror of a float32 array of any rank (element
 * strides).  mode 0 = "out" (j > i takes a[2i-j] when 2i-j >= 0), mode 1 =
 * "in" (j < i takes a[2i-j] when 2i-j < n).  Sources are never destinations,
 * so a serial loop gives the parallel kernel's result. */
void orc_mirror(float *arr, int ndim, const int64_t *shape, const int64_t *strides,
                int axis, int i, int mode) {
    int64_t size = 1;
    for (int d = 0; d < ndim; ++d) size *= shape[d];
    int64_t coords[16];
    for (int64_t idx = 0; idx < size; ++idx) {
        int64_t tmp = idx;
        for (int d = ndim - 1; d >= 0; --d) { coords[d] = tmp % shape[d]; tmp /= shape[d]; }
        int64_t j = coords[axis], n = shape[axis], dist = j - i, src;
        if (mode == 0 && dist > 0) { src = i - dist; if (src < 0) continue; }
        else if (mode == 1 && dist < 0) { src = i - dist; if (src >= n) continue; }
        else continue;
        int64_t od = 0, os = 0;
        for (int d = 0; d < ndim; ++d) {
            od += coords[d] * strides[d];
            os += (d == axis ? src : coords[d]) * strides[d];
        }
        arr[od] = arr[os];
    }
}

static int is_local_max(const float *image, int z, int x, int y, int depth, int height,
                        int width, int delta) {
    float v = image[((long)z * height + x) * width + y];
    for (int dz = -delta; dz <= delta; dz++)
        for (int dx = -delta; dx <= delta; dx++)
            for (int dy = -delta; dy <= delta; dy++) {
                if (dz == 0 && dx == 0 && dy == 0) continue;
                if (dz * dz + dx * dx + dy * dy > delta * delta) continue;
                int nz = reflect_idx(z + dz, depth);
                int nx = reflect_idx(x + dx, height);
                int ny = reflect_idx(y + dy, width);
                if (nz < 0 || nz >= depth || nx < 0 || nx >= height || ny < 0 || ny >= width) continue;
                if (v < image[((long)nz * height + nx) * width + ny]) return 0;
            }
    return 1;
}

/* maxima.cu:1-145: voxels strictly above threshold that no neighbour in the
 * sphere |d|^2 <= delta^2 exceeds.  Writes up to max_points (z, x, y) triples
 * in raster order and returns the total count. */
uint32_t orc_local_maxima(const float *image, float threshold, int delta, int depth, int height,
                          int width, uint16_t *z_out, uint16_t *x_out, uint16_t *y_out,
                          uint32_t max_points) {
    uint32_t *cnt = (uint32_t *)calloc((size_t)depth + 1, sizeof(uint32_t));
#pragma omp parallel for schedule(dynamic)
    for (int z = 0; z < depth; ++z) {
        uint32_t c = 0;
        for (int x = 0; x < height; ++x)
            for (int y = 0; y < width; ++y) {
                if (image[((long)z * height + x) * width + y] <= threshold) continue;
                c += (uint32_t)is_local_max(image, z, x, y, depth, height, width, delta);
            }
        cnt[z + 1] = c;
    }
    for (int z = 0; z < depth; ++z) cnt[z + 1] += cnt[z];
#pragma omp parallel for schedule(dynamic)
    for (int z = 0; z < depth; ++z) {
        uint32_t pos = cnt[z];
        if (pos >= max_points) continue;
        for (int x = 0; x < height; ++x)
            for (int y = 0; y < width; ++y) {
                if (image[((long)z * height + x) * width + y] <= threshold) continue;
                if (!is_local_max(image, z, x, y, depth, height, width, delta)) continue;
                if (pos < max_points) {
                    z_out[pos] = (uint16_t)z; x_out[pos] = (uint16_t)x; y_out[pos] = (uint16_t)y;
                }
                pos++;
            }
    }
    uint32_t total = cnt[depth];
    free(cnt);
    return total;
}

#define ORC_MAX_KERNEL_POINTS 600

/* maxima.cu:147-341 (delta_fit_cross_corr), float32 in the reference's order.
 * out row: [zc, xc, yc, background, a, habs, hn, h]. */
void orc_delta_fit(const float *image, const float *raw, const uint16_t *z_in,
                   const uint16_t *x_in, const uint16_t *y_in, float *output, int num_maxima,
                   int Z, int X, int Y, int delta_fit, float sigmaZ, float sigmaXY) {
#pragma omp parallel for schedule(dynamic, 64)
    for (int idx = 0; idx < num_maxima; ++idx) {
        int z0 = z_in[idx], x0 = x_in[idx], y0 = y_in[idx];
        float min_val = 1e20f;
        float norm_G[ORC_MAX_KERNEL_POINTS], sample_vals[ORC_MAX_KERNEL_POINTS],
            raw_vals[ORC_MAX_KERNEL_POINTS];
        int dz_vals[ORC_MAX_KERNEL_POINTS], dx_vals[ORC_MAX_KERNEL_POINTS],
            dy_vals[ORC_MAX_KERNEL_POINTS];
        int count = 0;
        for (int dz = -delta_fit; dz <= delta_fit; ++dz)
            for (int dx = -delta_fit; dx <= delta_fit; ++dx)
                for (int dy = -delta_fit; dy <= delta_fit; ++dy) {
                    if (dz * dz + dx * dx + dy * dy > delta_fit * delta_fit) continue;
                    if (count >= ORC_MAX_KERNEL_POINTS) continue;
                    int zz = reflect_idx(z0 + dz, Z);
                    int xx = reflect_idx(x0 + dx, X);
                    int yy = reflect_idx(y0 + dy, Y);
                    if (zz < 0 || zz >= Z || xx < 0 || xx >= X || yy < 0 || yy >= Y) continue;
                    long ii = ((long)zz * X + xx) * Y + yy;
                    float val = image[ii];
                    sample_vals[count] = val;
                    raw_vals[count] = raw[ii];
                    if (val < min_val) min_val = val;
                    dz_vals[count] = dz; dx_vals[count] = dx; dy_vals[count] = dy;
                    norm_G[count] = expf(-(dz * dz / (2 * sigmaZ * sigmaZ) +
                                           dx * dx / (2 * sigmaXY * sigmaXY) +
                                           dy * dy / (2 * sigmaXY * sigmaXY)));
                    count++;
                }
        if (count == 0) continue;
        float mean_G = 0.0f, var_G = 0.0f;
        for (int i = 0; i < count; i++) mean_G += norm_G[i];
        mean_G /= count;
        for (int i = 0; i < count; i++) { float d = norm_G[i] - mean_G; var_G += d * d; }
        var_G /= count;
        float std_G = sqrtf(var_G);
        for (int i = 0; i < count; i++) norm_G[i] = (norm_G[i] - mean_G) / std_G;
        float background = min_val;
        for (int i = 0; i < count; i++) sample_vals[i] -= background;
        float mean_s = 0.0f, var_s = 0.0f, mean_r = 0.0f, var_r = 0.0f;
        for (int i = 0; i < count; i++) { mean_s += sample_vals[i]; mean_r += raw_vals[i]; }
        mean_s /= count;
        mean_r /= count;
        for (int i = 0; i < count; i++) {
            float ds = sample_vals[i] - mean_s, dr = raw_vals[i] - mean_r;
            var_s += ds * ds;
            var_r += dr * dr;
        }
        var_s /= count;
        var_r /= count;
        float std_s = sqrtf(var_s), std_r = sqrtf(var_r);
        float hn = 0.0f, a = 0.0f;
        for (int i = 0; i < count; i++) {
            float ns = (sample_vals[i] - mean_s) / (std_s > 0 ? std_s : 1.0f);
            float nr = (raw_vals[i] - mean_r) / (std_r > 0 ? std_r : 1.0f);
            hn += ns * norm_G[i];
            a += nr * norm_G[i];
        }
        hn /= count;
        a /= count;
        float sw = 0.0f, cz = 0.0f, cx = 0.0f, cy = 0.0f;
        for (int i = 0; i < count; i++) {
            cz += (z0 + dz_vals[i]) * sample_vals[i];
            cx += (x0 + dx_vals[i]) * sample_vals[i];
            cy += (y0 + dy_vals[i]) * sample_vals[i];
            sw += sample_vals[i];
        }
        if (sw > 0) { cz /= sw; cx /= sw; cy /= sw; }
        else { cz = (float)z0; cx = (float)x0; cy = (float)y0; }
        long ci = ((long)z0 * X + x0) * Y + y0;
        float *o = output + (long)idx * 8;
        o[0] = cz; o[1] = cx; o[2] = cy; o[3] = background;
        o[4] = a; o[5] = raw[ci]; o[6] = hn; o[7] = image[ci];
    }
}
