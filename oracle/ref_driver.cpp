/* Serial launcher for the reference kernels compiled as C++ (see
 * ref_prelude.h).  Each ref_* function runs one "thread" per index, like a
 * 1-D launch with blockDim.x = 1.  Test infrastructure only. */
#include "ref_prelude.h"
mm_ref_dim3 threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1};

extern "C" void local_maxima_count(const float *, float, int, unsigned *, int, int, int, int);
extern "C" void local_maxima(const float *, float, int, int, unsigned short *, unsigned short *,
                             unsigned short *, unsigned *, int, int, int, int);
extern "C" void delta_fit_cross_corr(const float *, const float *, unsigned short *,
                                     unsigned short *, unsigned short *, float *, int, int, int,
                                     int, int, float, float);
extern "C" void box_1d(const float *, float *, int, int, int, int, int);

extern "C" unsigned ref_local_maxima(const float *im, float th, int delta, int d, int h, int w,
                                     unsigned short *zo, unsigned short *xo, unsigned short *yo,
                                     unsigned max_points) {
    unsigned count = 0;
    long n = (long)d * h * w;
    for (long i = 0; i < n; ++i) { blockIdx.x = (unsigned)i; local_maxima_count(im, th, delta, &count, d, h, w, (int)n); }
    unsigned total = count;
    count = 0;
    for (long i = 0; i < n; ++i) { blockIdx.x = (unsigned)i; local_maxima(im, th, delta, 0, zo, xo, yo, &count, d, h, w, (int)max_points); }
    return total;
}

extern "C" void ref_delta_fit(const float *im, const float *raw, unsigned short *zo,
                              unsigned short *xo, unsigned short *yo, float *out, int n, int Z,
                              int X, int Y, int delta_fit, float sz, float sxy) {
    for (int i = 0; i < n; ++i) { blockIdx.x = (unsigned)i; delta_fit_cross_corr(im, raw, zo, xo, yo, out, n, Z, X, Y, delta_fit, sz, sxy); }
}

extern "C" void ref_box_1d(const float *in, float *out, int sz, int sx, int sy, int delta, int axis) {
    long n = (long)sz * sx * sy;
    for (long i = 0; i < n; ++i) { blockIdx.x = (unsigned)i; box_1d(in, out, sz, sx, sy, delta, axis); }
}
