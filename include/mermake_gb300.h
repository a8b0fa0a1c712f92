/*
 * mermake_gb300 -- C ABI of the GB300 (sm_103a) implementation of MERMAKE's
 * per-FOV image path.
 *
 * Every entry point takes plain device pointers, element strides and sizes,
 * and a cudaStream_t passed as void* (NULL = legacy default stream); work is
 * enqueued on that stream.  Entry points that must report a count to the
 * host (maxima, spots) synchronise that stream once, at the end.  All device
 * buffers are owned by the caller; an mm_ctx owns only reusable scratch
 * (spectrum/tile workspaces, candidate lists, counters), grows it on demand
 * and frees it in mm_ctx_destroy.  An mm_ctx may be used by one host thread
 * at a time.  FFT plans (twiddle tables) are cached per device for the life
 * of the process; the first call at a new length uploads them synchronously,
 * so make it before any stream capture.
 *
 * Return value: MM_OK or an error code; mm_last_error() gives the message of
 * the calling thread's last failure.  Layouts follow the reference: volumes
 * are (z, x, y) with y contiguous; Xh rows are 8 float32
 * [zc, xc, yc, background, a, habs, hn, h].
 *
 * Each declaration cites the reference interface it replaces (paths inside
 * the deprekate/MERMAKE v0.0.74 tree).
 */
#ifndef MERMAKE_GB300_H
#define MERMAKE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MM_OK = 0,
    MM_EINVAL = 1,     /* bad argument: ValueError / TypeError / IndexError in the reference */
    MM_ENOMEM = 2,     /* device allocation of scratch failed */
    MM_EOVERFLOW = 3,  /* output capacity too small; *count holds the exact count, retry */
    MM_ETIMEOUT = 4,   /* a bounded device-side wait gave up */
    MM_EDEVICE = 5     /* CUDA runtime error */
};

/* element types of image / raw operands */
enum { MM_DTYPE_F32 = 0, MM_DTYPE_U16 = 1 };

typedef struct mm_ctx mm_ctx;

/* Version of this ABI (bumped on incompatible changes). */
int mm_abi_version(void);
/* Message of the calling thread's last error ("" if none). */
const char *mm_last_error(void);
/* Scratch owner for the calls below (no reference counterpart: it replaces
 * CuPy's memory pool and the per-call free_all_blocks, mermake/maxima.py:96). */
int mm_ctx_create(mm_ctx **out);
int mm_ctx_destroy(mm_ctx *ctx);
/* Device bytes of scratch the context holds (no reference counterpart; for
 * callers that budget device memory, e.g. a serving loop).  The scratch grows
 * on demand, in stream order on the calling stream, and is freed by
 * mm_ctx_destroy.  Safe to call while another thread uses the context. */
int mm_ctx_scratch_bytes(const mm_ctx *ctx, uint64_t *bytes);

/* Context options (no reference counterpart).  MM_OPT_BLUR_MODE selects how
 * the blur subtraction of tile_wise (mermake/deconvolver.py:160-163: the
 * result minus its box mean along x and y, the window truncated at the
 * padded tile's edges, mermake/blur.cu:1-52) is computed:
 *   MM_BLUR_AUTO (default): mm_hyb_spots / mm_dapi_spots (and their _async
 *     forms) fold it into the z step as the factor 1 - D(kx) D(ky) of each
 *     frequency (D: the box mean's frequency response), with no box means
 *     taken on the result, whenever they run the z kernel and every voxel
 *     they read lies at least the box half-width d inside the tile (hyb:
 *     overlap >= d + 1 + delta_fit + max(delta, delta_fit); DAPI: overlap >=
 *     d + 1).  There the truncated box mean equals the circular one, so the
 *     spots and the stitched buffer are those of the truncated blur up to
 *     float32 rounding.  mm_deconv_tiles keeps the truncated blur, whose
 *     edge voxels it returns.
 *   MM_BLUR_EXACT: every call takes the truncated box means on the result.
 *   MM_BLUR_SPECTRAL: as AUTO, and mm_deconv_tiles folds as well (overlap >=
 *     d + 1), so that it returns the volumes the drivers compute (its voxels
 *     within d of a tile edge then differ from the truncated blur's). */
enum { MM_OPT_BLUR_MODE = 1, MM_OPT_ZFORM = 2 };
enum { MM_BLUR_AUTO = 0, MM_BLUR_EXACT = 1, MM_BLUR_SPECTRAL = 2 };
/* MM_OPT_ZFORM selects how the z step of tile_wise (padding by reflection,
 * transforms over Zp, times W, crop; mermake/deconvolver.py:139-157) runs:
 *   MM_ZFORM_AUTO (default): the first form below that the batch qualifies for
 *     (over one shared spectrum, the matrix forms from batches of 10 tiles);
 *   MM_ZFORM_REGISTERS: one Z x Z matrix per frequency, formed in registers
 *     from the z kernel (Z a multiple of 5, 1 <= zpad <= Z - 1): over one
 *     spectrum shared by the batch, operands staged by TMA; or, with a
 *     spectrum per tile or a batch below 10 tiles, each tile's matrix from its
 *     own z kernel (Z <= 80);
 *   MM_ZFORM_SHARED: the same matrix summed into shared memory (one spectrum,
 *     Z <= 64, at most four copies of a plane);
 *   MM_ZFORM_DIRECT: the direct sum over the padded planes per tile;
 *   MM_ZFORM_TRANSFORMS: the reference's transforms over the padded depth;
 *   MM_ZFORM_TENSOR: the matrix of each frequency applied on the tensor
 *     cores (tcgen05, TF32 operands split in two so that the products keep
 *     float32 accuracy; one spectrum, Z <= 56, 1 <= zpad <= Z - 1, up to 32
 *     tiles).
 * A form the batch does not qualify for falls back to AUTO's choice.  All
 * forms give the same voxels within float32 rounding; the choice is a
 * performance setting (tune.autotune picks it per geometry). */
enum {
    MM_ZFORM_AUTO = 0,
    MM_ZFORM_REGISTERS = 1,
    MM_ZFORM_SHARED = 2,
    MM_ZFORM_DIRECT = 3,
    MM_ZFORM_TRANSFORMS = 4,
    MM_ZFORM_TENSOR = 5
};
int mm_ctx_set_option(mm_ctx *ctx, int option, int value);

/* fill.reflect (mermake/fill.py:54-111, kernel `mirror` fill.py:6-52), in place.
 * mode 0 = "out" (a[j] = a[2i-j] for j > i), 1 = "in" (for j < i).
 * shape/strides are host arrays of ndim int64 (strides in elements). */
int mm_reflect_f32(float *arr, int ndim, const int64_t *shape, const int64_t *strides, int axis, int i,
                   int mode, void *stream);

/* blur.box_1d (mermake/blur.py:157-188, kernel box_1d blur.cu:1-52): mean over
 * [c-delta, c+delta] clipped to the axis.  A 2-D image is (1, x, y).
 * in_strides/out_strides: host int64[3] (elements). */
int mm_box_1d_f32(const float *in, const int64_t *in_strides, float *out, const int64_t *out_strides,
                  int size_z, int size_x, int size_y, int delta, int axis, void *stream);

/* math.subtract_clamp (mode 0, mermake/math.py:4-17) and math.subtract_reflect
 * (mode 1, mermake/math.py:20-33) on uint16 arrays of any rank <= 8. */
int mm_subtract_u16(const uint16_t *x, const int64_t *x_strides, const uint16_t *y, const int64_t *y_strides,
                    uint16_t *z, const int64_t *z_strides, int ndim, const int64_t *shape, int mode,
                    void *stream);

/* cp.median of a float32 array as load_flats uses it (mermake/io.py:42-54):
 * writes the median to *median (host) -- the mean in float32 of the two middle
 * values when n is even -- and, when out is not NULL, out[i] = x[i] / median
 * (io.py:52).  Synchronises the stream. */
int mm_median_f32(mm_ctx *ctx, const float *x, int64_t n, float *median, float *out, void *stream);

/* Deconvolver.__init__ for one PSF (mermake/deconvolver.py:48-75 with
 * center_psf 238-270 and laplacian_3d 24-36): writes the Wiener spectrum
 * conj(H)/(|H|^2 + beta |L|^2), pre-divided by Zp*P*P, as the half spectrum
 * W[Zp][P][P/2+1] of complex64 (float2), Zp = tile_height + 2*zpad,
 * P = tile_size + 2*overlap.  psf: float32 (pz, px, py), device. */
int mm_wiener_spectrum(mm_ctx *ctx, const float *psf, int pz, int px, int py, int tile_height, int tile_size,
                       int zpad, int overlap, float beta, void *W, void *stream);

/* The z kernel of one spectrum, for the z step of tile_wise without the
 * padded-depth transforms (mermake/deconvolver.py:139-157: z padding by
 * reflection, FFT over Zp, times W, inverse FFT, keep planes
 * [zpad, zpad + Z)).  No counterpart in the reference, which transforms every
 * tile over the padded depth.  Writes zop, (Zp, P, P/2+1) complex64 like W:
 * the inverse DFT of W along z, so that output plane i of a tile is
 * sum_z zop[(zpad + i - z) mod Zp] x[map(z)] per frequency.  Passing zop
 * (one kernel per spectrum, laid out like W) to mm_deconv_tiles /
 * mm_hyb_spots / mm_dapi_spots replaces the two padded-depth transforms of
 * each tile: with one spectrum and batches of at least 10 tiles by one Z x Z
 * complex matrix per frequency over the batch (each entry a sum of at most
 * four kernel samples; tile_height <= 64 and no plane copied more than four
 * times by the padding), otherwise by that sum taken directly per tile
 * (tile_height <= 128).  Zp <= 400 (MM_EINVAL otherwise). */
int mm_wiener_zop(mm_ctx *ctx, const void *W, int tile_height, int zpad, int tile_size, int overlap, void *zop,
                  void *stream);

/* 1 when mm_wiener_zop accepts (tile_height, zpad), else 0. */
int mm_zkernel_supported(int tile_height, int zpad);

/* Deconvolver.tile_wise / apply (mermake/deconvolver.py:98-184) for tiles
 * [tile_begin, tile_begin + tile_count) of the x-major tile grid of a
 * (Z, X, Y) channel, uint16 or float32 (image_dtype; strides isz, isx, 1).  flat: float32 (X, Y) with row stride fsx, or NULL.
 * W: npsf spectra as made by mm_wiener_spectrum (tile i uses spectrum i when
 * npsf > 1).  zop: NULL, or the z kernels of the npsf spectra made by
 * mm_wiener_zop, laid out like W.  blur_radius < 0: no background subtraction.
 * Outputs (any may be NULL):
 *   res_out    (tile_count, Z, P, P) float32: tile_res after blur subtraction;
 *              the yielded view is [:, :xend, :yend]
 *   raw_out    (tile_count, Z, P, P) float32: the raw view tile_pad[zpad:-zpad]
 *              with the flat multiplied back (deconvolver.py:165-170)
 *   stitch_out (Z, X, Y) float32 with strides (osz, osx, 1): tile centres
 *              written as Deconvolver.apply does (deconvolver.py:179-183). */
int mm_deconv_tiles(mm_ctx *ctx, const void *image, int image_dtype, int Z, int X, int Y, int64_t isz, int64_t isx,
                    const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size,
                    int zpad, int overlap, int tile_begin, int tile_count, int blur_radius, float *res_out, float *raw_out,
                    float *stitch_out, int64_t osz, int64_t osx, void *stream);

/* find_local_maxima (mermake/maxima.py:17-98; kernels local_maxima_count,
 * local_maxima, delta_fit_cross_corr in mermake/maxima.cu) on one (Z, X, Y)
 * float32 volume with strides (isz, isx, 1).  raw: same shape, raw_dtype 0 =
 * float32 (MM_DTYPE_F32), 1 = uint16 (MM_DTYPE_U16), strides (rsz, rsx, 1).  norm_div != 0 reads the image
 * as v / norm_div (then negated if negate), bit-identical to dividing the
 * volume first (mermake/__main__.py:222-224).  Writes min(count, out_cap) rows
 * to out and the count to *count (host); MM_EOVERFLOW if count > out_cap.
 * delta > 5 -> MM_EINVAL (the reference raises TypeError). */
int mm_find_local_maxima(mm_ctx *ctx, const float *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                         const void *raw, int raw_dtype, int64_t rsz, int64_t rsx, float threshold, int delta,
                         int delta_fit, float sigmaZ, float sigmaXY, float norm_div, int negate, float *out,
                         uint32_t out_cap, uint32_t *count, void *stream);

/* find_local_maxima for callers that cannot allocate device memory while they
 * run (code inside another framework's memory pool or under a fixed memory
 * budget, real-time loops that must not take cudaMalloc's implicit device
 * synchronisation).  No counterpart in the reference: it is
 * mm_find_local_maxima with the candidate list held in a static device array
 * of the library instead of context scratch, so it takes no mm_ctx and calls
 * no allocating routine.  Same arguments and results as mm_find_local_maxima;
 * the caller still owns image, raw, out and count.  Limit: Z*X*Y <= 2,097,152
 * voxels (MM_EINVAL beyond); the array (16 MiB) is held by every GPU that
 * loads it until the process exits.  The CUDA runtime loads the library's
 * device code lazily, so the first call on a device (or the first use of any
 * maxima entry point there) reserves the array's device memory, uploads the
 * neighbour tables, looks the array up (cudaGetSymbolAddress) and synchronises
 * the device: make that first call at start-up, before any stream capture and
 * before the code that must not allocate.  Later calls allocate nothing.  All
 * calls share the array: calls that overlap on the GPU race and must be
 * serialised by the caller. */
int mm_find_local_maxima_noalloc(const float *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                                 const void *raw, int raw_dtype, int64_t rsz, int64_t rsx, float threshold,
                                 int delta, int delta_fit, float sigmaZ, float sigmaXY, float norm_div, int negate,
                                 float *out, uint32_t out_cap, uint32_t *count, void *stream);

/* One hyb colour (mermake/__main__.py:242-265): tile_wise over every tile,
 * find_local_maxima on each yielded tile with its raw view, keep rows with
 * overlap <= xc, yc < extent - overlap, shift by the tile origin, concatenate.
 * Tiles run `batch` at a time.  Rows are appended to out (row order is not
 * specified, as in the reference); *count = total rows; MM_EOVERFLOW if it
 * exceeds out_cap. */
int mm_hyb_spots(mm_ctx *ctx, const uint16_t *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                 const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size,
                 int zpad, int overlap, int blur_radius, float threshold, int delta, int delta_fit, float sigmaZ,
                 float sigmaXY, int batch, float *out, uint32_t out_cap, uint32_t *count, void *stream);

/* The DAPI block (mermake/__main__.py:215-225): Deconvolver.apply into `buffer`
 * (Z, X, Y) float32, divide by the RMS, find_local_maxima (+), negate,
 * find_local_maxima (-), both with the uint16 channel as raw.  The division
 * and negation are applied on read; `buffer` keeps the un-normalised result.
 * *rms receives the divisor used (float). */
int mm_dapi_spots(mm_ctx *ctx, const uint16_t *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                  const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size,
                  int zpad, int overlap, int blur_radius, float threshold, int delta, int delta_fit, float sigmaZ,
                  float sigmaXY, int batch, float *buffer, float *out_plus, uint32_t cap_plus, uint32_t *count_plus,
                  float *out_minus, uint32_t cap_minus, uint32_t *count_minus, float *rms, void *stream);

/* mm_hyb_spots / mm_dapi_spots without a host synchronisation, for capture in
 * a CUDA graph (no counterpart in the reference): the counts stay on the
 * device and nothing is retried.
 *   mm_hyb_spots_async: *count_dev = rows (rows past out_cap are dropped);
 *     *overflow_dev = 0, or the candidate count that did not fit the list.
 *   mm_dapi_spots_async: counts_dev[0..2] = rows (+), rows (-), candidate
 *     overflow (0 when none); *rms_dev (may be NULL) = the divisor.
 * A result is complete when the overflow is 0 and every count is within its
 * capacity; otherwise rerun with the synchronous call.  The context's scratch
 * is sized by the first call: capture a graph only after one eager call with
 * the same shapes, on a context that no other call grows while the graph
 * lives (its workspace addresses are baked into the graph). */
int mm_hyb_spots_async(mm_ctx *ctx, const uint16_t *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                       const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size,
                       int zpad, int overlap, int blur_radius, float threshold, int delta, int delta_fit,
                       float sigmaZ, float sigmaXY, int batch, float *out, uint32_t out_cap, uint32_t *count_dev,
                       uint32_t *overflow_dev, void *stream);
int mm_dapi_spots_async(mm_ctx *ctx, const uint16_t *image, int Z, int X, int Y, int64_t isz, int64_t isx,
                        const float *flat, int64_t fsx, const void *W, int npsf, const void *zop, int tile_size,
                        int zpad, int overlap, int blur_radius, float threshold, int delta, int delta_fit,
                        float sigmaZ, float sigmaXY, int batch, float *buffer, float *out_plus, uint32_t cap_plus,
                        float *out_minus, uint32_t cap_minus, uint32_t *counts_dev, float *rms_dev, void *stream);

/* Tile layout of Deconvolver.tiled / tile_wise (mermake/deconvolver.py:117-148,
 * 186-206), host only (no device work).  tile < 0 returns the number of tiles.
 * desc (13 int32): x, y, x0, y0, xd, yd, xstart, ystart, xend, yend, psf index,
 * P, Zp.  map_z (Zp), map_x (P), map_y (P): for each padded index, the source
 * index inside the tile after placement and the reference's reflect calls, or
 * -1 where the padded tile holds zero.  Any output may be NULL. */
int mm_tile_geometry(int Z, int X, int Y, int tile_size, int zpad, int overlap, int npsf, int tile, int32_t *desc,
                     int32_t *map_z, int32_t *map_x, int32_t *map_y);

/* Engine diagnostic, no reference counterpart (the reference calls cuFFT via
 * cp.fft.fftn/ifftn, mermake/deconvolver.py:155-157): in-place unnormalised
 * complex64 DFT of nlines lines of length n stored element-major
 * (element e of line l at data[e*nlines + l]); inverse uses exp(+i...). */
int mm_fft_c2c(void *data, int n, int nlines, int inverse, void *stream);

/* Drift alignment of maxima point sets (mermake/align.py:12-129, utils.py:10-36).
 * mm_aligner_create is Aligner.__init__(X_ref, resc, trim, th): rows of X_ref
 * (n rows of `cols` float32, row stride ld, device) whose last column exceeds
 * th are kept (th = NaN: all rows), their first three columns are the
 * reference points, and the reference's splat image (round(X/resc), trimmed in
 * x and y) stays resident on the device.  No row left -> MM_EINVAL (the
 * reference raises ValueError).  mm_aligner_translation is
 * get_best_translation_points(X, target, return_counts=True): same threshold
 * on X's last column, argmax of the full correlation of the two splat images
 * (computed exactly as a histogram of voxel-pair differences), five
 * nearest-neighbour refinements; writes tzxy[3] and npts (host) and
 * synchronises the stream.  mm_aligner_info reports the kept reference points,
 * the unique reference voxels and the image shape. */
typedef struct mm_aligner mm_aligner;
int mm_aligner_create(const float *X_ref, int n, int cols, int64_t ld, float th, int resc, int trim,
                      mm_aligner **out, void *stream);
int mm_aligner_translation(mm_aligner *al, const float *X, int n, int cols, int64_t ld, float target, float *tzxy,
                           int *npts, void *stream);
int mm_aligner_info(const mm_aligner *al, int *n_points, int *n_voxels, int *shape3);
int mm_aligner_destroy(mm_aligner *al);

/* Instrumentation, no reference counterpart (the reference has no timing on
 * this path).  mm_profile_enable(ctx, 1) resets and starts per-stage CUDA-event
 * timing of this context's launches (stages: rows_fwd, cols_fwd, zpass,
 * cols_inv, rows_inv_blur_y, blur_x_sub, make_raw, maxima_fit, sumsq, wiener);
 * mm_profile_read fills up to nmax entries of total milliseconds, algorithmic
 * bytes (the DRAM traffic each stage's function needs at minimum) and launch
 * counts, synchronising the recorded events, and returns the number of
 * stages.  mm_stage_name(i) names stage i.  mm_launch_count() is the number of
 * kernels this library has launched in the process. */
int mm_profile_enable(mm_ctx *ctx, int on);
int mm_profile_read(mm_ctx *ctx, int nmax, double *ms, double *bytes, int64_t *launches);
const char *mm_stage_name(int i);
uint64_t mm_launch_count(void);

#ifdef __cplusplus
}
#endif

#endif /* MERMAKE_GB300_H */
