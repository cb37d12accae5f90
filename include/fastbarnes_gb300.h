/*
 * fastbarnes_gb300.h -- C ABI of the GB300 fast Barnes interpolation library
 * (libfastbarnes_gb300.so).
 *
 * Every entry point takes plain pointers and sizes.  Arrays named d_* are
 * device pointers (CUDA global memory of the current device); everything else
 * is host memory.  `stream` is a cudaStream_t passed as void* (NULL = the
 * legacy default stream).  Device entry points are asynchronous on `stream`
 * and never allocate: the caller provides the workspace whose size
 * fb_workspace_size() reports.  Return value: FB_OK or one of the FB_ERR_*
 * codes; fb_last_error() then holds a message for the calling thread.
 *
 * Layout conventions are the reference's (MeteoSwiss/fast-barnes-py 2.0):
 *   pts  : N x dim float64, row-major (x, y[, z] of each sample)
 *   val  : N float64
 *   size : {nx[, ny[, nz]]} (x first), grid arrays are [nz][ny][nx], x fastest
 */
#ifndef FASTBARNES_GB300_H
#define FASTBARNES_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum fb_status {
    FB_OK = 0,
    FB_ERR_ARG = 1,          /* invalid argument (dimension, sizes, pointers)     */
    FB_ERR_KERNEL_SIZE = 2,  /* 2T+1 >= grid size in some axis                    */
    FB_ERR_WORKSPACE = 3,    /* workspace missing or smaller than required        */
    FB_ERR_CUDA = 4,         /* a CUDA runtime call failed                        */
    FB_ERR_UNSUPPORTED = 5,  /* a line cannot be tiled in shared memory           */
    FB_ERR_DEVICE = 6        /* a kernel reported an error through its status word */
};

enum fb_precision {
    FB_FP64 = 0,   /* float64 throughout: the drop-in form                          */
    FB_FP32C = 1   /* float32 running sums re-anchored on exact chunk sums, scaled  */
};

enum fb_method {
    FB_OPTIMIZED_CONVOLUTION = 0,  /* 'optimized_convolution' (rect kernel + tails) */
    FB_CONVOLUTION = 1,            /* 'convolution' (plain rect kernel)             */
    FB_NAIVE = 2                   /* 'naive' (direct Gaussian sums, O(N x grid))   */
};

/* Library version string. */
const char *fb_version(void);

/* Message describing the last failure of the calling thread ("" if none). */
const char *fb_last_error(void);

/* Launch-shape knob, no reference counterpart: name "chunk" = cells per
 * thread chunk of the float32 sliding passes for windows wider than 65 cells
 * (0 = automatic, 17 or 33).  Used by the autotuner. */
int fb_tune(const char *name, int value);

/* ---- kernel-size helpers (host only) --------------------------------------
 * Replace fastbarnes/interpolation.py:543-569 (get_half_kernel_size_opt,
 * get_tail_value) and :777-803 (get_half_kernel_size, get_sigma_effective). */
int fb_half_kernel_size_opt(double sigma, double step, int num_iter);
double fb_tail_value(double sigma, double step, int num_iter);
int fb_half_kernel_size(double sigma, double step, int num_iter);
double fb_sigma_effective(double sigma, double step, int num_iter);

/* ---- interpolation on a regular grid ---------------------------------------
 * Replaces fastbarnes/interpolation.py:328-367 (_interpolate_opt_convol, for
 * FB_OPTIMIZED_CONVOLUTION) and :575-612 (_interpolate_convol, for
 * FB_CONVOLUTION), i.e. the body of barnes(..., method=...) after its
 * argument checks (:31-199).  sigma, x0, step hold dim values, size dim
 * values; max_dist_weight = exp(-max_dist^2 / 2) as computed at :167.
 * d_out receives size[dim-1] x ... x size[0] values, float32 (out_f64 = 0,
 * the reference's return type) or float64 (out_f64 = 1, the quotient before
 * the float32 cast).  Grid points with too little weight are NaN (:420-430).
 * Returns FB_ERR_KERNEL_SIZE when 2T+1 >= size[m] (the check of :170-175). */
int fb_workspace_size(int method, int precision, int dim, int64_t n_pts, const double *sigma,
                      const double *step, const int64_t *size, int num_iter, size_t *bytes);

/* FB_NAIVE replaces _interpolate_naive (interpolation.py:861-938): every grid
 * point sums exp(-|d|^2 / 2 sigma^2) over all samples, NaN only where the
 * weights sum to zero (no max_dist mask, num_iter and max_dist_weight are
 * ignored); the float32 form keeps Kahan-compensated float32 sums. */
int fb_interpolate(int method, int precision, int dim, const double *d_pts, const double *d_val,
                   int64_t n_pts, const double *sigma, const double *x0, const double *step,
                   const int64_t *size, int num_iter, double max_dist_weight, void *d_out, int out_f64,
                   void *d_workspace, size_t workspace_bytes, void *stream);

/* Same computation from host buffers: copies pts / val to the device, runs
 * fb_interpolate on `stream` with a library-owned device buffer (grown on
 * demand, released by fb_release), copies the result into host `out`,
 * synchronizes the stream and checks the device status word (FB_ERR_DEVICE).
 * Pinned host memory (fb_host_alloc) makes the copies asynchronous DMA
 * transfers.  The library's device buffer is one per process: calls from
 * several host threads are serialized (one at a time, copies and
 * synchronization included). */
int fb_interpolate_host(int method, int precision, int dim, const double *pts, const double *val,
                        int64_t n_pts, const double *sigma, const double *x0, const double *step,
                        const int64_t *size, int num_iter, double max_dist_weight, void *out, int out_f64,
                        void *stream);

/* Replaces demo/quantinterpolation.py:66-155 (barnes with quant_bits): the
 * float64 result (d_out, size[dim-1] x ... x size[0] doubles) with its
 * quant_bits least significant mantissa bits dropped as demo/quantization.py
 * quant() does, applied in the last axis kernel.  quant_bits in [0, 52];
 * workspace as fb_workspace_size. */
int fb_interpolate_quant(int method, int precision, int dim, const double *d_pts, const double *d_val,
                         int64_t n_pts, const double *sigma, const double *x0, const double *step,
                         const int64_t *size, int num_iter, double max_dist_weight, int quant_bits, double *d_out,
                         void *d_workspace, size_t workspace_bytes, void *stream);

/* ---- gradients -------------------------------------------------------------
 * No reference counterpart (the reference has no derivatives).  The adjoint of
 * fb_interpolate: given dL/df in d_grad_out (same shape as d_out, float32 or
 * float64 with grad_f64 = 1), writes dL/dval into d_grad_val (n_pts doubles)
 * and, unless d_grad_pts is NULL, dL/dpts into d_grad_pts (n_pts x dim
 * doubles).  Masked (NaN) grid points carry no gradient; samples outside the
 * grid get zero; the value offset (min + max)/2 cancels in f and is treated
 * as a constant.  The box passes are symmetric, so the adjoint reuses them on
 * the seeded cells (dL/dV, dL/dW) = (g / W, -g V / W^2) and gathers the
 * result with the bilinear weights and their position derivatives.  Recomputes
 * the forward fields; workspace: fb_grad_workspace_size. */
int fb_grad_workspace_size(int method, int precision, int dim, int64_t n_pts, const double *sigma,
                           const double *step, const int64_t *size, int num_iter, size_t *bytes);
int fb_interpolate_grad(int method, int precision, int dim, const double *d_pts, const double *d_val,
                        int64_t n_pts, const double *sigma, const double *x0, const double *step,
                        const int64_t *size, int num_iter, double max_dist_weight, const void *d_grad_out,
                        int grad_f64, double *d_grad_val, double *d_grad_pts, void *d_workspace,
                        size_t workspace_bytes, void *stream);

/* No reference counterpart: the device status word of a workspace after a
 * call on `stream` (synchronizes the stream).  Kernels that stop early
 * instead of waiting on (a pipeline wait that ran out), and, in the
 * bounds-check build, kernels that skipped an out-of-range index, record a
 * bit there: 1 = a wait ran out, 2 = an index was skipped.  Returns FB_OK
 * and *status = 0 when the call ran to completion, else FB_ERR_DEVICE with
 * the bits in *status.  The word is cleared at the start of every call that
 * uses the workspace.  fb_interpolate_host checks it itself. */
int fb_workspace_status(const void *d_workspace, void *stream, int *status);

/* Pinned host memory for fb_interpolate_host buffers. */
void *fb_host_alloc(size_t bytes);
void fb_host_free(void *p);
/* Frees the device buffers fb_interpolate_host keeps between calls. */
void fb_release(void);

/* ---- stage timing ---------------------------------------------------------
 * No reference counterpart (the reference times whole calls with
 * time.perf_counter_ns, demo/timing1_table1_figure4.py:107-115).  Between
 * fb_profile_begin and fb_profile_end every interpolation records CUDA events
 * around its stages on its stream; fb_profile_end waits for them and returns
 * one record per stage: stage 0 = sample sort, 1 + m = the launch along axis
 * m, with its elapsed milliseconds. */
int fb_profile_begin(void);
int fb_profile_end(int *stages, float *ms, int max_records, int *n_records);

/* ---- batched 2D fields ------------------------------------------------------
 * No reference counterpart: the reference interpolates one field per call
 * (fastbarnes/interpolation.py:36 barnes; a batch is a Python loop over it,
 * demo/timing1_table1_figure4.py:107-115).  A plan holds many independent 2D
 * fields (each its own samples, sigma, grid and output, optimized convolution
 * or convolution) and runs all of them with one sample sort and, per axis
 * stage, one launch per kernel variant (chunk length and pass form): fields
 * of one shape share a launch description, fields of different grids,
 * samples and sigma go through a table of per-field descriptions in the same
 * launch.  Every field's result equals that of fb_interpolate on it.
 *
 * fb_batch_create checks the fields, plans the launches and allocates the
 * plan's device memory (tables, sort scratch, intermediate fields) on the
 * current device.  The device pointers in `fields` are kept: fb_batch_run
 * reads pts / val and writes out of every field each time (refill the input
 * buffers between runs to interpolate new data).  flags:
 *   FB_BATCH_GRAPH  capture the run's launches in a CUDA graph at the first
 *                   fb_batch_run and replay it afterwards;
 *   FB_BATCH_TUNE   time the candidate launch shapes on the given fields at
 *                   creation (runs the batch; inputs must be valid) and keep
 *                   the fastest; the choice is remembered for identical
 *                   batches in this process.
 * knobs (optional) pins the launch shape instead; fb_batch_knobs_of reports
 * the one in use. */
typedef struct fb_field2d {
    const double *pts;        /* device, n_pts x 2 */
    const double *val;        /* device, n_pts */
    int64_t n_pts;
    double sigma[2], x0[2], step[2];
    int64_t size[2];          /* (nx, ny); out is ny x nx */
    int num_iter;
    double max_dist_weight;
    int method;               /* FB_OPTIMIZED_CONVOLUTION or FB_CONVOLUTION */
    void *out;                /* device, float32 (or float64 with out_f64) */
} fb_field2d;

typedef struct fb_batch_knobs {
    int chunk;                /* 0 automatic, 17 or 33 (float32 windows wider than 65) */
    int rows_threads;         /* x-axis threads per CTA target: 0 (= 128), 128, 256 or 512 */
    int mixed;                /* 1: per-field descriptions even when the fields share one shape */
    int cols_pipe;            /* column stages: 0 library default for the precision, 1 the persistent
                                 TMA-pipelined kernel where it applies, 2 one CTA per column group */
    int interleave;           /* 1: per-field x and y launches on two streams (field f's y right after
                                 its x, beside field f+1's x) so that y reads an intermediate still in
                                 L2; 0: one launch per axis for all fields */
} fb_batch_knobs;

typedef struct fb_batch fb_batch;

enum { FB_BATCH_GRAPH = 1, FB_BATCH_TUNE = 2 };

int fb_batch_create(int precision, const fb_field2d *fields, int n_fields, int out_f64, int flags,
                    const fb_batch_knobs *knobs, fb_batch **plan);
/* Enqueues the whole batch on `stream` (0 = the legacy default stream). */
int fb_batch_run(fb_batch *plan, void *stream);
/* Host-buffer form: copies h_pts[f] (n_pts x 2) and h_val[f] of every field
 * into the plan's device inputs, runs the batch and copies every output into
 * h_out[f] (size[1] x size[0]); returns when the results are in host memory.
 * Pinned host buffers (fb_host_alloc) make the copies asynchronous. */
int fb_batch_run_host(fb_batch *plan, const double *const *h_pts, const double *const *h_val, void *const *h_out,
                      void *stream);
/* The same without waiting: everything is enqueued on `stream`, the results
 * are in h_out once the stream has completed.  With two plans on two streams
 * a caller overlaps one batch's copies with the other's interpolation. */
int fb_batch_enqueue_host(fb_batch *plan, const double *const *h_pts, const double *const *h_val,
                          void *const *h_out, void *stream);
int fb_batch_knobs_of(const fb_batch *plan, fb_batch_knobs *knobs);
/* The device status words of a plan's last run on `stream` (synchronizes
 * it), ORed over the fields: as fb_workspace_status. */
int fb_batch_status(const fb_batch *plan, void *stream, int *status);
/* Kernel launches and memsets one fb_batch_run enqueues, and the plan's
 * device bytes. */
int fb_batch_info(const fb_batch *plan, int *kernel_launches, int *memsets, size_t *device_bytes);
void fb_batch_destroy(fb_batch *plan);

/* ---- the 1D rect-kernel passes alone -----------------------------------------
 * Replaces _accumulate_tail_array (interpolation.py:484-533; rect_len = 2T+1,
 * tail weight alpha) and _accumulate_array (:729-772; alpha = 0): num_iter
 * passes over each of n_lines contiguous lines of length len, in place.  With
 * normalize = 0 the sums are unscaled like the reference's; with 1 every pass
 * is divided by rect_len + 2 alpha. */
int fb_accumulate_lines(int precision, void *d_lines, int64_t n_lines, int64_t len, int rect_len,
                        int num_iter, double alpha, int normalize, void *stream);

/* ---- the sphere ---------------------------------------------------------------
 * Replaces fastbarnes/interpolationS2.py:143-254 (_interpolate_opt_convol_S2:
 * projection to the fixed Lambert grid x0 = (-32, -2), size =
 * (int(64/step[0]), int(44/step[1])), optimized convolution there, and with
 * resample = 1 the bilinear resampling back to the lon/lat grid).  d_out:
 * size[1] x size[0] float32 (resample = 1) or the Lambert field
 * int(44/step[1]) x int(64/step[0]) float32 (resample = 0). */
int fb_s2_workspace_size(int precision, int64_t n_pts, const double *sigma, const double *step,
                         const int64_t *size, int num_iter, size_t *bytes);
int fb_interpolate_s2(int precision, const double *d_pts, const double *d_val, int64_t n_pts,
                      const double *sigma, const double *x0, const double *step, const int64_t *size,
                      int num_iter, double max_dist_weight, int resample, float *d_out, void *d_workspace,
                      size_t workspace_bytes, void *stream);

/* Replaces _interpolate_naive_S2 (fastbarnes/interpolationS2.py:259-301):
 * naive sums of the great-circle distance (degrees) on the lon/lat grid,
 * sigma[0] in both directions.  d_out: size[1] x size[0]; workspace: 256
 * bytes. */
int fb_interpolate_naive_s2(int precision, const double *d_pts, const double *d_val, int64_t n_pts,
                            const double *sigma, const double *x0, const double *step, const int64_t *size,
                            void *d_out, int out_f64, void *d_workspace, size_t workspace_bytes, void *stream);

/* Replaces _interpolate_radius (fastbarnes/interpolation.py:809-855) and
 * its kd-tree search (fastbarnes/util/kdtree.py:208-331): every grid point
 * sums exp(-d^2 / (2 sigma^2)) over the samples with d^2 <=
 * (sqrt(-2 ln(min_weight)) sigma)^2, NaN where the weights sum below
 * max_dist_weight.  2D, one sigma.  The samples may come in any order; sorted
 * by y (pts[:, 1]) most tiles of samples are out of reach of a block of grid
 * points and are skipped.  d_out: size[1] x size[0] (float64 for out_f64 = 1,
 * the reference's type, else float32); workspace: fb_radius_workspace_size(). */
int fb_radius_workspace_size(int64_t n_pts, size_t *bytes);
int fb_interpolate_radius(int precision, const double *d_pts, const double *d_val, int64_t n_pts, double sigma,
                          const double *x0, const double *step, const int64_t *size, double max_dist_weight,
                          double min_weight, void *d_out, int out_f64, void *d_workspace, size_t workspace_bytes,
                          void *stream);

/* Replaces fastbarnes/util/lambert_conformal.py:50-94 (create_proj):
 * proj[5] = {center_lon, n, n_inv, F, rho0}. */
void fb_lambert_create_proj(double center_lon, double center_lat, double lat1, double lat2, double *proj);

/* Replaces fastbarnes/util/lambert_conformal.py:113-123 (to_map) on the
 * device: d_geo (lon, lat) pairs -> d_map (x, y) pairs. */
int fb_lambert_to_map(const double *d_geo, double *d_map, int64_t n_pts, const double *proj, void *stream);

/* Replaces fastbarnes/interpolationS2.py:211-254 (_resample) on the device:
 * bilinear read of the float32 Lambert field d_lam (lam_h x lam_w, origin
 * lam_x0, spacing step) at the projection of every point of the lon/lat grid
 * (x0, step, size) into d_out (size[1] x size[0] float32).  d_tab is device
 * scratch of size[1] + 2 * size[0] doubles.  Points whose Lambert cell lies
 * outside the field are NaN (the reference does not check). */
int fb_resample(const float *d_lam, int64_t lam_w, int64_t lam_h, const double *lam_x0, const double *x0,
                const double *step, const int64_t *size, const double *proj, float *d_out, double *d_tab,
                void *stream);

/* No reference counterpart: fb_resample without the d_tab argument, for
 * callers that cannot allocate device memory at call time (code running while
 * another component owns the device allocator, or a loop whose latency budget
 * a cudaMalloc / cudaFree would break).  The tables live in a static device
 * array of 49152 doubles (384 KiB), so size[1] + 2 * size[0] <= 49152; larger
 * grids return FB_ERR_ARG.  The first call on a device looks the array up
 * (cudaGetSymbolAddress) -- make it once before any stream capture -- and
 * keeps the address for later calls on that device; the address is valid
 * for the lifetime of the device's primary context, so a process that
 * resets the device (cudaDeviceReset) must not call this entry again.  Calls
 * that overlap in time on one device share the array and race: serialize
 * them.  Allocates nothing. */
int fb_resample_noalloc(const float *d_lam, int64_t lam_w, int64_t lam_h, const double *lam_x0, const double *x0,
                        const double *step, const int64_t *size, const double *proj, float *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* FASTBARNES_GB300_H */
