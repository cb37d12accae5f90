// fb_kernels.cuh -- host-side entry points of the kernel translation units.
#pragma once
#include "fb_internal.cuh"

namespace fbg {

// fb_sort.cu
size_t sort_scratch_bytes(int64_t npts, uint32_t nbins, int precision);
cudaError_t sort_samples(int precision, const double *pts, const double *val, int64_t npts, const Geometry &g,
                         int bin_w, uint32_t nbins, FieldHeader *hdr, uint32_t *scratch, uint32_t *bin_start,
                         const uint32_t **sorted_idx, const void **recs, cudaStream_t st);

size_t batch_sort_scratch_bytes(int64_t ntot, uint32_t nbins, int precision);
// The sorted-index and record arrays batch_sort leaves in its scratch.
void batch_sort_views(int precision, int64_t ntot, uint32_t nbins, uint32_t *scratch, const uint32_t **sorted_idx,
                      const void **recs);
cudaError_t batch_sort(int precision, const BatchKeyField *d_fields, const uint2 *d_blocks, uint32_t nblocks,
                       int64_t ntot, uint32_t nbins, FieldHeader *hdrs, int nfields, uint32_t *scratch,
                       uint32_t *bin_start, const uint32_t **sorted_idx, const void **recs, cudaStream_t st);

// fb_axis.cu
// Dynamic shared memory one block may opt into on the current device (less a
// small reserve for static shared memory), and the device's SM count.
size_t axis_smem_limit();
int device_sm_count();
// Sets a kernel's dynamic shared-memory limit to axis_smem_limit() on the
// current device, once per (kernel, device); thread-safe.
cudaError_t ensure_smem_attr(const void *func);
struct AxisPlanLimits {
    int extent_max;        // longest line extent a rows-layout CTA holds
    int extent_max_cols;   // longest line extent a columns-layout CTA holds
    size_t smem_limit;     // dynamic shared memory per block
};
// Longest line extent one CTA holds for half kernel width T.
AxisPlanLimits axis_limits(int precision, int T, int kchunk = 0);
int axis_cols_chunk(int precision, int T, int64_t L, int kchunk);
// Lines per columns-layout CTA: 32 bytes of (v, w) cells per grid row.
int axis_col_group(int precision);
// Shared memory needed by one CTA of a launch.
size_t axis_smem_bytes(int precision, const AxisLaunch &a);
// Fills in lines_per_cta, extent_max, line_pitch, chunks_pad for a launch
// whose L / tile_len / halo are set; returns false if it cannot be held.
bool axis_shape(int precision, AxisLaunch &a);
cudaError_t launch_axis(int precision, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                        cudaStream_t st);
// Batched launches: fields of one launch share `a`, `g` and `sv` except for
// the pointers in fields[] (bpf blocks per field, nitems blocks in all).
// op 0: set the kernel's shared-memory limit and return the grid in *grid;
// op 1: launch it.
int axis_threads(int precision, const AxisLaunch &a);
cudaError_t launch_axis_batch(int op, int precision, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                              const TilePtrs *fields, uint32_t bpf, uint32_t nitems, int *grid, cudaStream_t st);
// Mixed batched launches: fields of different shapes sharing the kernel
// variant (chunk k, mode, splat dimension sd, layout); block x works on
// items[x] = (field, block).  op 0: set the shared-memory limit; op 1: launch.
int axis_variant_k(int precision, const AxisLaunch &a);
int axis_variant_mode(int precision, const AxisLaunch &a);
cudaError_t launch_axis_mixed(int op, int precision, int k, int mode, int sd, int layout, const MixedField *fields,
                              const uint2 *items, uint32_t nitems, size_t smem, int threads, cudaStream_t st);
// Tuning knobs ("chunk": 0 automatic, 17 or 33); returns 0 if accepted.
int axis_tune(const char *name, int value);
// Standalone n-pass box filter over contiguous device lines (no splat, no
// quotient): used for the reference's _accumulate_*_array entry points.
cudaError_t launch_lines(int precision, void *data, int64_t nlines, int64_t len, int T, double alpha,
                         int passes, int normalize, cudaStream_t st);

// fb_cols.cu: the pipelined columns kernel (whole lines of the y / z axis,
// TMA loads).  cols_pipe_plan fills the launch description for `nfields`
// fields of one shape and returns false when the kernel does not apply (tiled
// lines, splat fills, rows that are not a multiple of 16 bytes, or too little
// shared memory / registers); cols_pipe_map encodes the tensor map over the
// fields' source cells (field f at src0 + f * field_stride bytes).
// cols_pipe_tune: 0 off, 1 on, 2 automatic (the default: by precision);
// want: -1 follow that setting, 0 never, 1 wherever the kernel applies.
int cols_pipe_tune(int value);
bool cols_pipe_plan(int precision, const AxisLaunch &a, const Geometry &g, int nfields, ColsPipe &cp, int &K,
                    int &mode, int want = -1);
cudaError_t cols_pipe_map(int precision, const ColsPipe &cp, const Geometry &g, const void *src0,
                          int64_t field_stride, int nfields, CUtensorMap *map);
cudaError_t launch_cols_pipe(int precision, int k, int mode, const CUtensorMap &map, const ColsPipe &cp,
                             const TilePtrs *fields, cudaStream_t st);

// fb_grad.cu: seed (dL/dV, dL/dW) from dL/df in place over the final cells;
// gather the adjoint cells at every sample's corners.
cudaError_t launch_grad_seed(int precision, void *cells, int64_t npoints, const void *grad, int grad_f64, double thr,
                             cudaStream_t st);
cudaError_t launch_grad_gather(int precision, int dim, const void *rec, const uint32_t *keys, uint32_t skip_key,
                               int64_t npts, const void *A, const Geometry &g, const FieldHeader *hdr,
                               double *grad_val, double *grad_pts, cudaStream_t st);
// fb_sort.cu: the per-sample keys and records (by sample index) that
// sort_samples leaves in its scratch.
void sort_sample_arrays(int precision, int64_t npts, uint32_t nbins, uint32_t *scratch, const uint32_t **keys,
                        const void **rec);

// fb_naive.cu: value range into hdr, then the direct Gaussian sums (sphere:
// great-circle distances, 2D lon/lat)
cudaError_t launch_naive(int precision, int dim, int sphere, const double *pts, const double *val, int64_t n,
                         const double *sigma, const double *x0, const double *step, const int64_t *size,
                         FieldHeader *hdr, void *out, int out_f64, cudaStream_t st);
// method 'radius' (2D): value range and sample-tile boxes into the workspace,
// then the radius-limited sums
size_t radius_workspace_bytes(int64_t n);
cudaError_t launch_radius(int precision, const double *pts, const double *val, int64_t n, double sigma,
                          const double *x0, const double *step, const int64_t *size, double max_dist_weight,
                          double min_weight, void *ws, void *out, int out_f64, cudaStream_t st);

// fb_s2.cu
cudaError_t launch_lambert_to_map(const double *geo, double *map, int64_t n, const double *proj,
                                  cudaStream_t st);
cudaError_t launch_resample(const float *lam, int64_t lam_w, int64_t lam_h, const double *lam_x0,
                            const double *x0, const double *step, const int64_t *size,
                            const double *proj, float *out, double *tab, cudaStream_t st);

}  // namespace fbg
