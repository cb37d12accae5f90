// fb_axis_f64s.cu -- float64-form axis kernels with the 9-cell chunk, for
// sliding windows 2T + 1 < 17 (the sliding scheme needs 2T + 1 >= K).
#include "fb_axis_impl.cuh"

namespace fbg {

cudaError_t launch_axis_f64s(int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st)
{
    return launch_k<double, K9, 0>(sd, a, g, sv, st);
}

cudaError_t launch_axis_batch_f64s(int op, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                                   const TilePtrs *fields, uint32_t bpf, uint32_t nitems, int *grid,
                                   cudaStream_t st)
{
    return launch_batch_k<double, K9, 0>(op, sd, a, g, sv, fields, bpf, nitems, grid, st);
}

cudaError_t launch_axis_mixed_f64s(int op, int sd, int layout, const MixedField *fields, const uint2 *items,
                                   uint32_t nitems, size_t smem, int threads, cudaStream_t st)
{
    return launch_mixed_k<double, K9, 0>(op, sd, layout, fields, items, nitems, smem, threads, st);
}

}  // namespace fbg
