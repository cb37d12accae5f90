// fb_axis_f32l.cu -- float32-compensated axis kernels with the 33-cell chunk
// (sliding windows wider than 65 cells).
#include "fb_axis_impl.cuh"

namespace fbg {

cudaError_t launch_axis_f32l(int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st)
{
    return launch_k<float, K32, 0>(sd, a, g, sv, st);
}

cudaError_t launch_axis_batch_f32l(int op, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                                   const TilePtrs *fields, uint32_t bpf, uint32_t nitems, int *grid,
                                   cudaStream_t st)
{
    return launch_batch_k<float, K32, 0>(op, sd, a, g, sv, fields, bpf, nitems, grid, st);
}

cudaError_t launch_axis_mixed_f32l(int op, int sd, int layout, const MixedField *fields, const uint2 *items,
                                   uint32_t nitems, size_t smem, int threads, cudaStream_t st)
{
    return launch_mixed_k<float, K32, 0>(op, sd, layout, fields, items, nitems, smem, threads, st);
}

}  // namespace fbg
