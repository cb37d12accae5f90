// fb_axis_f32.cu -- float32-compensated instantiations of the axis kernels
// (chunk length 17 and the direct sums; the 33-cell chunk is in
// fb_axis_f32l.cu).
#include "fb_axis_impl.cuh"

namespace fbg {

cudaError_t launch_axis_f32l(int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv, cudaStream_t st);
cudaError_t launch_axis_batch_f32l(int op, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                                   const TilePtrs *fields, uint32_t bpf, uint32_t nitems, int *grid,
                                   cudaStream_t st);

cudaError_t launch_axis_f32(int k, int mode, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                            cudaStream_t st)
{
    if (mode == 1)
        return launch_k<float, K64, 1>(sd, a, g, sv, st);
    if (k == K64)
        return launch_k<float, K64, 0>(sd, a, g, sv, st);
    return launch_axis_f32l(sd, a, g, sv, st);
}

cudaError_t launch_axis_batch_f32(int op, int k, int mode, int sd, const AxisLaunch &a, const Geometry &g,
                                  const SampleView &sv, const TilePtrs *fields, uint32_t bpf, uint32_t nitems,
                                  int *grid, cudaStream_t st)
{
    if (mode == 1)
        return launch_batch_k<float, K64, 1>(op, sd, a, g, sv, fields, bpf, nitems, grid, st);
    if (k == K64)
        return launch_batch_k<float, K64, 0>(op, sd, a, g, sv, fields, bpf, nitems, grid, st);
    return launch_axis_batch_f32l(op, sd, a, g, sv, fields, bpf, nitems, grid, st);
}

cudaError_t launch_axis_mixed_f32l(int op, int sd, int layout, const MixedField *fields, const uint2 *items,
                                   uint32_t nitems, size_t smem, int threads, cudaStream_t st);

cudaError_t launch_axis_mixed_f32(int op, int k, int mode, int sd, int layout, const MixedField *fields,
                                  const uint2 *items, uint32_t nitems, size_t smem, int threads, cudaStream_t st)
{
    if (mode == 1)
        return launch_mixed_k<float, K64, 1>(op, sd, layout, fields, items, nitems, smem, threads, st);
    if (k == K64)
        return launch_mixed_k<float, K64, 0>(op, sd, layout, fields, items, nitems, smem, threads, st);
    return launch_axis_mixed_f32l(op, sd, layout, fields, items, nitems, smem, threads, st);
}

}  // namespace fbg
