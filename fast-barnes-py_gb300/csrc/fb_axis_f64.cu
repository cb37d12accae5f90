// fb_axis_f64.cu -- float64-form instantiations of the axis kernels.
#include "fb_axis_impl.cuh"

namespace fbg {

cudaError_t launch_axis_f64(int mode, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                            cudaStream_t st)
{
    if (mode == 1)
        return launch_k<double, K64, 1>(sd, a, g, sv, st);
    return launch_k<double, K64, 0>(sd, a, g, sv, st);
}

cudaError_t launch_axis_batch_f64(int op, int mode, int sd, int layout, const BatchAxisField *fields,
                                  const BatchItem *items, uint32_t nitems, uint32_t *counter, size_t smem,
                                  int threads, int *grid, cudaStream_t st)
{
    if (mode == 1)
        return launch_batch_k<double, K64, 1>(op, sd, layout, fields, items, nitems, counter, smem, threads, grid,
                                              st);
    return launch_batch_k<double, K64, 0>(op, sd, layout, fields, items, nitems, counter, smem, threads, grid, st);
}

}  // namespace fbg
