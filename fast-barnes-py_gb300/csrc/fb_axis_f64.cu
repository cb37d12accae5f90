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

}  // namespace fbg
