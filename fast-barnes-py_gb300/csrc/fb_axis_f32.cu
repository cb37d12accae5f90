// fb_axis_f32.cu -- float32-form instantiations of the axis kernels.
#include "fb_axis_impl.cuh"

namespace fbg {

cudaError_t launch_axis_f32(int k, int mode, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                            cudaStream_t st)
{
    if (mode == 1)
        return launch_k<float, K64, 1>(sd, a, g, sv, st);
    if (k == K64)
        return launch_k<float, K64, 0>(sd, a, g, sv, st);
    return launch_k<float, K32, 0>(sd, a, g, sv, st);
}

}  // namespace fbg
