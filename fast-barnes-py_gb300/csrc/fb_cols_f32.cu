// fb_cols_f32.cu -- float32-compensated instantiations of the pipelined
// columns kernel (fb_cols.cuh): the 33- and 17-cell sliding chunks and the
// direct sums.
#include "fb_cols.cuh"

namespace fbg {

cudaError_t launch_cols_pipe_f32(int k, int mode, const CUtensorMap &map, const ColsPipe &p, const TilePtrs *fields,
                                 int grid, cudaStream_t st)
{
    if (mode == 1)
        return launch_cols_pipe_t<float, K64, 1>(map, p, fields, grid, st);
    if (k == K32)
        return launch_cols_pipe_t<float, K32, 0>(map, p, fields, grid, st);
    return launch_cols_pipe_t<float, K64, 0>(map, p, fields, grid, st);
}

cudaError_t cols_pipe_regs_f32(int k, int mode, int *regs)
{
    if (mode == 1)
        return cols_pipe_regs_t<float, K64, 1>(regs);
    if (k == K32)
        return cols_pipe_regs_t<float, K32, 0>(regs);
    return cols_pipe_regs_t<float, K64, 0>(regs);
}

}  // namespace fbg
