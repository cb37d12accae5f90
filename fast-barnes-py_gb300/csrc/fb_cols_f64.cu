// fb_cols_f64.cu -- float64 instantiations of the pipelined columns kernel
// (fb_cols.cuh): the 17- and 9-cell sliding chunks and the direct sums.
#include "fb_cols.cuh"

namespace fbg {

cudaError_t launch_cols_pipe_f64(int k, int mode, const CUtensorMap &map, const ColsPipe &p, const TilePtrs *fields,
                                 int grid, cudaStream_t st)
{
    if (mode == 1)
        return launch_cols_pipe_t<double, K64, 1>(map, p, fields, grid, st);
    if (k == K9)
        return launch_cols_pipe_t<double, K9, 0>(map, p, fields, grid, st);
    return launch_cols_pipe_t<double, K64, 0>(map, p, fields, grid, st);
}

cudaError_t cols_pipe_regs_f64(int k, int mode, int *regs)
{
    if (mode == 1)
        return cols_pipe_regs_t<double, K64, 1>(regs);
    if (k == K9)
        return cols_pipe_regs_t<double, K9, 0>(regs);
    return cols_pipe_regs_t<double, K64, 0>(regs);
}

}  // namespace fbg
