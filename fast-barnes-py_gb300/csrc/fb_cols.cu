// fb_cols.cu -- host side of the pipelined columns kernel (fb_cols.cuh):
// launch geometry, the TMA tensor map over the intermediate cells, and the
// dispatch to the per-precision instantiations in fb_cols_f32.cu /
// fb_cols_f64.cu.
#include <string.h>

#include <algorithm>
#include <mutex>

#include "fb_cols.cuh"
#include "fb_kernels.cuh"

namespace fbg {

cudaError_t launch_cols_pipe_f32(int k, int mode, const CUtensorMap &map, const ColsPipe &p, const TilePtrs *fields,
                                 int grid, cudaStream_t st);
cudaError_t launch_cols_pipe_f64(int k, int mode, const CUtensorMap &map, const ColsPipe &p, const TilePtrs *fields,
                                 int grid, cudaStream_t st);
cudaError_t cols_pipe_regs_f32(int k, int mode, int *regs);
cudaError_t cols_pipe_regs_f64(int k, int mode, int *regs);

namespace {
// 0 off, 1 on, 2 automatic: on for float64 cells, off for float32 cells
// (measured on the GB300 headline batch: the float64 column stage 1% faster
// pipelined, the float32 one 3% slower; both kernels give identical results)
int g_pipe_mode = 2;

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link libcuda itself).
EncodeTiledFn encode_fn()
{
    static std::once_flag once;
    static EncodeTiledFn fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

int round_up(int64_t x, int m) { return (int)((x + m - 1) / m * m); }
}  // namespace

int cols_pipe_tune(int value)
{
    if (value < 0 || value > 2)
        return -1;
    g_pipe_mode = value;
    return 0;
}

bool cols_pipe_plan(int precision, const AxisLaunch &a, const Geometry &g, int nfields, ColsPipe &cp, int &K,
                    int &mode, int want)
{
    if (want < 0)
        want = g_pipe_mode == 2 ? (precision == 0 ? 1 : 0) : g_pipe_mode;
    if (!want || a.layout != 1 || a.ntiles != 1 || a.fill_splat || a.plain || a.passes < 1 || nfields < 1)
        return false;
    if (a.axis != 1 && a.axis != 2)
        return false;
    const int cs = precision == 0 ? 16 : 8;
    const int G = 32 / cs;
    // the tensor map's row stride (x extent of (v, w) cells) must be a
    // multiple of 16 bytes
    if ((g.size[0] * cs) % 16 != 0)
        return false;
    K = axis_variant_k(precision, a);
    mode = axis_variant_mode(precision, a);
    memset(&cp, 0, sizeof(cp));
    const int64_t E = a.L;
    const int T = a.T;
    const int nact = (int)(mode == 1 ? (E + K - 1) / K : (E + T + 1 + K - 1) / K);
    const int unit = 32 / G;
    cp.chunks_pad = round_up(nact, unit);
    cp.group_threads = G * cp.chunks_pad;
    cp.L = (int)E;
    // every read and every (zero) write of a chunk lies in
    // [-(T + 1 + K), E + T + K) of the line
    cp.line_pad = round_up(T + 1 + K, 4);
    cp.box_rows = E >= 256 ? 256 : round_up(E, 4);
    cp.nboxes = (int)((E + cp.box_rows - 1) / cp.box_rows);
    cp.line_pitch = round_up(std::max<int64_t>(cp.line_pad + E + T + K,
                                               (int64_t)cp.line_pad + (int64_t)cp.nboxes * cp.box_rows),
                             4);
    cp.stage_bytes = (uint32_t)round_up((int64_t)cp.line_pitch * 32, 128);
    const int q = (2 * T + 1) / K;
    cp.part_pad = q + 1;
    cp.part_pitch = round_up(cp.part_pad + cp.chunks_pad + q + 2, 2);
    cp.part_bytes = (uint32_t)round_up((int64_t)2 * cp.part_pitch * G * cs, 128);
    cp.axis = a.axis;
    cp.T = T;
    cp.passes = a.passes;
    cp.scaled = a.scaled;
    cp.store_quot = a.store_quot;
    cp.out_f64 = a.out_f64;
    cp.quant_bits = a.quant_bits;
    cp.alpha = a.alpha;
    cp.inv_norm = a.inv_norm;
    cp.thr = a.thr;
    cp.xblocks = (uint32_t)a.xblocks;
    cp.width = a.width;
    cp.elem_stride = a.elem_stride;
    cp.outer_stride = a.outer_stride;
    const int64_t tpf = a.outer_count * a.xblocks;
    if (tpf * nfields > (int64_t)0x7FFFFFFF)
        return false;
    cp.tiles_per_field = (uint32_t)tpf;
    cp.ntiles = (uint32_t)(tpf * nfields);
    int regs = 0;
    cudaError_t e = precision == 0 ? cols_pipe_regs_f64(K, mode, &regs) : cols_pipe_regs_f32(K, mode, &regs);
    if (e != cudaSuccess || regs <= 0)
        return false;
    const size_t lim = axis_smem_limit();
    // two consumer groups over three stages (the load of the next column
    // group always in flight), else one group over two stages, else one
    const int shapes[3][2] = {{2, 3}, {1, 2}, {1, 1}};
    for (const auto &sh : shapes) {
        cp.ngroups = sh[0];
        cp.nstages = sh[1];
        const int threads = cp.ngroups * cp.group_threads;
        if (threads > 1024 || (int64_t)threads * regs > 65536)
            continue;
        if (cols_pipe_smem(cp) > lim)
            continue;
        return true;
    }
    return false;
}

cudaError_t cols_pipe_map(int precision, const ColsPipe &cp, const Geometry &g, const void *src0,
                          int64_t field_stride, int nfields, CUtensorMap *map)
{
    EncodeTiledFn enc = encode_fn();
    if (!enc)
        return cudaErrorNotSupported;
    const cuuint64_t sz = precision == 0 ? 8 : 4;
    const cuuint64_t W = (cuuint64_t)g.size[0], H = (cuuint64_t)g.size[1], Z = (cuuint64_t)g.size[2];
    const cuuint64_t dims[4] = {2 * W, H, Z, (cuuint64_t)nfields};
    const cuuint64_t fs = nfields > 1 ? (cuuint64_t)field_stride : 2 * W * H * Z * sz;
    const cuuint64_t strides[3] = {2 * W * sz, 2 * W * H * sz, fs};
    const int G = precision == 0 ? 2 : 4;
    const cuuint32_t box[4] = {(cuuint32_t)(2 * G), cp.axis == 1 ? (cuuint32_t)cp.box_rows : 1u,
                               cp.axis == 2 ? (cuuint32_t)cp.box_rows : 1u, 1u};
    const cuuint32_t es[4] = {1u, 1u, 1u, 1u};
    CUresult r = enc(map, precision == 0 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4,
                     const_cast<void *>(src0), dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                     CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

cudaError_t launch_cols_pipe(int precision, int k, int mode, const CUtensorMap &map, const ColsPipe &cp,
                             const TilePtrs *fields, cudaStream_t st)
{
    if (cp.ntiles == 0)
        return cudaSuccess;
    const int grid = (int)std::min<int64_t>((int64_t)cp.ntiles, (int64_t)device_sm_count());
    if (precision == 0)
        return launch_cols_pipe_f64(k, mode, map, cp, fields, grid, st);
    return launch_cols_pipe_f32(k, mode, map, cp, fields, grid, st);
}

}  // namespace fbg
