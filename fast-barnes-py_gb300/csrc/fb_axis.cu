// fb_axis.cu -- launch shapes of the axis kernels (shared-memory extents,
// threads, lines per CTA) and the dispatch to the per-precision instantiations
// in fb_axis_f32.cu and fb_axis_f64.cu.
#include <string.h>

#include <algorithm>
#include <mutex>
#include <set>
#include <utility>

#include "fb_axis_impl.cuh"

namespace fbg {

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// Chunk length per launch.  Every output is at most K/2 sliding steps from an
// exact anchor; in float32 that distance must stay short against the window
// 2T+1, so windows up to 65 cells use the short chunk; wider windows use the
// long chunk (half the anchor overhead) unless fb_tune("chunk", 17) asks for
// the short one.
static int g_chunk_choice = 0;   // 0 = automatic, 17, 33

static int chunk_k(int precision, int T)
{
    if (precision == 0 || T <= 32)
        return K64;
    return g_chunk_choice == K64 ? K64 : K32;
}

static bool direct_mode(int precision, int T) { return T <= (precision == 0 ? DirectMax<double>::T : DirectMax<float>::T); }

// Chunk length of one launch: the direct-sum kernels and float64 use the
// short chunk; a plan may pin 17 or 33 for float32 sliding sums.
static int kchunk_of(int precision, int T, int kchunk)
{
    if (direct_mode(precision, T))
        return K64;
    if (precision == 0)
        return 2 * T + 1 >= K64 ? K64 : K9;
    if (T <= 32)
        return K64;
    if (kchunk == K64 || kchunk == K32)
        return kchunk;
    return chunk_k(precision, T);
}

static int cell_size(int precision) { return precision == 0 ? 16 : 8; }
static int col_g(int precision) { return (precision == 0 ? kColBytesF64 : kColBytesF32) / cell_size(precision); }
int axis_col_group(int precision) { return col_g(precision); }
constexpr int kMaxThreads = 512;

// Per-device properties and kernel attributes.  A process may drive several
// devices (and several host threads): the shared-memory opt-in limit and the
// SM count are looked up once per device, and a kernel's dynamic
// shared-memory attribute, which applies to one device only, is set once per
// (kernel, device), all under one lock.
namespace {
constexpr int kMaxDevices = 64;
std::mutex g_dev_mu;
int g_smem_optin[kMaxDevices];
int g_sm_count[kMaxDevices];
std::set<std::pair<const void *, int>> g_attr_set;

int cur_device()
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        dev = 0;
    return dev;
}
}  // namespace

size_t axis_smem_limit()
{
    const int dev = cur_device();
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (g_smem_optin[dev] <= 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess || v <= 0)
            v = 227 * 1024;
        // keep room for the kernels' few bytes of static shared memory
        g_smem_optin[dev] = v - 1024;
    }
    return (size_t)g_smem_optin[dev];
}

int device_sm_count()
{
    const int dev = cur_device();
    std::lock_guard<std::mutex> lk(g_dev_mu);
    if (g_sm_count[dev] <= 0) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
            v = 1;
        g_sm_count[dev] = v;
    }
    return g_sm_count[dev];
}

cudaError_t ensure_smem_attr(const void *func)
{
    const size_t lim = axis_smem_limit();
    const int dev = cur_device();
    std::lock_guard<std::mutex> lk(g_dev_mu);
    const auto key = std::make_pair(func, dev);
    if (g_attr_set.count(key))
        return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lim);
    if (e == cudaSuccess)
        g_attr_set.insert(key);
    return e;
}

static int even(int64_t x) { return (int)((x + 1) / 2 * 2); }

// Shared-memory geometry of a launch whose longest line extent is E.  Chunk
// slots: ceil(E/K) for direct sums, ceil((E + T + 1)/K) for sliding passes
// (their chunks alternate between two grids T + 1 cells apart; a chunk that
// lies wholly outside [0, E) in a pass reads clamped cells and is cleared).
// Every read lies in [-(T + 1 + K), E + T + K): the line buffer has
// T + 1 + K zero cells before the line (one more when that is odd, so that
// cell 0 of a float32 line is 16-byte aligned for vector stores) and T + K
// after it.  The two partial-sum arrays (S, X) have q + 1
// zero slots on both sides, q = floor((2T + 1)/K).
static void set_geometry(int precision, AxisLaunch &a, int K, int64_t E)
{
    const bool direct = direct_mode(precision, a.T);
    const int nact = (int)(direct ? (E + K - 1) / K : (E + a.T + 1 + K - 1) / K);
    const int unit = a.layout == 0 ? 32 : 32 / col_g(precision);
    a.chunks_pad = (nact + unit - 1) / unit * unit;
    a.extent_max = (int)E;
    a.line_pad = (a.T + 1 + K + 1) & ~1;
    a.line_pitch = even((int64_t)a.line_pad + E + a.T + K);
    const int q = (2 * a.T + 1) / K;
    a.part_pad = q + 1;
    a.part_pitch = even((int64_t)a.part_pad + a.chunks_pad + q + 2);
}

size_t axis_smem_bytes(int precision, const AxisLaunch &a)
{
    const size_t cs = cell_size(precision);
    const size_t nlc = a.layout == 0 ? (size_t)a.lines_per_cta : (size_t)col_g(precision);
    size_t b = nlc * ((size_t)a.line_pitch + 2 * (size_t)a.part_pitch) * cs;
    if (a.fill_splat)
        b += nlc * kStage * (precision == 0 ? sizeof(StageRec<double>) : sizeof(StageRec<float>));
    return b;
}

int axis_threads(int precision, const AxisLaunch &a)
{
    if (a.layout == 0)
        return a.lines_per_cta * a.chunks_pad;
    return col_g(precision) * a.chunks_pad;
}

// Chunk length of a columns launch over whole lines of L cells: the plan's
// choice, except that a float32 sliding launch whose CTA would need more
// than eight warps with the long chunk (lines longer than 64 chunks once
// the T + 1 shift of the sliding grids is added) takes the short one.  Its
// 126-register threads would then leave room for one CTA an SM; with the
// short chunk (64 registers) two 512-thread CTAs fit (measured on a batch of
// 8 fields of 4096 x 2048, T = 94 / 66: y axis 371 -> 261 us, 454 -> 287 us).
int axis_cols_chunk(int precision, int T, int64_t L, int kchunk)
{
    if (precision == 0 || direct_mode(precision, T) || kchunk_of(precision, T, kchunk) != K32)
        return kchunk;
    AxisLaunch a{};
    a.layout = 1;
    a.T = T;
    set_geometry(precision, a, K32, L);
    if (axis_threads(precision, a) <= 256)
        return kchunk;
    AxisLaunch b{};
    b.layout = 1;
    b.T = T;
    set_geometry(precision, b, K64, L);
    if (axis_threads(precision, b) > kMaxThreads || axis_smem_bytes(precision, b) > axis_smem_limit())
        return kchunk;
    return K64;
}

AxisPlanLimits axis_limits(int precision, int T, int kchunk)
{
    // the longest extent a rows-layout CTA (one line) and a columns-layout CTA
    // (G lines) can hold; the plan uses the one of its layout
    AxisPlanLimits l;
    l.smem_limit = axis_smem_limit();
    const int K = kchunk_of(precision, T, kchunk);
    int best[2] = {0, 0};
    for (int lay = 0; lay < 2; lay++) {
        int lo = 0, hi = kMaxThreads * K;
        while (lo < hi) {
            int mid = (lo + hi + 1) / 2;
            AxisLaunch a{};
            a.layout = lay;
            a.lines_per_cta = 1;
            a.fill_splat = lay == 0;
            a.T = T;
            set_geometry(precision, a, K, mid);
            if (axis_threads(precision, a) <= kMaxThreads && axis_smem_bytes(precision, a) <= l.smem_limit)
                lo = mid;
            else
                hi = mid - 1;
        }
        best[lay] = lo;
    }
    l.extent_max = best[0];
    l.extent_max_cols = best[1];
    return l;
}

bool axis_shape(int precision, AxisLaunch &a)
{
    const int K = kchunk_of(precision, a.T, a.kchunk);
    int64_t E = a.tile_len + 2 * (int64_t)a.halo;
    if (E > a.L)
        E = a.L;
    set_geometry(precision, a, K, E);
    if (a.layout == 1) {
        a.lines_per_cta = col_g(precision);
        return axis_threads(precision, a) <= kMaxThreads && axis_smem_bytes(precision, a) <= axis_smem_limit();
    }
    // rows: ~128 threads per CTA (the batch autotuner's usual choice: five
    // CTAs an SM, one line each for lines of ~4k cells) unless the plan asks
    // for another target
    const int target = a.rows_threads > 0 ? a.rows_threads : 128;
    int nl = std::max(1, std::min<int>(std::max(1, target / a.chunks_pad), kMaxThreads / a.chunks_pad));
    if (nl > a.nlines)
        nl = (int)a.nlines;
    for (; nl >= 1; nl--) {
        a.lines_per_cta = nl;
        if (axis_smem_bytes(precision, a) <= axis_smem_limit() && axis_threads(precision, a) <= kMaxThreads)
            return true;
    }
    return false;
}

cudaError_t launch_axis_f32(int k, int mode, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                            cudaStream_t st);
cudaError_t launch_axis_f64(int k, int mode, int sd, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                            cudaStream_t st);

cudaError_t launch_axis_batch_f32(int op, int k, int mode, int sd, const AxisLaunch &a, const Geometry &g,
                                  const SampleView &sv, const TilePtrs *fields, uint32_t bpf, uint32_t nitems,
                                  int *grid, cudaStream_t st);
cudaError_t launch_axis_batch_f64(int op, int k, int mode, int sd, const AxisLaunch &a, const Geometry &g,
                                  const SampleView &sv, const TilePtrs *fields, uint32_t bpf, uint32_t nitems,
                                  int *grid, cudaStream_t st);


cudaError_t launch_axis_mixed_f32(int op, int k, int mode, int sd, int layout, const MixedField *fields,
                                  const uint2 *items, uint32_t nitems, size_t smem, int threads, cudaStream_t st);
cudaError_t launch_axis_mixed_f64(int op, int k, int mode, int sd, int layout, const MixedField *fields,
                                  const uint2 *items, uint32_t nitems, size_t smem, int threads, cudaStream_t st);

int axis_variant_k(int precision, const AxisLaunch &a) { return kchunk_of(precision, a.T, a.kchunk); }
int axis_variant_mode(int precision, const AxisLaunch &a) { return direct_mode(precision, a.T) ? 1 : 0; }

cudaError_t launch_axis_mixed(int op, int precision, int k, int mode, int sd, int layout, const MixedField *fields,
                              const uint2 *items, uint32_t nitems, size_t smem, int threads, cudaStream_t st)
{
    if (layout == 1 && sd != 0)
        return cudaErrorInvalidValue;
    if (precision == 0)
        return launch_axis_mixed_f64(op, k, mode, sd, layout, fields, items, nitems, smem, threads, st);
    return launch_axis_mixed_f32(op, k, mode, sd, layout, fields, items, nitems, smem, threads, st);
}

cudaError_t launch_axis_batch(int op, int precision, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                              const TilePtrs *fields, uint32_t bpf, uint32_t nitems, int *grid, cudaStream_t st)
{
    const int sd = a.fill_splat ? g.dim : 0;
    if (a.layout == 1 && a.fill_splat)
        return cudaErrorInvalidValue;
    const int mode = direct_mode(precision, a.T) ? 1 : 0;
    if (precision == 0)
        return launch_axis_batch_f64(op, kchunk_of(precision, a.T, a.kchunk), mode, sd, a, g, sv, fields, bpf,
                                     nitems, grid, st);
    return launch_axis_batch_f32(op, kchunk_of(precision, a.T, a.kchunk), mode, sd, a, g, sv, fields, bpf, nitems,
                                 grid, st);
}

cudaError_t launch_axis(int precision, const AxisLaunch &a, const Geometry &g, const SampleView &sv,
                        cudaStream_t st)
{
    const int sd = a.fill_splat ? g.dim : 0;
    if (a.layout == 1 && a.fill_splat)
        return cudaErrorInvalidValue;
    if (a.layout == 1) {
        ColsPipe cp;
        int k = 0, mode = 0;
        CUtensorMap map;
        if (cols_pipe_plan(precision, a, g, 1, cp, k, mode) &&
            cols_pipe_map(precision, cp, g, a.src_v, 0, 1, &map) == cudaSuccess) {
            cp.single.src = a.src_v;
            cp.single.dst = a.dst_v;
            cp.single.out = a.out;
            cp.single.bin_start = sv.bin_start;
            cp.single.hdr = sv.hdr;
            cp.status = sv.hdr ? reinterpret_cast<uint32_t *>(const_cast<int *>(&sv.hdr->error)) : nullptr;
            return launch_cols_pipe(precision, k, mode, map, cp, nullptr, st);
        }
    }
    const int mode = direct_mode(precision, a.T) ? 1 : 0;
    if (precision == 0)
        return launch_axis_f64(kchunk_of(precision, a.T, a.kchunk), mode, sd, a, g, sv, st);
    return launch_axis_f32(kchunk_of(precision, a.T, a.kchunk), mode, sd, a, g, sv, st);
}

int axis_tune(const char *name, int value)
{
    if (strcmp(name, "chunk") == 0 && (value == 0 || value == K64 || value == K32)) {
        g_chunk_choice = value;
        return 0;
    }
    if (strcmp(name, "cols_pipe") == 0)
        return cols_pipe_tune(value);
    return -1;
}

cudaError_t launch_lines(int precision, void *data, int64_t nlines, int64_t len, int T, double alpha, int passes,
                         int normalize, cudaStream_t st)
{
    AxisLaunch a{};
    a.axis = 0;
    a.layout = 0;
    a.L = len;
    a.elem_stride = 1;
    a.nlines = nlines;
    a.tile_len = len;
    a.ntiles = 1;
    a.halo = 0;
    a.passes = passes;
    a.T = T;
    a.alpha = alpha;
    a.scaled = normalize ? 1 : 0;
    a.inv_norm = 1.0 / (2.0 * T + 1.0 + 2.0 * alpha);
    a.fill_splat = 0;
    a.store_quot = 0;
    a.plain = 1;
    a.src_v = data;
    a.dst_v = data;
    if (!axis_shape(precision, a))
        return cudaErrorInvalidValue;
    Geometry g{};
    g.dim = 1;
    g.size[0] = len;
    g.size[1] = g.size[2] = 1;
    SampleView sv{};
    return launch_axis(precision, a, g, sv, st);
}

}  // namespace fbg
