// fb_capi.cu -- the C ABI: argument checks, kernel-size parameters, workspace
// layout and the per-axis launch plan of one interpolation.
//
// Host arithmetic (T, alpha, the NaN threshold) follows the reference's float64
// expressions operation by operation; this file is compiled without FMA
// contraction so the host results are identical on x86 and aarch64.
#include <math.h>
#include <stddef.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/fastbarnes_gb300.h"
#include "fb_internal.cuh"
#include "fb_kernels.cuh"

using namespace fbg;

// NVTX range around the launches of one stage (the sample sort, one axis),
// so that Nsight tools group and filter the kernels by stage (for example
// ncu --nvtx --nvtx-include "fb axis 1/"); without an attached tool a push
// or a pop costs a test of one pointer.
struct StageRange {
    explicit StageRange(const char *name) { nvtxRangePushA(name); }
    ~StageRange() { nvtxRangePop(); }
    StageRange(const StageRange &) = delete;
    StageRange &operator=(const StageRange &) = delete;
};
static const char *axis_range_name(int axis)
{
    static const char *const names[3] = {"fb axis 0", "fb axis 1", "fb axis 2"};
    return names[axis <= 0 ? 0 : (axis >= 2 ? 2 : axis)];
}

static thread_local char g_err[512];

static int fail(int code, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

static int cuda_fail(cudaError_t e, const char *where)
{
    return fail(FB_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

// FB_ERR_DEVICE with a message naming the status bits a kernel recorded.
static int device_fail(uint32_t bits, const char *where)
{
    return fail(FB_ERR_DEVICE, "%s: device status 0x%x%s%s", where, bits,
                (bits & FB_DEVICE_TIMEOUT) ? " (a pipeline wait ran out: the kernel stopped early)" : "",
                (bits & FB_DEVICE_BOUNDS) ? " (an out-of-range index was skipped: bounds-check build)" : "");
}

extern "C" const char *fb_version(void)
{
    return kBoundsCheck ? "fastbarnes_gb300 0.1 (sm_103a, bounds-check build)" : "fastbarnes_gb300 0.1 (sm_103a)";
}
extern "C" const char *fb_last_error(void) { return g_err; }

extern "C" int fb_tune(const char *name, int value)
{
    if (!name || axis_tune(name, value) != 0)
        return fail(FB_ERR_ARG, "unknown tuning knob or value");
    return FB_OK;
}

// ---------------------------------------------------------------------------
// kernel-size helpers: fastbarnes/interpolation.py:543-569, :777-803
// ---------------------------------------------------------------------------

extern "C" int fb_half_kernel_size_opt(double sigma, double step, int num_iter)
{
    double s = sigma / step;
    return (int)((sqrt(1.0 + 12.0 * s * s / (double)num_iter) - 1.0) / 2.0);
}

extern "C" double fb_tail_value(double sigma, double step, int num_iter)
{
    int hks = fb_half_kernel_size_opt(sigma, step, num_iter);
    int ks = 2 * hks + 1;
    double sigma_rect_sqr = (double)((hks + 1) * hks) / 3.0 * (step * step);
    double s2n = sigma * sigma / (double)num_iter;
    double d = (double)(hks + 1) * step;
    return 0.5 * (double)ks * (s2n - sigma_rect_sqr) / (d * d - s2n);
}

extern "C" int fb_half_kernel_size(double sigma, double step, int num_iter)
{
    return (int)(sqrt(3.0 / (double)num_iter) * sigma / step + 0.5);
}

extern "C" double fb_sigma_effective(double sigma, double step, int num_iter)
{
    int hks = fb_half_kernel_size(sigma, step, num_iter);
    return sqrt((double)num_iter / 3.0 * (double)hks * (double)(hks + 1)) * step;
}

// ---------------------------------------------------------------------------
// planning
// ---------------------------------------------------------------------------

namespace {

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

struct Plan {
    Geometry g;
    int precision = 1;
    int64_t npts = 0;
    int64_t npoints = 0;     // grid points
    uint32_t nbins = 0;
    int bin_w = 1;
    std::vector<AxisLaunch> launches;
    int pairs = 0;           // intermediate value/weight field pairs needed
    bool naive = false;      // method FB_NAIVE: one direct-sum kernel, no launches
    double sigma[3] = {1, 1, 1};
    // workspace layout
    size_t off_hdr = 0, off_bins = 0, off_sort = 0, off_pair[2] = {0, 0}, total = 0;
};

// Half kernel size, tail value and the reference's NaN threshold for one axis
// (interpolation.py:351-353, :424-425 / :669-670).
void axis_params(int method, double sigma, double step, int n, int &T, double &alpha, double &factor)
{
    if (method == FB_OPTIMIZED_CONVOLUTION) {
        T = fb_half_kernel_size_opt(sigma, step, n);
        alpha = fb_tail_value(sigma, step, n);
        double ks = (double)(2 * T + 1);
        factor = pow(ks + 2.0 * alpha, (double)n) / sqrt(2.0 * 3.14159265358979311600) / (sigma / step);
    } else {
        T = fb_half_kernel_size(sigma, step, n);
        alpha = 0.0;
        // int32 kernel size raised to the power n in int32 arithmetic, as the
        // reference's numpy expression does (wraps for large kernels)
        uint32_t p = 1u;
        for (int e = 0; e < n; e++)
            p *= (uint32_t)(2 * T + 1);
        factor = (double)(int32_t)p / sqrt(2.0 * 3.14159265358979311600) / (sigma / step);
    }
}

int make_plan(int method, int precision, int dim, int64_t npts, const double *sigma, const double *x0,
              const double *step, const int64_t *size, int num_iter, double max_dist_weight, Plan &p,
              int kchunk = 0, int rows_threads = 0)
{
    if (dim < 1 || dim > 3)
        return fail(FB_ERR_ARG, "dim must be 1, 2 or 3 (got %d)", dim);
    if (precision != FB_FP64 && precision != FB_FP32C)
        return fail(FB_ERR_ARG, "unknown precision %d", precision);
    if (method != FB_OPTIMIZED_CONVOLUTION && method != FB_CONVOLUTION && method != FB_NAIVE)
        return fail(FB_ERR_ARG, "unknown method %d", method);
    if (num_iter < 1)
        return fail(FB_ERR_ARG, "num_iter must be >= 1 (got %d)", num_iter);
    if (npts < 0 || npts > (int64_t)0xFFFFFFF0ll)
        return fail(FB_ERR_ARG, "number of samples out of range (%lld)", (long long)npts);
    if (!sigma || !step || !size)
        return fail(FB_ERR_ARG, "sigma, step and size are required");
    p = Plan();
    p.precision = precision;
    p.npts = npts;
    if (method == FB_NAIVE) {
        // interpolation.py:861-938: no kernel size, no mask level; the
        // workspace holds the value range only
        p.naive = true;
        p.g.dim = dim;
        p.npoints = 1;
        for (int m = 0; m < 3; m++) {
            p.g.size[m] = m < dim ? size[m] : 1;
            p.g.x0[m] = (m < dim && x0) ? x0[m] : 0.0;
            p.g.step[m] = m < dim ? step[m] : 1.0;
            p.sigma[m] = m < dim ? sigma[m] : 1.0;
            if (m < dim && size[m] < 1)
                return fail(FB_ERR_ARG, "size[%d] must be positive (got %lld)", m, (long long)size[m]);
            p.npoints *= p.g.size[m];
        }
        p.off_hdr = 0;
        p.total = align_up(sizeof(FieldHeader));
        return FB_OK;
    }
    Geometry &g = p.g;
    g.dim = dim;
    g.num_iter = num_iter;
    double thr = 1.0, scale = 1.0;
    double inv[3] = {1, 1, 1};
    for (int m = 0; m < 3; m++) {
        g.size[m] = m < dim ? size[m] : 1;
        g.x0[m] = (m < dim && x0) ? x0[m] : 0.0;
        g.step[m] = m < dim ? step[m] : 1.0;
        g.T[m] = 0;
        g.alpha[m] = 0.0;
    }
    p.npoints = 1;
    for (int m = 0; m < dim; m++) {
        if (size[m] < 1)
            return fail(FB_ERR_ARG, "size[%d] must be positive (got %lld)", m, (long long)size[m]);
        double factor;
        axis_params(method, sigma[m], step[m], num_iter, g.T[m], g.alpha[m], factor);
        if (2 * (int64_t)g.T[m] + 1 >= size[m])
            return fail(FB_ERR_KERNEL_SIZE,
                        "resulting rectangular kernel size should be smaller w.r.t. specified grid: "
                        "axis %d kernel %d vs. size %lld",
                        m, 2 * g.T[m] + 1, (long long)size[m]);
        thr = (m == 0) ? factor : thr * factor;
        inv[m] = 1.0 / (2.0 * g.T[m] + 1.0 + 2.0 * g.alpha[m]);
        scale *= pow(inv[m], (double)num_iter);
        p.npoints *= size[m];
    }
    thr = thr * max_dist_weight;
    g.thr = thr;

    // bins of the sample sort: rows (2D), (z, y) rows (3D), x ranges (1D)
    if (dim == 1) {
        p.bin_w = (int)std::max<int64_t>(64, (size[0] + 65535) / 65536);
        p.nbins = (uint32_t)((size[0] + p.bin_w - 1) / p.bin_w);
    } else if (dim == 2) {
        p.nbins = (uint32_t)size[1];
    } else {
        if (size[1] * size[2] > (int64_t)0x7FFFFFFF)
            return fail(FB_ERR_ARG, "grid too large");
        p.nbins = (uint32_t)(size[1] * size[2]);
    }

    // float32 sums are left unscaled (like the reference's float64 ones)
    // unless the kernel growth prod_m (2T+1+2a)^n could overflow float32
    double growth = 1.0;
    for (int m = 0; m < dim; m++)
        growth *= pow(1.0 / inv[m], (double)num_iter);
    const bool scaled = precision == FB_FP32C && growth * (double)std::max<int64_t>(npts, 1) > 1e24;

    // per-axis launches; `cur` tracks which buffer pair holds the data
    int cur = -1;   // -1: nothing yet (first launch splats)
    for (int m = 0; m < dim; m++) {
        const int64_t L = size[m];
        const int T = g.T[m];
        const int kc = m == 0 ? kchunk : axis_cols_chunk(precision, T, L, kchunk);
        const AxisPlanLimits lim = axis_limits(precision, T, kc);
        const int64_t emax = m == 0 ? lim.extent_max : lim.extent_max_cols;
        std::vector<AxisLaunch> axl;
        AxisLaunch a{};
        a.axis = m;
        a.layout = m == 0 ? 0 : 1;
        a.L = L;
        a.elem_stride = m == 0 ? 1 : (m == 1 ? size[0] : size[0] * size[1]);
        a.nlines = p.npoints / L;
        a.width = size[0];
        a.xblocks = (size[0] + axis_col_group(precision) - 1) / axis_col_group(precision);
        a.outer_count = m == 1 ? (dim > 2 ? size[2] : 1) : (m == 2 ? size[1] : 1);
        a.outer_stride = m == 1 ? size[0] * size[1] : size[0];
        a.T = T;
        a.alpha = g.alpha[m];
        a.scaled = scaled ? 1 : 0;
        a.inv_norm = inv[m];
        a.kchunk = kc;
        a.rows_threads = rows_threads;
        bool ok = false;
        if (L <= emax) {
            a.tile_len = L;
            a.ntiles = 1;
            a.halo = 0;
            a.passes = num_iter;
            ok = axis_shape(precision, a);
            if (ok)
                axl.push_back(a);
        }
        if (!ok) {
            const int64_t h = (int64_t)num_iter * (T + 1);
            const int64_t tl = emax - 2 * h;
            if (tl >= std::max<int64_t>(1024, emax / 4)) {
                a.tile_len = tl;
                a.ntiles = (L + tl - 1) / tl;
                a.halo = (int)h;
                a.passes = num_iter;
                ok = axis_shape(precision, a);
                if (ok)
                    axl.push_back(a);
            }
        }
        if (!ok) {
            const int64_t h = T + 1;
            const int64_t tl = emax - 2 * h;
            if (tl >= 256) {
                a.tile_len = tl;
                a.ntiles = (L + tl - 1) / tl;
                a.halo = (int)h;
                a.passes = 1;
                ok = axis_shape(precision, a);
                for (int it = 0; ok && it < num_iter; it++)
                    axl.push_back(a);
            }
        }
        if (!ok)
            return fail(FB_ERR_UNSUPPORTED,
                        "axis %d: kernel half width %d too large to tile a line of %lld cells", m, T,
                        (long long)L);
        for (size_t q = 0; q < axl.size(); q++) {
            AxisLaunch &x = axl[q];
            const bool first = (cur == -1);
            const bool last = (m == dim - 1) && (q + 1 == axl.size());
            x.fill_splat = first ? 1 : 0;
            x.store_quot = last ? 1 : 0;
            x.thr = scaled ? thr * scale : thr;
            int src = cur, dst;
            if (last)
                dst = -2;
            else if (first)
                dst = 0;
            else if (x.ntiles == 1)
                dst = src;   // whole lines: each CTA reads its lines before writing them
            else
                dst = 1 - src;
            // encode pair indices for resolve_pointers
            x.src_v = (const void *)(intptr_t)(src + 16);
            x.dst_v = (void *)(intptr_t)(dst + 16);
            if (dst >= 0)
                p.pairs = std::max(p.pairs, dst + 1);
            if (src >= 0)
                p.pairs = std::max(p.pairs, src + 1);
            cur = dst;
            p.launches.push_back(x);
        }
    }

    // workspace layout
    const size_t sz = precision == FB_FP64 ? 8 : 4;
    size_t off = 0;
    p.off_hdr = off;
    off = align_up(off + sizeof(FieldHeader));
    p.off_bins = off;
    off = align_up(off + sizeof(uint32_t) * ((size_t)p.nbins + 1));
    p.off_sort = off;
    off = align_up(off + sort_scratch_bytes(npts, p.nbins, precision));
    for (int q = 0; q < p.pairs; q++) {
        p.off_pair[q] = off;
        off = align_up(off + 2 * sz * (size_t)p.npoints);
    }
    p.total = off;
    return FB_OK;
}

void resolve_pointers(const Plan &p, char *ws, void *out, AxisLaunch &a)
{
    const size_t sz = p.precision == FB_FP64 ? 8 : 4;
    auto pair = [&](intptr_t code, int f) -> void * {
        int idx = (int)code - 16;
        if (idx < 0)
            return nullptr;
        return ws + p.off_pair[idx] + (size_t)f * sz * (size_t)p.npoints;
    };
    // intermediate fields are interleaved (v, w) cells: one buffer per pair
    intptr_t s = (intptr_t)a.src_v, d = (intptr_t)a.dst_v;
    a.src_v = pair(s, 0);
    a.src_w = nullptr;
    a.dst_v = pair(d, 0);
    a.dst_w = nullptr;
    a.out = out;
}

}  // namespace

// ---------------------------------------------------------------------------
// adjoint plan: the forward launches storing the final (V, W) cells, the seed,
// then the same launches again (loading cells instead of splatting) over the
// seeded gradient cells; routes the cell buffers through the pair slots
// ---------------------------------------------------------------------------

namespace {

struct GradPlan {
    Plan p;                    // p.launches = forward then adjoint launches
    size_t nfwd = 0;           // forward launches
    int seed_pair = 0;         // buffer holding the final cells / the seed
    int final_pair = 0;        // buffer holding the adjoint cells
    double thr = 0.0;          // mask level in the units of the stored weights
};

int make_grad_plan(int method, int precision, int dim, int64_t npts, const double *sigma, const double *x0,
                   const double *step, const int64_t *size, int num_iter, double max_dist_weight, GradPlan &gp)
{
    if (method == FB_NAIVE)
        return fail(FB_ERR_UNSUPPORTED, "gradients are provided for the convolution methods");
    int rc = make_plan(method, precision, dim, npts, sigma, x0, step, size, num_iter, max_dist_weight, gp.p);
    if (rc != FB_OK)
        return rc;
    Plan &p = gp.p;
    std::vector<AxisLaunch> fwd = p.launches;
    gp.nfwd = fwd.size();
    gp.thr = fwd.back().thr;
    std::vector<AxisLaunch> all = fwd;
    for (AxisLaunch x : fwd) {
        x.fill_splat = 0;
        all.push_back(x);
    }
    int cur = -1, maxp = 0;
    for (size_t q = 0; q < all.size(); q++) {
        AxisLaunch &x = all[q];
        const bool first = cur == -1;
        x.store_quot = 0;
        x.plain = 0;
        const int src = cur;
        const int dst = first ? 0 : (x.ntiles == 1 ? src : 1 - src);
        x.src_v = (const void *)(intptr_t)(src + 16);
        x.dst_v = (void *)(intptr_t)(dst + 16);
        maxp = std::max(maxp, dst + 1);
        cur = dst;
        if (q + 1 == gp.nfwd)
            gp.seed_pair = cur;
    }
    gp.final_pair = cur;
    p.launches = all;
    // cell buffers the forward plan did not need (a 1D forward plan needs
    // none; tiled adjoint launches may need a second one)
    const size_t sz = precision == FB_FP64 ? 8 : 4;
    for (int q = p.pairs; q < maxp; q++) {
        p.off_pair[q] = p.total;
        p.total = align_up(p.total + 2 * sz * (size_t)p.npoints);
    }
    p.pairs = std::max(p.pairs, maxp);
    return FB_OK;
}

}  // namespace

extern "C" int fb_grad_workspace_size(int method, int precision, int dim, int64_t n_pts, const double *sigma,
                                      const double *step, const int64_t *size, int num_iter, size_t *bytes)
{
    GradPlan gp;
    int rc = make_grad_plan(method, precision, dim, n_pts, sigma, nullptr, step, size, num_iter, 0.0, gp);
    if (rc != FB_OK)
        return rc;
    if (bytes)
        *bytes = gp.p.total;
    return FB_OK;
}

extern "C" int fb_interpolate_grad(int method, int precision, int dim, const double *d_pts, const double *d_val,
                                   int64_t n_pts, const double *sigma, const double *x0, const double *step,
                                   const int64_t *size, int num_iter, double max_dist_weight, const void *d_grad_out,
                                   int grad_f64, double *d_grad_val, double *d_grad_pts, void *d_workspace,
                                   size_t workspace_bytes, void *stream)
{
    g_err[0] = 0;
    GradPlan gp;
    int rc = make_grad_plan(method, precision, dim, n_pts, sigma, x0, step, size, num_iter, max_dist_weight, gp);
    if (rc != FB_OK)
        return rc;
    Plan &p = gp.p;
    if (!x0)
        return fail(FB_ERR_ARG, "x0 is required");
    if (!d_grad_out || !d_grad_val || (n_pts > 0 && (!d_pts || !d_val)))
        return fail(FB_ERR_ARG, "null device pointer");
    if (!d_workspace || workspace_bytes < p.total)
        return fail(FB_ERR_WORKSPACE, "workspace of %zu bytes required, %zu given", p.total, workspace_bytes);
    char *ws = (char *)d_workspace;
    cudaStream_t st = (cudaStream_t)stream;
    FieldHeader *hdr = reinterpret_cast<FieldHeader *>(ws + p.off_hdr);
    uint32_t *bins = reinterpret_cast<uint32_t *>(ws + p.off_bins);
    uint32_t *scratch = reinterpret_cast<uint32_t *>(ws + p.off_sort);
    const uint32_t *sorted = nullptr;
    const void *recs = nullptr;
    cudaError_t e;
    {
        StageRange r("fb sort");
        e = sort_samples(p.precision, d_pts, d_val, p.npts, p.g, p.bin_w, p.nbins, hdr, scratch, bins, &sorted,
                         &recs, st);
    }
    if (e != cudaSuccess)
        return cuda_fail(e, "sample sort");
    SampleView sv{};
    sv.rec = recs;
    sv.npts = p.npts;
    sv.sorted_idx = sorted;
    sv.bin_start = bins;
    sv.nbins = p.nbins;
    sv.bin_w = p.bin_w;
    sv.hdr = hdr;
    const size_t sz = precision == FB_FP64 ? 8 : 4;
    for (size_t q = 0; q < p.launches.size(); q++) {
        if (q == gp.nfwd) {
            e = launch_grad_seed(precision, ws + p.off_pair[gp.seed_pair], p.npoints, d_grad_out, grad_f64, gp.thr,
                                 st);
            if (e != cudaSuccess)
                return cuda_fail(e, "gradient seed");
        }
        AxisLaunch a = p.launches[q];
        resolve_pointers(p, ws, nullptr, a);
        {
            StageRange r(q < gp.nfwd ? axis_range_name(a.axis) : "fb adjoint axis");
            e = launch_axis(p.precision, a, p.g, sv, st);
        }
        if (e != cudaSuccess)
            return cuda_fail(e, "axis kernel");
    }
    const uint32_t *keys = nullptr;
    const void *rec = nullptr;
    sort_sample_arrays(precision, p.npts, p.nbins, scratch, &keys, &rec);
    {
        StageRange r("fb adjoint gather");
        e = launch_grad_gather(precision, dim, rec, keys, p.nbins, p.npts, ws + p.off_pair[gp.final_pair], p.g,
                               hdr, d_grad_val, d_grad_pts, st);
    }
    (void)sz;
    return e == cudaSuccess ? FB_OK : cuda_fail(e, "gradient gather");
}

extern "C" int fb_workspace_size(int method, int precision, int dim, int64_t n_pts, const double *sigma,
                                 const double *step, const int64_t *size, int num_iter, size_t *bytes)
{
    Plan p;
    int rc = make_plan(method, precision, dim, n_pts, sigma, nullptr, step, size, num_iter, 0.0, p);
    if (rc != FB_OK)
        return rc;
    if (bytes)
        *bytes = p.total;
    return FB_OK;
}

// Optional stage timing: when enabled, run_plan records a CUDA event before
// the sample sort, after it, and after every axis launch, on the work stream.
namespace {
struct StageProfile {
    std::mutex mu;
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    struct Rec {
        int stage;   // 0 = sample sort, 1 + axis = axis launch of that axis
        size_t e0, e1;
    };
    std::vector<Rec> recs;
};
StageProfile g_prof;

size_t prof_event(cudaStream_t st)
{
    if (g_prof.used == g_prof.pool.size()) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        g_prof.pool.push_back(e);
    }
    cudaEventRecord(g_prof.pool[g_prof.used], st);
    return g_prof.used++;
}
}  // namespace

extern "C" int fb_profile_begin(void)
{
    std::lock_guard<std::mutex> lk(g_prof.mu);
    g_prof.on = true;
    g_prof.used = 0;
    g_prof.recs.clear();
    return FB_OK;
}

extern "C" int fb_profile_end(int *stages, float *ms, int max_records, int *n_records)
{
    std::lock_guard<std::mutex> lk(g_prof.mu);
    g_prof.on = false;
    int n = 0;
    for (const auto &r : g_prof.recs) {
        if (n >= max_records)
            break;
        cudaError_t e = cudaEventSynchronize(g_prof.pool[r.e1]);
        if (e != cudaSuccess)
            return cuda_fail(e, "profile event");
        float t = 0.f;
        cudaEventElapsedTime(&t, g_prof.pool[r.e0], g_prof.pool[r.e1]);
        if (stages)
            stages[n] = r.stage;
        if (ms)
            ms[n] = t;
        n++;
    }
    if (n_records)
        *n_records = n;
    return FB_OK;
}

static int run_plan(Plan &p, const double *d_pts, const double *d_val, void *d_out, int out_f64, char *ws,
                    cudaStream_t st)
{
    if (p.naive) {
        cudaError_t e = launch_naive(p.precision, p.g.dim, 0, d_pts, d_val, p.npts, p.sigma, p.g.x0, p.g.step,
                                     p.g.size, reinterpret_cast<FieldHeader *>(ws + p.off_hdr), d_out, out_f64, st);
        return e == cudaSuccess ? FB_OK : cuda_fail(e, "naive kernel");
    }
    std::unique_lock<std::mutex> plk(g_prof.mu, std::defer_lock);
    const bool prof = g_prof.on;
    if (prof)
        plk.lock();
    size_t ev = prof ? prof_event(st) : 0;
    FieldHeader *hdr = reinterpret_cast<FieldHeader *>(ws + p.off_hdr);
    uint32_t *bins = reinterpret_cast<uint32_t *>(ws + p.off_bins);
    uint32_t *scratch = reinterpret_cast<uint32_t *>(ws + p.off_sort);
    const uint32_t *sorted = nullptr;
    const void *recs = nullptr;
    cudaError_t e;
    {
        StageRange r("fb sort");
        e = sort_samples(p.precision, d_pts, d_val, p.npts, p.g, p.bin_w, p.nbins, hdr, scratch, bins, &sorted,
                         &recs, st);
    }
    if (e != cudaSuccess)
        return cuda_fail(e, "sample sort");
    if (prof) {
        size_t e1 = prof_event(st);
        g_prof.recs.push_back({0, ev, e1});
        ev = e1;
    }
    SampleView sv{};
    sv.rec = recs;
    sv.npts = p.npts;
    sv.sorted_idx = sorted;
    sv.bin_start = bins;
    sv.nbins = p.nbins;
    sv.bin_w = p.bin_w;
    sv.hdr = hdr;
    for (AxisLaunch a : p.launches) {
        resolve_pointers(p, ws, d_out, a);
        a.out_f64 = out_f64;
        {
            StageRange r(axis_range_name(a.axis));
            e = launch_axis(p.precision, a, p.g, sv, st);
        }
        if (e != cudaSuccess)
            return cuda_fail(e, "axis kernel");
        if (prof) {
            size_t e1 = prof_event(st);
            g_prof.recs.push_back({1 + a.axis, ev, e1});
            ev = e1;
        }
    }
    return FB_OK;
}

extern "C" int fb_interpolate(int method, int precision, int dim, const double *d_pts, const double *d_val,
                              int64_t n_pts, const double *sigma, const double *x0, const double *step,
                              const int64_t *size, int num_iter, double max_dist_weight, void *d_out,
                              int out_f64, void *d_workspace, size_t workspace_bytes, void *stream)
{
    g_err[0] = 0;
    Plan p;
    int rc = make_plan(method, precision, dim, n_pts, sigma, x0, step, size, num_iter, max_dist_weight, p);
    if (rc != FB_OK)
        return rc;
    if (!x0)
        return fail(FB_ERR_ARG, "x0 is required");
    if (!d_out || (n_pts > 0 && (!d_pts || !d_val)))
        return fail(FB_ERR_ARG, "null device pointer");
    if (!d_workspace || workspace_bytes < p.total)
        return fail(FB_ERR_WORKSPACE, "workspace of %zu bytes required, %zu given", p.total, workspace_bytes);
    return run_plan(p, d_pts, d_val, d_out, out_f64, (char *)d_workspace, (cudaStream_t)stream);
}

// Quantised result (demo/quantinterpolation.py:149-153): the float64 quotient
// with its `quant_bits` least significant mantissa bits dropped in the last
// axis kernel.
extern "C" int fb_interpolate_quant(int method, int precision, int dim, const double *d_pts, const double *d_val,
                                    int64_t n_pts, const double *sigma, const double *x0, const double *step,
                                    const int64_t *size, int num_iter, double max_dist_weight, int quant_bits,
                                    double *d_out, void *d_workspace, size_t workspace_bytes, void *stream)
{
    g_err[0] = 0;
    if (quant_bits < 0 || quant_bits > 52)
        return fail(FB_ERR_ARG, "quant_bits must be in [0, 52] (got %d)", quant_bits);
    if (method == FB_NAIVE)
        return fail(FB_ERR_UNSUPPORTED, "quantisation is provided for the convolution methods");
    Plan p;
    int rc = make_plan(method, precision, dim, n_pts, sigma, x0, step, size, num_iter, max_dist_weight, p);
    if (rc != FB_OK)
        return rc;
    if (!x0)
        return fail(FB_ERR_ARG, "x0 is required");
    if (!d_out || (n_pts > 0 && (!d_pts || !d_val)))
        return fail(FB_ERR_ARG, "null device pointer");
    if (!d_workspace || workspace_bytes < p.total)
        return fail(FB_ERR_WORKSPACE, "workspace of %zu bytes required, %zu given", p.total, workspace_bytes);
    p.launches.back().quant_bits = quant_bits;
    return run_plan(p, d_pts, d_val, d_out, 1, (char *)d_workspace, (cudaStream_t)stream);
}

// ---------------------------------------------------------------------------
// host-buffer entry
// ---------------------------------------------------------------------------

namespace {
struct DevPool {
    std::mutex mu;
    void *ptr = nullptr;
    size_t cap = 0;
    int device = -1;
};
DevPool g_pool;

int pool_get(size_t bytes, char **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "cudaGetDevice");
    if (g_pool.ptr && (g_pool.cap < bytes || g_pool.device != dev)) {
        cudaFree(g_pool.ptr);
        g_pool.ptr = nullptr;
        g_pool.cap = 0;
    }
    if (!g_pool.ptr) {
        e = cudaMalloc(&g_pool.ptr, bytes);
        if (e != cudaSuccess) {
            g_pool.ptr = nullptr;
            return cuda_fail(e, "cudaMalloc (host-buffer entry)");
        }
        g_pool.cap = bytes;
        g_pool.device = dev;
    }
    *out = (char *)g_pool.ptr;
    return FB_OK;
}
}  // namespace

extern "C" int fb_interpolate_host(int method, int precision, int dim, const double *pts, const double *val,
                                   int64_t n_pts, const double *sigma, const double *x0, const double *step,
                                   const int64_t *size, int num_iter, double max_dist_weight, void *out,
                                   int out_f64, void *stream)
{
    g_err[0] = 0;
    Plan p;
    int rc = make_plan(method, precision, dim, n_pts, sigma, x0, step, size, num_iter, max_dist_weight, p);
    if (rc != FB_OK)
        return rc;
    if (!x0 || !out || (n_pts > 0 && (!pts || !val)))
        return fail(FB_ERR_ARG, "null host pointer");
    const size_t in_pts = align_up(sizeof(double) * dim * (size_t)n_pts);
    const size_t in_val = align_up(sizeof(double) * (size_t)n_pts);
    const size_t out_b = (out_f64 ? 8 : 4) * (size_t)p.npoints;
    std::lock_guard<std::mutex> lk(g_pool.mu);
    char *base = nullptr;
    rc = pool_get(in_pts + in_val + align_up(out_b) + p.total, &base);
    if (rc != FB_OK)
        return rc;
    cudaStream_t st = (cudaStream_t)stream;
    double *d_pts = (double *)base;
    double *d_val = (double *)(base + in_pts);
    void *d_out = base + in_pts + in_val;
    char *ws = base + in_pts + in_val + align_up(out_b);
    cudaError_t e;
    if (n_pts > 0) {
        e = cudaMemcpyAsync(d_pts, pts, sizeof(double) * dim * (size_t)n_pts, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(d_val, val, sizeof(double) * (size_t)n_pts, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess)
            return cuda_fail(e, "copy to device");
    }
    rc = run_plan(p, d_pts, d_val, d_out, out_f64, ws, st);
    if (rc != FB_OK)
        return rc;
    e = cudaMemcpyAsync(out, d_out, out_b, cudaMemcpyDeviceToHost, st);
    int status = 0;
    if (e == cudaSuccess && !p.naive)
        e = cudaMemcpyAsync(&status, ws + p.off_hdr + offsetof(FieldHeader, error), sizeof(int),
                            cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return cuda_fail(e, "copy to host");
    if (status != 0)
        return device_fail((uint32_t)status, "fb_interpolate_host");
    return FB_OK;
}

extern "C" int fb_workspace_status(const void *d_workspace, void *stream, int *status)
{
    g_err[0] = 0;
    if (!d_workspace)
        return fail(FB_ERR_ARG, "null workspace");
    int bits = 0;
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(&bits, static_cast<const char *>(d_workspace) + offsetof(FieldHeader, error),
                                    sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return cuda_fail(e, "fb_workspace_status");
    if (status)
        *status = bits;
    return bits ? device_fail((uint32_t)bits, "fb_workspace_status") : FB_OK;
}

extern "C" void *fb_host_alloc(size_t bytes)
{
    void *p = nullptr;
    if (cudaMallocHost(&p, bytes) != cudaSuccess)
        return nullptr;
    return p;
}

extern "C" void fb_host_free(void *p)
{
    if (p)
        cudaFreeHost(p);
}

extern "C" void fb_release(void)
{
    std::lock_guard<std::mutex> lk(g_pool.mu);
    if (g_pool.ptr)
        cudaFree(g_pool.ptr);
    g_pool.ptr = nullptr;
    g_pool.cap = 0;
}

// ---------------------------------------------------------------------------
// 1D passes alone
// ---------------------------------------------------------------------------

extern "C" int fb_accumulate_lines(int precision, void *d_lines, int64_t n_lines, int64_t len, int rect_len,
                                   int num_iter, double alpha, int normalize, void *stream)
{
    g_err[0] = 0;
    if (precision != FB_FP64 && precision != FB_FP32C)
        return fail(FB_ERR_ARG, "unknown precision %d", precision);
    if (!d_lines || n_lines < 0 || len < 1 || rect_len < 1 || (rect_len & 1) == 0 || num_iter < 0)
        return fail(FB_ERR_ARG, "invalid line arguments");
    if (n_lines == 0 || num_iter == 0)
        return FB_OK;
    const AxisPlanLimits lim = axis_limits(precision, (rect_len - 1) / 2);
    if (len > lim.extent_max)
        return fail(FB_ERR_UNSUPPORTED, "line length %lld exceeds %d", (long long)len, lim.extent_max);
    cudaError_t e = launch_lines(precision, d_lines, n_lines, len, (rect_len - 1) / 2, alpha, num_iter, normalize,
                                 (cudaStream_t)stream);
    if (e != cudaSuccess)
        return cuda_fail(e, "line passes");
    return FB_OK;
}

// ---------------------------------------------------------------------------
// sphere
// ---------------------------------------------------------------------------

static const double kRad = 3.14159265358979311600 / 180.0;

extern "C" void fb_lambert_create_proj(double center_lon, double center_lat, double lat1, double lat2,
                                       double *proj)
{
    const double hrad = kRad / 2.0;
    double n;
    if (lat1 != lat2)
        n = log(cos(lat1 * kRad) / cos(lat2 * kRad)) / log(tan((90.0 + lat2) * hrad) / tan((90.0 + lat1) * hrad));
    else
        n = sin(lat1 * kRad);
    double F = cos(lat1 * kRad) * pow(tan((90.0 + lat1) * hrad), n) / n;
    double rho0 = F / pow(tan((90.0 + center_lat) * hrad), n);
    proj[0] = center_lon;
    proj[1] = n;
    proj[2] = 1.0 / n;
    proj[3] = F;
    proj[4] = rho0;
}

extern "C" int fb_lambert_to_map(const double *d_geo, double *d_map, int64_t n_pts, const double *proj,
                                 void *stream)
{
    g_err[0] = 0;
    if (n_pts < 0 || !proj || (n_pts > 0 && (!d_geo || !d_map)))
        return fail(FB_ERR_ARG, "invalid projection arguments");
    cudaError_t e = launch_lambert_to_map(d_geo, d_map, n_pts, proj, (cudaStream_t)stream);
    return e == cudaSuccess ? FB_OK : cuda_fail(e, "lambert to_map");
}

namespace {
// interpolationS2.py:187-188: the fixed Lambert grid
void s2_lambert_grid(const double *step, double *lam_x0, int64_t *lam_size)
{
    lam_x0[0] = -32.0;
    lam_x0[1] = -2.0;
    lam_size[0] = (int64_t)(64.0 / step[0]);
    lam_size[1] = (int64_t)(44.0 / step[1]);
}
}  // namespace

extern "C" int fb_s2_workspace_size(int precision, int64_t n_pts, const double *sigma, const double *step,
                                    const int64_t *size, int num_iter, size_t *bytes)
{
    if (!size || size[0] < 1 || size[1] < 1)
        return fail(FB_ERR_ARG, "invalid output size");
    double lx0[2];
    int64_t ls[2];
    s2_lambert_grid(step, lx0, ls);
    size_t inner = 0;
    int rc = fb_workspace_size(FB_OPTIMIZED_CONVOLUTION, precision, 2, n_pts, sigma, step, ls, num_iter, &inner);
    if (rc != FB_OK)
        return rc;
    if (bytes)
        *bytes = align_up(sizeof(double) * 2 * (size_t)n_pts) + align_up(sizeof(float) * ls[0] * ls[1]) +
                 align_up(sizeof(double) * (size_t)(size[1] + 2 * size[0])) + inner;
    return FB_OK;
}

extern "C" int fb_interpolate_s2(int precision, const double *d_pts, const double *d_val, int64_t n_pts,
                                 const double *sigma, const double *x0, const double *step, const int64_t *size,
                                 int num_iter, double max_dist_weight, int resample, float *d_out,
                                 void *d_workspace, size_t workspace_bytes, void *stream)
{
    g_err[0] = 0;
    if (!sigma || !x0 || !step || !size || !d_out)
        return fail(FB_ERR_ARG, "null argument");
    double lx0[2];
    int64_t ls[2];
    s2_lambert_grid(step, lx0, ls);
    size_t need = 0;
    int rc = fb_s2_workspace_size(precision, n_pts, sigma, step, size, num_iter, &need);
    if (rc != FB_OK)
        return rc;
    if (!d_workspace || workspace_bytes < need)
        return fail(FB_ERR_WORKSPACE, "workspace of %zu bytes required, %zu given", need, workspace_bytes);
    cudaStream_t st = (cudaStream_t)stream;
    char *ws = (char *)d_workspace;
    double *lam_pts = (double *)ws;
    float *lam = (float *)(ws + align_up(sizeof(double) * 2 * (size_t)n_pts));
    double *tab = (double *)(ws + align_up(sizeof(double) * 2 * (size_t)n_pts) + align_up(sizeof(float) * ls[0] * ls[1]));
    char *inner = (char *)tab + align_up(sizeof(double) * (size_t)(size[1] + 2 * size[0]));
    double proj[5];
    fb_lambert_create_proj(11.5, 34.5, 42.5, 65.5, proj);
    cudaError_t e = launch_lambert_to_map(d_pts, lam_pts, n_pts, proj, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "lambert to_map");
    float *lam_out = resample ? lam : d_out;
    rc = fb_interpolate(FB_OPTIMIZED_CONVOLUTION, precision, 2, lam_pts, d_val, n_pts, sigma, lx0, step, ls,
                        num_iter, max_dist_weight, lam_out, 0, inner, need - (size_t)(inner - ws), stream);
    if (rc != FB_OK)
        return rc;
    if (resample) {
        e = launch_resample(lam, ls[0], ls[1], lx0, x0, step, size, proj, d_out, tab, st);
        if (e != cudaSuccess)
            return cuda_fail(e, "resample");
    }
    return FB_OK;
}

extern "C" int fb_interpolate_naive_s2(int precision, const double *d_pts, const double *d_val, int64_t n_pts,
                                       const double *sigma, const double *x0, const double *step,
                                       const int64_t *size, void *d_out, int out_f64, void *d_workspace,
                                       size_t workspace_bytes, void *stream)
{
    g_err[0] = 0;
    if (precision != FB_FP64 && precision != FB_FP32C)
        return fail(FB_ERR_ARG, "unknown precision %d", precision);
    if (!sigma || !x0 || !step || !size || size[0] < 1 || size[1] < 1 || n_pts < 0)
        return fail(FB_ERR_ARG, "invalid naive S2 arguments");
    if (!d_out || (n_pts > 0 && (!d_pts || !d_val)))
        return fail(FB_ERR_ARG, "null device pointer");
    if (!d_workspace || workspace_bytes < sizeof(FieldHeader))
        return fail(FB_ERR_WORKSPACE, "workspace of %zu bytes required, %zu given", sizeof(FieldHeader),
                    workspace_bytes);
    const double sig[2] = {sigma[0], sigma[0]};
    cudaError_t e = launch_naive(precision, 2, 1, d_pts, d_val, n_pts, sig, x0, step, size,
                                 reinterpret_cast<FieldHeader *>(d_workspace), d_out, out_f64, (cudaStream_t)stream);
    return e == cudaSuccess ? FB_OK : cuda_fail(e, "naive S2 kernel");
}

extern "C" int fb_radius_workspace_size(int64_t n_pts, size_t *bytes)
{
    g_err[0] = 0;
    if (!bytes || n_pts < 0)
        return fail(FB_ERR_ARG, "invalid radius workspace arguments");
    *bytes = radius_workspace_bytes(n_pts);
    return FB_OK;
}

extern "C" int fb_interpolate_radius(int precision, const double *d_pts, const double *d_val, int64_t n_pts,
                                     double sigma, const double *x0, const double *step, const int64_t *size,
                                     double max_dist_weight, double min_weight, void *d_out, int out_f64,
                                     void *d_workspace, size_t workspace_bytes, void *stream)
{
    g_err[0] = 0;
    if (precision != FB_FP64 && precision != FB_FP32C)
        return fail(FB_ERR_ARG, "unknown precision %d", precision);
    if (!x0 || !step || !size || size[0] < 1 || size[1] < 1 || n_pts < 0 || !(sigma > 0.0))
        return fail(FB_ERR_ARG, "invalid radius arguments");
    if (size[0] > 65535LL * 16 || size[1] > 65535LL * 16)
        return fail(FB_ERR_KERNEL_SIZE, "radius grid of %lld x %lld points is too large", (long long)size[0],
                    (long long)size[1]);
    if (!d_out || (n_pts > 0 && (!d_pts || !d_val)))
        return fail(FB_ERR_ARG, "null device pointer");
    const size_t need = radius_workspace_bytes(n_pts);
    if (!d_workspace || workspace_bytes < need)
        return fail(FB_ERR_WORKSPACE, "workspace of %zu bytes required, %zu given", need, workspace_bytes);
    cudaError_t e = launch_radius(precision, d_pts, d_val, n_pts, sigma, x0, step, size, max_dist_weight, min_weight,
                                  d_workspace, d_out, out_f64, (cudaStream_t)stream);
    return e == cudaSuccess ? FB_OK : cuda_fail(e, "radius kernel");
}

extern "C" int fb_resample(const float *d_lam, int64_t lam_w, int64_t lam_h, const double *lam_x0, const double *x0,
                           const double *step, const int64_t *size, const double *proj, float *d_out, double *d_tab,
                           void *stream)
{
    g_err[0] = 0;
    if (!d_lam || !lam_x0 || !x0 || !step || !size || !proj || !d_out || !d_tab || size[0] < 1 || size[1] < 1 ||
        lam_w < 2 || lam_h < 2)
        return fail(FB_ERR_ARG, "invalid resample arguments");
    cudaError_t e = launch_resample(d_lam, lam_w, lam_h, lam_x0, x0, step, size, proj, d_out, d_tab,
                                    (cudaStream_t)stream);
    return e == cudaSuccess ? FB_OK : cuda_fail(e, "resample");
}

// ---------------------------------------------------------------------------
// batched 2D fields: one sample sort and one launch per axis stage
// for all fields of a plan
// ---------------------------------------------------------------------------

namespace {

// One persistent launch: the s-th axis launch of every field whose launch
// has the same shape and parameters (everything but the pointers), as one
// shared launch description and a table of per-field pointers.
struct BatchStage {
    bool mixed = false;       // fields of different shapes: MixedField table + items
    AxisLaunch a{};           // homogeneous: the shared launch description
    Geometry g{};
    SampleView sv{};
    int k = 0, mode = 0, sd = 0, layout = 0;   // kernel variant
    size_t smem = 0;          // mixed: largest shared memory of its fields
    int threads = 0;          // mixed: most threads of its fields
    int axis = 0;
    int grid = 0;
    size_t off_fields = 0;    // TilePtrs[nf] (homogeneous) or MixedField[nf] (mixed)
    size_t off_items = 0;     // mixed: uint2 (field, block)[nitems]
    uint32_t nf = 0, bpf = 0, nitems = 0;
    // homogeneous column stages of whole lines: the pipelined TMA kernel
    bool pipe = false;
    int pk = 0, pmode = 0;
    ColsPipe cp{};
    CUtensorMap map{};
};

bool same_launch(const AxisLaunch &x, const AxisLaunch &y)
{
    AxisLaunch u = x, v = y;
    u.src_v = v.src_v = nullptr;
    u.src_w = v.src_w = nullptr;
    u.dst_v = v.dst_v = nullptr;
    u.dst_w = v.dst_w = nullptr;
    u.out = v.out = nullptr;
    // compare field by field (no padding bytes involved)
    return u.axis == v.axis && u.layout == v.layout && u.L == v.L && u.elem_stride == v.elem_stride &&
           u.nlines == v.nlines && u.outer_count == v.outer_count && u.outer_stride == v.outer_stride &&
           u.xblocks == v.xblocks && u.width == v.width && u.lines_per_cta == v.lines_per_cta &&
           u.tile_len == v.tile_len && u.ntiles == v.ntiles && u.halo == v.halo && u.extent_max == v.extent_max &&
           u.line_pitch == v.line_pitch && u.line_pad == v.line_pad && u.chunks_pad == v.chunks_pad &&
           u.part_pitch == v.part_pitch && u.part_pad == v.part_pad && u.passes == v.passes && u.T == v.T &&
           u.alpha == v.alpha && u.scaled == v.scaled && u.inv_norm == v.inv_norm && u.fill_splat == v.fill_splat &&
           u.store_quot == v.store_quot && u.out_f64 == v.out_f64 && u.plain == v.plain && u.thr == v.thr &&
           u.kchunk == v.kchunk && u.rows_threads == v.rows_threads;
}

bool same_geometry(const Geometry &x, const Geometry &y)
{
    return x.dim == y.dim && x.size[0] == y.size[0] && x.size[1] == y.size[1] && x.size[2] == y.size[2];
}

std::mutex g_batch_tune_mu;
std::map<std::string, fb_batch_knobs> g_batch_tuned;

}  // namespace

struct fb_batch {
    int precision = 1, out_f64 = 0, flags = 0, device = 0;
    fb_batch_knobs knobs{0, 0, 0};
    int nfields = 0;
    int64_t ntot = 0;
    uint32_t nbins = 0, nblocks = 0;
    char *dev = nullptr;
    size_t dev_bytes = 0;
    size_t off_keyf = 0, off_blocks = 0, off_hdrs = 0, off_bins = 0, off_sort = 0;
    std::vector<BatchStage> stages;
    std::vector<fb_field2d> fields;
    cudaStream_t cap = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // interleaved runs: the second stream and the events ordering field f's
    // y launch after its x launch
    bool interleave = false;
    cudaStream_t side = nullptr;
    std::vector<cudaEvent_t> ev_field;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // host-buffer runs: result copies spread over several streams (copy
    // engines), made at the first fb_batch_run_host
    static constexpr int kCopyStreams = 4;
    cudaStream_t copy_st[kCopyStreams] = {};
    cudaEvent_t copy_ev[kCopyStreams + 1] = {};
};

namespace {

void batch_free(fb_batch *b)
{
    if (b->exec)
        cudaGraphExecDestroy(b->exec);
    if (b->graph)
        cudaGraphDestroy(b->graph);
    if (b->cap)
        cudaStreamDestroy(b->cap);
    if (b->side)
        cudaStreamDestroy(b->side);
    for (cudaEvent_t ev : b->ev_field)
        cudaEventDestroy(ev);
    b->ev_field.clear();
    if (b->ev_fork)
        cudaEventDestroy(b->ev_fork);
    if (b->ev_join)
        cudaEventDestroy(b->ev_join);
    b->side = nullptr;
    b->ev_fork = b->ev_join = nullptr;
    for (int q = 0; q < fb_batch::kCopyStreams; q++) {
        if (b->copy_st[q])
            cudaStreamDestroy(b->copy_st[q]);
        b->copy_st[q] = nullptr;
    }
    for (int q = 0; q <= fb_batch::kCopyStreams; q++) {
        if (b->copy_ev[q])
            cudaEventDestroy(b->copy_ev[q]);
        b->copy_ev[q] = nullptr;
    }
    if (b->dev)
        cudaFree(b->dev);
    b->exec = nullptr;
    b->graph = nullptr;
    b->cap = nullptr;
    b->dev = nullptr;
}

int batch_build(int precision, const fb_field2d *fields, int nf, int out_f64, fb_batch_knobs kn, fb_batch *b)
{
    if (nf < 1 || !fields)
        return fail(FB_ERR_ARG, "a batch needs at least one field");
    if (kn.chunk != 0 && kn.chunk != 17 && kn.chunk != 33)
        return fail(FB_ERR_ARG, "chunk must be 0, 17 or 33 (got %d)", kn.chunk);
    if (kn.rows_threads != 0 && kn.rows_threads != 128 && kn.rows_threads != 256 && kn.rows_threads != 512)
        return fail(FB_ERR_ARG, "rows_threads must be 0, 128, 256 or 512 (got %d)", kn.rows_threads);
    if (kn.mixed != 0 && kn.mixed != 1)
        return fail(FB_ERR_ARG, "mixed must be 0 or 1 (got %d)", kn.mixed);
    if (kn.cols_pipe < 0 || kn.cols_pipe > 2)
        return fail(FB_ERR_ARG, "cols_pipe must be 0, 1 or 2 (got %d)", kn.cols_pipe);
    if (kn.interleave != 0 && kn.interleave != 1)
        return fail(FB_ERR_ARG, "interleave must be 0 or 1 (got %d)", kn.interleave);
    b->precision = precision;
    b->out_f64 = out_f64 ? 1 : 0;
    b->knobs = kn;
    b->nfields = nf;
    b->fields.assign(fields, fields + nf);
    std::vector<Plan> plans((size_t)nf);
    int64_t ntot = 0, nbins = 0;
    std::vector<int64_t> sample_off((size_t)nf), bin_off((size_t)nf);
    for (int f = 0; f < nf; f++) {
        const fb_field2d &F = fields[f];
        if (F.method == FB_NAIVE)
            return fail(FB_ERR_UNSUPPORTED, "field %d: batches take the convolution methods", f);
        int rc = make_plan(F.method, precision, 2, F.n_pts, F.sigma, F.x0, F.step, F.size, F.num_iter,
                           F.max_dist_weight, plans[f], kn.chunk, kn.rows_threads);
        if (rc != FB_OK) {
            char msg[sizeof(g_err)];
            snprintf(msg, sizeof(msg), "%s", g_err);
            return fail(rc, "field %d: %s", f, msg);
        }
        if (!F.out || (F.n_pts > 0 && (!F.pts || !F.val)))
            return fail(FB_ERR_ARG, "field %d: null device pointer", f);
        sample_off[f] = ntot;
        bin_off[f] = nbins;
        ntot += F.n_pts;
        // the field's rows and one more bin for its skipped samples, so
        // that its bins cover its own samples exactly
        nbins += (int64_t)plans[f].nbins + 1;
    }
    if (ntot > (int64_t)0xFFFFFFF0ll)
        return fail(FB_ERR_ARG, "batch has too many samples (%lld)", (long long)ntot);
    if (nbins > (int64_t)0xFFFFFFF0ll)
        return fail(FB_ERR_ARG, "batch has too many grid rows (%lld)", (long long)nbins);
    b->ntot = ntot;
    b->nbins = (uint32_t)nbins;

    // sample blocks of the bin-key kernel
    std::vector<uint2> blocks;
    for (int f = 0; f < nf; f++)
        for (int64_t s0 = 0; s0 < fields[f].n_pts; s0 += kBatchKeysPerBlock)
            blocks.push_back(make_uint2((unsigned)f, (unsigned)s0));
    b->nblocks = (uint32_t)blocks.size();

    // stages: the s-th launch of every field, grouped by kernel variant; a
    // group whose fields all have the same shape and parameters shares one
    // launch description (unless the knobs ask for mixed launches), any
    // other group goes through a table of per-field descriptions
    size_t nstage_max = 0;
    for (const Plan &p : plans)
        nstage_max = std::max(nstage_max, p.launches.size());
    struct Group {
        BatchStage st;
        std::vector<int> f;
        std::vector<uint32_t> fblocks;   // blocks of each field's launch
        size_t q = 0;
    };
    auto blocks_of = [](const AxisLaunch &a) -> int64_t {
        const int64_t grp = a.layout == 0 ? (a.nlines + a.lines_per_cta - 1) / a.lines_per_cta
                                          : a.outer_count * a.xblocks;
        return grp * a.ntiles;
    };
    std::vector<Group> groups;
    for (size_t q = 0; q < nstage_max; q++) {
        const size_t first = groups.size();
        for (int f = 0; f < nf; f++) {
            if (q >= plans[f].launches.size())
                continue;
            const AxisLaunch &a = plans[f].launches[q];
            const int k = axis_variant_k(precision, a), mode = axis_variant_mode(precision, a);
            const int sd = a.fill_splat ? 2 : 0;
            Group *g = nullptr;
            for (size_t x = first; x < groups.size(); x++)
                if (groups[x].st.k == k && groups[x].st.mode == mode && groups[x].st.sd == sd &&
                    groups[x].st.layout == a.layout)
                    g = &groups[x];
            if (!g) {
                Group ng;
                ng.st.a = a;
                ng.st.g = plans[f].g;
                ng.st.sv.nbins = plans[f].nbins;
                ng.st.sv.bin_w = plans[f].bin_w;
                ng.st.k = k;
                ng.st.mode = mode;
                ng.st.sd = sd;
                ng.st.layout = a.layout;
                ng.st.axis = a.axis;
                ng.q = q;
                groups.push_back(ng);
                g = &groups.back();
            }
            const int64_t nb = blocks_of(a);
            if (nb > (int64_t)0x7FFFFFFF)
                return fail(FB_ERR_ARG, "field %d: too many blocks in one launch", f);
            if (!(same_launch(g->st.a, a) && same_geometry(g->st.g, plans[f].g) &&
                  g->st.sv.nbins == plans[f].nbins && g->st.sv.bin_w == plans[f].bin_w))
                g->st.mixed = true;
            g->st.smem = std::max(g->st.smem, axis_smem_bytes(precision, a));
            g->st.threads = std::max(g->st.threads, axis_threads(precision, a));
            g->f.push_back(f);
            g->fblocks.push_back((uint32_t)nb);
        }
    }
    for (Group &g : groups) {
        if (kn.mixed)
            g.st.mixed = true;
        int64_t items = 0;
        for (uint32_t nb : g.fblocks)
            items += nb;
        if (items > (int64_t)0x7FFFFFFF)
            return fail(FB_ERR_ARG, "batch stage too large");
        g.st.nf = (uint32_t)g.f.size();
        g.st.nitems = (uint32_t)items;
        g.st.bpf = g.st.mixed ? 0 : g.fblocks[0];
    }

    // device layout
    const size_t sz = precision == FB_FP64 ? 8 : 4;
    size_t off = 0;
    b->off_keyf = off;
    off = align_up(off + sizeof(BatchKeyField) * (size_t)nf);
    b->off_blocks = off;
    off = align_up(off + sizeof(uint2) * std::max<size_t>(1, blocks.size()));
    b->off_hdrs = off;
    off = align_up(off + sizeof(FieldHeader) * (size_t)nf);
    b->off_bins = off;
    off = align_up(off + sizeof(uint32_t) * ((size_t)nbins + 1));
    b->off_sort = off;
    off = align_up(off + batch_sort_scratch_bytes(ntot, (uint32_t)nbins, precision));
    for (Group &g : groups) {
        g.st.off_fields = off;
        off = align_up(off + (g.st.mixed ? sizeof(MixedField) : sizeof(TilePtrs)) * g.f.size());
        if (g.st.mixed) {
            g.st.off_items = off;
            off = align_up(off + sizeof(uint2) * (size_t)g.st.nitems);
        }
    }
    const size_t tables_end = off;
    std::vector<size_t> pair_off((size_t)nf);
    std::vector<size_t> pair_bytes((size_t)nf);
    for (int f = 0; f < nf; f++) {
        pair_off[f] = off;
        pair_bytes[f] = align_up(2 * sz * (size_t)plans[f].npoints);
        off += (size_t)plans[f].pairs * pair_bytes[f];
    }
    b->dev_bytes = off;
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess)
        e = cudaMalloc(&b->dev, b->dev_bytes);
    // zeroed once: the bin counts and tickets of the sort are kept zero
    // between runs by the kernels that consume them
    if (e == cudaSuccess)
        e = cudaMemset(b->dev, 0, b->dev_bytes);
    if (e != cudaSuccess) {
        if (b->dev)
            cudaFree(b->dev);
        b->dev = nullptr;
        return cuda_fail(e, "batch plan memory");
    }
    char *dv = b->dev;

    // host image of the tables
    std::vector<char> img(tables_end, 0);
    BatchKeyField *kf = reinterpret_cast<BatchKeyField *>(img.data() + b->off_keyf);
    for (int f = 0; f < nf; f++) {
        const fb_field2d &F = fields[f];
        kf[f].pts = F.pts;
        kf[f].val = F.val;
        kf[f].npts = F.n_pts;
        kf[f].sample_offset = sample_off[f];
        kf[f].bin_offset = (uint32_t)bin_off[f];
        kf[f].pad = 0;
        for (int m = 0; m < 2; m++) {
            kf[f].x0[m] = F.x0[m];
            kf[f].step[m] = F.step[m];
            kf[f].inv_step[m] = 1.0 / F.step[m];
            kf[f].size[m] = F.size[m];
        }
    }
    if (!blocks.empty())
        memcpy(img.data() + b->off_blocks, blocks.data(), sizeof(uint2) * blocks.size());
    // bin starts: every bin of a field at the field's first sample (empty);
    // the key pass rewrites those of fields with samples every run, those
    // of fields without samples keep these
    {
        uint32_t *bs = reinterpret_cast<uint32_t *>(img.data() + b->off_bins);
        for (int f = 0; f < nf; f++)
            for (int64_t i = 0; i <= (int64_t)plans[f].nbins; i++)
                bs[bin_off[f] + i] = (uint32_t)sample_off[f];
        bs[nbins] = (uint32_t)ntot;
    }
    const uint32_t *sorted = nullptr;
    const void *recs = nullptr;
    batch_sort_views(precision, ntot, (uint32_t)nbins, reinterpret_cast<uint32_t *>(dv + b->off_sort), &sorted,
                     &recs);
    b->stages.clear();
    for (Group &g : groups) {
        auto ptrs = [&](int f) {
            const AxisLaunch &a = plans[f].launches[g.q];
            auto pair = [&](const void *code) -> void * {
                const int idx = (int)(intptr_t)code - 16;
                return idx < 0 ? nullptr : dv + pair_off[f] + (size_t)idx * pair_bytes[f];
            };
            TilePtrs t;
            t.src = pair(a.src_v);
            t.dst = pair(a.dst_v);
            t.out = fields[f].out;
            t.bin_start = reinterpret_cast<const uint32_t *>(dv + b->off_bins) + bin_off[f];
            t.hdr = reinterpret_cast<const FieldHeader *>(dv + b->off_hdrs) + f;
            return t;
        };
        auto view = [&](int f) {
            SampleView sv{};
            sv.rec = recs;
            sv.npts = ntot;
            sv.sorted_idx = sorted;
            sv.nbins = plans[f].nbins;
            sv.bin_w = plans[f].bin_w;
            return sv;
        };
        BatchStage st = g.st;
        if (st.mixed) {
            MixedField *mf = reinterpret_cast<MixedField *>(img.data() + st.off_fields);
            for (size_t mi = 0; mi < g.f.size(); mi++) {
                const int f = g.f[mi];
                mf[mi].a = plans[f].launches[g.q];
                mf[mi].a.out_f64 = b->out_f64;
                mf[mi].g = plans[f].g;
                mf[mi].sv = view(f);
                mf[mi].fp = ptrs(f);
                mf[mi].sv.bin_start = mf[mi].fp.bin_start;
                mf[mi].sv.hdr = mf[mi].fp.hdr;
                mf[mi].a.src_v = mf[mi].fp.src;
                mf[mi].a.dst_v = mf[mi].fp.dst;
                mf[mi].a.out = mf[mi].fp.out;
                mf[mi].a.src_w = mf[mi].a.dst_w = nullptr;
            }
            // items, the fields with most blocks first
            std::vector<size_t> order(g.f.size());
            for (size_t mi = 0; mi < order.size(); mi++)
                order[mi] = mi;
            std::stable_sort(order.begin(), order.end(),
                             [&](size_t x, size_t y) { return g.fblocks[x] > g.fblocks[y]; });
            uint2 *it = reinterpret_cast<uint2 *>(img.data() + st.off_items);
            size_t ni = 0;
            for (size_t mi : order)
                for (uint32_t bl = 0; bl < g.fblocks[mi]; bl++)
                    it[ni++] = make_uint2((unsigned)mi, bl);
            st.grid = (int)st.nitems;
            e = launch_axis_mixed(0, precision, st.k, st.mode, st.sd, st.layout, nullptr, nullptr, st.nitems,
                                  st.smem, st.threads, nullptr);
        } else {
            TilePtrs *tp = reinterpret_cast<TilePtrs *>(img.data() + st.off_fields);
            for (size_t mi = 0; mi < g.f.size(); mi++)
                tp[mi] = ptrs(g.f[mi]);
            st.a.src_v = st.a.src_w = nullptr;
            st.a.dst_v = st.a.dst_w = nullptr;
            st.a.out = nullptr;
            st.a.out_f64 = b->out_f64;
            st.sv = view(g.f[0]);
            e = launch_axis_batch(0, precision, st.a, st.g, st.sv, nullptr, st.bpf, st.nitems, &st.grid, nullptr);
            // column stages: the pipelined kernel when the fields' source
            // cells are evenly spaced (one tensor map over all of them)
            if (e == cudaSuccess && st.a.layout == 1 &&
                cols_pipe_plan(precision, st.a, st.g, (int)g.f.size(), st.cp, st.pk, st.pmode,
                               kn.interleave ? 0 : (kn.cols_pipe == 0 ? -1 : (kn.cols_pipe == 1 ? 1 : 0)))) {
                const char *s0 = static_cast<const char *>(tp[0].src);
                const int64_t fstride = g.f.size() > 1 ? static_cast<const char *>(tp[1].src) - s0 : 0;
                bool even = fstride >= 0 && fstride % 16 == 0;
                for (size_t mi = 1; even && mi < g.f.size(); mi++)
                    even = static_cast<const char *>(tp[mi].src) == s0 + (int64_t)mi * fstride;
                if (even &&
                    cols_pipe_map(precision, st.cp, st.g, s0, fstride, (int)g.f.size(), &st.map) == cudaSuccess) {
                    st.pipe = true;
                    st.cp.status =
                        reinterpret_cast<uint32_t *>(&reinterpret_cast<FieldHeader *>(dv + b->off_hdrs)->error);
                    st.grid = st.cp.ntiles > 0 ? 1 : 0;
                }
            }
        }
        if (e != cudaSuccess)
            return cuda_fail(e, "batch axis kernel setup");
        b->stages.push_back(st);
    }
    e = cudaMemcpy(dv, img.data(), tables_end, cudaMemcpyHostToDevice);
    if (e != cudaSuccess)
        return cuda_fail(e, "batch tables upload");
    // interleaved schedule: an x stage and a y stage, one field shape
    b->interleave = kn.interleave && b->stages.size() == 2 && !b->stages[0].mixed && !b->stages[1].mixed &&
                    b->stages[0].axis == 0 && b->stages[1].axis == 1 && b->stages[0].nf == (uint32_t)nf &&
                    b->stages[1].nf == (uint32_t)nf;
    if (b->interleave) {
        e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
        if (e == cudaSuccess)
            e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
        b->ev_field.assign((size_t)nf, nullptr);
        for (int f = 0; f < nf && e == cudaSuccess; f++)
            e = cudaEventCreateWithFlags(&b->ev_field[f], cudaEventDisableTiming);
        if (e != cudaSuccess)
            return cuda_fail(e, "batch interleave streams");
    }
    return FB_OK;
}

int batch_enqueue(fb_batch *b, cudaStream_t st, bool prof)
{
    char *dv = b->dev;
    size_t ev = prof ? prof_event(st) : 0;
    cudaError_t e;
    const uint32_t *sorted = nullptr;
    const void *recs = nullptr;
    {
        StageRange r("fb sort");
        e = batch_sort(b->precision, reinterpret_cast<const BatchKeyField *>(dv + b->off_keyf),
                       reinterpret_cast<const uint2 *>(dv + b->off_blocks), b->nblocks, b->ntot, b->nbins,
                       reinterpret_cast<FieldHeader *>(dv + b->off_hdrs), b->nfields,
                       reinterpret_cast<uint32_t *>(dv + b->off_sort), reinterpret_cast<uint32_t *>(dv + b->off_bins),
                       &sorted, &recs, st);
    }
    if (e != cudaSuccess)
        return cuda_fail(e, "batch sample sort");
    if (prof) {
        size_t e1 = prof_event(st);
        g_prof.recs.push_back({0, ev, e1});
        ev = e1;
    }
    if (b->interleave) {
        // field f: x on `st`, then y on the side stream once its x is done,
        // beside field f + 1's x; the side stream joins back at the end
        BatchStage &sx = b->stages[0], &sy = b->stages[1];
        const TilePtrs *tx = reinterpret_cast<const TilePtrs *>(dv + sx.off_fields);
        const TilePtrs *ty = reinterpret_cast<const TilePtrs *>(dv + sy.off_fields);
        e = cudaEventRecord(b->ev_fork, st);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(b->side, b->ev_fork, 0);
        for (int f = 0; f < b->nfields && e == cudaSuccess; f++) {
            {
                StageRange r(axis_range_name(0));
                e = launch_axis_batch(1, b->precision, sx.a, sx.g, sx.sv, tx + f, sx.bpf, sx.bpf, &sx.grid, st);
            }
            if (e == cudaSuccess)
                e = cudaEventRecord(b->ev_field[f], st);
            if (e == cudaSuccess)
                e = cudaStreamWaitEvent(b->side, b->ev_field[f], 0);
            if (e == cudaSuccess) {
                StageRange r(axis_range_name(1));
                e = launch_axis_batch(1, b->precision, sy.a, sy.g, sy.sv, ty + f, sy.bpf, sy.bpf, &sy.grid, b->side);
            }
        }
        if (e == cudaSuccess)
            e = cudaEventRecord(b->ev_join, b->side);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(st, b->ev_join, 0);
        if (e != cudaSuccess)
            return cuda_fail(e, "batch interleaved axis kernels");
        if (prof) {
            // x and y overlap: one stage (3) for both axes
            size_t e1 = prof_event(st);
            g_prof.recs.push_back({3, ev, e1});
        }
        return FB_OK;
    }
    for (size_t i = 0; i < b->stages.size(); i++) {
        BatchStage &s = b->stages[i];
        StageRange r(axis_range_name(s.axis));
        if (s.pipe)
            e = launch_cols_pipe(b->precision, s.pk, s.pmode, s.map, s.cp,
                                 reinterpret_cast<const TilePtrs *>(dv + s.off_fields), st);
        else if (s.mixed)
            e = launch_axis_mixed(1, b->precision, s.k, s.mode, s.sd, s.layout,
                                  reinterpret_cast<const MixedField *>(dv + s.off_fields),
                                  reinterpret_cast<const uint2 *>(dv + s.off_items), s.nitems, s.smem, s.threads,
                                  st);
        else
            e = launch_axis_batch(1, b->precision, s.a, s.g, s.sv,
                                  reinterpret_cast<const TilePtrs *>(dv + s.off_fields), s.bpf, s.nitems, &s.grid,
                                  st);
        if (e != cudaSuccess)
            return cuda_fail(e, "batch axis kernel");
        if (prof) {
            size_t e1 = prof_event(st);
            g_prof.recs.push_back({1 + s.axis, ev, e1});
            ev = e1;
        }
    }
    return FB_OK;
}

std::string batch_signature(int precision, const fb_field2d *fields, int nf, int out_f64)
{
    std::string sig;
    char buf[256];
    snprintf(buf, sizeof(buf), "p%d o%d n%d", precision, out_f64, nf);
    sig += buf;
    for (int f = 0; f < nf; f++) {
        const fb_field2d &F = fields[f];
        snprintf(buf, sizeof(buf), "|%d %lld %lld %d %d %d %lld", F.method, (long long)F.size[0],
                 (long long)F.size[1], fb_half_kernel_size_opt(F.sigma[0], F.step[0], F.num_iter),
                 fb_half_kernel_size_opt(F.sigma[1], F.step[1], F.num_iter), F.num_iter, (long long)F.n_pts);
        sig += buf;
    }
    return sig;
}

// Times each candidate launch shape on the given fields (2 warm-up runs,
// best of 5) and returns the fastest.
int batch_tune(int precision, const fb_field2d *fields, int nf, int out_f64, fb_batch_knobs *best)
{
    bool wide = false;
    for (int f = 0; f < nf && precision == FB_FP32C; f++)
        for (int m = 0; m < 2; m++)
            if (fb_half_kernel_size_opt(fields[f].sigma[m], fields[f].step[m], fields[f].num_iter) > 32)
                wide = true;
    std::vector<int> chunks = wide ? std::vector<int>{17, 33} : std::vector<int>{0};
    const int rows[3] = {128, 256, 512};
    const int mixes[2] = {0, 1};
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e0);
    if (e == cudaSuccess)
        e = cudaEventCreate(&e1);
    float best_ms = 1e30f;
    *best = fb_batch_knobs{0, 0, 0, 0, 0};
    int rc = e == cudaSuccess ? FB_OK : cuda_fail(e, "tuning stream");
    // best of 5 timed runs (after 2 warm-up runs) of one candidate
    auto try_knobs = [&](fb_batch_knobs kn) {
        if (rc != FB_OK)
            return;
        fb_batch tb;
        rc = batch_build(precision, fields, nf, out_f64, kn, &tb);
        float t_best = 1e30f;
        for (int it = 0; rc == FB_OK && it < 7; it++) {
            if (it >= 2)
                cudaEventRecord(e0, st);
            rc = batch_enqueue(&tb, st, false);
            if (rc == FB_OK && it >= 2) {
                cudaEventRecord(e1, st);
                e = cudaEventSynchronize(e1);
                float ms = 0.f;
                if (e == cudaSuccess)
                    e = cudaEventElapsedTime(&ms, e0, e1);
                if (e != cudaSuccess)
                    rc = cuda_fail(e, "tuning run");
                t_best = std::min(t_best, ms);
            }
        }
        if (rc == FB_OK && t_best < best_ms) {
            best_ms = t_best;
            *best = kn;
        }
        cudaStreamSynchronize(st);
        batch_free(&tb);
    };
    for (int c : chunks)
        for (int r : rows)
            for (int mx : mixes)
                try_knobs(fb_batch_knobs{c, r, mx, 0, 0});
    // then the column kernel both ways, and the interleaved schedule, on the
    // best launch shape
    const fb_batch_knobs shape = *best;
    if (!shape.mixed) {
        for (int pipe = 1; pipe <= 2; pipe++)
            try_knobs(fb_batch_knobs{shape.chunk, shape.rows_threads, 0, pipe, 0});
        try_knobs(fb_batch_knobs{shape.chunk, shape.rows_threads, 0, 2, 1});
    }
    if (e0)
        cudaEventDestroy(e0);
    if (e1)
        cudaEventDestroy(e1);
    if (st)
        cudaStreamDestroy(st);
    return rc;
}

}  // namespace

extern "C" int fb_batch_create(int precision, const fb_field2d *fields, int n_fields, int out_f64, int flags,
                               const fb_batch_knobs *knobs, fb_batch **plan)
{
    g_err[0] = 0;
    if (!plan)
        return fail(FB_ERR_ARG, "plan pointer is required");
    *plan = nullptr;
    if (precision != FB_FP64 && precision != FB_FP32C)
        return fail(FB_ERR_ARG, "unknown precision %d", precision);
    if (flags & ~(FB_BATCH_GRAPH | FB_BATCH_TUNE))
        return fail(FB_ERR_ARG, "unknown batch flags 0x%x", flags);
    fb_batch_knobs kn{0, 0, 0};
    if (knobs) {
        kn = *knobs;
    } else if (flags & FB_BATCH_TUNE) {
        if (n_fields < 1 || !fields)
            return fail(FB_ERR_ARG, "a batch needs at least one field");
        const std::string sig = batch_signature(precision, fields, n_fields, out_f64);
        std::lock_guard<std::mutex> lk(g_batch_tune_mu);
        auto it = g_batch_tuned.find(sig);
        if (it != g_batch_tuned.end()) {
            kn = it->second;
        } else {
            int rc = batch_tune(precision, fields, n_fields, out_f64, &kn);
            if (rc != FB_OK)
                return rc;
            g_batch_tuned[sig] = kn;
        }
    }
    fb_batch *b = new fb_batch();
    b->flags = flags;
    int rc = batch_build(precision, fields, n_fields, out_f64, kn, b);
    if (rc == FB_OK && (flags & FB_BATCH_GRAPH)) {
        cudaError_t e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
        if (e != cudaSuccess)
            rc = cuda_fail(e, "batch capture stream");
    }
    if (rc != FB_OK) {
        batch_free(b);
        delete b;
        return rc;
    }
    *plan = b;
    return FB_OK;
}

extern "C" int fb_batch_run(fb_batch *b, void *stream)
{
    g_err[0] = 0;
    if (!b)
        return fail(FB_ERR_ARG, "null plan");
    cudaStream_t st = (cudaStream_t)stream;
    if (!(b->flags & FB_BATCH_GRAPH)) {
        std::unique_lock<std::mutex> plk(g_prof.mu, std::defer_lock);
        const bool prof = g_prof.on;
        if (prof)
            plk.lock();
        return batch_enqueue(b, st, prof);
    }
    if (!b->exec) {
        cudaError_t e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess)
            return cuda_fail(e, "batch graph capture");
        int rc = batch_enqueue(b, b->cap, false);
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(b->cap, &g);
        if (rc != FB_OK) {
            if (g)
                cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess)
            return cuda_fail(e, "batch graph capture");
        b->graph = g;
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) {
            b->exec = nullptr;
            return cuda_fail(e, "batch graph instantiate");
        }
    }
    cudaError_t e = cudaGraphLaunch(b->exec, st);
    if (e != cudaSuccess)
        return cuda_fail(e, "batch graph launch");
    return FB_OK;
}

extern "C" int fb_batch_enqueue_host(fb_batch *b, const double *const *h_pts, const double *const *h_val,
                                     void *const *h_out, void *stream)
{
    g_err[0] = 0;
    if (!b || !h_pts || !h_val || !h_out)
        return fail(FB_ERR_ARG, "null argument");
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaSuccess;
    for (int f = 0; f < b->nfields && e == cudaSuccess; f++) {
        const fb_field2d &F = b->fields[f];
        if (F.n_pts == 0)
            continue;
        if (!h_pts[f] || !h_val[f])
            return fail(FB_ERR_ARG, "field %d: null host pointer", f);
        e = cudaMemcpyAsync((void *)F.pts, h_pts[f], sizeof(double) * 2 * (size_t)F.n_pts, cudaMemcpyHostToDevice,
                            st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync((void *)F.val, h_val[f], sizeof(double) * (size_t)F.n_pts, cudaMemcpyHostToDevice,
                                st);
    }
    if (e != cudaSuccess)
        return cuda_fail(e, "batch inputs to device");
    int rc = fb_batch_run(b, stream);
    if (rc != FB_OK)
        return rc;
    // results back in 16 MiB pieces over several streams, so that several
    // copy engines share the transfer
    if (!b->copy_st[0]) {
        for (int q = 0; q < fb_batch::kCopyStreams && e == cudaSuccess; q++)
            e = cudaStreamCreateWithFlags(&b->copy_st[q], cudaStreamNonBlocking);
        for (int q = 0; q <= fb_batch::kCopyStreams && e == cudaSuccess; q++)
            e = cudaEventCreateWithFlags(&b->copy_ev[q], cudaEventDisableTiming);
        if (e != cudaSuccess)
            return cuda_fail(e, "batch copy streams");
    }
    e = cudaEventRecord(b->copy_ev[fb_batch::kCopyStreams], st);
    for (int q = 0; q < fb_batch::kCopyStreams && e == cudaSuccess; q++)
        e = cudaStreamWaitEvent(b->copy_st[q], b->copy_ev[fb_batch::kCopyStreams], 0);
    const size_t osz = b->out_f64 ? 8 : 4;
    const size_t piece = (size_t)16 << 20;
    int next = 0;
    for (int f = 0; f < b->nfields && e == cudaSuccess; f++) {
        const fb_field2d &F = b->fields[f];
        if (!h_out[f])
            return fail(FB_ERR_ARG, "field %d: null host pointer", f);
        const size_t bytes = osz * (size_t)F.size[0] * (size_t)F.size[1];
        for (size_t o = 0; o < bytes && e == cudaSuccess; o += piece) {
            const size_t len = std::min(piece, bytes - o);
            e = cudaMemcpyAsync((char *)h_out[f] + o, (const char *)F.out + o, len, cudaMemcpyDeviceToHost,
                                b->copy_st[next]);
            next = (next + 1) % fb_batch::kCopyStreams;
        }
    }
    for (int q = 0; q < fb_batch::kCopyStreams && e == cudaSuccess; q++) {
        e = cudaEventRecord(b->copy_ev[q], b->copy_st[q]);
        if (e == cudaSuccess)
            e = cudaStreamWaitEvent(st, b->copy_ev[q], 0);
    }
    if (e != cudaSuccess)
        return cuda_fail(e, "batch results to host");
    return FB_OK;
}

extern "C" int fb_batch_run_host(fb_batch *b, const double *const *h_pts, const double *const *h_val,
                                 void *const *h_out, void *stream)
{
    int rc = fb_batch_enqueue_host(b, h_pts, h_val, h_out, stream);
    if (rc != FB_OK)
        return rc;
    cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
    return e == cudaSuccess ? FB_OK : cuda_fail(e, "batch results to host");
}

extern "C" int fb_batch_knobs_of(const fb_batch *b, fb_batch_knobs *knobs)
{
    if (!b || !knobs)
        return fail(FB_ERR_ARG, "null argument");
    *knobs = b->knobs;
    return FB_OK;
}

extern "C" int fb_batch_status(const fb_batch *b, void *stream, int *status)
{
    g_err[0] = 0;
    if (!b)
        return fail(FB_ERR_ARG, "null plan");
    std::vector<FieldHeader> h((size_t)b->nfields);
    cudaStream_t st = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(h.data(), b->dev + b->off_hdrs, sizeof(FieldHeader) * h.size(),
                                    cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return cuda_fail(e, "fb_batch_status");
    int bits = 0;
    for (const FieldHeader &x : h)
        bits |= x.error;
    if (status)
        *status = bits;
    return bits ? device_fail((uint32_t)bits, "fb_batch_status") : FB_OK;
}

extern "C" int fb_batch_info(const fb_batch *b, int *kernel_launches, int *memsets, size_t *device_bytes)
{
    if (!b)
        return fail(FB_ERR_ARG, "null plan");
    // batch_sort: a memset of the field headers, k_batch_keys (every
    // field's bin starts scanned by its last block) when there are samples,
    // then k_bin_scatter and k_sort_bins (which also puts the records in
    // sorted order); then one axis launch per stage with work
    int k = (b->nblocks > 0 ? 1 : 0) + (b->ntot > 0 ? 2 : 0);
    for (const BatchStage &s : b->stages)
        k += s.grid > 0 ? 1 : 0;
    if (kernel_launches)
        *kernel_launches = k;
    if (memsets)
        *memsets = 1;
    if (device_bytes)
        *device_bytes = b->dev_bytes;
    return FB_OK;
}

extern "C" void fb_batch_destroy(fb_batch *b)
{
    if (!b)
        return;
    batch_free(b);
    delete b;
}

// ---------------------------------------------------------------------------
// resampling without allocation
// ---------------------------------------------------------------------------
//
// fb_resample needs device scratch for its row / column tables (size[1] +
// 2 size[0] doubles), which the caller allocates.  Some callers cannot
// allocate at call time: code that runs while another component owns the
// device allocator, or a loop with a latency budget that cudaMalloc /
// cudaFree (which may synchronize the device) would break.  For them
// fb_resample_noalloc keeps the tables in one file-scope device array of
// fixed size, located once per device with cudaGetSymbolAddress.
//
// Every table entry the resample kernel reads is written by the table
// kernels of the same call first, so nothing in the array has to start at
// zero.  The array is shared by every call on a device: two calls that
// overlap in time (different streams or host threads) race on it.

namespace {
constexpr int64_t kResampleScratchDoubles = 49152;   // 384 KiB: size[1] + 2 * size[0] <= 49152
constexpr int kMaxScratchDevices = 64;
static __device__ __align__(256) double g_resample_scratch[kResampleScratchDoubles];
std::mutex g_scratch_mu;
double *g_scratch_ptr[kMaxScratchDevices] = {};

// Address of the scratch array on the current device; the first call for a
// device looks it up (no allocation).  The cached address stays valid for
// the lifetime of the device's primary context (a cudaDeviceReset would
// reload the module, possibly elsewhere).
int resample_scratch(double **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess)
        return cuda_fail(e, "fb_resample_noalloc: current device");
    if (dev < 0 || dev >= kMaxScratchDevices)
        return fail(FB_ERR_ARG, "fb_resample_noalloc: device %d beyond the %d supported", dev, kMaxScratchDevices);
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_resample_scratch);
        if (e != cudaSuccess)
            return cuda_fail(e, "fb_resample_noalloc: scratch address");
        g_scratch_ptr[dev] = static_cast<double *>(p);
    }
    *out = g_scratch_ptr[dev];
    return FB_OK;
}
}  // namespace

extern "C" int fb_resample_noalloc(const float *d_lam, int64_t lam_w, int64_t lam_h, const double *lam_x0,
                                   const double *x0, const double *step, const int64_t *size, const double *proj,
                                   float *d_out, void *stream)
{
    g_err[0] = 0;
    if (!d_lam || !lam_x0 || !x0 || !step || !size || !proj || !d_out || size[0] < 1 || size[1] < 1 ||
        lam_w < 2 || lam_h < 2)
        return fail(FB_ERR_ARG, "invalid resample arguments");
    if (size[0] > kResampleScratchDoubles || size[1] > kResampleScratchDoubles ||
        size[1] + 2 * size[0] > kResampleScratchDoubles)
        return fail(FB_ERR_ARG,
                    "fb_resample_noalloc: grid %lld x %lld needs %lld table doubles, more than the static "
                    "scratch of %lld (size[1] + 2 * size[0] <= %lld); use fb_resample with a caller workspace",
                    (long long)size[0], (long long)size[1], (long long)(size[1] + 2 * size[0]),
                    (long long)kResampleScratchDoubles, (long long)kResampleScratchDoubles);
    double *tab = nullptr;
    int rc = resample_scratch(&tab);
    if (rc != FB_OK)
        return rc;
    cudaError_t e = launch_resample(d_lam, lam_w, lam_h, lam_x0, x0, step, size, proj, d_out, tab,
                                    (cudaStream_t)stream);
    return e == cudaSuccess ? FB_OK : cuda_fail(e, "resample");
}
