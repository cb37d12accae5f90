// fb_capi.cu -- the C ABI: argument checks, kernel-size parameters, workspace
// layout and the per-axis launch plan of one interpolation.
//
// Host arithmetic (T, alpha, the NaN threshold) follows the reference's float64
// expressions operation by operation; this file is compiled without FMA
// contraction so the host results are identical on x86 and aarch64.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "../../include/fastbarnes_gb300.h"
#include "fb_internal.cuh"
#include "fb_kernels.cuh"

using namespace fbg;

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

extern "C" const char *fb_version(void) { return "fastbarnes_gb300 0.1 (sm_103a)"; }
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
              const double *step, const int64_t *size, int num_iter, double max_dist_weight, Plan &p)
{
    if (dim < 1 || dim > 3)
        return fail(FB_ERR_ARG, "dim must be 1, 2 or 3 (got %d)", dim);
    if (precision != FB_FP64 && precision != FB_FP32C)
        return fail(FB_ERR_ARG, "unknown precision %d", precision);
    if (method != FB_OPTIMIZED_CONVOLUTION && method != FB_CONVOLUTION)
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
        const AxisPlanLimits lim = axis_limits(precision, T);
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
    cudaError_t e = sort_samples(p.precision, d_pts, d_val, p.npts, p.g, p.bin_w, p.nbins, hdr, scratch, bins,
                                 &sorted, &recs, st);
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
        e = launch_axis(p.precision, a, p.g, sv, st);
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
    if (e == cudaSuccess)
        e = cudaStreamSynchronize(st);
    if (e != cudaSuccess)
        return cuda_fail(e, "copy to host");
    return FB_OK;
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
