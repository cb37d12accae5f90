/*
 * barnes_oracle.c -- CPU oracle for the fast Barnes interpolation path.
 *
 * TEST INFRASTRUCTURE, NOT PRODUCT CODE.  This file restates, in plain C and
 * in the reference's own floating-point operation order, the algorithms of
 * MeteoSwiss/fast-barnes-py that the GPU library replaces.  It exists only to
 * check the GPU results (tests/, the smoke check) and to time the reference's
 * CPU algorithm beside the GPU (bench.py's cpu_baseline / --impl reference
 * arm).  Nothing in the product library links or calls it.
 *
 * Build: gcc -O2 -ffp-contract=off -fno-fast-math -fopenmp -shared -fPIC
 * (-ffp-contract=off keeps gcc from fusing a*b+c into an FMA on aarch64, which
 * would change the rounding of the reference's separate multiply and add).
 *
 * Parity is pinned: tests/golden/make_golden.py runs the reference itself (as
 * pure Python/NumPy) and stores its outputs; tests/test_oracle_golden.py checks
 * that this file reproduces them bit for bit (float32 output and float64
 * quotient) for the 1D/2D/3D paths and to 1e-12 for the sphere path, whose
 * trigonometry the reference evaluates with NumPy's vectorised functions.
 *
 * Threading: the row / column loops of the convolution are independent lines,
 * so they run in parallel under OpenMP when nthreads > 1.  Each line is still
 * computed by exactly the reference's sequential loop, so the result does not
 * depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FBO_EXPORT __attribute__((visibility("default")))

static const double RAD_PER_DEGREE = 3.14159265358979311600 / 180.0;

/* ------------------------------------------------------------------------- */
/* kernel-size helpers                                                        */
/* ------------------------------------------------------------------------- */

/* fastbarnes/interpolation.py:548-552 (_get_half_kernel_size_opt):
 * T = int32((sqrt(1 + 12 s^2 / n) - 1) / 2), s = sigma / step.  NumPy
 * evaluates 12*s*s/num_iter left to right. */
FBO_EXPORT int fbo_half_kernel_size_opt(double sigma, double step, int num_iter)
{
    double s = sigma / step;
    double t = (sqrt(1.0 + 12.0 * s * s / (double)num_iter) - 1.0) / 2.0;
    return (int)t;
}

/* fastbarnes/interpolation.py:560-569 (_get_tail_value). */
FBO_EXPORT double fbo_tail_value(double sigma, double step, int num_iter)
{
    int hks = fbo_half_kernel_size_opt(sigma, step, num_iter);
    int ks = 2 * hks + 1;
    double sigma_rect_sqr = (double)((hks + 1) * hks) / 3.0 * (step * step);
    double s2n = sigma * sigma / (double)num_iter;
    double d = (double)(hks + 1) * step;
    return 0.5 * (double)ks * (s2n - sigma_rect_sqr) / (d * d - s2n);
}

/* fastbarnes/interpolation.py:783-785 (_get_half_kernel_size, plain method). */
FBO_EXPORT int fbo_half_kernel_size(double sigma, double step, int num_iter)
{
    double t = sqrt(3.0 / (double)num_iter) * sigma / step + 0.5;
    return (int)t;
}

/* fastbarnes/interpolation.py:796-803 (_get_sigma_effective). */
FBO_EXPORT double fbo_sigma_effective(double sigma, double step, int num_iter)
{
    int hks = fbo_half_kernel_size(sigma, step, num_iter);
    return sqrt((double)num_iter / 3.0 * (double)hks * (double)(hks + 1)) * step;
}

/* ------------------------------------------------------------------------- */
/* 1D rect-kernel passes                                                      */
/* ------------------------------------------------------------------------- */

/* fastbarnes/interpolation.py:484-533 (_accumulate_tail_array): num_iter
 * passes of a running window sum of length rect_len plus tail weight alpha at
 * +-(T+1), zero outside [0, arr_len), ping-ponging between the two buffers.
 * Returns whichever buffer holds the result, as the reference does. */
FBO_EXPORT double *fbo_accumulate_tail_array(double *in_arr, double *h_arr, int arr_len,
                                             int rect_len, int num_iter, double alpha)
{
    int h0 = (rect_len - 1) / 2;
    int h0_1 = h0 + 1;
    int h1 = rect_len - h0;
    for (int it = 0; it < num_iter; it++) {
        double accu = 0.0;
        for (int k = -h0; k < 0; k++)
            accu += in_arr[k + h0];
        for (int k = 0; k < h1; k++) {
            accu += in_arr[k + h0];
            h_arr[k] = accu + alpha * in_arr[k + h0_1];
        }
        for (int k = h1; k < arr_len - h0_1; k++) {
            accu += (in_arr[k + h0] - in_arr[k - h1]);
            h_arr[k] = accu + alpha * (in_arr[k - h1] + in_arr[k + h0_1]);
        }
        {
            int k = arr_len - h0_1;
            accu += (in_arr[k + h0] - in_arr[k - h1]);
            h_arr[k] = accu + alpha * in_arr[k - h1];
        }
        for (int k = arr_len - h0; k < arr_len; k++) {
            accu -= in_arr[k - h1];
            h_arr[k] = accu + alpha * in_arr[k - h1];
        }
        double *t = in_arr;
        in_arr = h_arr;
        h_arr = t;
    }
    return in_arr;
}

/* fastbarnes/interpolation.py:729-772 (_accumulate_array): the same without
 * tails (the plain 'convolution' method). */
FBO_EXPORT double *fbo_accumulate_array(double *in_arr, double *h_arr, int arr_len,
                                        int rect_len, int num_iter)
{
    int h0 = (rect_len - 1) / 2;
    int h1 = rect_len - h0;
    for (int it = 0; it < num_iter; it++) {
        double accu = 0.0;
        for (int k = -h0; k < 0; k++)
            accu += in_arr[k + h0];
        for (int k = 0; k < h1; k++) {
            accu += in_arr[k + h0];
            h_arr[k] = accu;
        }
        for (int k = h1; k < arr_len - h0; k++) {
            accu += (in_arr[k + h0] - in_arr[k - h1]);
            h_arr[k] = accu;
        }
        for (int k = arr_len - h0; k < arr_len; k++) {
            accu -= in_arr[k - h1];
            h_arr[k] = accu;
        }
        double *t = in_arr;
        in_arr = h_arr;
        h_arr = t;
    }
    return in_arr;
}

/* Not a restatement: the same num_iter passes as fbo_accumulate_tail_array,
 * but every output summed directly over its window (2T + 1 cells plus the
 * two tails, zero outside [0, arr_len)), so no rounding is carried from one
 * output to the next.  The reference's running sum carries its rounding along
 * the whole line; on very long lines this direct form is the more accurate
 * float64 value of the same quantity and serves as the truth both are
 * measured against.  Cells run in parallel (nthreads). */
FBO_EXPORT double *fbo_direct_tail_passes(double *in_arr, double *h_arr, int64_t arr_len, int rect_len,
                                          int num_iter, double alpha, int nthreads)
{
    const int64_t T = (rect_len - 1) / 2;
    (void)nthreads;
    for (int it = 0; it < num_iter; it++) {
#pragma omp parallel for num_threads(nthreads) schedule(static)
        for (int64_t k = 0; k < arr_len; k++) {
            const int64_t lo = k - T < 0 ? 0 : k - T;
            const int64_t hi = k + T > arr_len - 1 ? arr_len - 1 : k + T;
            double acc = 0.0;
            for (int64_t m = lo; m <= hi; m++)
                acc += in_arr[m];
            double tails = 0.0;
            if (k - T - 1 >= 0)
                tails += in_arr[k - T - 1];
            if (k + T + 1 < arr_len)
                tails += in_arr[k + T + 1];
            h_arr[k] = acc + alpha * tails;
        }
        double *t = in_arr;
        in_arr = h_arr;
        h_arr = t;
    }
    return in_arr;
}

/* ------------------------------------------------------------------------- */
/* splat                                                                      */
/* ------------------------------------------------------------------------- */

/* fastbarnes/interpolation.py:218-322 (_inject_data_1d/2d/3d).  Fields are
 * laid out [z][y][x] with x fastest; corner order and skip rule as there. */
static void inject(int dim, double *vg, double *wg, const double *pts, const double *val,
                   int64_t npts, const double *x0, const double *step, const int64_t *size)
{
    const int64_t W = size[0];
    const int64_t H = dim > 1 ? size[1] : 1;
    for (int64_t k = 0; k < npts; k++) {
        const double *p = pts + k * dim;
        if (dim == 1) {
            double xc = (p[0] - x0[0]) / step[0];
            if (xc < 0.0 || xc >= (double)(size[0] - 1))
                continue;
            int64_t xi = (int64_t)xc;
            double xw = xc - (double)xi;
            double w = (1.0 - xw);
            vg[xi] += w * val[k];
            wg[xi] += w;
            w = xw;
            vg[xi + 1] += w * val[k];
            wg[xi + 1] += w;
        } else if (dim == 2) {
            double xc = (p[0] - x0[0]) / step[0];
            double yc = (p[1] - x0[1]) / step[1];
            if (xc < 0.0 || yc < 0.0 || xc >= (double)(size[0] - 1) || yc >= (double)(size[1] - 1))
                continue;
            int64_t xi = (int64_t)xc, yi = (int64_t)yc;
            double xw = xc - (double)xi, yw = yc - (double)yi;
            int64_t b = yi * W + xi;
            double w;
            w = (1.0 - xw) * (1.0 - yw); vg[b] += w * val[k];         wg[b] += w;
            w = xw * (1.0 - yw);         vg[b + 1] += w * val[k];     wg[b + 1] += w;
            w = xw * yw;                 vg[b + W + 1] += w * val[k]; wg[b + W + 1] += w;
            w = (1.0 - xw) * yw;         vg[b + W] += w * val[k];     wg[b + W] += w;
        } else {
            double xc = (p[0] - x0[0]) / step[0];
            double yc = (p[1] - x0[1]) / step[1];
            double zc = (p[2] - x0[2]) / step[2];
            if (xc < 0.0 || yc < 0.0 || zc < 0.0 || xc >= (double)(size[0] - 1) ||
                yc >= (double)(size[1] - 1) || zc >= (double)(size[2] - 1))
                continue;
            int64_t xi = (int64_t)xc, yi = (int64_t)yc, zi = (int64_t)zc;
            double xw = xc - (double)xi, yw = yc - (double)yi, zw = zc - (double)zi;
            int64_t b = (zi * H + yi) * W + xi, S = W * H;
            double w;
            w = (1.0 - xw) * (1.0 - yw) * (1.0 - zw); vg[b] += w * val[k];             wg[b] += w;
            w = xw * (1.0 - yw) * (1.0 - zw);         vg[b + 1] += w * val[k];         wg[b + 1] += w;
            w = xw * yw * (1.0 - zw);                 vg[b + W + 1] += w * val[k];     wg[b + W + 1] += w;
            w = (1.0 - xw) * yw * (1.0 - zw);         vg[b + W] += w * val[k];         wg[b + W] += w;
            w = (1.0 - xw) * (1.0 - yw) * zw;         vg[b + S] += w * val[k];         wg[b + S] += w;
            w = xw * (1.0 - yw) * zw;                 vg[b + S + 1] += w * val[k];     wg[b + S + 1] += w;
            w = xw * yw * zw;                         vg[b + S + W + 1] += w * val[k]; wg[b + S + W + 1] += w;
            w = (1.0 - xw) * yw * zw;                 vg[b + S + W] += w * val[k];     wg[b + S + W] += w;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* n-fold convolution along every axis                                        */
/* ------------------------------------------------------------------------- */

/* Runs the 1D passes over every line of one axis of a [D][H][W] field, in the
 * axis order of _convolve_tail_{1,2,3}d (interpolation.py:372-479) and
 * _convolve_{1,2,3}d (:617-724).  Lines are gathered with their stride, as the
 * reference's .copy() does, and written back. */
static void convolve_axis(double *f, const int64_t *shape_xyz, int axis, int rect_len,
                          int num_iter, double alpha, int tail, int nthreads, int direct)
{
    int64_t W = shape_xyz[0], H = shape_xyz[1], D = shape_xyz[2];
    int64_t len = axis == 0 ? W : (axis == 1 ? H : D);
    int64_t stride = axis == 0 ? 1 : (axis == 1 ? W : W * H);
    int64_t nlines = (W * H * D) / len;
    (void)nthreads;
    if (direct) {
        /* the drift-free truth (test use): lines one after another, the
         * cells of a line in parallel */
        double *a = (double *)malloc(sizeof(double) * len);
        double *h = (double *)malloc(sizeof(double) * len);
        for (int64_t li = 0; li < nlines; li++) {
            int64_t base = axis == 0 ? li * W : (axis == 1 ? (li / W) * W * H + li % W : li);
            for (int64_t k = 0; k < len; k++)
                a[k] = f[base + k * stride];
            double *r = fbo_direct_tail_passes(a, h, len, rect_len, num_iter, tail ? alpha : 0.0, nthreads);
            for (int64_t k = 0; k < len; k++)
                f[base + k * stride] = r[k];
        }
        free(a);
        free(h);
        return;
    }
#pragma omp parallel num_threads(nthreads)
    {
        double *a = (double *)malloc(sizeof(double) * len);
        double *h = (double *)malloc(sizeof(double) * len);
#pragma omp for schedule(static)
        for (int64_t li = 0; li < nlines; li++) {
            int64_t base;
            if (axis == 0) {
                base = li * W;
            } else if (axis == 1) {
                int64_t z = li / W, x = li % W;
                base = z * W * H + x;
            } else {
                base = li;
            }
            for (int64_t k = 0; k < len; k++)
                a[k] = f[base + k * stride];
            double *r = tail ? fbo_accumulate_tail_array(a, h, (int)len, rect_len, num_iter, alpha)
                             : fbo_accumulate_array(a, h, (int)len, rect_len, num_iter);
            for (int64_t k = 0; k < len; k++)
                f[base + k * stride] = r[k];
        }
        free(a);
        free(h);
    }
}

/* fastbarnes/interpolation.py:328-367 (_interpolate_opt_convol) and :575-612
 * (_interpolate_convol).  method 0 = 'optimized_convolution', 1 =
 * 'convolution'.  val is not modified (the reference works on a copy).
 *   out_f32 : the reference's return value, (vg / wg + offset).astype(float32)
 *   q64     : optional, the float64 quotient before the float32 cast
 *   wg_out  : optional, the convolved weight field before the NaN mask
 * Returns the NaN threshold applied to the weight field. */
static double interpolate_impl(int method, int dim, const double *pts, const double *val, int64_t npts,
                               const double *sigma, const double *x0, const double *step, const int64_t *size,
                               int num_iter, double max_dist_weight, int nthreads, float *out_f32, double *q64,
                               double *wg_out, int direct);

FBO_EXPORT double fbo_interpolate(int method, int dim, const double *pts, const double *val,
                                  int64_t npts, const double *sigma, const double *x0,
                                  const double *step, const int64_t *size, int num_iter,
                                  double max_dist_weight, int nthreads, float *out_f32,
                                  double *q64, double *wg_out)
{
    return interpolate_impl(method, dim, pts, val, npts, sigma, x0, step, size, num_iter, max_dist_weight,
                            nthreads, out_f32, q64, wg_out, 0);
}

/* Not a restatement: fbo_interpolate with every pass summed directly over its
 * window (fbo_direct_tail_passes) instead of the reference's running sums --
 * the drift-free float64 truth for very long lines. */
FBO_EXPORT double fbo_interpolate_direct(int method, int dim, const double *pts, const double *val,
                                         int64_t npts, const double *sigma, const double *x0,
                                         const double *step, const int64_t *size, int num_iter,
                                         double max_dist_weight, int nthreads, float *out_f32,
                                         double *q64, double *wg_out)
{
    return interpolate_impl(method, dim, pts, val, npts, sigma, x0, step, size, num_iter, max_dist_weight,
                            nthreads, out_f32, q64, wg_out, 1);
}

static double interpolate_impl(int method, int dim, const double *pts, const double *val, int64_t npts,
                               const double *sigma, const double *x0, const double *step, const int64_t *size,
                               int num_iter, double max_dist_weight, int nthreads, float *out_f32, double *q64,
                               double *wg_out, int direct)
{
    int64_t shp[3] = {size[0], dim > 1 ? size[1] : 1, dim > 2 ? size[2] : 1};
    int64_t total = shp[0] * shp[1] * shp[2];

    /* _normalize_values (interpolation.py:204-212) on a copy of val */
    double *v = (double *)malloc(sizeof(double) * (npts > 0 ? npts : 1));
    double mn = npts > 0 ? val[0] : 0.0, mx = mn;
    for (int64_t k = 0; k < npts; k++) {
        v[k] = val[k];
        if (isnan(val[k])) { mn = val[k]; mx = val[k]; }
        if (!isnan(mn) && val[k] < mn) mn = val[k];
        if (!isnan(mx) && val[k] > mx) mx = val[k];
    }
    double offset = (mn + mx) / 2.0;
    for (int64_t k = 0; k < npts; k++)
        v[k] -= offset;

    double *vg = (double *)calloc((size_t)total, sizeof(double));
    double *wg = (double *)calloc((size_t)total, sizeof(double));
    inject(dim, vg, wg, pts, v, npts, x0, step, size);

    double factor[3] = {1.0, 1.0, 1.0};
    for (int m = 0; m < dim; m++) {
        int hks, ks;
        double alpha;
        if (method == 0) {
            hks = fbo_half_kernel_size_opt(sigma[m], step[m], num_iter);
            alpha = fbo_tail_value(sigma[m], step[m], num_iter);
        } else {
            hks = fbo_half_kernel_size(sigma[m], step[m], num_iter);
            alpha = 0.0;
        }
        ks = 2 * hks + 1;
        convolve_axis(vg, shp, m, ks, num_iter, alpha, method == 0, nthreads, direct);
        convolve_axis(wg, shp, m, ks, num_iter, alpha, method == 0, nthreads, direct);
        /* interpolation.py:424 / :669.  The plain method raises the int32
         * kernel size to the power n in int32 arithmetic, which wraps around
         * for large kernels; the product is reproduced modulo 2^32. */
        double pw;
        if (method == 0) {
            pw = pow((double)ks + 2.0 * alpha, (double)num_iter);
        } else {
            uint32_t p = 1u;
            for (int e = 0; e < num_iter; e++)
                p *= (uint32_t)ks;
            pw = (double)(int32_t)p;
        }
        factor[m] = pw / sqrt(2.0 * 3.14159265358979311600) / (sigma[m] / step[m]);
    }
    double thr = factor[0];
    for (int m = 1; m < dim; m++)
        thr = thr * factor[m];
    thr = thr * max_dist_weight;

    if (wg_out)
        memcpy(wg_out, wg, sizeof(double) * total);
#pragma omp parallel for num_threads(nthreads) schedule(static)
    for (int64_t i = 0; i < total; i++) {
        double w = wg[i];
        if (w < thr)
            w = NAN;
        double q = vg[i] / w + offset;
        if (q64)
            q64[i] = q;
        out_f32[i] = (float)q;
    }
    free(v);
    free(vg);
    free(wg);
    return thr;
}

/* fastbarnes/interpolation.py:861-938 (_interpolate_naive), sequential sums.
 * The reference evaluates the weighted sums with NumPy's dot / sum, whose
 * summation order is not specified, so this is a tolerance-level oracle (the
 * exact Barnes interpolation, used to measure approximation error). */
FBO_EXPORT void fbo_interpolate_naive(int dim, const double *pts, const double *val, int64_t npts,
                                      const double *sigma, const double *x0, const double *step,
                                      const int64_t *size, int nthreads, double *out)
{
    double mn = npts > 0 ? val[0] : 0.0, mx = mn;
    for (int64_t k = 0; k < npts; k++) {
        if (val[k] < mn) mn = val[k];
        if (val[k] > mx) mx = val[k];
    }
    double offset = (mn + mx) / 2.0;
    double scale[3];
    for (int m = 0; m < dim; m++)
        scale[m] = 2.0 * sigma[m] * sigma[m];
    int64_t W = size[0], H = dim > 1 ? size[1] : 1, D = dim > 2 ? size[2] : 1;
    int64_t total = W * H * D;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for (int64_t g = 0; g < total; g++) {
        int64_t i = g % W, j = (g / W) % H, kz = g / (W * H);
        double c[3] = {x0[0] + (double)i * step[0], dim > 1 ? x0[1] + (double)j * step[1] : 0.0,
                       dim > 2 ? x0[2] + (double)kz * step[2] : 0.0};
        double ws = 0.0, wt = 0.0;
        for (int64_t k = 0; k < npts; k++) {
            double d2 = 0.0;
            for (int m = 0; m < dim; m++) {
                double d = pts[k * dim + m] - c[m];
                d2 += d * d / scale[m];
            }
            double w = exp(-d2);
            ws += w * (val[k] - offset);
            wt += w;
        }
        out[g] = wt > 0.0 ? ws / wt + offset : NAN;
    }
}

/* fastbarnes/interpolation.py:809-855 (_interpolate_radius) with the
 * kd-tree radius search of fastbarnes/util/kdtree.py:208-331 replaced by a
 * scan over all samples under the same test: squared distance
 * (c0 - p0)^2 + (c1 - p1)^2 <= radius^2, radius = sqrt(-2 ln(min_weight))
 * sigma; weight exp(-d^2 / (2 sigma^2)); NaN where the weights sum below
 * max_dist_weight.  Sums in sample order (the reference's follow the tree's
 * order), so this is a tolerance-level oracle.  2D, one sigma. */
FBO_EXPORT void fbo_interpolate_radius(const double *pts, const double *val, int64_t npts, double sigma,
                                       const double *x0, const double *step, const int64_t *size,
                                       double max_dist_weight, double min_weight, int nthreads, double *out)
{
    double mn = npts > 0 ? val[0] : 0.0, mx = mn;
    for (int64_t k = 0; k < npts; k++) {
        if (val[k] < mn) mn = val[k];
        if (val[k] > mx) mx = val[k];
    }
    const double offset = (mn + mx) / 2.0;
    const double radius = sqrt(-2.0 * log(min_weight)) * sigma;
    const double r2 = radius * radius;
    const double scale = 2.0 * sigma * sigma;
    const int64_t W = size[0], H = size[1];
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 64)
    for (int64_t g = 0; g < W * H; g++) {
        const int64_t i = g % W, j = g / W;
        const double c0 = x0[0] + (double)i * step[0], c1 = x0[1] + (double)j * step[1];
        double ws = 0.0, wt = 0.0;
        for (int64_t k = 0; k < npts; k++) {
            const double dx = c0 - pts[2 * k], dy = c1 - pts[2 * k + 1];
            const double d2 = dx * dx + dy * dy;
            if (d2 <= r2) {
                const double w = exp(-d2 / scale);
                ws += w * (val[k] - offset);
                wt += w;
            }
        }
        out[g] = wt >= max_dist_weight ? ws / wt + offset : NAN;
    }
}

/* demo/quantization.py:23-37 (quant): drops the nbits least significant bits
 * of every non-NaN float64, m = frexp mantissa, int(m * 2^(53-nbits) + 0.5)
 * (a truncation toward zero), ldexp back. */
FBO_EXPORT void fbo_quant(double *arr, int64_t n, int nbits)
{
    if (nbits <= 0)
        return;
    int shift = 53 - nbits;
    for (int64_t i = 0; i < n; i++) {
        if (arr[i] == arr[i]) {
            int e;
            double m = frexp(arr[i], &e);
            double mi = trunc(m * ldexp(1.0, shift) + 0.5);
            arr[i] = ldexp(mi, e - shift);
        }
    }
}

/* fastbarnes/interpolationS2.py:259-301 (_interpolate_naive_S2, _dist_S2):
 * Gaussian weights of the great-circle distance (degrees) of every sample to
 * every lon/lat grid point; sigma[0] for both directions. */
FBO_EXPORT void fbo_interpolate_naive_s2(const double *pts, const double *val, int64_t npts,
                                         const double *sigma, const double *x0, const double *step,
                                         const int64_t *size, int nthreads, double *out)
{
    double mn = npts > 0 ? val[0] : 0.0, mx = mn;
    for (int64_t k = 0; k < npts; k++) {
        if (val[k] < mn) mn = val[k];
        if (val[k] > mx) mx = val[k];
    }
    double offset = (mn + mx) / 2.0;
    double scale = 2.0 * sigma[0] * sigma[0];
    int64_t W = size[0], H = size[1];
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 16)
    for (int64_t g = 0; g < W * H; g++) {
        int64_t i = g % W, j = g / W;
        double xc = x0[0] + (double)i * step[0], yc = x0[1] + (double)j * step[1];
        double lat0 = yc * RAD_PER_DEGREE;
        double ws = 0.0, wt = 0.0;
        for (int64_t k = 0; k < npts; k++) {
            double lat1 = pts[2 * k + 1] * RAD_PER_DEGREE;
            double arg = sin(lat0) * sin(lat1) + cos(lat0) * cos(lat1) * cos((pts[2 * k] - xc) * RAD_PER_DEGREE);
            if (arg > 1.0)
                arg = 1.0;
            double dist = acos(arg) / RAD_PER_DEGREE;
            double w = exp(-dist * dist / scale);
            ws += w * (val[k] - offset);
            wt += w;
        }
        out[g] = wt > 0.0 ? ws / wt + offset : NAN;
    }
}

/* ------------------------------------------------------------------------- */
/* sphere: Lambert conformal projection + resampling                          */
/* ------------------------------------------------------------------------- */

/* fastbarnes/util/lambert_conformal.py:50-94 (create_proj).
 * proj = {center_lon, n, n_inv, F, rho0}. */
FBO_EXPORT void fbo_lambert_create_proj(double center_lon, double center_lat, double lat1,
                                        double lat2, double *proj)
{
    const double HRAD = RAD_PER_DEGREE / 2.0;
    double n;
    if (lat1 != lat2)
        n = log(cos(lat1 * RAD_PER_DEGREE) / cos(lat2 * RAD_PER_DEGREE)) /
            log(tan((90.0 + lat2) * HRAD) / tan((90.0 + lat1) * HRAD));
    else
        n = sin(lat1 * RAD_PER_DEGREE);
    double F = cos(lat1 * RAD_PER_DEGREE) * pow(tan((90.0 + lat1) * HRAD), n) / n;
    double rho0 = F / pow(tan((90.0 + center_lat) * HRAD), n);
    proj[0] = center_lon;
    proj[1] = n;
    proj[2] = 1.0 / n;
    proj[3] = F;
    proj[4] = rho0;
}

/* fastbarnes/util/lambert_conformal.py:113-123 (to_map), geo (lon, lat) ->
 * map (x, y), both N x 2. */
FBO_EXPORT void fbo_lambert_to_map(const double *geo, double *map, int64_t npts, const double *proj)
{
    const double HRAD = RAD_PER_DEGREE / 2.0;
    for (int64_t k = 0; k < npts; k++) {
        double lon = geo[2 * k], lat = geo[2 * k + 1];
        double rho = proj[3] / pow(tan((90.0 + lat) * HRAD), proj[1]);
        double arg = proj[1] * (lon - proj[0]) * RAD_PER_DEGREE;
        map[2 * k] = rho * sin(arg) / RAD_PER_DEGREE;
        map[2 * k + 1] = (proj[4] - rho * cos(arg)) / RAD_PER_DEGREE;
    }
}

/* fastbarnes/interpolationS2.py:211-254 (_resample) with to_map2
 * (lambert_conformal.py:127-136): bilinear read of the float32 Lambert field
 * (lam_h x lam_w) at the projection of every lon/lat grid point.  Points whose
 * cell falls outside the Lambert grid (the reference has no bounds check) are
 * written as NaN. */
FBO_EXPORT void fbo_resample(const float *lam, int64_t lam_w, int64_t lam_h, const double *lam_x0,
                             const double *x0, const double *step, const int64_t *size,
                             const double *proj, float *out)
{
    const double HRAD = RAD_PER_DEGREE / 2.0;
    int64_t W = size[0], H = size[1];
    for (int64_t j = 0; j < H; j++) {
        double geoy = (double)j * step[1] + x0[1];
        double rho = proj[3] / pow(tan((90.0 + geoy) * HRAD), proj[1]);
        for (int64_t i = 0; i < W; i++) {
            double geox = x0[0] + (double)i * step[0];
            double arg = proj[1] * (geox - proj[0]) * RAD_PER_DEGREE;
            double mapx = rho * sin(arg) / RAD_PER_DEGREE;
            double mapy = (proj[4] - rho * cos(arg)) / RAD_PER_DEGREE;
            mapx -= lam_x0[0];
            mapx /= step[0];
            mapy -= lam_x0[1];
            mapy /= step[1];
            int32_t ix = (int32_t)mapx, iy = (int32_t)mapy;
            mapx -= (double)ix;
            mapy -= (double)iy;
            if (ix < 0 || iy < 0 || ix + 1 >= lam_w || iy + 1 >= lam_h) {
                out[j * W + i] = NAN;
                continue;
            }
            const float *r0 = lam + (int64_t)iy * lam_w + ix;
            const float *r1 = r0 + lam_w;
            double v = (1.0 - mapy) * (1.0 - mapx) * (double)r0[0] + mapy * (1.0 - mapx) * (double)r1[0] +
                       mapy * mapx * (double)r1[1] + (1.0 - mapy) * mapx * (double)r0[1];
            out[j * W + i] = (float)v;
        }
    }
}

/* fastbarnes/interpolationS2.py:143-202: part 1 projects the samples onto the
 * fixed Lambert grid (x0 = (-32, -2), size = (int(64/step_x), int(44/step_y)))
 * and runs the optimized convolution there; part 2 resamples to lon/lat.
 * lam_out must hold int(44/step_y) * int(64/step_x) floats; out (if resample)
 * size[1] * size[0]. */
FBO_EXPORT void fbo_interpolate_s2(const double *pts, const double *val, int64_t npts,
                                   const double *sigma, const double *x0, const double *step,
                                   const int64_t *size, int num_iter, double max_dist_weight,
                                   int nthreads, float *lam_out, float *out)
{
    double proj[5];
    fbo_lambert_create_proj(11.5, 34.5, 42.5, 65.5, proj);
    double lam_x0[2] = {-32.0, -2.0};
    int64_t lam_size[2] = {(int64_t)(64.0 / step[0]), (int64_t)(44.0 / step[1])};
    double *lam_pts = (double *)malloc(sizeof(double) * 2 * (npts > 0 ? npts : 1));
    fbo_lambert_to_map(pts, lam_pts, npts, proj);
    fbo_interpolate(0, 2, lam_pts, val, npts, sigma, lam_x0, step, lam_size, num_iter,
                    max_dist_weight, nthreads, lam_out, NULL, NULL);
    if (out)
        fbo_resample(lam_out, lam_size[0], lam_size[1], lam_x0, x0, step, size, proj, out);
    free(lam_pts);
}
