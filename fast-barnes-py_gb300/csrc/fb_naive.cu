// fb_naive.cu -- the naive O(N x grid) Barnes interpolation on the GPU.
//
// Replaces _interpolate_naive (fastbarnes/interpolation.py:861-938) and
// _interpolate_naive_S2 (fastbarnes/interpolationS2.py:259-283): every grid
// point sums exp(-d^2 / (2 sigma^2)) weights over all samples (Euclidean d in
// 1/2/3D, the great-circle distance in degrees on the sphere), value =
// sum(w (val - offset)) / sum(w) + offset, NaN where the weights sum to zero.
// The samples stream through shared memory in tiles; every thread owns one
// grid point.  The float64 form accumulates in float64; the float32 form
// computes weights in float32 and keeps Kahan-compensated float32 sums.
//
// Also replaces _interpolate_radius (fastbarnes/interpolation.py:809-855)
// and its kd-tree radius search (fastbarnes/util/kdtree.py:257-331): the same
// sums over the samples within sqrt(-2 ln(min_weight)) sigma of the grid point
// only, NaN where the weights sum below max_dist_weight.  Instead of a tree,
// the samples stream through in tiles with precomputed bounding boxes, and a
// block of grid points skips every tile whose box is out of reach.
#include <math.h>

#include <algorithm>

#include "fb_internal.cuh"
#include "fb_kernels.cuh"

namespace fbg {

namespace {

constexpr int kNaiveThreads = 256;
constexpr int kNaiveTile = 256;
constexpr double kRadPerDeg = 3.14159265358979311600 / 180.0;

struct NaiveParams {
    int dim;
    int sphere;
    int64_t size[3];
    double x0[3], step[3];
    double inv_scale[3];   // 1 / (2 sigma^2)
};

// Kahan-compensated running sum (float32) / plain sum (float64).
template <typename Real>
struct Acc {
    Real s = 0, c = 0;
    __device__ __forceinline__ void add(Real x)
    {
        if (sizeof(Real) == 8) {
            s += x;
        } else {
            const Real y = x - c;
            const Real t = s + y;
            c = (t - s) - y;
            s = t;
        }
    }
};

}  // namespace

__global__ void k_value_range(const double *__restrict__ val, int64_t n, FieldHeader *__restrict__ hdr)
{
    __shared__ unsigned long long s_min[32], s_max[32];
    __shared__ int s_nan[32];
    unsigned long long kmin = ~0ull, kmax = 0ull;
    int nan = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double v = val[k];
        if (isnan(v)) {
            nan = 1;
        } else {
            const unsigned long long o = dbl_to_ordered(v);
            kmin = o < kmin ? o : kmin;
            kmax = o > kmax ? o : kmax;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned long long a = __shfl_xor_sync(0xffffffffu, kmin, o);
        const unsigned long long b = __shfl_xor_sync(0xffffffffu, kmax, o);
        kmin = a < kmin ? a : kmin;
        kmax = b > kmax ? b : kmax;
    }
    nan = __any_sync(0xffffffffu, nan);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
        s_min[w] = kmin;
        s_max[w] = kmax;
        s_nan[w] = nan;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int q = 1; q < (int)(blockDim.x >> 5); q++) {
            kmin = s_min[q] < kmin ? s_min[q] : kmin;
            kmax = s_max[q] > kmax ? s_max[q] : kmax;
            nan |= s_nan[q];
        }
        if (kmin != ~0ull)
            atomicMax(&hdr->vmin_key, ~kmin);
        if (kmax != 0ull)
            atomicMax(&hdr->vmax_key, kmax);
        if (nan)
            atomicExch(&hdr->nan_seen, 1);
    }
}

template <int DIM, bool SPHERE, typename Real>
__global__ void __launch_bounds__(kNaiveThreads) k_naive(const double *__restrict__ pts, const double *__restrict__ val,
                                                         int64_t n, NaiveParams p, const FieldHeader *__restrict__ hdr,
                                                         void *__restrict__ out, int out_f64)
{
    // per sample: coordinates (or lon, sin lat, cos lat on the sphere) and the
    // centred value
    __shared__ Real s_c[kNaiveTile][3];
    __shared__ Real s_v[kNaiveTile];
    const double offset = field_offset(hdr);
    const int64_t npoints = p.size[0] * (DIM > 1 ? p.size[1] : 1) * (DIM > 2 ? p.size[2] : 1);
    const int64_t gidx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const bool live = gidx < npoints;
    const int64_t i = live ? gidx % p.size[0] : 0;
    const int64_t j = DIM > 1 && live ? (gidx / p.size[0]) % p.size[1] : 0;
    const int64_t kz = DIM > 2 && live ? gidx / (p.size[0] * p.size[1]) : 0;
    double c[3] = {p.x0[0] + (double)i * p.step[0], DIM > 1 ? p.x0[1] + (double)j * p.step[1] : 0.0,
                   DIM > 2 ? p.x0[2] + (double)kz * p.step[2] : 0.0};
    Real gc[3];
    if (SPHERE) {
        // grid point: lon (radians), sin lat, cos lat
        const double lat = c[1] * kRadPerDeg;
        gc[0] = (Real)(c[0] * kRadPerDeg);
        gc[1] = (Real)sin(lat);
        gc[2] = (Real)cos(lat);
    } else {
        for (int m = 0; m < 3; m++)
            gc[m] = (Real)c[m];
    }
    const Real inv0 = (Real)p.inv_scale[0], inv1 = (Real)p.inv_scale[1], inv2 = (Real)p.inv_scale[2];
    Acc<Real> ws, wt;
    for (int64_t t0 = 0; t0 < n; t0 += kNaiveTile) {
        const int cnt = (int)min((int64_t)kNaiveTile, n - t0);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int64_t k = t0 + q;
            if (SPHERE) {
                const double lat = pts[2 * k + 1] * kRadPerDeg;
                s_c[q][0] = (Real)(pts[2 * k] * kRadPerDeg);
                s_c[q][1] = (Real)sin(lat);
                s_c[q][2] = (Real)cos(lat);
            } else {
                for (int m = 0; m < DIM; m++)
                    s_c[q][m] = (Real)pts[k * DIM + m];
            }
            s_v[q] = (Real)(val[k] - offset);
        }
        __syncthreads();
        if (live) {
            for (int q = 0; q < cnt; q++) {
                Real d2;
                if (SPHERE) {
                    Real arg = gc[1] * s_c[q][1] + gc[2] * s_c[q][2] * cos(s_c[q][0] - gc[0]);
                    arg = arg > (Real)1 ? (Real)1 : arg;
                    const Real dist = acos(arg) / (Real)kRadPerDeg;
                    d2 = dist * dist * inv0;
                } else {
                    const Real dx = s_c[q][0] - gc[0];
                    d2 = dx * dx * inv0;
                    if (DIM > 1) {
                        const Real dy = s_c[q][1] - gc[1];
                        d2 += dy * dy * inv1;
                    }
                    if (DIM > 2) {
                        const Real dz = s_c[q][2] - gc[2];
                        d2 += dz * dz * inv2;
                    }
                }
                const Real w = exp(-d2);
                ws.add(w * s_v[q]);
                wt.add(w);
            }
        }
    }
    if (live) {
        const double r = wt.s > (Real)0 ? (double)ws.s / (double)wt.s + offset : (double)NAN;
        if (out_f64)
            reinterpret_cast<double *>(out)[gidx] = r;
        else
            reinterpret_cast<float *>(out)[gidx] = (float)r;
    }
}

cudaError_t launch_naive(int precision, int dim, int sphere, const double *pts, const double *val, int64_t n,
                         const double *sigma, const double *x0, const double *step, const int64_t *size,
                         FieldHeader *hdr, void *out, int out_f64, cudaStream_t st)
{
    NaiveParams p{};
    p.dim = dim;
    p.sphere = sphere;
    int64_t npoints = 1;
    for (int m = 0; m < 3; m++) {
        p.size[m] = m < dim ? size[m] : 1;
        p.x0[m] = m < dim ? x0[m] : 0.0;
        p.step[m] = m < dim ? step[m] : 1.0;
        p.inv_scale[m] = m < dim ? 1.0 / (2.0 * sigma[m] * sigma[m]) : 0.0;
        npoints *= p.size[m];
    }
    cudaError_t e = cudaMemsetAsync(hdr, 0, sizeof(FieldHeader), st);
    if (e != cudaSuccess)
        return e;
    if (n > 0)
        k_value_range<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 4), 256, 0, st>>>(val, n, hdr);
    const unsigned blocks = (unsigned)((npoints + kNaiveThreads - 1) / kNaiveThreads);
#define FBG_N(D, S, R) k_naive<D, S, R><<<blocks, kNaiveThreads, 0, st>>>(pts, val, n, p, hdr, out, out_f64)
    if (sphere) {
        if (precision == 0)
            FBG_N(2, true, double);
        else
            FBG_N(2, true, float);
    } else if (precision == 0) {
        if (dim == 1)
            FBG_N(1, false, double);
        else if (dim == 2)
            FBG_N(2, false, double);
        else
            FBG_N(3, false, double);
    } else {
        if (dim == 1)
            FBG_N(1, false, float);
        else if (dim == 2)
            FBG_N(2, false, float);
        else
            FBG_N(3, false, float);
    }
#undef FBG_N
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------
// method 'radius': the naive sums restricted to a search radius
// ---------------------------------------------------------------------------

namespace {

constexpr int kRadiusSide = 16;   // a CTA covers 16 x 16 grid points

struct RadiusParams {
    int64_t size[2];
    double x0[2], step[2];
    double r2;                // (sqrt(-2 ln(min_weight)) sigma)^2
    double scale;             // 2 sigma^2
    double max_dist_weight;
};

}  // namespace

// Bounding box {xmin, xmax, ymin, ymax} of every tile of kNaiveTile samples.
__global__ void __launch_bounds__(kNaiveTile) k_tile_boxes(const double *__restrict__ pts, int64_t n,
                                                           double4 *__restrict__ boxes)
{
    __shared__ double s_b[4][kNaiveTile / 32];
    const int64_t k = (int64_t)blockIdx.x * kNaiveTile + threadIdx.x;
    double b[4];
    if (k < n) {
        b[0] = b[1] = pts[2 * k];
        b[2] = b[3] = pts[2 * k + 1];
    } else {
        b[0] = b[2] = INFINITY;
        b[1] = b[3] = -INFINITY;
    }
    for (int o = 16; o > 0; o >>= 1)
        for (int m = 0; m < 4; m++) {
            const double v = __shfl_xor_sync(0xffffffffu, b[m], o);
            b[m] = (m & 1) ? fmax(b[m], v) : fmin(b[m], v);
        }
    if ((threadIdx.x & 31) == 0)
        for (int m = 0; m < 4; m++)
            s_b[m][threadIdx.x >> 5] = b[m];
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < kNaiveTile / 32; w++)
            for (int m = 0; m < 4; m++)
                b[m] = (m & 1) ? fmax(b[m], s_b[m][w]) : fmin(b[m], s_b[m][w]);
        boxes[blockIdx.x] = make_double4(b[0], b[1], b[2], b[3]);
    }
}

// One thread per grid point of a 16 x 16 block.  Sample tiles whose bounding
// box lies farther than the radius from the block's points are skipped by the
// whole CTA.  Float64: the reference's arithmetic (squared distance without
// fused products, compared with the squared radius, weight exp(-d^2 / scale)).
// Float32: coordinates relative to the block's corner (exact in float64,
// then rounded), Kahan-compensated sums; a squared distance within 1e-4 of
// the radius is decided again in float64 from the original coordinates.
template <typename Real>
__global__ void __launch_bounds__(kRadiusSide *kRadiusSide)
    k_radius(const double *__restrict__ pts, const double *__restrict__ val, int64_t n, RadiusParams p,
             const double4 *__restrict__ boxes, const FieldHeader *__restrict__ hdr, void *__restrict__ out,
             int out_f64)
{
    __shared__ Real s_x[kNaiveTile], s_y[kNaiveTile], s_v[kNaiveTile];
    const double offset = field_offset(hdr);
    const int64_t i0 = (int64_t)blockIdx.x * kRadiusSide, j0 = (int64_t)blockIdx.y * kRadiusSide;
    const int64_t i = i0 + (threadIdx.x % kRadiusSide), j = j0 + (threadIdx.x / kRadiusSide);
    const bool live = i < p.size[0] && j < p.size[1];
    const double ox = p.x0[0] + (double)i0 * p.step[0], oy = p.x0[1] + (double)j0 * p.step[1];
    const double ex = p.x0[0] + (double)(i0 + kRadiusSide - 1) * p.step[0];
    const double ey = p.x0[1] + (double)(j0 + kRadiusSide - 1) * p.step[1];
    // the reference's grid point c = x0 + index * step
    const double cx = p.x0[0] + (double)i * p.step[0], cy = p.x0[1] + (double)j * p.step[1];
    constexpr bool F64 = sizeof(Real) == 8;
    const Real gx = F64 ? (Real)cx : (Real)(cx - ox), gy = F64 ? (Real)cy : (Real)(cy - oy);
    const float r2f = (float)p.r2, band = 1e-4f * r2f;
    const float inv_scale_f = (float)(1.0 / p.scale);
    Acc<Real> ws, wt;
    const int64_t ntiles = (n + kNaiveTile - 1) / kNaiveTile;
    for (int64_t t = 0; t < ntiles; t++) {
        const double4 b = boxes[t];
        const double gapx = fmax(0.0, fmax(b.x - ex, ox - b.y));
        const double gapy = fmax(0.0, fmax(b.z - ey, oy - b.w));
        if (gapx * gapx + gapy * gapy > p.r2 * (1.0 + 1e-9))
            continue;   // the same decision in every thread of the CTA
        const int64_t t0 = t * kNaiveTile;
        const int cnt = (int)min((int64_t)kNaiveTile, n - t0);
        __syncthreads();
        for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int64_t k = t0 + q;
            s_x[q] = F64 ? (Real)pts[2 * k] : (Real)(pts[2 * k] - ox);
            s_y[q] = F64 ? (Real)pts[2 * k + 1] : (Real)(pts[2 * k + 1] - oy);
            s_v[q] = (Real)(val[k] - offset);
        }
        __syncthreads();
        if (!live)
            continue;
        for (int q = 0; q < cnt; q++) {
            if (F64) {
                const double dx = (double)gx - (double)s_x[q], dy = (double)gy - (double)s_y[q];
                const double d2 = __dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy));
                if (d2 <= p.r2) {
                    const double w = exp(-d2 / p.scale);
                    ws.add((Real)__dmul_rn(w, (double)s_v[q]));
                    wt.add((Real)w);
                }
            } else {
                const float dx = (float)gx - (float)s_x[q], dy = (float)gy - (float)s_y[q];
                const float d2 = dx * dx + dy * dy;
                bool in = d2 <= r2f;
                if (fabsf(d2 - r2f) <= band) {
                    const int64_t k = t0 + q;
                    const double ddx = cx - pts[2 * k], ddy = cy - pts[2 * k + 1];
                    in = __dadd_rn(__dmul_rn(ddx, ddx), __dmul_rn(ddy, ddy)) <= p.r2;
                }
                if (in) {
                    const float w = expf(-d2 * inv_scale_f);
                    ws.add((Real)(w * (float)s_v[q]));
                    wt.add((Real)w);
                }
            }
        }
    }
    if (live) {
        const double r = (double)wt.s >= p.max_dist_weight ? (double)ws.s / (double)wt.s + offset : (double)NAN;
        const int64_t gidx = j * p.size[0] + i;
        if (out_f64)
            reinterpret_cast<double *>(out)[gidx] = r;
        else
            reinterpret_cast<float *>(out)[gidx] = (float)r;
    }
}

size_t radius_workspace_bytes(int64_t n)
{
    const int64_t ntiles = (n + kNaiveTile - 1) / kNaiveTile;
    return 256 + (size_t)ntiles * sizeof(double4);
}

cudaError_t launch_radius(int precision, const double *pts, const double *val, int64_t n, double sigma,
                          const double *x0, const double *step, const int64_t *size, double max_dist_weight,
                          double min_weight, void *ws, void *out, int out_f64, cudaStream_t st)
{
    RadiusParams p{};
    for (int m = 0; m < 2; m++) {
        p.size[m] = size[m];
        p.x0[m] = x0[m];
        p.step[m] = step[m];
    }
    // interpolation.py:825 and util/kdtree.py:249
    const double radius = sqrt(-2.0 * log(min_weight)) * sigma;
    p.r2 = radius * radius;
    p.scale = 2.0 * sigma * sigma;
    p.max_dist_weight = max_dist_weight;
    FieldHeader *hdr = reinterpret_cast<FieldHeader *>(ws);
    double4 *boxes = reinterpret_cast<double4 *>(reinterpret_cast<char *>(ws) + 256);
    cudaError_t e = cudaMemsetAsync(hdr, 0, sizeof(FieldHeader), st);
    if (e != cudaSuccess)
        return e;
    const int64_t ntiles = (n + kNaiveTile - 1) / kNaiveTile;
    if (n > 0) {
        k_value_range<<<(unsigned)std::min<int64_t>((n + 255) / 256, 152 * 4), 256, 0, st>>>(val, n, hdr);
        k_tile_boxes<<<(unsigned)ntiles, kNaiveTile, 0, st>>>(pts, n, boxes);
    }
    const dim3 grid((unsigned)((size[0] + kRadiusSide - 1) / kRadiusSide),
                    (unsigned)((size[1] + kRadiusSide - 1) / kRadiusSide));
    if (precision == 0)
        k_radius<double><<<grid, kRadiusSide * kRadiusSide, 0, st>>>(pts, val, n, p, boxes, hdr, out, out_f64);
    else
        k_radius<float><<<grid, kRadiusSide * kRadiusSide, 0, st>>>(pts, val, n, p, boxes, hdr, out, out_f64);
    return cudaGetLastError();
}

}  // namespace fbg
