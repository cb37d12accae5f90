// fb_s2.cu -- the sphere path: Lambert conformal projection of the samples and
// bilinear resampling of the Lambert field onto the lon/lat grid.
//
// Replaces fastbarnes/util/lambert_conformal.py:113-136 (to_map, to_map2) and
// fastbarnes/interpolationS2.py:211-254 (_resample).  This translation unit
// is compiled with -fmad=false so every product and sum rounds separately, as
// in the reference's float64 expressions; the transcendental functions are
// CUDA's (within a few ulp of libm's).
#include <algorithm>

#include "fb_internal.cuh"
#include "fb_kernels.cuh"

namespace fbg {

__constant__ double c_rad_per_degree = 3.14159265358979311600 / 180.0;

struct Proj {
    double center_lon, n, n_inv, F, rho0;
};

__global__ void k_to_map(const double *__restrict__ geo, double *__restrict__ map, int64_t n, Proj pj)
{
    const double RAD = c_rad_per_degree;
    const double HRAD = RAD / 2.0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n; k += (int64_t)gridDim.x * blockDim.x) {
        const double lon = geo[2 * k], lat = geo[2 * k + 1];
        const double rho = pj.F / pow(tan((90.0 + lat) * HRAD), pj.n);
        const double arg = pj.n * (lon - pj.center_lon) * RAD;
        map[2 * k] = rho * sin(arg) / RAD;
        map[2 * k + 1] = (pj.rho0 - rho * cos(arg)) / RAD;
    }
}

// Per output row j the projection radius depends on the latitude only, per
// column i the angle on the longitude only: both are tabulated first.
__global__ void k_resample_rows(double *__restrict__ rho, int64_t H, double y0, double sy, Proj pj)
{
    const double HRAD = c_rad_per_degree / 2.0;
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < H; j += (int64_t)gridDim.x * blockDim.x) {
        const double geoy = (double)j * sy + y0;
        rho[j] = pj.F / pow(tan((90.0 + geoy) * HRAD), pj.n);
    }
}

__global__ void k_resample_cols(double *__restrict__ sn, double *__restrict__ cs, int64_t W, double x0, double sx,
                                Proj pj)
{
    const double RAD = c_rad_per_degree;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < W; i += (int64_t)gridDim.x * blockDim.x) {
        const double geox = x0 + (double)i * sx;
        const double arg = pj.n * (geox - pj.center_lon) * RAD;
        sn[i] = sin(arg);
        cs[i] = cos(arg);
    }
}

__global__ void k_resample(const float *__restrict__ lam, int64_t lam_w, int64_t lam_h, double lx0, double ly0,
                           double sx, double sy, const double *__restrict__ rho, const double *__restrict__ sn,
                           const double *__restrict__ cs, int64_t W, int64_t H, double rho0,
                           float *__restrict__ out)
{
    const double RAD = c_rad_per_degree;
    const int64_t total = W * H;
    for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < total;
         g += (int64_t)gridDim.x * blockDim.x) {
        const int64_t j = g / W, i = g - j * W;
        const double r = rho[j];
        double mapx = r * sn[i] / RAD;
        double mapy = (rho0 - r * cs[i]) / RAD;
        mapx -= lx0;
        mapx /= sx;
        mapy -= ly0;
        mapy /= sy;
        const int ix = (int)mapx, iy = (int)mapy;
        mapx -= (double)ix;
        mapy -= (double)iy;
        float res;
        if (ix < 0 || iy < 0 || ix + 1 >= lam_w || iy + 1 >= lam_h) {
            res = __int_as_float(0x7fc00000);   // outside the Lambert grid
        } else {
            const float *r0 = lam + (int64_t)iy * lam_w + ix;
            const float *r1 = r0 + lam_w;
            const double v = (1.0 - mapy) * (1.0 - mapx) * (double)r0[0] + mapy * (1.0 - mapx) * (double)r1[0] +
                             mapy * mapx * (double)r1[1] + (1.0 - mapy) * mapx * (double)r0[1];
            res = (float)v;
        }
        out[g] = res;
    }
}

static Proj to_proj(const double *p) { return Proj{p[0], p[1], p[2], p[3], p[4]}; }

cudaError_t launch_lambert_to_map(const double *geo, double *map, int64_t n, const double *proj, cudaStream_t st)
{
    if (n <= 0)
        return cudaSuccess;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 16);
    k_to_map<<<blocks, 256, 0, st>>>(geo, map, n, to_proj(proj));
    return cudaGetLastError();
}

cudaError_t launch_resample(const float *lam, int64_t lam_w, int64_t lam_h, const double *lam_x0, const double *x0,
                            const double *step, const int64_t *size, const double *proj, float *out, double *tab,
                            cudaStream_t st)
{
    // tab: H row radii, then W sines and W cosines (workspace)
    const int64_t W = size[0], H = size[1];
    Proj pj = to_proj(proj);
    k_resample_rows<<<(int)((H + 255) / 256), 256, 0, st>>>(tab, H, x0[1], step[1], pj);
    k_resample_cols<<<(int)((W + 255) / 256), 256, 0, st>>>(tab + H, tab + H + W, W, x0[0], step[0], pj);
    const int64_t total = W * H;
    int blocks = (int)std::min<int64_t>((total + 255) / 256, 152 * 32);
    k_resample<<<blocks, 256, 0, st>>>(lam, lam_w, lam_h, lam_x0[0], lam_x0[1], step[0], step[1], tab, tab + H,
                                      tab + H + W, W, H, pj.rho0, out);
    return cudaGetLastError();
}

}  // namespace fbg
