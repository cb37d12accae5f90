// fb_grad.cu -- the adjoint of the interpolation (no reference counterpart:
// the reference has no gradients).  With f = V / W + offset on the unmasked
// grid points (V = C S (val - offset), W = C S 1, S the bilinear splat, C the
// n box passes of every axis), a loss gradient g = dL/df gives
//   dL/dV = g / W,  dL/dW = -g V / W^2       (seed, per grid point)
//   A = C^T (dL/dV, dL/dW) = C (dL/dV, dL/dW) (C is symmetric with the
//                                              line's zero padding)
//   dL/dval_k = sum_c w_kc A_V[c]            (gather at the sample's corners)
//   dL/dx_k   = sum_c dw_kc/dx_k (val'_k A_V[c] + A_W[c]),  val' = val - offset
// The offset cancels in f, so it is a constant here.  Masked grid points
// (W below the mask level) carry no gradient.
#include "fb_axis_impl.cuh"

namespace fbg {

template <typename Real>
__global__ void k_grad_seed(typename CellOf<Real>::T *__restrict__ cells, int64_t npoints,
                            const void *__restrict__ grad, int grad_f64, double thr)
{
    using C = typename CellOf<Real>::T;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < npoints;
         i += (int64_t)gridDim.x * blockDim.x) {
        const C c = cells[i];
        const double g = grad_f64 ? reinterpret_cast<const double *>(grad)[i]
                                  : (double)reinterpret_cast<const float *>(grad)[i];
        const double v = (double)c.x, w = (double)c.y;
        C s;
        if (!(c.y >= (Real)thr) || isnan(g)) {   // the forward mask, in the form's precision
            s.x = (Real)0;
            s.y = (Real)0;
        } else {
            s.x = (Real)(g / w);
            s.y = (Real)(-g * v / (w * w));
        }
        cells[i] = s;
    }
}

template <int DIM, typename Real>
__global__ void k_grad_gather(const SampleRec<Real> *__restrict__ rec, const uint32_t *__restrict__ keys,
                              uint32_t skip_key, int64_t npts, const typename CellOf<Real>::T *__restrict__ A,
                              Geometry g, const FieldHeader *__restrict__ hdr, double *__restrict__ grad_val,
                              double *__restrict__ grad_pts)
{
    const double offset = field_offset(hdr);
    const int64_t W = g.size[0], H = g.size[1];
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < npts;
         k += (int64_t)gridDim.x * blockDim.x) {
        double gv = 0.0, gp[3] = {0.0, 0.0, 0.0};
        if (keys[k] < skip_key) {
            const SampleRec<Real> r = rec[k];
            const double vp = r.val - offset;
            const double xw = (double)r.xw, yw = (double)r.yw, zw = (double)r.zw;
            for (int cz = 0; cz < (DIM == 3 ? 2 : 1); cz++) {
                const double wz = DIM == 3 ? (cz ? zw : 1.0 - zw) : 1.0, dz = cz ? 1.0 : -1.0;
                for (int cy = 0; cy < (DIM >= 2 ? 2 : 1); cy++) {
                    const double wy = DIM >= 2 ? (cy ? yw : 1.0 - yw) : 1.0, dy = cy ? 1.0 : -1.0;
                    for (int cx = 0; cx < 2; cx++) {
                        const double wx = cx ? xw : 1.0 - xw, dx = cx ? 1.0 : -1.0;
                        const int64_t idx = (((int64_t)r.zi + cz) * H + ((int64_t)r.yi + cy)) * W + r.xi + cx;
                        const double av = (double)A[idx].x, aw = (double)A[idx].y;
                        double w = wx;
                        if (DIM >= 2)
                            w = w * wy;
                        if (DIM == 3)
                            w = w * wz;
                        gv += w * av;
                        const double t = vp * av + aw;
                        gp[0] += dx * (DIM >= 2 ? wy : 1.0) * (DIM == 3 ? wz : 1.0) * t;
                        if (DIM >= 2)
                            gp[1] += wx * dy * (DIM == 3 ? wz : 1.0) * t;
                        if (DIM == 3)
                            gp[2] += wx * wy * dz * t;
                    }
                }
            }
        }
        grad_val[k] = gv;
        if (grad_pts)
            for (int m = 0; m < DIM; m++)
                grad_pts[k * DIM + m] = gp[m] / g.step[m];
    }
}

cudaError_t launch_grad_seed(int precision, void *cells, int64_t npoints, const void *grad, int grad_f64, double thr,
                             cudaStream_t st)
{
    const int blocks = (int)std::min<int64_t>((npoints + 255) / 256, 152 * 16);
    if (precision == 0)
        k_grad_seed<double><<<blocks, 256, 0, st>>>(reinterpret_cast<double2 *>(cells), npoints, grad, grad_f64, thr);
    else
        k_grad_seed<float><<<blocks, 256, 0, st>>>(reinterpret_cast<float2 *>(cells), npoints, grad, grad_f64, thr);
    return cudaGetLastError();
}

cudaError_t launch_grad_gather(int precision, int dim, const void *rec, const uint32_t *keys, uint32_t skip_key,
                               int64_t npts, const void *A, const Geometry &g, const FieldHeader *hdr,
                               double *grad_val, double *grad_pts, cudaStream_t st)
{
    if (npts < 1)
        return cudaSuccess;
    const int blocks = (int)std::min<int64_t>((npts + 255) / 256, 152 * 16);
#define FBG_G(D, R)                                                                                               \
    k_grad_gather<D, R><<<blocks, 256, 0, st>>>(reinterpret_cast<const SampleRec<R> *>(rec), keys, skip_key, npts, \
                                                reinterpret_cast<const typename CellOf<R>::T *>(A), g, hdr,        \
                                                grad_val, grad_pts)
    if (precision == 0) {
        if (dim == 1)
            FBG_G(1, double);
        else if (dim == 2)
            FBG_G(2, double);
        else
            FBG_G(3, double);
    } else {
        if (dim == 1)
            FBG_G(1, float);
        else if (dim == 2)
            FBG_G(2, float);
        else
            FBG_G(3, float);
    }
#undef FBG_G
    return cudaGetLastError();
}

}  // namespace fbg
