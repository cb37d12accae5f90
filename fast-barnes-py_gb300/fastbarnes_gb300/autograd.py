"""Differentiable Barnes interpolation (GB300 extension; the reference has no
derivatives).

``barnes(pts, val, ...)`` takes CUDA float64 tensors and returns the
interpolated field as a tensor that torch.autograd can differentiate with
respect to ``val`` and ``pts``.  The backward pass is the hand-written adjoint
in libfastbarnes_gb300 (``fb_interpolate_grad``): the seed (dL/dV, dL/dW) =
(g / W, -g V / W^2) on the unmasked grid points, the same symmetric box passes
again, and a gather with the bilinear weights and their position derivatives.
NaN-masked grid points carry no gradient; the value offset cancels in the
result and is treated as a constant.
"""
import ctypes
from math import exp

import numpy as np

from . import _lib
from .interpolation import _check_args, _get_half_kernel_size, _get_half_kernel_size_opt, _kernel_guard, \
    _precision_code

__all__ = ["barnes", "BarnesFunction"]

_METHODS = {"optimized_convolution": _lib.FB_OPTIMIZED_CONVOLUTION, "convolution": _lib.FB_CONVOLUTION}


class _Params:
    def __init__(self, method, prec, dim, sigma, x0, step, size, num_iter, max_dist_weight, out_f64):
        self.method, self.prec, self.dim = method, prec, dim
        self.c_sigma = _lib.dvec([float(s) for s in sigma])
        self.c_x0 = _lib.dvec([float(s) for s in x0])
        self.c_step = _lib.dvec([float(s) for s in step])
        self.c_size = _lib.dvec([int(s) for s in size], ctypes.c_int64)
        self.size = tuple(int(s) for s in size)
        self.num_iter = int(num_iter)
        self.mdw = float(max_dist_weight)
        self.out_f64 = out_f64


def _torch():
    return _lib.torch_cuda()


class BarnesFunction:
    """torch.autograd.Function wrapper (built lazily so that importing this
    module does not need torch)."""
    _fn = None

    @classmethod
    def get(cls):
        if cls._fn is not None:
            return cls._fn
        torch = _torch()

        class _F(torch.autograd.Function):
            @staticmethod
            def forward(ctx, pts, val, prm):
                L = _lib.lib()
                dev = val.device
                n = int(val.shape[0])
                out = torch.empty(prm.size[::-1], dtype=torch.float64 if prm.out_f64 else torch.float32, device=dev)
                need = ctypes.c_size_t(0)
                with torch.cuda.device(dev):
                    _lib.check(L.fb_workspace_size(prm.method, prm.prec, prm.dim, n, prm.c_sigma, prm.c_step,
                                                   prm.c_size, prm.num_iter, ctypes.byref(need)), "fb_workspace_size")
                    ws = _lib.workspace(need.value, dev)
                    _lib.check(L.fb_interpolate(prm.method, prm.prec, prm.dim, pts.data_ptr(), val.data_ptr(), n,
                                                prm.c_sigma, prm.c_x0, prm.c_step, prm.c_size, prm.num_iter, prm.mdw,
                                                out.data_ptr(), int(prm.out_f64), ws.data_ptr(), ws.numel(),
                                                _lib.stream_ptr(torch, dev)), "fb_interpolate")
                ctx.save_for_backward(pts, val)
                ctx.prm = prm
                return out

            @staticmethod
            def backward(ctx, grad_out):
                pts, val = ctx.saved_tensors
                prm = ctx.prm
                L = _lib.lib()
                dev = val.device
                n = int(val.shape[0])
                g = grad_out.contiguous()
                g_f64 = 1 if g.dtype == torch.float64 else 0
                if not g_f64:
                    g = g.to(torch.float32)
                grad_val = torch.empty(n, dtype=torch.float64, device=dev)
                want_pts = ctx.needs_input_grad[0]
                grad_pts = torch.empty((n, prm.dim), dtype=torch.float64, device=dev) if want_pts else None
                need = ctypes.c_size_t(0)
                with torch.cuda.device(dev):
                    _lib.check(L.fb_grad_workspace_size(prm.method, prm.prec, prm.dim, n, prm.c_sigma, prm.c_step,
                                                        prm.c_size, prm.num_iter, ctypes.byref(need)),
                               "fb_grad_workspace_size")
                    ws = torch.empty(max(int(need.value), 256), dtype=torch.uint8, device=dev)
                    _lib.check(L.fb_interpolate_grad(prm.method, prm.prec, prm.dim, pts.data_ptr(), val.data_ptr(),
                                                     n, prm.c_sigma, prm.c_x0, prm.c_step, prm.c_size,
                                                     prm.num_iter, prm.mdw, g.data_ptr(), g_f64,
                                                     grad_val.data_ptr(),
                                                     grad_pts.data_ptr() if want_pts else None, ws.data_ptr(),
                                                     ws.numel(), _lib.stream_ptr(torch, dev)),
                               "fb_interpolate_grad")
                gp = grad_pts.reshape(pts.shape) if want_pts else None
                return gp, grad_val if ctx.needs_input_grad[1] else None, None

        cls._fn = _F
        return _F


def barnes(pts, val, sigma, x0, step, size, method='optimized_convolution', num_iter=4, max_dist=3.5, *,
           precision='fp64', out_dtype=np.float64):
    """Differentiable Barnes interpolation: pts (N x dim) and val (N) are CUDA
    float64 tensors (with requires_grad as needed); returns a tensor of shape
    size[::-1] (float64 by default) that autograd differentiates with respect
    to val and pts.  Arguments and checks as interpolation.barnes."""
    torch = _torch()
    p2, v2, dim, sigma, x0, step, size, _ = _check_args(pts, val, sigma, x0, step, size)
    if len(v2) == 0:
        raise ValueError('zero-size array to reduction operation minimum which has no identity')
    if method not in _METHODS:
        raise RuntimeError("encountered invalid Barnes interpolation method: " + str(method))
    if method == 'optimized_convolution':
        ks = 2 * _get_half_kernel_size_opt(sigma, step, num_iter) + 1
    else:
        ks = 2 * _get_half_kernel_size(sigma, step, num_iter) + 1
    _kernel_guard(ks, size, dim)
    if not (isinstance(pts, torch.Tensor) and isinstance(val, torch.Tensor) and pts.is_cuda and val.is_cuda
            and pts.dtype == torch.float64 and val.dtype == torch.float64):
        raise TypeError("pts and val must be CUDA float64 tensors")
    prm = _Params(_METHODS[method], _precision_code(precision), dim, sigma, x0, step, size, num_iter,
                  exp(-max_dist ** 2 / 2), np.dtype(out_dtype) == np.float64)
    p = pts.reshape(-1, dim)
    if not p.is_contiguous():
        p = p.contiguous()
    v = val if val.is_contiguous() else val.contiguous()
    return BarnesFunction.get().apply(p, v, prm)
