"""Barnes interpolation on the unit sphere, computed on a GB300.

Drop-in for ``fastbarnes.interpolationS2`` (MeteoSwiss/fast-barnes-py 2.0):
``barnes_S2`` keeps the reference's simplified argument checks and messages
(fastbarnes/interpolationS2.py:84-138), including its default
``method='optimized_convolution'``, which its own dispatcher rejects: callers
pass ``method='optimized_convolution_S2'`` there and here.  The samples are
projected to the fixed Lambert grid, interpolated there with the optimized
convolution and resampled to the lon/lat grid, all on the GPU.
'naive_S2' (direct Gaussian sums of great-circle distances, float64 result
like the reference's) runs on the GPU as well.
"""
import ctypes
from math import exp

import numpy as np

from . import _lib
from .interpolation import _is_tensor, _per_dim, _precision_code
from .util import lambert_conformal

__all__ = ["barnes_S2", "interpolate_opt_convol_S2_part1", "interpolate_opt_convol_S2_part2", "get_lambert_proj"]


def get_lambert_proj():
    """The projection of the reference's European domain
    (interpolationS2.py:205-208)."""
    return lambert_conformal.create_proj(11.5, 34.5, 42.5, 65.5)


def _lambert_grid(step):
    """interpolationS2.py:187-188: the fixed Lambert grid."""
    lam_x0 = np.asarray([-32.0, -2.0])
    lam_size = (int(64.0 / step[0]), int(44.0 / step[1]))
    return lam_x0, lam_size


def barnes_S2(pts, val, sigma, x0, step, size, method='optimized_convolution', num_iter=4, max_dist=3.5,
              resample=True, *, precision='fp64'):
    """Barnes interpolation on S^2 of the lon/lat samples (pts, val) onto the
    lon/lat grid (x0, step, size); see fastbarnes/interpolationS2.py:32-83.
    Returns a float32 array of shape size[::-1] (resample=True) or the Lambert
    field (resample=False)."""
    dim = pts.shape[1]
    sigma = _per_dim('sigma', sigma, dim)
    x0 = _per_dim('x0', x0, dim)
    step = _per_dim('step', step, dim)
    if isinstance(size, (list, tuple, np.ndarray)):
        if len(size) != dim:
            raise RuntimeError('specified size with invalid length: ' + str(len(size)))
        size = tuple(size)
    elif dim != 1:
        raise RuntimeError('array size should be array-like of length: ' + str(dim))
    else:
        size = (size,)
    max_dist_weight = exp(-max_dist ** 2 / 2)
    if method == 'optimized_convolution_S2':
        return _run_s2(pts, val, sigma, x0, step, size, num_iter, max_dist_weight, resample,
                       _precision_code(precision))
    elif method == 'naive_S2':
        return _run_naive_s2(pts, val, sigma, x0, step, size, _precision_code(precision))
    else:
        raise RuntimeError("encountered invalid Barnes interpolation method: " + str(method))


def _run_naive_s2(pts, val, sigma, x0, step, size, prec):
    """interpolationS2.py:259-283 on the GPU; float64 result."""
    torch = _lib.torch_cuda()
    tensor_in = _is_tensor(pts) or _is_tensor(val)
    dev = pts.device if _is_tensor(pts) and pts.is_cuda else torch.device("cuda", torch.cuda.current_device())
    n = int(val.shape[0])
    if n == 0:
        raise ValueError('zero-size array to reduction operation minimum which has no identity')
    tp = torch.as_tensor(pts).to(device=dev, dtype=torch.float64).reshape(n, 2).contiguous()
    tv = torch.as_tensor(val).to(device=dev, dtype=torch.float64).contiguous()
    out = torch.empty((int(size[1]), int(size[0])), dtype=torch.float64, device=dev)
    c_sigma, c_x0, c_step = (_lib.dvec([float(s) for s in a]) for a in (sigma, x0, step))
    c_size = _lib.dvec([int(s) for s in size], ctypes.c_int64)
    with torch.cuda.device(dev):
        ws = _lib.workspace(256, dev)
        _lib.check(_lib.lib().fb_interpolate_naive_s2(prec, tp.data_ptr(), tv.data_ptr(), n, c_sigma, c_x0, c_step,
                                                      c_size, out.data_ptr(), 1, ws.data_ptr(), ws.numel(),
                                                      _lib.stream_ptr(torch, dev)), "fb_interpolate_naive_s2")
    return out if tensor_in else out.cpu().numpy()


def _run_s2(pts, val, sigma, x0, step, size, num_iter, max_dist_weight, resample, prec):
    torch = _lib.torch_cuda()
    tensor_in = _is_tensor(pts) or _is_tensor(val)
    dev = pts.device if _is_tensor(pts) and pts.is_cuda else torch.device("cuda", torch.cuda.current_device())
    n = int(val.shape[0])
    if n == 0:
        raise ValueError('zero-size array to reduction operation minimum which has no identity')
    tp = torch.as_tensor(pts).to(device=dev, dtype=torch.float64).reshape(n, 2).contiguous()
    tv = torch.as_tensor(val).to(device=dev, dtype=torch.float64).contiguous()
    lam_x0, lam_size = _lambert_grid(step)
    shape = (int(size[1]), int(size[0])) if resample else (lam_size[1], lam_size[0])
    out = torch.empty(shape, dtype=torch.float32, device=dev)
    L = _lib.lib()
    c_sigma, c_x0, c_step = (_lib.dvec([float(s) for s in a]) for a in (sigma, x0, step))
    c_size = _lib.dvec([int(s) for s in size], ctypes.c_int64)
    need = ctypes.c_size_t(0)
    with torch.cuda.device(dev):
        _lib.check(L.fb_s2_workspace_size(prec, n, c_sigma, c_step, c_size, int(num_iter), ctypes.byref(need)),
                   "fb_s2_workspace_size")
        ws = _lib.workspace(need.value, dev)
        rc = L.fb_interpolate_s2(prec, tp.data_ptr(), tv.data_ptr(), n, c_sigma, c_x0, c_step, c_size,
                                 int(num_iter), float(max_dist_weight), int(bool(resample)), out.data_ptr(),
                                 ws.data_ptr(), ws.numel(), _lib.stream_ptr(torch, dev))
        _lib.check(rc, "fb_interpolate_s2")
    return out if tensor_in else out.cpu().numpy()


def interpolate_opt_convol_S2_part1(pts, val, sigma, x0, step, size, num_iter, max_dist_weight):
    """The convolution part in Lambert space (interpolationS2.py:180-196):
    returns (lam_field, lam_x0, x0, step, size, lambert_proj)."""
    sigma = np.asarray(sigma, np.float64)
    step = np.asarray(step, np.float64)
    lam_x0, _ = _lambert_grid(step)
    torch = _lib.torch_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    n = int(len(val))
    tp = torch.as_tensor(pts).to(device=dev, dtype=torch.float64).reshape(n, 2).contiguous()
    tv = torch.as_tensor(val).to(device=dev, dtype=torch.float64).contiguous()
    lam_size = (int(64.0 / step[0]), int(44.0 / step[1]))
    lam = torch.empty((lam_size[1], lam_size[0]), dtype=torch.float32, device=dev)
    L = _lib.lib()
    c_sigma, c_x0, c_step = (_lib.dvec([float(s) for s in a]) for a in (sigma, x0, step))
    c_size = _lib.dvec([int(s) for s in size], ctypes.c_int64)
    need = ctypes.c_size_t(0)
    with torch.cuda.device(dev):
        _lib.check(L.fb_s2_workspace_size(_lib.FB_FP64, n, c_sigma, c_step, c_size, int(num_iter),
                                          ctypes.byref(need)), "fb_s2_workspace_size")
        ws = _lib.workspace(need.value, dev)
        _lib.check(L.fb_interpolate_s2(_lib.FB_FP64, tp.data_ptr(), tv.data_ptr(), n, c_sigma, c_x0, c_step, c_size,
                                       int(num_iter), float(max_dist_weight), 0, lam.data_ptr(), ws.data_ptr(),
                                       ws.numel(), _lib.stream_ptr(torch, dev)), "fb_interpolate_s2")
    return (lam.cpu().numpy(), lam_x0, x0, step, size, get_lambert_proj())


def interpolate_opt_convol_S2_part2(lam_field, lam_x0, x0, step, size, lambert_proj):
    """The back-projection part (interpolationS2.py:199-202): resamples the
    Lambert field to the lon/lat grid on the GPU."""
    torch = _lib.torch_cuda()
    dev = torch.device("cuda", torch.cuda.current_device())
    lam = torch.as_tensor(np.ascontiguousarray(lam_field, np.float32)).to(dev)
    step = np.broadcast_to(np.asarray(step, np.float64), (2,))
    x0 = np.broadcast_to(np.asarray(x0, np.float64), (2,))
    out = torch.empty((int(size[1]), int(size[0])), dtype=torch.float32, device=dev)
    tab = torch.empty(int(size[1]) + 2 * int(size[0]), dtype=torch.float64, device=dev)
    c = lambda a: _lib.dvec([float(s) for s in a])  # noqa: E731
    with torch.cuda.device(dev):
        _lib.check(_lib.lib().fb_resample(lam.data_ptr(), lam.shape[1], lam.shape[0], c(lam_x0), c(x0), c(step),
                                          _lib.dvec([int(size[0]), int(size[1])], ctypes.c_int64),
                                          c(lambert_proj), out.data_ptr(), tab.data_ptr(),
                                          _lib.stream_ptr(torch, dev)), "fb_resample")
    return out.cpu().numpy()
