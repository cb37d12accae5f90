"""Quantised Barnes interpolation (drop-in for the reference's
demo/quantinterpolation.py): the 'convolution' algorithm whose float64 result
keeps only 53 - quant_bits mantissa bits, rounded as demo/quantization.py
quant() does.  The quantisation is fused into the last axis kernel
(fb_interpolate_quant).

``barnes(pts, val, sigma, x0, step, size, quant_bits, num_iter=4,
max_dist=3.5)`` keeps the demo's simplified argument checks and returns a
float64 array of shape size[::-1].
"""
import ctypes
from math import exp

import numpy as np

from . import _lib
from .interpolation import _is_tensor, _per_dim, _precision_code

__all__ = ["barnes"]


def barnes(pts, val, sigma, x0, step, size, quant_bits, num_iter=4, max_dist=3.5, *, precision='fp64'):
    """demo/quantinterpolation.py:21-117 on the GPU."""
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
    torch = _lib.torch_cuda()
    tensor_in = _is_tensor(pts) or _is_tensor(val)
    dev = pts.device if _is_tensor(pts) and pts.is_cuda else torch.device("cuda", torch.cuda.current_device())
    n = int(val.shape[0])
    if n == 0:
        raise ValueError('zero-size array to reduction operation minimum which has no identity')
    tp = torch.as_tensor(pts).to(device=dev, dtype=torch.float64).reshape(n, dim).contiguous()
    tv = torch.as_tensor(val).to(device=dev, dtype=torch.float64).contiguous()
    out = torch.empty(tuple(int(s) for s in size[::-1]), dtype=torch.float64, device=dev)
    L = _lib.lib()
    prec = _precision_code(precision)
    c_sigma, c_x0, c_step = (_lib.dvec([float(s) for s in a]) for a in (sigma, x0, step))
    c_size = _lib.dvec([int(s) for s in size], ctypes.c_int64)
    need = ctypes.c_size_t(0)
    with torch.cuda.device(dev):
        _lib.check(L.fb_workspace_size(_lib.FB_CONVOLUTION, prec, dim, n, c_sigma, c_step, c_size, int(num_iter),
                                       ctypes.byref(need)), "fb_workspace_size")
        ws = _lib.workspace(need.value, dev)
        _lib.check(L.fb_interpolate_quant(_lib.FB_CONVOLUTION, prec, dim, tp.data_ptr(), tv.data_ptr(), n, c_sigma,
                                          c_x0, c_step, c_size, int(num_iter), float(max_dist_weight),
                                          int(quant_bits), out.data_ptr(), ws.data_ptr(), ws.numel(),
                                          _lib.stream_ptr(torch, dev)), "fb_interpolate_quant")
    return out if tensor_in else out.cpu().numpy()
