"""Barnes interpolation on regular 1D / 2D / 3D grids, computed on a GB300.

Drop-in for ``fastbarnes.interpolation`` (MeteoSwiss/fast-barnes-py 2.0):
``barnes()`` takes the same arguments, performs the same argument checks with
the same RuntimeError messages (fastbarnes/interpolation.py:103-199) and
returns the same float32 array of shape ``size[::-1]``.  The work itself runs
in libfastbarnes_gb300 (sm_103a CUDA kernels): a stable bin sort of the
samples, a splat fused into the first axis's box passes, and the n box-and-tail
passes of every axis held in shared memory, with the NaN mask and the quotient
fused into the last axis.

Extensions beyond the reference's signature (keyword-only):
  precision : 'fp64' (default; float64 throughout, the drop-in) or 'fp32c'
              (float32 running sums re-anchored on exact chunk sums).
  out_dtype : np.float32 (default, the reference's return type) or
              np.float64 (the quotient before the cast).
``pts`` / ``val`` may also be CUDA torch tensors; the result is then a CUDA
torch tensor and nothing crosses the host.

Methods: 'optimized_convolution', 'convolution', 'naive' (direct Gaussian
sums) and 'radius' (the same sums over the samples within
sqrt(-2 ln(min_weight)) sigma; the reference's kd-tree search becomes tiles of
y-sorted samples that a block of grid points skips when out of reach) all run
on the GPU; 'naive' and 'radius' return float64 like the reference's.
"""
import ctypes
from math import exp

import numpy as np

from . import _lib

__all__ = ["barnes", "get_half_kernel_size_opt", "get_tail_value", "get_half_kernel_size",
           "get_sigma_effective"]


# ---------------------------------------------------------------------------
# kernel-size helpers (interpolation.py:538-569, :777-803)
# ---------------------------------------------------------------------------

def _to_np(value):
    """Converts a scalar to a numpy array (interpolation.py:538-540)."""
    return np.asarray([value], dtype=np.float64)


def _get_half_kernel_size_opt(sigma, step, num_iter):
    """T = int32((sqrt(1 + 12 s^2 / n) - 1) / 2), s = sigma / step, per axis."""
    s = sigma / step
    return ((np.sqrt(1.0 + 12 * s * s / num_iter) - 1.0) / 2.0).astype(np.int32)


def _get_tail_value(sigma, step, num_iter):
    """Tail weight alpha of the optimized rect kernel, per axis."""
    T = _get_half_kernel_size_opt(sigma, step, num_iter)
    ks = 2 * T + 1
    sigma_rect_sqr = (T + 1) * T / 3.0 * step ** 2
    return 0.5 * ks * (sigma ** 2 / num_iter - sigma_rect_sqr) / (((T + 1) * step) ** 2 - sigma ** 2 / num_iter)


def _get_half_kernel_size(sigma, step, num_iter):
    """T of the plain rect kernel, per axis."""
    return (np.sqrt(3.0 / num_iter) * sigma / step + 0.5).astype(np.int32)


def _get_sigma_effective(sigma, step, num_iter):
    T = _get_half_kernel_size(sigma, step, num_iter)
    return np.sqrt(num_iter / 3.0 * T * (T + 1)) * step


def get_half_kernel_size_opt(sigma, step, num_iter):
    """Half kernel size T of the optimized convolution (scalar arguments)."""
    return _get_half_kernel_size_opt(_to_np(sigma), _to_np(step), num_iter)[0]


def get_tail_value(sigma, step, num_iter):
    """Tail value alpha of the optimized convolution (scalar arguments)."""
    return _get_tail_value(_to_np(sigma), _to_np(step), num_iter)[0]


def get_half_kernel_size(sigma, step, num_iter):
    """Half kernel size T of the plain convolution (scalar arguments)."""
    return _get_half_kernel_size(_to_np(sigma), _to_np(step), num_iter)[0]


def get_sigma_effective(sigma, step, num_iter):
    """Effective sigma of the num_iter-fold plain rect kernel (scalar arguments)."""
    return _get_sigma_effective(_to_np(sigma), _to_np(step), num_iter)[0]


# ---------------------------------------------------------------------------
# argument checks (interpolation.py:103-164)
# ---------------------------------------------------------------------------

def _is_tensor(x):
    try:
        import torch
        return isinstance(x, torch.Tensor)
    except ImportError:
        return False


def _per_dim(name, x, dim, dtype=np.float64):
    if isinstance(x, (list, tuple, np.ndarray)):
        if len(x) != dim:
            raise RuntimeError('specified ' + name + ' with invalid length: ' + str(len(x)))
        return np.asarray(x, dtype=dtype)
    return np.full(dim, x, dtype=dtype)


def _check_args(pts, val, sigma, x0, step, size):
    tensor_in = _is_tensor(pts) or _is_tensor(val)
    if not (isinstance(pts, np.ndarray) or _is_tensor(pts)):
        raise RuntimeError('specified pts is not a numpy ndarray')
    if len(pts.shape) > 2:
        raise RuntimeError('expected pts array of shape (N, M) but was: ' + str(tuple(pts.shape)))
    if len(pts.shape) == 1:
        pts = pts.reshape(-1, 1)
    dim = pts.shape[1]
    if dim < 1 or dim > 3:
        raise RuntimeError('Barnes interpolation supports only sample points in dimensions 1, 2 or 3')
    if not (isinstance(val, np.ndarray) or _is_tensor(val)):
        raise RuntimeError('specified val is not a numpy ndarray')
    if len(val.shape) > 1:
        raise RuntimeError('expected val array of shape (N) but was: ' + str(tuple(val.shape)))
    if val.shape[0] != pts.shape[0]:
        raise RuntimeError('pts and val arrays have inconsistent shapes: ' + str(tuple(pts.shape)) + ' vs. '
                           + str(tuple(val.shape)))
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
    return pts, val, dim, sigma, x0, step, size, tensor_in


def _kernel_guard(kernel_size, size, dim):
    """interpolation.py:170-175 / :179-184."""
    for m in range(dim):
        if kernel_size[m] >= size[m]:
            raise RuntimeError('resulting rectangular kernel size should be smaller w.r.t. specified grid: '
                               + str(kernel_size) + ' vs. ' + str(size))


def _precision_code(precision):
    try:
        return _lib.PRECISIONS[precision]
    except KeyError:
        raise ValueError("precision must be 'fp64' or 'fp32c', got " + repr(precision)) from None


# ---------------------------------------------------------------------------
# device execution
# ---------------------------------------------------------------------------

def _run_grid_host(method_code, prec, dim, pts, val, sigma, x0, step, size, num_iter, max_dist_weight, out_dtype):
    """numpy in, numpy out: one call of the C ABI's host-buffer entry
    (fb_interpolate_host: copies in, the interpolation and the copy out on
    torch's current stream, with the library's device buffer; no torch
    tensors), which also checks the device status word.  The result array
    wraps a page-locked buffer of the library's pool, so the result comes
    back as one DMA transfer."""
    torch = _lib.torch_cuda()
    npts = int(val.shape[0])
    hp = np.ascontiguousarray(pts, dtype=np.float64).reshape(npts, dim)
    hv = np.ascontiguousarray(val, dtype=np.float64)
    out_f64 = 1 if np.dtype(out_dtype) == np.float64 else 0
    out = _lib.pinned.empty(tuple(int(s) for s in size[::-1]), np.float64 if out_f64 else np.float32)
    L = _lib.lib()
    dev = torch.device("cuda", torch.cuda.current_device())
    with torch.cuda.device(dev):
        rc = L.fb_interpolate_host(method_code, prec, dim, hp.ctypes.data, hv.ctypes.data, npts,
                                   _lib.dvec([float(s) for s in sigma]), _lib.dvec([float(s) for s in x0]),
                                   _lib.dvec([float(s) for s in step]), _lib.dvec([int(s) for s in size], ctypes.c_int64),
                                   int(num_iter), float(max_dist_weight), out.ctypes.data, out_f64,
                                   _lib.stream_ptr(torch, dev))
        _lib.check(rc, "fb_interpolate_host")
    return out


def _run_grid(method_code, prec, dim, pts, val, sigma, x0, step, size, num_iter, max_dist_weight, out_dtype,
              tensor_in):
    """Runs fb_interpolate on the current CUDA device; returns numpy or torch."""
    torch = _lib.torch_cuda()
    if not tensor_in:
        return _run_grid_host(method_code, prec, dim, pts, val, sigma, x0, step, size, num_iter, max_dist_weight,
                              out_dtype)
    if tensor_in:
        dev = pts.device if _is_tensor(pts) and pts.is_cuda else torch.device("cuda", torch.cuda.current_device())
    else:
        dev = torch.device("cuda", torch.cuda.current_device())
    npts = int(val.shape[0])
    tp = torch.as_tensor(pts).to(device=dev, dtype=torch.float64).reshape(npts, dim).contiguous()
    tv = torch.as_tensor(val).to(device=dev, dtype=torch.float64).contiguous()
    out_f64 = 1 if np.dtype(out_dtype) == np.float64 else 0
    out = torch.empty(tuple(int(s) for s in size[::-1]), dtype=torch.float64 if out_f64 else torch.float32,
                      device=dev)
    L = _lib.lib()
    c_sigma = _lib.dvec([float(s) for s in sigma])
    c_x0 = _lib.dvec([float(s) for s in x0])
    c_step = _lib.dvec([float(s) for s in step])
    c_size = _lib.dvec([int(s) for s in size], ctypes.c_int64)
    need = ctypes.c_size_t(0)
    with torch.cuda.device(dev):
        _lib.check(L.fb_workspace_size(method_code, prec, dim, npts, c_sigma, c_step, c_size, int(num_iter),
                                       ctypes.byref(need)), "fb_workspace_size")
        ws = _lib.workspace(need.value, dev)
        rc = L.fb_interpolate(method_code, prec, dim, tp.data_ptr(), tv.data_ptr(), npts, c_sigma, c_x0, c_step,
                              c_size, int(num_iter), float(max_dist_weight), out.data_ptr(), out_f64, ws.data_ptr(),
                              ws.numel(), _lib.stream_ptr(torch, dev))
        _lib.check(rc, "fb_interpolate")
    if tensor_in:
        return out
    return out.cpu().numpy()


def barnes(pts, val, sigma, x0, step, size, method='optimized_convolution', num_iter=4, max_dist=3.5,
           min_weight=0.001, *, precision='fp64', out_dtype=np.float32):
    """Barnes interpolation of the samples (pts, val) onto the regular grid
    (x0, step, size) with Gaussian width sigma; see the module docstring and
    fastbarnes/interpolation.py:31-101 for the parameters.  Returns an array
    of shape size[::-1] ([y, x] in 2D, [z, y, x] in 3D) with NaN where the
    nearest samples are farther than max_dist * sigma."""
    pts, val, dim, sigma, x0, step, size, tensor_in = _check_args(pts, val, sigma, x0, step, size)
    if len(val) == 0:
        # the reference's np.amin on an empty array raises this ValueError
        raise ValueError('zero-size array to reduction operation minimum which has no identity')
    max_dist_weight = exp(-max_dist ** 2 / 2)
    prec = _precision_code(precision)

    if method == 'optimized_convolution':
        kernel_size = 2 * _get_half_kernel_size_opt(sigma, step, num_iter) + 1
        _kernel_guard(kernel_size, size, dim)
        return _run_grid(_lib.FB_OPTIMIZED_CONVOLUTION, prec, dim, pts, val, sigma, x0, step, size, num_iter,
                         max_dist_weight, out_dtype, tensor_in)
    elif method == 'convolution':
        kernel_size = 2 * _get_half_kernel_size(sigma, step, num_iter) + 1
        _kernel_guard(kernel_size, size, dim)
        return _run_grid(_lib.FB_CONVOLUTION, prec, dim, pts, val, sigma, x0, step, size, num_iter,
                         max_dist_weight, out_dtype, tensor_in)
    elif method == 'radius':
        if dim != 2:
            raise RuntimeError('radius algorithm works only in 2D but data is: ' + str(dim) + 'D')
        if sigma[0] != sigma[1]:
            raise RuntimeError('radius algorithm in 2D works only for scalar sigma value but sigma is: '
                               + str(sigma))
        return _run_radius(prec, pts, val, float(sigma[0]), x0, step, size, max_dist_weight, float(min_weight),
                           tensor_in)
    elif method == 'naive':
        # interpolation.py:861-938: no kernel-size check, no max_dist mask,
        # float64 result like the reference's
        return _run_grid(_lib.FB_NAIVE, prec, dim, pts, val, sigma, x0, step, size, num_iter, max_dist_weight,
                         np.float64, tensor_in)
    else:
        raise RuntimeError("encountered invalid Barnes interpolation method: " + method)


def _run_radius(prec, pts, val, sigma, x0, step, size, max_dist_weight, min_weight, tensor_in):
    """fb_interpolate_radius on the samples sorted by y (a stable device sort,
    so that the kernel's sample tiles are narrow in y); float64 result."""
    torch = _lib.torch_cuda()
    if tensor_in:
        dev = pts.device if _is_tensor(pts) and pts.is_cuda else torch.device("cuda", torch.cuda.current_device())
    else:
        dev = torch.device("cuda", torch.cuda.current_device())
    npts = int(val.shape[0])
    tp = torch.as_tensor(pts).to(device=dev, dtype=torch.float64).reshape(npts, 2)
    tv = torch.as_tensor(val).to(device=dev, dtype=torch.float64)
    order = torch.argsort(tp[:, 1], stable=True)
    tp = tp[order].contiguous()
    tv = tv[order].contiguous()
    out = torch.empty((int(size[1]), int(size[0])), dtype=torch.float64, device=dev)
    L = _lib.lib()
    c_x0 = _lib.dvec([float(s) for s in x0])
    c_step = _lib.dvec([float(s) for s in step])
    c_size = _lib.dvec([int(s) for s in size], ctypes.c_int64)
    need = ctypes.c_size_t(0)
    with torch.cuda.device(dev):
        _lib.check(L.fb_radius_workspace_size(npts, ctypes.byref(need)), "fb_radius_workspace_size")
        ws = _lib.workspace(need.value, dev)
        rc = L.fb_interpolate_radius(prec, tp.data_ptr(), tv.data_ptr(), npts, sigma, c_x0, c_step, c_size,
                                     float(max_dist_weight), min_weight, out.data_ptr(), 1, ws.data_ptr(),
                                     ws.numel(), _lib.stream_ptr(torch, dev))
        _lib.check(rc, "fb_interpolate_radius")
    if tensor_in:
        return out
    return out.cpu().numpy()


# ---------------------------------------------------------------------------
# the 1D passes alone (interpolation.py:484-533, :729-772)
# ---------------------------------------------------------------------------

def accumulate_lines(lines, rect_len, num_iter, alpha=0.0, *, precision='fp64', normalize=False):
    """num_iter passes of the rect kernel of length rect_len (plus tail weight
    alpha at +-(T+1)) over every row of the 2D array `lines`, zero outside the
    row, computed on the GPU; the device counterpart of the reference's
    _accumulate_tail_array (alpha != 0) and _accumulate_array (alpha = 0).
    Returns a new float64 numpy array (or a CUDA tensor for tensor input)."""
    torch = _lib.torch_cuda()
    tensor_in = _is_tensor(lines)
    a = torch.as_tensor(lines)
    if a.dim() == 1:
        a = a.reshape(1, -1)
    prec = _precision_code(precision)
    dt = torch.float64 if prec == _lib.FB_FP64 else torch.float32
    dev = a.device if a.is_cuda else torch.device("cuda", torch.cuda.current_device())
    buf = a.to(device=dev, dtype=dt).contiguous().clone()
    with torch.cuda.device(dev):
        rc = _lib.lib().fb_accumulate_lines(prec, buf.data_ptr(), buf.shape[0], buf.shape[1], int(rect_len),
                                            int(num_iter), float(alpha), int(bool(normalize)),
                                            _lib.stream_ptr(torch, dev))
        _lib.check(rc, "fb_accumulate_lines")
    if tensor_in:
        return buf.reshape(tuple(lines.shape))
    return buf.cpu().numpy().astype(np.float64).reshape(np.shape(lines))
