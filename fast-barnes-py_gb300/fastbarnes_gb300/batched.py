"""Many 2D Barnes interpolations in one plan (GB300 extension, no reference
counterpart: the reference interpolates one field per ``barnes()`` call,
fastbarnes/interpolation.py:36).

A :class:`BatchPlan` holds the device inputs and outputs of many independent
2D fields -- each with its own samples, sigma, grid and method -- and runs all
of them with one sample sort and one launch per axis stage, optionally
replayed from a CUDA graph.  Each field's result equals
``interpolation.barnes(..., precision=p)`` of that field.

    plan = BatchPlan([dict(pts=p0, val=v0, sigma=1.0, x0=(-9, 47), step=0.01, size=(4096, 2048)),
                      dict(pts=p1, val=v1, sigma=0.5, x0=(0, 0), step=0.1, size=(300, 200))],
                     precision='fp32c', graph=True)
    outs = plan.run()          # list of CUDA tensors, shape size[::-1]
    p0.copy_(new_pts); ...     # refill inputs in place, then run again
"""
import ctypes
from math import exp

import numpy as np

from . import _lib
from .interpolation import _check_args, _get_half_kernel_size, _get_half_kernel_size_opt, _kernel_guard, \
    _precision_code

__all__ = ["BatchPlan", "barnes_batch"]

_METHODS = {"optimized_convolution": _lib.FB_OPTIMIZED_CONVOLUTION, "convolution": _lib.FB_CONVOLUTION}


class BatchPlan:
    """A batch of 2D fields on one CUDA device.

    fields    : sequence of dicts with keys pts (N x 2), val (N), sigma, x0,
                step, size (nx, ny), and optionally method
                ('optimized_convolution' default or 'convolution'), num_iter
                (4), max_dist (3.5), out (a preallocated CUDA tensor).
                pts / val are used in place when they are contiguous float64
                CUDA tensors (refill them between runs); anything else is
                copied to the device once.
    precision : 'fp32c' (default) or 'fp64'.
    out_dtype : np.float32 (default) or np.float64.
    graph     : capture the launches in a CUDA graph at the first run.
    tune      : time the candidate launch shapes at creation (runs the batch).
    knobs     : (chunk, rows_threads[, mixed[, cols_pipe[, interleave]]]) to
                pin the launch shape instead (cols_pipe: 0 library default,
                1 the pipelined TMA column kernel, 2 one CTA per column
                group; interleave 1: per-field x and y launches on two
                streams, y reading its field from L2).
    """

    def __init__(self, fields, *, precision='fp32c', out_dtype=np.float32, graph=True, tune=False, knobs=None,
                 device=None):
        torch = _lib.torch_cuda()
        self._torch = torch
        self.device = torch.device(device) if device is not None else torch.device("cuda",
                                                                                  torch.cuda.current_device())
        prec = _precision_code(precision)
        self.out_f64 = 1 if np.dtype(out_dtype) == np.float64 else 0
        odt = torch.float64 if self.out_f64 else torch.float32
        n = len(fields)
        if n < 1:
            raise ValueError("a batch needs at least one field")
        arr = (_lib.Field2D * n)()
        self.pts, self.val, self.outs = [], [], []
        for k, f in enumerate(fields):
            pts, val, dim, sigma, x0, step, size, _ = _check_args(f["pts"], f["val"], f["sigma"], f["x0"],
                                                                  f["step"], f["size"])
            if dim != 2:
                raise RuntimeError("batched fields must be 2D (field %d is %dD)" % (k, dim))
            if len(val) == 0:
                raise ValueError('zero-size array to reduction operation minimum which has no identity')
            method = f.get("method", "optimized_convolution")
            if method not in _METHODS:
                raise RuntimeError("encountered invalid Barnes interpolation method: " + str(method))
            num_iter = int(f.get("num_iter", 4))
            if method == "optimized_convolution":
                ks = 2 * _get_half_kernel_size_opt(sigma, step, num_iter) + 1
            else:
                ks = 2 * _get_half_kernel_size(sigma, step, num_iter) + 1
            _kernel_guard(ks, size, dim)
            tp = torch.as_tensor(pts).to(device=self.device, dtype=torch.float64).reshape(-1, 2).contiguous()
            tv = torch.as_tensor(val).to(device=self.device, dtype=torch.float64).contiguous()
            out = f.get("out")
            shape = (int(size[1]), int(size[0]))
            if out is None:
                out = torch.empty(shape, dtype=odt, device=self.device)
            elif tuple(out.shape) != shape or out.dtype != odt or not out.is_contiguous() or out.device != self.device:
                raise ValueError("field %d: out must be a contiguous %s tensor of shape %s on %s"
                                 % (k, odt, shape, self.device))
            self.pts.append(tp)
            self.val.append(tv)
            self.outs.append(out)
            F = arr[k]
            F.pts, F.val, F.n_pts = tp.data_ptr(), tv.data_ptr(), int(tv.shape[0])
            for m in range(2):
                F.sigma[m], F.x0[m], F.step[m], F.size[m] = float(sigma[m]), float(x0[m]), float(step[m]), int(size[m])
            F.num_iter = num_iter
            F.max_dist_weight = exp(-float(f.get("max_dist", 3.5)) ** 2 / 2)
            F.method = _METHODS[method]
            F.out = out.data_ptr()
        self._fields = arr
        flags = (_lib.FB_BATCH_GRAPH if graph else 0) | (_lib.FB_BATCH_TUNE if tune else 0)
        kn = None
        if knobs is not None:
            kn = _lib.BatchKnobs(*[int(knobs[q]) if len(knobs) > q else 0 for q in range(5)])
        L = _lib.lib()
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(L.fb_batch_create(prec, arr, n, self.out_f64, flags, ctypes.byref(kn) if kn else None,
                                         ctypes.byref(h)), "fb_batch_create")
        self._h = h

    @property
    def knobs(self):
        k = _lib.BatchKnobs()
        _lib.check(_lib.lib().fb_batch_knobs_of(self._h, ctypes.byref(k)), "fb_batch_knobs_of")
        return (k.chunk, k.rows_threads, k.mixed, k.cols_pipe, k.interleave)

    @property
    def info(self):
        """(kernel launches per run, memsets per run, plan device bytes)."""
        k, m, b = ctypes.c_int(), ctypes.c_int(), ctypes.c_size_t()
        _lib.check(_lib.lib().fb_batch_info(self._h, ctypes.byref(k), ctypes.byref(m), ctypes.byref(b)),
                   "fb_batch_info")
        return k.value, m.value, b.value

    def run(self, stream=None):
        """Enqueues the batch on `stream` (default: torch's current stream);
        returns the output tensors."""
        torch = self._torch
        if self._h is None:
            raise RuntimeError("plan is closed")
        with torch.cuda.device(self.device):
            sp = ctypes.c_void_p(stream.cuda_stream if stream is not None
                                 else torch.cuda.current_stream(self.device).cuda_stream)
            _lib.check(_lib.lib().fb_batch_run(self._h, sp), "fb_batch_run")
        return self.outs

    def close(self):
        if getattr(self, "_h", None) is not None:
            _lib.lib().fb_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def barnes_batch(fields, *, precision='fp32c', out_dtype=np.float32):
    """One-shot batch: interpolates every field of `fields` (see BatchPlan)
    and returns the list of CUDA output tensors."""
    plan = BatchPlan(fields, precision=precision, out_dtype=out_dtype, graph=False)
    outs = plan.run()
    plan._torch.cuda.current_stream(plan.device).synchronize()
    plan.close()
    return outs
