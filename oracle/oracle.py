"""ctypes front end of the CPU oracle (barnes_oracle.c).

TEST INFRASTRUCTURE, NOT PRODUCT CODE: only tests/, the smoke check in
__graft_entry__.py and bench.py's CPU-baseline / reference arm use this module,
and only to compare the GPU results against or as the timed CPU baseline.
The GPU library never imports it.

Every function mirrors one of the reference's (MeteoSwiss/fast-barnes-py) in
its float64 operation order; see the citations in barnes_oracle.c.
"""
import ctypes
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "barnes_oracle.c")
LIB = os.path.join(HERE, "libbarnes_oracle.so")

_lib = None


def build(force=False):
    """Compile barnes_oracle.c into libbarnes_oracle.so (gcc, no FMA contraction)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-shared", "-fPIC",
           "-o", LIB, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        d, i, i64 = ctypes.c_double, ctypes.c_int, ctypes.c_int64
        P = ctypes.c_void_p
        L.fbo_half_kernel_size_opt.argtypes = [d, d, i]
        L.fbo_half_kernel_size_opt.restype = i
        L.fbo_tail_value.argtypes = [d, d, i]
        L.fbo_tail_value.restype = d
        L.fbo_half_kernel_size.argtypes = [d, d, i]
        L.fbo_half_kernel_size.restype = i
        L.fbo_sigma_effective.argtypes = [d, d, i]
        L.fbo_sigma_effective.restype = d
        L.fbo_accumulate_tail_array.argtypes = [P, P, i, i, i, d]
        L.fbo_accumulate_tail_array.restype = P
        L.fbo_accumulate_array.argtypes = [P, P, i, i, i]
        L.fbo_accumulate_array.restype = P
        L.fbo_interpolate.argtypes = [i, i, P, P, i64, P, P, P, P, i, d, i, P, P, P]
        L.fbo_interpolate.restype = d
        L.fbo_interpolate_direct.argtypes = [i, i, P, P, i64, P, P, P, P, i, d, i, P, P, P]
        L.fbo_interpolate_direct.restype = d
        L.fbo_interpolate_naive.argtypes = [i, P, P, i64, P, P, P, P, i, P]
        L.fbo_interpolate_naive.restype = None
        L.fbo_interpolate_naive_s2.argtypes = [P, P, i64, P, P, P, P, i, P]
        L.fbo_interpolate_radius.argtypes = [P, P, i64, d, P, P, P, d, d, i, P]
        L.fbo_interpolate_radius.restype = None
        L.fbo_quant.argtypes = [P, i64, i]
        L.fbo_quant.restype = None
        L.fbo_interpolate_naive_s2.restype = None
        L.fbo_lambert_create_proj.argtypes = [d, d, d, d, P]
        L.fbo_lambert_to_map.argtypes = [P, P, i64, P]
        L.fbo_resample.argtypes = [P, i64, i64, P, P, P, P, P, P]
        L.fbo_interpolate_s2.argtypes = [P, P, i64, P, P, P, P, i, d, i, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def half_kernel_size_opt(sigma, step, num_iter):
    return lib().fbo_half_kernel_size_opt(float(sigma), float(step), int(num_iter))


def tail_value(sigma, step, num_iter):
    return lib().fbo_tail_value(float(sigma), float(step), int(num_iter))


def half_kernel_size(sigma, step, num_iter):
    return lib().fbo_half_kernel_size(float(sigma), float(step), int(num_iter))


def sigma_effective(sigma, step, num_iter):
    return lib().fbo_sigma_effective(float(sigma), float(step), int(num_iter))


def accumulate_tail_array(arr, rect_len, num_iter, alpha):
    a = np.ascontiguousarray(arr, dtype=np.float64).copy()
    h = np.empty_like(a)
    r = lib().fbo_accumulate_tail_array(_p(a), _p(h), len(a), int(rect_len), int(num_iter), float(alpha))
    return a.copy() if r == a.ctypes.data else h.copy()


def accumulate_array(arr, rect_len, num_iter):
    a = np.ascontiguousarray(arr, dtype=np.float64).copy()
    h = np.empty_like(a)
    r = lib().fbo_accumulate_array(_p(a), _p(h), len(a), int(rect_len), int(num_iter))
    return a.copy() if r == a.ctypes.data else h.copy()


def _vec(x, dim, dtype=np.float64):
    return np.ascontiguousarray(np.broadcast_to(np.asarray(x, dtype), (dim,)))


def interpolate(pts, val, sigma, x0, step, size, num_iter=4, max_dist=3.5,
                method="optimized_convolution", nthreads=1, direct=False):
    """Returns (out_f32, q64, wg, thr) exactly as the reference computes them:
    out_f32 is barnes()'s return value, q64 the float64 quotient before the
    cast, wg the convolved weights before the NaN mask, thr the mask level.

    direct=True computes every box pass by summing each output's window
    directly instead of the reference's running sums (fbo_direct_tail_passes):
    not the reference's rounding, but the drift-free float64 value of the
    same quantity, used as the truth on very long lines."""
    pts = np.asarray(pts, np.float64)
    if pts.ndim == 1:
        pts = pts.reshape(-1, 1)
    pts = np.ascontiguousarray(pts)
    dim = pts.shape[1]
    val = np.ascontiguousarray(val, np.float64)
    sz = _vec(size, dim, np.int64)
    # the reference's kernel-size check (interpolation.py:170-175, :179-184):
    # the C restatement below assumes it and would index past its buffers
    sg, st = _vec(sigma, dim), _vec(step, dim)
    half = half_kernel_size_opt if method == "optimized_convolution" else half_kernel_size
    for a in range(dim):
        if 2 * half(sg[a], st[a], num_iter) + 1 >= sz[a]:
            raise RuntimeError("kernel size not smaller than the grid along axis %d" % a)
    shape = tuple(int(s) for s in sz[::-1])
    out = np.empty(shape, np.float32)
    q = np.empty(shape, np.float64)
    wg = np.empty(shape, np.float64)
    m = 0 if method == "optimized_convolution" else 1
    mdw = math.exp(-max_dist ** 2 / 2)
    fn = lib().fbo_interpolate_direct if direct else lib().fbo_interpolate
    thr = fn(m, dim, _p(pts), _p(val), len(val), _p(_vec(sigma, dim)),
                                _p(_vec(x0, dim)), _p(_vec(step, dim)), _p(sz), int(num_iter),
                                mdw, int(nthreads), _p(out), _p(q), _p(wg))
    return out, q, wg, thr


def interpolate_naive(pts, val, sigma, x0, step, size, nthreads=1):
    pts = np.asarray(pts, np.float64)
    if pts.ndim == 1:
        pts = pts.reshape(-1, 1)
    pts = np.ascontiguousarray(pts)
    dim = pts.shape[1]
    val = np.ascontiguousarray(val, np.float64)
    sz = _vec(size, dim, np.int64)
    out = np.empty(tuple(int(s) for s in sz[::-1]), np.float64)
    lib().fbo_interpolate_naive(dim, _p(pts), _p(val), len(val), _p(_vec(sigma, dim)),
                                _p(_vec(x0, dim)), _p(_vec(step, dim)), _p(sz), int(nthreads), _p(out))
    return out


def interpolate_naive_s2(pts, val, sigma, x0, step, size, nthreads=1):
    g = np.ascontiguousarray(pts, np.float64)
    v = np.ascontiguousarray(val, np.float64)
    sz = _vec(size, 2, np.int64)
    out = np.empty((int(sz[1]), int(sz[0])), np.float64)
    lib().fbo_interpolate_naive_s2(_p(g), _p(v), len(v), _p(_vec(sigma, 2)), _p(_vec(x0, 2)), _p(_vec(step, 2)),
                                   _p(sz), int(nthreads), _p(out))
    return out


def interpolate_radius(pts, val, sigma, x0, step, size, max_dist=3.5, min_weight=0.001, nthreads=1):
    g = np.ascontiguousarray(pts, np.float64)
    v = np.ascontiguousarray(val, np.float64)
    sz = _vec(size, 2, np.int64)
    out = np.empty((int(sz[1]), int(sz[0])), np.float64)
    lib().fbo_interpolate_radius(_p(g), _p(v), len(v), float(sigma), _p(_vec(x0, 2)), _p(_vec(step, 2)), _p(sz),
                                 math.exp(-max_dist ** 2 / 2), float(min_weight), int(nthreads), _p(out))
    return out


def quant(arr, nbits):
    """demo/quantization.py quant() on a copy of arr (float64)."""
    a = np.array(arr, np.float64, copy=True, order="C")
    lib().fbo_quant(_p(a), a.size, int(nbits))
    return a


def lambert_proj(center_lon=11.5, center_lat=34.5, lat1=42.5, lat2=65.5):
    p = np.empty(5, np.float64)
    lib().fbo_lambert_create_proj(center_lon, center_lat, lat1, lat2, _p(p))
    return p


def lambert_to_map(pts, proj=None):
    proj = lambert_proj() if proj is None else np.ascontiguousarray(proj, np.float64)
    g = np.ascontiguousarray(pts, np.float64)
    m = np.empty_like(g)
    lib().fbo_lambert_to_map(_p(g), _p(m), len(g), _p(proj))
    return m


def interpolate_s2(pts, val, sigma, x0, step, size, num_iter=4, max_dist=3.5, resample=True, nthreads=1):
    """barnes_S2(method='optimized_convolution_S2'): returns the resampled
    lon/lat field if resample else the Lambert field."""
    pts = np.ascontiguousarray(pts, np.float64)
    val = np.ascontiguousarray(val, np.float64)
    stp = _vec(step, 2)
    sz = _vec(size, 2, np.int64)
    lam = np.empty((int(44.0 / stp[1]), int(64.0 / stp[0])), np.float32)
    out = np.empty((int(sz[1]), int(sz[0])), np.float32)
    mdw = math.exp(-max_dist ** 2 / 2)
    lib().fbo_interpolate_s2(_p(pts), _p(val), len(val), _p(_vec(sigma, 2)), _p(_vec(x0, 2)), _p(stp),
                             _p(sz), int(num_iter), mdw, int(nthreads), _p(lam),
                             _p(out) if resample else None)
    return out if resample else lam
