"""ctypes binding of libfastbarnes_gb300.so (the C ABI in include/fastbarnes_gb300.h).

The library is built in-tree (``build.py`` next to this package, or
``__graft_entry__.build()`` at the repository root).  There is no CPU
fallback: if the library or a CUDA device is missing, every entry point that
needs them raises.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
# FASTBARNES_GB300_LIB selects another build of the library (for instance the
# bounds-check variant, libfastbarnes_gb300_checked.so)
LIB_PATH = os.environ.get("FASTBARNES_GB300_LIB") or os.path.join(HERE, "libfastbarnes_gb300.so")

FB_OK = 0
FB_ERR_ARG, FB_ERR_KERNEL_SIZE, FB_ERR_WORKSPACE, FB_ERR_CUDA, FB_ERR_UNSUPPORTED, FB_ERR_DEVICE = 1, 2, 3, 4, 5, 6
FB_FP64, FB_FP32C = 0, 1
FB_OPTIMIZED_CONVOLUTION, FB_CONVOLUTION, FB_NAIVE = 0, 1, 2

PRECISIONS = {"fp64": FB_FP64, "float64": FB_FP64, "fp32c": FB_FP32C}

_lib = None
_lock = threading.Lock()


class Field2D(ctypes.Structure):
    """fb_field2d: one field of a batch (device pointers, grid, parameters)."""
    _fields_ = [
        ("pts", ctypes.c_void_p),
        ("val", ctypes.c_void_p),
        ("n_pts", ctypes.c_int64),
        ("sigma", ctypes.c_double * 2),
        ("x0", ctypes.c_double * 2),
        ("step", ctypes.c_double * 2),
        ("size", ctypes.c_int64 * 2),
        ("num_iter", ctypes.c_int),
        ("max_dist_weight", ctypes.c_double),
        ("method", ctypes.c_int),
        ("out", ctypes.c_void_p),
    ]


class BatchKnobs(ctypes.Structure):
    """fb_batch_knobs: launch shape of a batch plan."""
    _fields_ = [("chunk", ctypes.c_int), ("rows_threads", ctypes.c_int), ("mixed", ctypes.c_int),
                ("cols_pipe", ctypes.c_int), ("interleave", ctypes.c_int)]


FB_BATCH_GRAPH, FB_BATCH_TUNE = 1, 2


class FastBarnesError(RuntimeError):
    """A call into libfastbarnes_gb300 failed; the message is the library's."""


def build(force=False):
    """Compile the CUDA library for sm_103a (nvcc must be on PATH)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_fbg_build", os.path.join(os.path.dirname(HERE), "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise FastBarnesError(
                f"{LIB_PATH} is missing: build it with fast-barnes-py_gb300/build.py "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        P, d, i, i64, sz = ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_int64, ctypes.c_size_t
        sig = {
            "fb_version": ([], ctypes.c_char_p),
            "fb_last_error": ([], ctypes.c_char_p),
            "fb_half_kernel_size_opt": ([d, d, i], i),
            "fb_tail_value": ([d, d, i], d),
            "fb_half_kernel_size": ([d, d, i], i),
            "fb_sigma_effective": ([d, d, i], d),
            "fb_workspace_size": ([i, i, i, i64, P, P, P, i, ctypes.POINTER(sz)], i),
            "fb_interpolate": ([i, i, i, P, P, i64, P, P, P, P, i, d, P, i, P, sz, P], i),
            "fb_interpolate_host": ([i, i, i, P, P, i64, P, P, P, P, i, d, P, i, P], i),
            "fb_interpolate_quant": ([i, i, i, P, P, i64, P, P, P, P, i, d, i, P, P, sz, P], i),
            "fb_grad_workspace_size": ([i, i, i, i64, P, P, P, i, ctypes.POINTER(sz)], i),
            "fb_interpolate_grad": ([i, i, i, P, P, i64, P, P, P, P, i, d, P, i, P, P, P, sz, P], i),
            "fb_host_alloc": ([sz], P),
            "fb_host_free": ([P], None),
            "fb_release": ([], None),
            "fb_accumulate_lines": ([i, P, i64, i64, i, i, d, i, P], i),
            "fb_s2_workspace_size": ([i, i64, P, P, P, i, ctypes.POINTER(sz)], i),
            "fb_interpolate_s2": ([i, P, P, i64, P, P, P, P, i, d, i, P, P, sz, P], i),
            "fb_lambert_create_proj": ([d, d, d, d, P], None),
            "fb_lambert_to_map": ([P, P, i64, P, P], i),
            "fb_resample": ([P, i64, i64, P, P, P, P, P, P, P, P], i),
            "fb_interpolate_naive_s2": ([i, P, P, i64, P, P, P, P, P, i, P, sz, P], i),
            "fb_radius_workspace_size": ([i64, ctypes.POINTER(sz)], i),
            "fb_interpolate_radius": ([i, P, P, i64, d, P, P, P, d, d, P, i, P, sz, P], i),
            "fb_resample_noalloc": ([P, i64, i64, P, P, P, P, P, P, P], i),
            "fb_tune": ([ctypes.c_char_p, i], i),
            "fb_profile_begin": ([], i),
            "fb_profile_end": ([P, P, i, ctypes.POINTER(i)], i),
            "fb_batch_create": ([i, ctypes.POINTER(Field2D), i, i, i, ctypes.POINTER(BatchKnobs),
                                 ctypes.POINTER(P)], i),
            "fb_batch_run": ([P, P], i),
            "fb_batch_run_host": ([P, P, P, P, P], i),
            "fb_batch_enqueue_host": ([P, P, P, P, P], i),
            "fb_batch_knobs_of": ([P, ctypes.POINTER(BatchKnobs)], i),
            "fb_batch_status": ([P, P, ctypes.POINTER(i)], i),
            "fb_workspace_status": ([P, P, ctypes.POINTER(i)], i),
            "fb_batch_info": ([P, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(sz)], i),
            "fb_batch_destroy": ([P], None),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
        return L


def check(rc, what="fastbarnes_gb300"):
    if rc != FB_OK:
        msg = lib().fb_last_error().decode(errors="replace")
        raise FastBarnesError(f"{what} failed (status {rc}): {msg}")


def version():
    return lib().fb_version().decode()


# ---------------------------------------------------------------------------
# device plumbing (torch provides device memory and the current stream)
# ---------------------------------------------------------------------------

def torch_cuda():
    import torch
    if not torch.cuda.is_available():
        raise FastBarnesError("no CUDA device available (fastbarnes_gb300 has no CPU fallback)")
    return torch


def workspace(nbytes, device):
    """A uint8 device buffer of at least nbytes on `device` for one call.

    Every call gets its own buffer from torch's caching allocator, which is
    stream-ordered: a freed block is handed out again only to work on the
    stream it was allocated on (after that stream's earlier work), so calls
    from several host threads or on several torch streams never share
    scratch memory.  After the first call of a size the allocation is a cache
    hit (no cudaMalloc)."""
    torch = torch_cuda()
    return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=device)


class _PinnedPool:
    """Page-locked host buffers (fb_host_alloc) for numpy results: a result
    array wraps one buffer, so the device-to-host copy is one DMA straight
    into it; when the array is freed the buffer returns here (up to
    `keep` free buffers are cached, the rest released)."""

    def __init__(self, keep=4):
        self.keep = keep
        self.free = {}
        self.lock = threading.Lock()

    def empty(self, shape, dtype):
        import weakref
        import numpy as np
        dtype = np.dtype(dtype)
        nbytes = max(int(np.prod(shape)) * dtype.itemsize, 16)
        with self.lock:
            bucket = self.free.get(nbytes)
            ptr = bucket.pop() if bucket else None
        if ptr is None:
            ptr = lib().fb_host_alloc(nbytes)
            if not ptr:
                raise FastBarnesError(f"fb_host_alloc({nbytes}) failed")
        buf = (ctypes.c_char * nbytes).from_address(ptr)
        arr = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
        weakref.finalize(buf, self._put, ptr, nbytes)
        return arr

    def _put(self, ptr, nbytes):
        with self.lock:
            bucket = self.free.setdefault(nbytes, [])
            if sum(len(b) for b in self.free.values()) < self.keep:
                bucket.append(ptr)
                return
        lib().fb_host_free(ptr)


pinned = _PinnedPool()


def stream_ptr(torch, device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def dvec(values, ctype=ctypes.c_double):
    arr = (ctype * len(values))(*values)
    return arr
