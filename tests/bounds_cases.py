"""A fixed set of small interpolations run with whichever build of the
library FASTBARNES_GB300_LIB selects; the results go to the .npz file named on
the command line.  tests/test_gpu_bounds_check.py runs this once with the
bounds-check build and once with the normal one.  Every case checks the
device status word (the host-buffer entry does so itself; batches through
fb_batch_status), so an index the bounds-check build found out of range
fails the run."""
import ctypes
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "fast-barnes-py_gb300"))

import numpy as np  # noqa: E402
import torch  # noqa: E402

from fastbarnes_gb300 import _lib  # noqa: E402
from fastbarnes_gb300 import interpolation as I  # noqa: E402
from fastbarnes_gb300.batched import BatchPlan  # noqa: E402


def main(path):
    torch.cuda.set_device(0)
    L = _lib.lib()
    rng = np.random.default_rng(77)
    out = {"version": np.array(_lib.version())}
    # 2D: the reference example's shape, both precisions and methods, both
    # column kernels
    n = 3490
    pts = np.c_[rng.uniform(-26, 49, n), rng.uniform(34.5, 72, n)]
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) + rng.normal(0, 2, n)
    for prec in ("fp64", "fp32c"):
        for pipe in (1, 0):
            _lib.check(L.fb_tune(b"cols_pipe", pipe))
            for method in ("optimized_convolution", "convolution"):
                out[f"2d_{prec}_{method}_{pipe}"] = I.barnes(pts, val, 1.0, (-26.0, 34.5), 1 / 32, (2400, 1200),
                                                             method=method, precision=prec,
                                                             out_dtype=np.float64)
    _lib.check(L.fb_tune(b"cols_pipe", 2))
    # the headline field's shape (33-cell chunks), direct sums (T <= 8), 1D, 3D
    n = 100_000
    pts = np.c_[rng.uniform(-26, 49, n), rng.uniform(34.5, 72, n)]
    val = 1000 + rng.normal(0, 2, n)
    out["headline_fp32c"] = I.barnes(pts, val, 1.0, (-26.0, 34.5), (75 / 4096, 37.5 / 2048), (4096, 2048),
                                     precision="fp32c")
    out["direct_fp64"] = I.barnes(pts[:5000], val[:5000], 0.1, (-26.0, 34.5), 0.05, (400, 300))
    p1 = rng.uniform(0, 100, 20_000)
    out["1d_fp64"] = I.barnes(p1, np.sin(p1) + rng.normal(0, 0.1, len(p1)), 0.5, 0.0, 1 / 64, 6400,
                              out_dtype=np.float64)
    p3 = rng.uniform(0, 40, (20_000, 3))
    out["3d_fp32c"] = I.barnes(p3, p3.sum(axis=1), 2.0, (0.0, 0.0, 0.0), (0.5, 0.5, 0.5), (80, 80, 80),
                               precision="fp32c")
    # a batch of three fields (mixed launch shapes), status checked
    dev = torch.device("cuda", 0)
    fields = []
    for f in range(3):
        q = rng.uniform(0, [16, 8], (20_000, 2))
        fields.append(dict(pts=torch.as_tensor(q, device=dev), val=torch.as_tensor(np.cos(q[:, 0]), device=dev),
                           sigma=0.3 + 0.2 * f, x0=(0.0, 0.0), step=1 / 64, size=(1024, 512)))
    plan = BatchPlan(fields, precision="fp32c", graph=False, device=dev)
    outs = plan.run()
    st = ctypes.c_int(0)
    _lib.check(L.fb_batch_status(plan._h, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream),
                                 ctypes.byref(st)), "fb_batch_status")
    for f, o in enumerate(outs):
        out[f"batch_{f}"] = o.cpu().numpy()
    plan.close()
    np.savez(path, **out)


if __name__ == "__main__":
    main(sys.argv[1])
