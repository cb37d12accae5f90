"""GPU parity of the batched form (fb_batch_*): every field of a batch equals
the single-field call on it, and the oracle within the stated tolerances.

Tolerances: a batch runs the same kernels' arithmetic per field as the
single-field path with the same launch shape, so with equal knobs the two are
compared for exact equality (NaN positions included); against the oracle the
FP64 form is within 1e-9 * max(|ref|, range(val)) and the FP32C form within
1e-5 relative max error (see test_gpu_parity.py).
"""
import numpy as np
import pytest

from fastbarnes_gb300 import interpolation as I
from fastbarnes_gb300.batched import BatchPlan, barnes_batch
from oracle import oracle

from test_gpu_parity import check_fp32c, check_fp64

pytestmark = pytest.mark.gpu


def uneven_fields(torch, seed=7):
    """Fields of different grids, sigma, n, sample counts and methods,
    including a 20000-cell row that the x axis must tile."""
    rng = np.random.default_rng(seed)
    specs = [
        dict(N=6000, sigma=1.0, x0=(-26.0, 34.5), step=1 / 32, size=(1200, 600), n=4, method="optimized_convolution"),
        dict(N=300, sigma=0.4, x0=(0.0, 0.0), step=0.1, size=(130, 90), n=3, method="optimized_convolution"),
        dict(N=2500, sigma=(0.01, 0.004), x0=(0.0, 0.0), step=1e-3, size=(20000, 64), n=3,
             method="optimized_convolution"),
        dict(N=4000, sigma=0.8, x0=(-5.0, -3.0), step=(0.05, 0.04), size=(400, 350), n=5, method="convolution"),
        dict(N=1, sigma=0.3, x0=(0.0, 0.0), step=0.1, size=(40, 30), n=4, method="optimized_convolution"),
    ]
    fields, host = [], []
    for s in specs:
        size = s["size"]
        step = np.broadcast_to(np.asarray(s["step"], float), (2,))
        lo = np.asarray(s["x0"]) - 2 * step
        hi = np.asarray(s["x0"]) + step * (np.asarray(size) + 2)
        pts = rng.uniform(lo, hi, (s["N"], 2))
        val = 50 + 10 * np.sin(pts[:, 0] * 3) + rng.normal(0, 1, s["N"])
        host.append((pts, val, s))
        fields.append(dict(pts=torch.as_tensor(pts, device="cuda"), val=torch.as_tensor(val, device="cuda"),
                           sigma=s["sigma"], x0=s["x0"], step=s["step"], size=size, num_iter=s["n"],
                           method=s["method"]))
    return fields, host


def same(a, b):
    """Exact equality, NaN positions included; the message says how they differ."""
    if np.array_equal(a, b, equal_nan=True):
        return True, ""
    na, nb = np.isnan(a), np.isnan(b)
    m = ~na & ~nb
    d = np.abs(a[m] - b[m])
    idx = np.argwhere((np.abs(np.nan_to_num(a) - np.nan_to_num(b)) > 0) | (na != nb))
    return False, (f"{int(np.sum(na != nb))} NaN mismatches, {int(np.sum(d > 0))} differing values, "
                   f"max diff {float(d.max()) if d.size else 0.0:.3e}, first at {idx[:3].tolist()}")


def single(pts, val, s, precision, out_dtype=np.float64):
    return I.barnes(pts, val, s["sigma"], s["x0"], s["step"], s["size"], method=s["method"], num_iter=s["n"],
                    precision=precision, out_dtype=out_dtype)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("graph", [False, True])
def test_batch_equals_single(precision, graph):
    import torch
    fields, host = uneven_fields(torch)
    plan = BatchPlan(fields, precision=precision, out_dtype=np.float64, graph=graph)
    for rep in range(2):
        outs = [o.cpu().numpy() for o in plan.run()]
        for (pts, val, s), o in zip(host, outs):
            ref = single(pts, val, s, precision)
            assert o.shape == ref.shape
            ok, msg = same(o, ref)
            assert ok, (s, rep, msg)
    plan.close()


def test_batch_refill_inputs():
    """New data written into the plan's input tensors is picked up by the
    next run (graph replay included)."""
    import torch
    fields, host = uneven_fields(torch, seed=8)
    plan = BatchPlan(fields, precision="fp32c", out_dtype=np.float64, graph=True)
    plan.run()
    rng = np.random.default_rng(99)
    for k, (pts, val, s) in enumerate(host):
        nv = val[::-1].copy() + rng.normal(0, 1, len(val))
        plan.val[k].copy_(torch.as_tensor(nv))
        host[k] = (pts, nv, s)
    outs = [o.cpu().numpy() for o in plan.run()]
    for (pts, val, s), o in zip(host, outs):
        ok, msg = same(o, single(pts, val, s, "fp32c"))
        assert ok, (s, msg)
    plan.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_batch_vs_oracle(precision):
    import torch
    fields, host = uneven_fields(torch, seed=9)
    outs = barnes_batch(fields, precision=precision, out_dtype=np.float64)
    outs32 = barnes_batch(fields, precision=precision)
    for (pts, val, s), q, q32 in zip(host, outs, outs32):
        ref_out, ref_q, wg, thr = oracle.interpolate(pts, val, s["sigma"], s["x0"], s["step"], s["size"], s["n"],
                                                     method=s["method"], nthreads=8)
        q = q.cpu().numpy()
        if precision == "fp64":
            check_fp64(q, q32.cpu().numpy(), ref_q, ref_out, wg, thr, val)
        else:
            check_fp32c(q, ref_q, wg, thr)


def test_batch_headline_shape_knobs_and_tuning():
    """Three 1024 x 512 fields with a window wider than 65 cells: every pinned
    launch shape and the tuned one stay within the FP32C bound of the oracle
    and agree with the single-field call for equal knobs.  The plan launches
    7 kernels: bin keys, the bin-start scan (one block for 1536 bins),
    scatter, two bin sorts, and one launch per axis."""
    import torch
    rng = np.random.default_rng(4)
    B, N = 3, 20000
    size, step, x0, sigma = (1024, 512), 1 / 64, (0.0, 0.0), 1.0
    host = []
    for b in range(B):
        pts = rng.uniform(0, [16, 8], (N, 2))
        val = 280 + 15 * np.cos(pts[:, 0] / 3 + b) + rng.normal(0, 1, N)
        host.append((pts, val))
    fields = [dict(pts=torch.as_tensor(p, device="cuda"), val=torch.as_tensor(v, device="cuda"), sigma=sigma, x0=x0,
                   step=step, size=size, num_iter=4) for p, v in host]
    refs = [oracle.interpolate(p, v, sigma, x0, step, size, 4, nthreads=8) for p, v in host]
    seen = set()
    for knobs in ((17, 128), (33, 256), (33, 512), (33, 128, 1), None):
        plan = BatchPlan(fields, precision="fp32c", out_dtype=np.float64, graph=True, tune=knobs is None,
                         knobs=knobs)
        got = plan.knobs
        assert got[0] in (17, 33) and got[1] in (128, 256, 512)
        seen.add(got)
        outs = [o.cpu().numpy() for o in plan.run()]
        for (p, v), (ref_out, ref_q, wg, thr), o in zip(host, refs, outs):
            check_fp32c(o, ref_q, wg, thr)
        launches, memsets, nbytes = plan.info
        # keys with the bin-start scan, scatter, bin sort, x axis, y axis;
        # one memset (field headers)
        assert launches == 5 and memsets == 1 and nbytes > 0
        plan.close()
    assert len(seen) >= 3


def test_many_uneven_fields_one_launch_per_variant():
    """Forty fields of random grids, sample counts and sigma (some narrow
    enough for direct sums, some wide): every field equals its single call,
    and the plan needs one launch per kernel variant and stage."""
    import torch
    rng = np.random.default_rng(12)
    grids = ((96, 64), (256, 128), (300, 200), (512, 256))
    fields, host = [], []
    for k in range(40):
        W, H = grids[rng.integers(len(grids))]
        N = int(rng.integers(50, 3000))
        step = 1.0 / 16
        sigma = float(rng.uniform(0.15, 1.2))
        n = int(rng.choice([3, 4, 5]))
        pts = rng.uniform([-0.5, -0.5], [W * step + 0.5, H * step + 0.5], (N, 2))
        val = 20 * np.cos(pts[:, 0]) + rng.normal(0, 1, N)
        s = dict(sigma=sigma, x0=(0.0, 0.0), step=step, size=(W, H), n=n, method="optimized_convolution")
        host.append((pts, val, s))
        fields.append(dict(pts=torch.as_tensor(pts, device="cuda"), val=torch.as_tensor(val, device="cuda"),
                           sigma=sigma, x0=(0.0, 0.0), step=step, size=(W, H), num_iter=n))
    for precision in ("fp32c", "fp64"):
        plan = BatchPlan(fields, precision=precision, out_dtype=np.float64, graph=True)
        launches, _, _ = plan.info
        assert launches <= 8 + 2 * 3, launches   # sort kernels + at most 3 variants per stage
        outs = [o.cpu().numpy() for o in plan.run()]
        for (pts, val, s), o in zip(host, outs):
            ok, msg = same(o, single(pts, val, s, precision))
            assert ok, (s, msg)
        plan.close()


def test_homogeneous_fields_shared_and_mixed_launches_agree():
    import torch
    rng = np.random.default_rng(13)
    fields = []
    for b in range(3):
        pts = rng.uniform(0, [16, 8], (5000, 2))
        val = rng.normal(0, 1, 5000)
        fields.append(dict(pts=torch.as_tensor(pts, device="cuda"), val=torch.as_tensor(val, device="cuda"),
                           sigma=0.5, x0=(0.0, 0.0), step=1 / 32, size=(512, 256), num_iter=4))
    a = BatchPlan(fields, precision="fp32c", out_dtype=np.float64, knobs=(0, 256, 0))
    b = BatchPlan(fields, precision="fp32c", out_dtype=np.float64, knobs=(0, 256, 1))
    oa = [o.cpu().numpy() for o in a.run()]
    ob = [o.cpu().numpy() for o in b.run()]
    for x, y in zip(oa, ob):
        ok, msg = same(x, y)
        assert ok, msg


def test_host_buffer_batch_matches_device_run():
    """fb_batch_run_host (samples copied in, results copied out over several
    streams in 16 MiB pieces) gives the device run's results."""
    import ctypes
    import torch
    from fastbarnes_gb300 import _lib
    fields, host = uneven_fields(torch, seed=14)
    plan = BatchPlan(fields, precision="fp32c", graph=True)
    ref = [o.cpu().numpy() for o in plan.run()]
    L = _lib.lib()
    n = len(host)
    h_pts = [np.ascontiguousarray(p, np.float64) for p, _, _ in host]
    h_val = [np.ascontiguousarray(v[::-1] * 1.5, np.float64) for _, v, _ in host]   # new values
    outs = [np.full((s["size"][1], s["size"][0]), -7.0, np.float32) for _, _, s in host]
    a_pts = (ctypes.c_void_p * n)(*[p.ctypes.data for p in h_pts])
    a_val = (ctypes.c_void_p * n)(*[v.ctypes.data for v in h_val])
    a_out = (ctypes.c_void_p * n)(*[o.ctypes.data for o in outs])
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(L.fb_batch_run_host(plan._h, a_pts, a_val, a_out, sp), "fb_batch_run_host")
    for k, (pts, _, s) in enumerate(host):
        exp_ = I.barnes(pts, h_val[k], s["sigma"], s["x0"], s["step"], s["size"], method=s["method"],
                        num_iter=s["n"], precision="fp32c")
        assert np.array_equal(outs[k], exp_, equal_nan=True), k
    # the device tensors now hold the new inputs' results too
    assert np.array_equal(plan.outs[0].cpu().numpy(), outs[0], equal_nan=True)
    assert not np.array_equal(ref[0], outs[0], equal_nan=True)
    plan.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_batch_with_empty_and_all_skipped_fields(precision):
    """Every field's bins cover its own range of sample slots (its rows plus
    one bin for the samples the reference skips): fields without samples
    (through the C ABI; the Python front door refuses them like the
    reference's empty np.amin), a field whose samples all lie outside its
    grid and a field with a single sample sit between ordinary ones, and
    every field still equals its own single-field call; fields without
    weight anywhere come out all NaN."""
    import ctypes
    import torch
    from fastbarnes_gb300 import _lib
    rng = np.random.default_rng(21)
    specs = [
        dict(N=3000, sigma=1.0, x0=(0.0, 0.0), step=0.05, size=(300, 200)),
        dict(N=0, sigma=1.0, x0=(0.0, 0.0), step=0.05, size=(260, 180)),
        dict(N=500, sigma=0.7, x0=(0.0, 0.0), step=0.05, size=(240, 160), outside=True),
        dict(N=1, sigma=0.6, x0=(1.0, 1.0), step=0.05, size=(200, 150)),
        dict(N=2000, sigma=0.9, x0=(-2.0, 3.0), step=0.04, size=(320, 240)),
        dict(N=0, sigma=0.5, x0=(0.0, 0.0), step=0.05, size=(120, 100)),
    ]
    L = _lib.lib()
    arr = (_lib.Field2D * len(specs))()
    keep, host = [], []
    for k, s in enumerate(specs):
        size, step, x0 = np.asarray(s["size"]), s["step"], np.asarray(s["x0"])
        if s.get("outside"):
            pts = x0 + step * np.c_[rng.uniform(size[0] + 1, size[0] + 50, s["N"]), rng.uniform(0, size[1], s["N"])]
        else:
            pts = x0 + step * rng.uniform(0, size - 1, (s["N"], 2))
        val = 20 + 5 * np.cos(pts.sum(axis=1)) + rng.normal(0, 1, s["N"])
        tp = torch.as_tensor(pts.reshape(-1, 2), device="cuda").contiguous()
        tv = torch.as_tensor(val, device="cuda").contiguous()
        out = torch.empty((int(size[1]), int(size[0])), dtype=torch.float64, device="cuda")
        keep += [tp, tv, out]
        host.append((pts, val, s, out))
        F = arr[k]
        F.pts = tp.data_ptr() if s["N"] else None
        F.val = tv.data_ptr() if s["N"] else None
        F.n_pts = s["N"]
        for m in range(2):
            F.sigma[m], F.x0[m], F.step[m], F.size[m] = float(s["sigma"]), float(x0[m]), float(step), int(size[m])
        F.num_iter = 4
        F.max_dist_weight = np.exp(-3.5 ** 2 / 2)
        F.method = _lib.FB_OPTIMIZED_CONVOLUTION
        F.out = out.data_ptr()
    prec = _lib.PRECISIONS[precision]
    h = ctypes.c_void_p()
    _lib.check(L.fb_batch_create(prec, arr, len(specs), 1, _lib.FB_BATCH_GRAPH, None, ctypes.byref(h)),
               "fb_batch_create")
    try:
        for rep in range(2):
            _lib.check(L.fb_batch_run(h, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "fb_batch_run")
            torch.cuda.synchronize()
            for pts, val, s, out in host:
                o = out.cpu().numpy()
                if s["N"] == 0 or s.get("outside"):
                    assert np.isnan(o).all(), (s, rep)
                    continue
                ref = I.barnes(pts, val, s["sigma"], s["x0"], s["step"], s["size"], num_iter=4,
                               precision=precision, out_dtype=np.float64)
                ok, msg = same(o, ref)
                assert ok, (s, rep, msg)
    finally:
        L.fb_batch_destroy(h)
    with pytest.raises(ValueError):
        BatchPlan([dict(pts=np.zeros((0, 2)), val=np.zeros(0), sigma=1.0, x0=(0.0, 0.0), step=0.05,
                        size=(100, 100))])
