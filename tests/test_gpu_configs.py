"""The benchmark configurations at their full sizes, through properties that do
not need a CPU result of the same size, plus the oracle where it finishes in
seconds.

- Sweep (2D grids up to 16384 x 8192, N up to 1M, uniform and 3-cluster
  locations, sigma 0.5 / 1 / 4 grid-degrees, n 3 / 4 / 6): the FP32C form
  within 1e-5 relative max error of the FP64 form (the stated tolerance), NaN
  masks equal except within 1e-4 of the mask level.
- Batched: 512 fields of uneven grids, N and sigma in one plan; a sample of the
  fields equals the single calls bit for bit.
- 1D L = 2^26, N = 4M: FP64 against the oracle on sub-lines (1e-9 relative
  to the value range) and on the whole line (1e-7: the reference's single
  running sum drifts over 2^26 cells), FP32C against FP64 (1e-5).
- 3D 512 x 512 x 256, N = 2M: FP64 against the oracle on the whole volume
  (1e-9), FP32C against FP64 (1e-5); a constant field stays constant wherever
  it is not masked (exact property of V / W).
"""
import numpy as np
import pytest

from fastbarnes_gb300 import interpolation as I
from fastbarnes_gb300.batched import BatchPlan
from oracle import oracle

pytestmark = pytest.mark.gpu


def rel_err(a, b):
    m = ~np.isnan(a) & ~np.isnan(b)
    return float(np.max(np.abs(a[m] - b[m])) / np.max(np.abs(b[m])))


def check_fp64_vs_oracle(q64, out32, ref_out, ref_q, wg, thr, val):
    """The float64 quotient within 1e-9 of max(|ref|, range(val)); the float32
    result within 1 ulp plus that float64 tolerance (where values cross zero a
    float32 ulp is far below it, and rounding two float64 values to float32
    keeps them within their distance plus an ulp); NaN masks equal but where
    the weight is within 1e-9 of the mask level."""
    diff = np.isnan(q64) != np.isnan(ref_q)
    assert np.all(np.abs(wg[diff] - thr) <= 1e-9 * abs(thr))
    m = ~np.isnan(q64) & ~np.isnan(ref_q)
    assert m.any()
    scale = np.maximum(np.abs(ref_q[m]), np.ptp(val))
    assert np.max(np.abs(q64[m] - ref_q[m]) / scale) <= 1e-9
    m32 = ~np.isnan(out32) & ~np.isnan(ref_out)
    tol32 = np.spacing(np.abs(ref_out[m32])).astype(np.float64) + 1e-9 * np.maximum(np.abs(ref_q[m32]), np.ptp(val))
    assert np.all(np.abs(out32[m32].astype(np.float64) - ref_out[m32]) <= tol32)


def locations(rng, N, kind):
    if kind == "uniform":
        return np.c_[rng.uniform(-26, 49, N), rng.uniform(34.5, 72, N)]
    c = rng.uniform([-20, 40], [40, 65], (3, 2))
    s = rng.uniform(3, 8, 3)
    lab = rng.integers(0, 3, N)
    return c[lab] + rng.normal(0, 1, (N, 2)) * s[lab][:, None]


@pytest.mark.parametrize("W,H", [(1024, 512), (4096, 2048), (16384, 8192)])
def test_sweep_fp32c_within_tolerance(W, H):
    import torch
    rng = np.random.default_rng(W)
    x0, step = (-26.0, 34.5), (75.0 / W, 37.5 / H)
    worst = 0.0
    for N, kind, sigma, n in ((10_000, "uniform", 0.5, 3), (100_000, "cluster", 1.0, 4),
                              (1_000_000, "uniform", 4.0, 6), (1_000_000, "cluster", 1.0, 3)):
        pts = locations(rng, N, kind)
        val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
        tp = torch.as_tensor(pts, device="cuda")
        tv = torch.as_tensor(val, device="cuda")
        if 2 * int(I.get_half_kernel_size_opt(sigma, step[1], n)) + 1 >= H:
            continue
        q64 = I.barnes(tp, tv, sigma, x0, step, (W, H), num_iter=n, out_dtype=np.float64).cpu().numpy()
        q32 = I.barnes(tp, tv, sigma, x0, step, (W, H), num_iter=n, out_dtype=np.float64,
                       precision="fp32c").cpu().numpy()
        mism = np.isnan(q64) != np.isnan(q32)
        assert mism.sum() <= 1e-6 * q64.size, int(mism.sum())
        e = rel_err(q32, q64)
        worst = max(worst, e)
        assert e <= 1e-5, (N, kind, sigma, n, e)
    assert worst > 0.0


def test_sweep_full_factorial_fp32c_4096x2048():
    """All 54 combinations of N {10k, 100k, 1M} x {uniform, 3-cluster} x
    sigma {0.5, 1, 4} degrees x n {3, 4, 6} on the 4096 x 2048 grid: the
    FP32C form within 1e-5 relative max error of the FP64 form, masks equal
    but for at most 1e-6 of the points."""
    import torch
    W, H = 4096, 2048
    rng = np.random.default_rng(2048)
    x0, step = (-26.0, 34.5), (75.0 / W, 37.5 / H)
    worst = 0.0
    for N in (10_000, 100_000, 1_000_000):
        for kind in ("uniform", "cluster"):
            pts = locations(rng, N, kind)
            val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
            tp = torch.as_tensor(pts, device="cuda")
            tv = torch.as_tensor(val, device="cuda")
            for sigma in (0.5, 1.0, 4.0):
                for n in (3, 4, 6):
                    q64 = I.barnes(tp, tv, sigma, x0, step, (W, H), num_iter=n, out_dtype=np.float64)
                    q32 = I.barnes(tp, tv, sigma, x0, step, (W, H), num_iter=n, out_dtype=np.float64,
                                   precision="fp32c")
                    nan64, nan32 = torch.isnan(q64), torch.isnan(q32)
                    assert int((nan64 != nan32).sum()) <= 1e-6 * W * H, (N, kind, sigma, n)
                    both = ~nan64 & ~nan32
                    e = float((q32[both] - q64[both]).abs().max() / q64[both].abs().max())
                    worst = max(worst, e)
                    assert e <= 1e-5, (N, kind, sigma, n, e)
    assert worst > 0.0


@pytest.mark.parametrize("W,H,N", [(4096, 2048, 100_000), (16384, 8192, 1_000_000)])
def test_full_grids_vs_oracle(W, H, N):
    """The headline field (4096 x 2048, N = 100k) and the sweep's largest grid
    (16384 x 8192, N = 1M), uniform samples, sigma = 1 degree, n = 4: FP64
    against the oracle over the whole grid, FP32C within 1e-5 relative of the
    oracle (masks equal but within 1e-4 of the mask level)."""
    import torch
    rng = np.random.default_rng(W + N)
    x0, step, sigma, n = (-26.0, 34.5), (75.0 / W, 37.5 / H), 1.0, 4
    pts = locations(rng, N, "uniform")
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
    tp, tv = torch.as_tensor(pts, device="cuda"), torch.as_tensor(val, device="cuda")
    ref_out, ref_q, wg, thr = oracle.interpolate(pts, val, sigma, np.array(x0), np.array(step), (W, H), n,
                                                 nthreads=16)
    q64 = I.barnes(tp, tv, sigma, x0, step, (W, H), num_iter=n, out_dtype=np.float64).cpu().numpy()
    out32 = I.barnes(tp, tv, sigma, x0, step, (W, H), num_iter=n).cpu().numpy()
    check_fp64_vs_oracle(q64, out32, ref_out, ref_q, wg, thr, val)
    del q64, out32
    q32 = I.barnes(tp, tv, sigma, x0, step, (W, H), num_iter=n, out_dtype=np.float64,
                   precision="fp32c").cpu().numpy()
    diff = np.isnan(q32) != np.isnan(ref_q)
    assert np.all(np.abs(wg[diff] - thr) <= 1e-4 * abs(thr))
    assert rel_err(q32, ref_q) <= 1e-5


def test_batch_of_512_uneven_fields():
    import torch
    rng = np.random.default_rng(512)
    grids = ((256, 256), (1024, 512), (2048, 1024))
    fields, host = [], []
    for k in range(512):
        W, H = grids[rng.integers(3)]
        N = int(np.exp(rng.uniform(np.log(500), np.log(50000))))
        step = 1.0 / 64
        sigma = float(rng.uniform(0.5, 4.0)) * step
        pts = rng.uniform([0, 0], [W * step, H * step], (N, 2))
        ph = rng.uniform(0, 2 * np.pi, 8)
        val = sum(np.sin(pts[:, 0] * (q + 1) + ph[q]) for q in range(8)) + rng.normal(0, 1, N)
        host.append((pts, val, sigma, step, (W, H)))
        fields.append(dict(pts=torch.as_tensor(pts, device="cuda"), val=torch.as_tensor(val, device="cuda"),
                           sigma=sigma, x0=(0.0, 0.0), step=step, size=(W, H), num_iter=4))
    plan = BatchPlan(fields, precision="fp32c", out_dtype=np.float64, graph=True)
    launches, _, _ = plan.info
    assert launches <= 8 + 2 * 3
    outs = plan.run()
    torch.cuda.synchronize()
    for k in rng.choice(512, 12, replace=False):
        pts, val, sigma, step, size = host[k]
        ref = I.barnes(pts, val, sigma, (0.0, 0.0), step, size, num_iter=4, precision="fp32c",
                       out_dtype=np.float64)
        assert np.array_equal(outs[k].cpu().numpy(), ref, equal_nan=True), k
    plan.close()


def test_1d_full_length():
    """L = 2^26 cells, N = 4M.  The reference carries one running sum along the
    whole line, so its float64 rounding grows with the line; the GPU's sums
    are re-anchored every few cells.  The truth is the same interpolation with
    every pass summed directly over each output's window (no rounding carried
    between outputs; oracle direct=True).  Asserted over the whole line: the
    GPU float64 result is within 1e-9 of the value range of the truth, the
    reference's own deviation from the truth is the larger of the two, and
    FP32C is within 1e-5 of FP64.  The GPU also equals the reference's loops
    on short sub-lines cut around several windows (samples within the window
    and a margin; the passes only reach n (T + 1) cells, so the window's
    interior is unaffected by the cut) to 1e-9 of the value range."""
    import torch
    rng = np.random.default_rng(26)
    L, N = 2 ** 26, 4_000_000
    step = 1.0 / 1024
    sigma, n = 0.01, 4
    pts = rng.uniform(0, L * step, N)
    val = rng.normal(10.0, 3.0, N)
    tp, tv = torch.as_tensor(pts, device="cuda"), torch.as_tensor(val, device="cuda")
    q64 = I.barnes(tp, tv, sigma, 0.0, step, L, num_iter=n, out_dtype=np.float64).cpu().numpy()
    q32 = I.barnes(tp, tv, sigma, 0.0, step, L, num_iter=n, out_dtype=np.float64, precision="fp32c").cpu().numpy()
    assert rel_err(q32, q64) <= 1e-5
    _, ref, _, _ = oracle.interpolate(pts, val, sigma, 0.0, step, L, n, nthreads=8)
    _, truth, _, _ = oracle.interpolate(pts, val, sigma, 0.0, step, L, n, nthreads=16, direct=True)
    assert np.array_equal(np.isnan(q64), np.isnan(truth))
    m = ~np.isnan(truth) & ~np.isnan(ref)
    gpu_dev = float(np.max(np.abs(q64[m] - truth[m])))
    ref_dev = float(np.max(np.abs(ref[m] - truth[m])))
    assert gpu_dev <= 1e-9 * np.ptp(val), gpu_dev
    assert ref_dev >= gpu_dev, (ref_dev, gpu_dev)
    # the offset is the full sample set's, so sub-lines get one extra sample
    # at each extreme value far away from the window (outside the sub-grid)
    lo, hi = int(np.argmin(val)), int(np.argmax(val))
    reach = n * (int(I.get_half_kernel_size_opt(sigma, step, n)) + 1) + 2
    for c0 in (1000, L // 3, L // 2 + 12345, L - 30000):
        a, b = c0, c0 + 20000
        sel = (pts >= (a - 2 * reach) * step) & (pts < (b + 2 * reach) * step)
        sub_pts = np.r_[pts[sel] - (a - 2 * reach) * step, -10.0, -10.0]
        sub_val = np.r_[val[sel], val[lo], val[hi]]
        sub_len = b - a + 4 * reach
        _, sref, _, _ = oracle.interpolate(sub_pts, sub_val, sigma, 0.0, step, sub_len, n)
        mine = q64[a - 2 * reach + reach:b + 2 * reach - reach]
        theirs = sref[reach:sub_len - reach]
        mm = ~np.isnan(theirs)
        assert np.array_equal(np.isnan(mine), np.isnan(theirs)), c0
        assert np.max(np.abs(mine[mm] - theirs[mm])) <= 1e-9 * np.ptp(val), c0


def test_3d_full_size_and_constant_field():
    import torch
    rng = np.random.default_rng(33)
    N = 2_000_000
    c = rng.uniform([0.1, 0.1, 0.1], [0.9, 0.9, 0.9], (8, 3))
    lab = rng.integers(0, 8, N)
    pts = c[lab] + rng.normal(0, 0.08, (N, 3))
    val = rng.normal(0, 1, N) + pts[:, 0]
    size = (512, 512, 256)
    step = (1 / 512, 1 / 512, 1 / 256)
    sigma = (3 / 512, 3 / 512, 3 / 256)
    tp, tv = torch.as_tensor(pts, device="cuda"), torch.as_tensor(val, device="cuda")
    q64 = I.barnes(tp, tv, sigma, (0, 0, 0), step, size, num_iter=4, out_dtype=np.float64)
    q32 = I.barnes(tp, tv, sigma, (0, 0, 0), step, size, num_iter=4, out_dtype=np.float64, precision="fp32c")
    a, b = q32.cpu().numpy(), q64.cpu().numpy()
    assert rel_err(a, b) <= 1e-5
    # FP64 against the oracle on the whole volume
    ref_out, ref_q, wg, thr = oracle.interpolate(pts, val, np.array(sigma), np.zeros(3), np.array(step), size, 4,
                                                 nthreads=16)
    out32 = I.barnes(tp, tv, sigma, (0, 0, 0), step, size, num_iter=4).cpu().numpy()
    check_fp64_vs_oracle(b, out32, ref_out, ref_q, wg, thr, val)
    del ref_out, ref_q, wg, out32
    const = torch.full_like(tv, 7.25)
    for prec in ("fp64", "fp32c"):
        f = I.barnes(tp, const, sigma, (0, 0, 0), step, size, num_iter=4, out_dtype=np.float64,
                     precision=prec).cpu().numpy()
        m = ~np.isnan(f)
        assert m.any()
        assert np.all(f[m] == 7.25), prec


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
@pytest.mark.parametrize("knobs", ["pinned", "tuned"])
def test_headline_batch_plan_vs_oracle(precision, knobs):
    """The benchmark's own plan: 8 fields of 4096 x 2048, N = 100k, sigma =
    1 deg, n = 4 (bench.field_inputs, bench's seeds), with the pinned knobs
    (chunk 33, 128-thread rows) and with the autotuner's choice, every field
    against the oracle: float64 within 1e-9 of max(|ref|, range(val)) (float32
    result within an ulp), fp32c within 1e-5 relative max error, NaN masks
    equal but where the weight lies within 1e-9 (fp64) / 1e-4 (fp32c) of the
    mask level."""
    import torch
    import bench
    dev = torch.device("cuda", 0)
    B = 8
    host = [bench.field_inputs(bench.field_seed(0, f)) for f in range(B)]
    fields = [dict(pts=torch.as_tensor(p, device=dev), val=torch.as_tensor(v, device=dev), sigma=bench.SIGMA,
                   x0=bench.X0, step=bench.STEP, size=(bench.W, bench.H), num_iter=bench.NITER,
                   max_dist=bench.MAX_DIST) for p, v in host]
    kn = (33, 128, 0) if knobs == "pinned" else None
    plan = BatchPlan(fields, precision=precision, out_dtype=np.float64, graph=True, tune=kn is None, knobs=kn,
                     device=dev)
    plan.run()
    plan32 = BatchPlan(fields, precision=precision, graph=True, knobs=plan.knobs, device=dev)
    plan32.run()
    torch.cuda.synchronize()
    for f in range(B):
        pts, val = host[f]
        ref_out, ref_q, wg, thr = oracle.interpolate(pts, val, bench.SIGMA, bench.X0, bench.STEP,
                                                     (bench.W, bench.H), bench.NITER, bench.MAX_DIST, nthreads=16)
        q = plan.outs[f].cpu().numpy()
        if precision == "fp64":
            check_fp64_vs_oracle(q, plan32.outs[f].cpu().numpy(), ref_out, ref_q, wg, thr, val)
        else:
            diff = np.isnan(q) != np.isnan(ref_q)
            assert np.all(np.abs(wg[diff] - thr) <= 1e-4 * abs(thr)), f
            assert rel_err(q, ref_q) <= 1e-5, f
    plan.close()
    plan32.close()
