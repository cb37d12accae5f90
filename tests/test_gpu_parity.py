"""GPU parity: libfastbarnes_gb300 against the reference's own results.

The references are the golden fixtures produced by running the reference
(tests/golden/make_golden.py) and, at larger sizes, the CPU oracle that those
fixtures pin bit for bit (oracle/barnes_oracle.c).

Tolerances (stated here, used below):
  FP64 form   : |gpu - ref| <= 1e-9 * max(|ref|, range(val)) on the float64
                quotient; the float32 result within 1 float32 ulp; NaN masks
                equal except where the weight lies within 1e-9 of the mask level.
  FP32C form  : max |gpu - ref| / max |ref| <= 1e-5 (relative max error against
                the float64 result); NaN masks equal except within 1e-4 of the
                mask level.
"""
import ctypes
import math

import numpy as np
import pytest

from fastbarnes_gb300 import _lib
from fastbarnes_gb300 import interpolation as I
from fastbarnes_gb300 import interpolationS2 as S2
from fastbarnes_gb300.util import lambert_conformal as LC
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL64 = 1e-9
TOL32 = 1e-5


def masks_agree(mine, ref_q, ref_wg, thr, band):
    """NaN masks equal except where the reference weight is within `band`
    (relative) of the mask level."""
    a, b = np.isnan(mine), np.isnan(ref_q)
    diff = a != b
    if not diff.any():
        return True
    near = np.abs(ref_wg - thr) <= band * abs(thr)
    return bool(np.all(near[diff]))


def check_fp64(q, out32, ref_q, ref_out, ref_wg, thr, val):
    assert masks_agree(q, ref_q, ref_wg, thr, 1e-9)
    m = ~np.isnan(q) & ~np.isnan(ref_q)
    if not m.any():
        return 0.0
    scale = np.maximum(np.abs(ref_q[m]), np.ptp(val))
    err = np.abs(q[m] - ref_q[m])
    assert np.all(err <= TOL64 * scale), f"max scaled err {np.max(err / scale):.3e}"
    m32 = ~np.isnan(out32) & ~np.isnan(ref_out)
    ulp = np.spacing(np.abs(ref_out[m32]).astype(np.float32))
    assert np.all(np.abs(out32[m32] - ref_out[m32]) <= ulp)
    return float(np.max(err / scale))


def check_fp32c(q, ref_q, ref_wg, thr):
    assert masks_agree(q, ref_q, ref_wg, thr, 1e-4)
    m = ~np.isnan(q) & ~np.isnan(ref_q)
    if not m.any():
        return 0.0
    rel = float(np.max(np.abs(q[m].astype(np.float64) - ref_q[m])) / np.max(np.abs(ref_q[m])))
    assert rel <= TOL32, f"relative max error {rel:.3e}"
    return rel


def gpu(pts, val, sigma, x0, step, size, n, max_dist=3.5, method="optimized_convolution", precision="fp64",
        out_dtype=np.float32):
    return I.barnes(pts, val, sigma, x0, step, size, method=method, num_iter=n, max_dist=max_dist,
                    precision=precision, out_dtype=out_dtype)


# ---------------------------------------------------------------------------
# 1D passes (the reference's AccumulationTest / GaussianApproximationTest)
# ---------------------------------------------------------------------------

def test_accumulate_golden(golden):
    g = golden("accumulate.npz")
    for k in range(len(g["kind"])):
        L = int(g["length"][k])
        a = g["inp"][k][:L]
        alpha = float(g["alpha"][k]) if g["kind"][k] == 1 else 0.0
        out = I.accumulate_lines(a[None, :], int(g["rect"][k]), int(g["n"][k]), alpha)[0]
        ref = g["out"][k][:L]
        if np.all(np.mod(a * 4, 1) == 0) and alpha in (0.0, 0.25, 0.5, 1.0):
            # impulse inputs of the reference's AccumulationTest: exact
            np.testing.assert_array_equal(out, ref, err_msg=f"case {k}")
        else:
            np.testing.assert_allclose(out, ref, rtol=0, atol=1e-12 * np.max(np.abs(ref)), err_msg=f"case {k}")


def test_accumulate_fp32c_matches_scaled(golden):
    g = golden("accumulate.npz")
    for k in range(len(g["kind"])):
        L = int(g["length"][k])
        a = g["inp"][k][:L]
        rect, n = int(g["rect"][k]), int(g["n"][k])
        alpha = float(g["alpha"][k]) if g["kind"][k] == 1 else 0.0
        out = I.accumulate_lines(a[None, :], rect, n, alpha, precision="fp32c", normalize=True)[0]
        ref = g["out"][k][:L] / (rect + 2 * alpha) ** n
        np.testing.assert_allclose(out, ref, rtol=0, atol=2e-6 * max(np.max(np.abs(ref)), 1e-30))


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_gaussian_convergence(precision):
    """The methodology of the reference's GaussianApproximationTest: a Dirac
    impulse through the n-fold tailed rect kernel approaches the Gaussian."""
    for sigma in (0.6, 0.8, 1.0, 1.5, 2.0):
        for n, max_diff in ((3, 0.02395), (4, 0.01405), (5, 0.012325), (6, 0.010045)):
            delta = 1.0 / 512.0
            width = 3.5 * sigma
            grid = np.arange(-width, width + 0.000001, delta)
            gaussian = np.exp(-(grid / sigma) ** 2 / 2) / math.sqrt(2 * math.pi) / sigma
            values = np.zeros(len(grid))
            values[len(grid) // 2] = 1.0 / delta
            T = I.get_half_kernel_size_opt(sigma, delta, n)
            alpha = I.get_tail_value(sigma, delta, n)
            out = I.accumulate_lines(values[None, :], 2 * int(T) + 1, n, alpha, precision=precision)[0]
            out = out * (delta / 2 / math.sqrt(3 / n) / sigma) ** n
            assert np.max(np.abs(out - gaussian)) <= max_diff / sigma + 1e-6


# ---------------------------------------------------------------------------
# barnes() against the golden fixtures
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("tag", ["opt", "conv"])
def test_barnes_golden_fp64(golden, dim, tag):
    g = golden(f"barnes_{dim}d.npz")
    method = "optimized_convolution" if tag == "opt" else "convolution"
    for c in range(int(g["count"])):
        pts = g[f"c{c}_pts"]
        args = (pts if dim > 1 else pts[:, 0], g[f"c{c}_val"], g[f"c{c}_sigma"], g[f"c{c}_x0"], g[f"c{c}_step"],
                tuple(int(s) for s in g[f"c{c}_size"]), int(g[f"c{c}_n"]), float(g[f"c{c}_max_dist"]), method)
        out32 = gpu(*args)
        q = gpu(*args, out_dtype=np.float64)
        _, _, wg, thr = oracle.interpolate(*args[:-1], method=method)
        check_fp64(q, out32, g[f"c{c}_{tag}_q64"], g[f"c{c}_{tag}_out"], wg, thr, g[f"c{c}_val"])


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_barnes_golden_fp32c(golden, dim):
    g = golden(f"barnes_{dim}d.npz")
    for c in range(int(g["count"])):
        pts = g[f"c{c}_pts"]
        args = (pts if dim > 1 else pts[:, 0], g[f"c{c}_val"], g[f"c{c}_sigma"], g[f"c{c}_x0"], g[f"c{c}_step"],
                tuple(int(s) for s in g[f"c{c}_size"]), int(g[f"c{c}_n"]), float(g[f"c{c}_max_dist"]))
        q = gpu(*args, precision="fp32c", out_dtype=np.float64)
        _, _, wg, thr = oracle.interpolate(*args)
        check_fp32c(q, g[f"c{c}_opt_q64"], wg, thr)


# ---------------------------------------------------------------------------
# larger cases against the oracle
# ---------------------------------------------------------------------------

def config1_inputs(N=3490, seed=1):
    """The reference's CPU-runnable example shape: N samples over the European
    domain, grid 2400 x 1200 at 1/32 degree, sigma 1, n 4."""
    rng = np.random.default_rng(seed)
    lon = rng.uniform(-26, 49, N)
    lat = rng.uniform(34.5, 72, N)
    val = 1000 + 20 * np.sin(lon / 10) * np.cos(lat / 8) + rng.normal(0, 2, N)
    return np.c_[lon, lat], val, 1.0, np.array([-26.0, 34.5]), 1 / 32, (2400, 1200)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_config1_vs_oracle(precision):
    pts, val, sigma, x0, step, size = config1_inputs()
    ref_out, ref_q, wg, thr = oracle.interpolate(pts, val, sigma, x0, step, size, 4, nthreads=8)
    q = gpu(pts, val, sigma, x0, step, size, 4, precision=precision, out_dtype=np.float64)
    if precision == "fp64":
        out32 = gpu(pts, val, sigma, x0, step, size, 4)
        check_fp64(q, out32, ref_q, ref_out, wg, thr, val)
    else:
        check_fp32c(q, ref_q, wg, thr)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_deterministic(precision):
    pts, val, sigma, x0, step, size = config1_inputs(N=20000, seed=5)
    a = gpu(pts, val, sigma, x0, step, size, 4, precision=precision, out_dtype=np.float64)
    b = gpu(pts, val, sigma, x0, step, size, 4, precision=precision, out_dtype=np.float64)
    assert np.array_equal(a, b, equal_nan=True)


def test_clustered_sweep_vs_oracle():
    """Clustered samples, several sigma / n on a 1024 x 512 grid."""
    rng = np.random.default_rng(11)
    N = 30000
    c = rng.uniform([-20, 40], [40, 65], (3, 2))
    s = rng.uniform(3, 8, 3)
    lab = rng.integers(0, 3, N)
    pts = c[lab] + rng.normal(0, 1, (N, 2)) * s[lab][:, None]
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
    x0, size = np.array([-26.0, 34.5]), (1024, 512)
    step = np.array([75.0 / 1024, 37.5 / 512])
    for sigma, n in ((0.5, 3), (1.0, 4), (4.0, 6)):
        ref_out, ref_q, wg, thr = oracle.interpolate(pts, val, sigma, x0, step, size, n, nthreads=8)
        q = gpu(pts, val, sigma, x0, step, size, n, out_dtype=np.float64)
        out32 = gpu(pts, val, sigma, x0, step, size, n)
        check_fp64(q, out32, ref_q, ref_out, wg, thr, val)
        q32 = gpu(pts, val, sigma, x0, step, size, n, precision="fp32c", out_dtype=np.float64)
        check_fp32c(q32, ref_q, wg, thr)


def test_sweep_full_factorial_vs_oracle():
    """Every combination of the 2D precision sweep's parameters on its
    1024 x 512 grid (European domain, step 75/1024 x 37.5/512 degrees): N in
    {10k, 100k, 1M}, uniform or 3-cluster locations, sigma in {0.5, 1, 4}
    degrees, n in {3, 4, 6} -- 54 fields.  The float64 form within 1e-9 of
    the oracle (its float32 result within 1 ulp), the float32-compensated
    form within 1e-5 relative (both modes: sigma = 4, n = 6 at N = 1M grows
    past the float32 limit, so its passes run scaled)."""
    rng = np.random.default_rng(54)
    x0, size = np.array([-26.0, 34.5]), (1024, 512)
    step = np.array([75.0 / 1024, 37.5 / 512])
    worst64 = worst32 = 0.0
    for N in (10_000, 100_000, 1_000_000):
        for kind in ("uniform", "cluster"):
            if kind == "uniform":
                pts = np.c_[rng.uniform(-26, 49, N), rng.uniform(34.5, 72, N)]
            else:
                c = rng.uniform([-20, 40], [40, 65], (3, 2))
                s = rng.uniform(3, 8, 3)
                lab = rng.integers(0, 3, N)
                pts = c[lab] + rng.normal(0, 1, (N, 2)) * s[lab][:, None]
            val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
            for sigma in (0.5, 1.0, 4.0):
                for n in (3, 4, 6):
                    ref_out, ref_q, wg, thr = oracle.interpolate(pts, val, sigma, x0, step, size, n, nthreads=8)
                    q = gpu(pts, val, sigma, x0, step, size, n, out_dtype=np.float64)
                    out32 = gpu(pts, val, sigma, x0, step, size, n)
                    worst64 = max(worst64, check_fp64(q, out32, ref_q, ref_out, wg, thr, val))
                    q32 = gpu(pts, val, sigma, x0, step, size, n, precision="fp32c", out_dtype=np.float64)
                    worst32 = max(worst32, check_fp32c(q32, ref_q, wg, thr))
    assert worst32 > 0.0


def test_3d_vs_oracle():
    rng = np.random.default_rng(21)
    N = 5000
    pts = rng.normal([2.0, 2.0, 1.0], [0.8, 0.6, 0.4], (N, 3))
    val = rng.normal(0, 1, N) + pts[:, 0]
    args = (pts, val, (0.3, 0.3, 0.2), (0.0, 0.0, 0.0), (1 / 16, 1 / 16, 1 / 16), (64, 56, 40), 4)
    ref_out, ref_q, wg, thr = oracle.interpolate(*args, nthreads=8)
    q = gpu(*args, out_dtype=np.float64)
    check_fp64(q, gpu(*args), ref_q, ref_out, wg, thr, val)
    check_fp32c(gpu(*args, precision="fp32c", out_dtype=np.float64), ref_q, wg, thr)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_long_lines_tiled(precision):
    """Lines longer than one CTA's shared memory are cut into tiles with a
    halo of n (T + 1) cells; with a very wide kernel every pass is its own
    launch with a halo of T + 1."""
    rng = np.random.default_rng(3)
    for L, sigma in ((60000, 0.05), (30000, 3.0)):
        N = 4000
        pts = rng.uniform(-1, L / 1000 + 1, N)
        val = rng.normal(10, 3, N)
        args = (pts, val, sigma, 0.0, 1e-3, L, 4)
        ref_out, ref_q, wg, thr = oracle.interpolate(*args)
        q = gpu(*args, precision=precision, out_dtype=np.float64)
        if precision == "fp64":
            check_fp64(q, gpu(*args), ref_q, ref_out, wg, thr, val)
        else:
            check_fp32c(q, ref_q, wg, thr)
    # 2D rows wider than one CTA in float64
    N = 3000
    pts = np.c_[rng.uniform(0, 20, N), rng.uniform(0, 0.064, N)]
    val = rng.normal(0, 1, N)
    args = (pts, val, (0.01, 0.004), (0.0, 0.0), (1e-3, 1e-3), (20000, 64), 3)
    ref_out, ref_q, wg, thr = oracle.interpolate(*args)
    q = gpu(*args, precision=precision, out_dtype=np.float64)
    if precision == "fp64":
        check_fp64(q, gpu(*args), ref_q, ref_out, wg, thr, val)
    else:
        check_fp32c(q, ref_q, wg, thr)


# ---------------------------------------------------------------------------
# edge cases
# ---------------------------------------------------------------------------

def test_edge_cases():
    x0, step, size = (0.0, 0.0), 0.1, (40, 30)
    # all samples outside the grid: everything masked
    pts = np.array([[-1.0, -1.0], [10.0, 10.0], [3.95, 1.0], [1.0, 2.95]])
    out = gpu(pts, np.array([1.0, 2.0, 3.0, 4.0]), 0.3, x0, step, size, 4)
    assert np.all(np.isnan(out))
    # a NaN value poisons the offset, as in the reference
    pts = np.array([[1.0, 1.0], [2.0, 1.5]])
    out = gpu(pts, np.array([1.0, np.nan]), 0.3, x0, step, size, 4)
    assert np.all(np.isnan(out))
    # one sample, on a cell corner: constant value where defined
    out = gpu(np.array([[2.0, 1.5]]), np.array([7.25]), 0.3, x0, step, size, 4)
    m = ~np.isnan(out)
    assert m.any() and np.all(out[m] == np.float32(7.25))
    # tiny sigma: T = 0 and only the tails act
    rng = np.random.default_rng(9)
    pts = np.c_[rng.uniform(0, 3.9, 200), rng.uniform(0, 2.9, 200)]
    val = rng.normal(0, 1, 200)
    for n in (1, 4):
        args = (pts, val, 0.01, x0, step, size, n)
        assert I.get_half_kernel_size_opt(0.01, 0.1, n) == 0
        ref_out, ref_q, wg, thr = oracle.interpolate(*args)
        check_fp64(gpu(*args, out_dtype=np.float64), gpu(*args), ref_q, ref_out, wg, thr, val)


def test_val_not_modified():
    pts, val, sigma, x0, step, size = config1_inputs(N=500)
    v0 = val.copy()
    gpu(pts, val, sigma, x0, step, size, 4)
    assert np.array_equal(val, v0)


@pytest.mark.parametrize("method", ["convolution", "optimized_convolution"])
def test_basic_ranges(method):
    """The property of the reference's BasicTest: 0/1 samples give results in
    [0, 1] or NaN, for 1D, 2D and 3D and many sigma / n."""
    rng = np.random.default_rng(17)
    step = 1.0 / 64
    cases = [(rng.uniform(0.1, 1.9, 16), 129, (1, 2, 3, 4, 5, 6, 8, 10), 1e-15),
             (rng.uniform(0.0, 2.0, (60, 2)), (129, 129), (1, 2, 3, 4, 5, 6, 8, 10), 5e-13),
             (2.0 * rng.random((307, 3)), (129, 129, 129), (1, 3, 4, 6, 10), 1e-12)]
    for pts, size, iters, eps in cases:
        val = rng.integers(2, size=len(pts)).astype(np.float64)
        for sigma in (0.5, 0.2, 0.05):
            for n in iters:
                for precision, e in (("fp64", eps), ("fp32c", 1e-5)):
                    r = gpu(pts, val, sigma, 0.0, step, size, n, method=method, precision=precision)
                    ok = np.isnan(r) | ((r >= -e) & (r <= 1 + e))
                    assert np.all(ok)


# ---------------------------------------------------------------------------
# other entry points
# ---------------------------------------------------------------------------

def test_c_abi_host_entry_matches():
    pts, val, sigma, x0, step, size = config1_inputs(N=2000, seed=4)
    ref = gpu(pts, val, sigma, x0, step, size, 4)
    L = _lib.lib()
    out = np.empty(ref.shape, np.float32)
    d = _lib.dvec
    p = np.ascontiguousarray(pts)
    v = np.ascontiguousarray(val)
    rc = L.fb_interpolate_host(0, 0, 2, p.ctypes.data, v.ctypes.data, len(v), d([sigma, sigma]), d(list(x0)),
                               d([step, step]), d(list(size), ctypes.c_int64), 4, math.exp(-3.5 ** 2 / 2),
                               out.ctypes.data, 0, None)
    _lib.check(rc)
    assert np.array_equal(out, ref, equal_nan=True)


def test_torch_tensors_stay_on_device():
    import torch
    pts, val, sigma, x0, step, size = config1_inputs(N=2000, seed=8)
    ref = gpu(pts, val, sigma, x0, step, size, 4)
    t = I.barnes(torch.as_tensor(pts, device="cuda"), torch.as_tensor(val, device="cuda"), sigma, x0, step, size)
    assert t.is_cuda and t.dtype == torch.float32
    assert np.array_equal(t.cpu().numpy(), ref, equal_nan=True)


def test_lambert_to_map_vs_oracle():
    rng = np.random.default_rng(2)
    geo = np.c_[rng.uniform(-26, 49, 1000), rng.uniform(34.5, 72, 1000)]
    proj = LC.create_proj(11.5, 34.5, 42.5, 65.5)
    assert np.array_equal(np.array(proj), oracle.lambert_proj())
    m = LC.to_map(geo, geo.copy(), *proj)
    ref = oracle.lambert_to_map(geo)
    np.testing.assert_allclose(m, ref, rtol=1e-13, atol=1e-12)


def test_s2_golden(golden):
    g = golden("barnes_s2.npz")
    kw = dict(method="optimized_convolution_S2", num_iter=int(g["n"]), max_dist=float(g["max_dist"]))
    args = (g["pts"], g["val"], float(g["sigma"]), g["x0"], float(g["step"]), tuple(int(s) for s in g["size"]))
    for resample, ref in ((False, g["lam"]), (True, g["out"])):
        out = S2.barnes_S2(*args, resample=resample, **kw)
        assert out.shape == ref.shape
        m = ~np.isnan(ref) & ~np.isnan(out)
        assert np.mean(np.isnan(out) != np.isnan(ref)) < 1e-3
        ulp = np.spacing(np.abs(ref[m]).astype(np.float32))
        assert np.max(np.abs(out[m] - ref[m]) / ulp) <= 2.0


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_s2_vs_oracle_full_resolution(precision):
    """The sphere at 1/32 degree: Lambert grid 2048 x 1408, output 2400 x 1200."""
    rng = np.random.default_rng(12)
    N = 50000
    pts = np.c_[rng.uniform(-26, 49, N), rng.uniform(34.5, 72, N)]
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
    step = 1.0 / 32
    x0 = np.array([-26.0 + step, 34.5])
    size = (int(75.0 / step), int(37.5 / step))
    ref = oracle.interpolate_s2(pts, val, 1.0, x0, step, size, 4, nthreads=8)
    out = S2.barnes_S2(pts, val, 1.0, x0, step, size, method="optimized_convolution_S2", precision=precision)
    m = ~np.isnan(ref) & ~np.isnan(out)
    assert np.mean(np.isnan(out) != np.isnan(ref)) < 1e-4
    rel = np.max(np.abs(out[m].astype(np.float64) - ref[m])) / np.max(np.abs(ref[m]))
    assert rel <= (1.5e-7 if precision == "fp64" else TOL32)


def test_s2_parts_match_whole():
    rng = np.random.default_rng(13)
    N = 500
    pts = np.c_[rng.uniform(-26, 49, N), rng.uniform(34.5, 72, N)]
    val = rng.normal(1000, 5, N)
    step = 0.25
    x0 = np.array([-26.0 + step, 34.5])
    size = (300, 150)
    whole = S2.barnes_S2(pts, val, 1.0, x0, step, size, method="optimized_convolution_S2")
    res1 = S2.interpolate_opt_convol_S2_part1(pts, val.copy(), np.full(2, 1.0), x0, np.full(2, step), size, 4,
                                              math.exp(-3.5 ** 2 / 2))
    parts = S2.interpolate_opt_convol_S2_part2(*res1)
    assert np.array_equal(whole, parts, equal_nan=True)
