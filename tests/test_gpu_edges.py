"""Edge cases against the oracle, seeded and randomised over shapes.

The reference's indexing edges (fastbarnes/interpolation.py:249-270: the
skip rule xc < 0 or xc >= size - 1 and the corner writes; :505-523: the
border phases of the running sum) are exercised by:
  - samples exactly on cell borders, exactly on the grid's lower edge
    (xc = 0 and -0.0), and at xc = size - 1 and one ulp either side of it
    (kept below, skipped at and above), plus samples outside the grid;
  - T = 0 in one axis (anisotropic sigma), N = 1, and grids of exactly
    2T + 2 cells (the smallest the kernel-size check admits);
  - random grid shapes, sigma, num_iter, both convolution methods, in 1D, 2D
    and 3D.
Tolerances are the parity tests': float64 quotient within 1e-9 of
max(|ref|, range(val)), fp32c within 1e-5 relative max error, NaN masks equal
except where the weight lies within 1e-9 (fp64) / 1e-4 (fp32c) of the mask
level.
"""
import math

import numpy as np
import pytest

from fastbarnes_gb300 import interpolation as I
from oracle import oracle

pytestmark = pytest.mark.gpu


def check(q, ref_q, ref_wg, thr, val, precision):
    band = 1e-9 if precision == "fp64" else 1e-4
    diff = np.isnan(q) != np.isnan(ref_q)
    assert np.all(np.abs(ref_wg[diff] - thr) <= band * abs(thr)), "mask differs away from the mask level"
    m = ~np.isnan(q) & ~np.isnan(ref_q)
    if not m.any():
        return
    if precision == "fp64":
        scale = np.maximum(np.abs(ref_q[m]), np.ptp(val) if len(val) > 1 else 0.0)
        scale = np.where(scale > 0, scale, 1.0)
        err = np.max(np.abs(q[m] - ref_q[m]) / scale)
        assert err <= 1e-9, err
    else:
        rel = np.max(np.abs(q[m] - ref_q[m])) / max(np.max(np.abs(ref_q[m])), 1e-300)
        assert rel <= 1e-5, rel


def edge_samples(rng, x0, step, size, n_uniform):
    """Uniform samples plus the edge positions along every axis."""
    dim = len(size)
    x0 = np.asarray(x0, np.float64)
    step = np.asarray(step, np.float64)
    size = np.asarray(size)
    pts = [x0 + step * rng.uniform(-0.5, size + 0.5, (n_uniform, dim))]
    for m in range(dim):
        base = x0 + step * rng.uniform(0, size - 1, (12, dim))
        top = x0[m] + (size[m] - 1) * step[m]
        specials = [x0[m], -0.0 if x0[m] == 0 else x0[m], np.nextafter(x0[m], -np.inf),
                    top, np.nextafter(top, -np.inf), np.nextafter(top, np.inf),
                    x0[m] + step[m] * rng.integers(0, size[m], 6)]
        cols = np.concatenate([np.atleast_1d(np.asarray(v, np.float64)) for v in specials])
        b = np.repeat(base[:1], len(cols), axis=0)
        b[:, m] = cols
        # the other coordinates on cell borders too, half of the time
        for mm in range(dim):
            if mm != m:
                b[::2, mm] = x0[mm] + step[mm] * rng.integers(0, size[mm] - 1, len(b[::2]))
        pts.append(b)
    pts = np.concatenate(pts)
    val = 10.0 + 5.0 * np.sin(pts.sum(axis=1)) + rng.normal(0, 1, len(pts))
    return pts, val


def run_case(pts, val, sigma, x0, step, size, n, method, precision):
    ref_out, ref_q, wg, thr = oracle.interpolate(pts, val, sigma, x0, step, size, n, method=method, nthreads=4)
    q = I.barnes(pts, val, sigma, x0, step, size, method=method, num_iter=n, precision=precision,
                 out_dtype=np.float64)
    check(q, ref_q, wg, thr, val, precision)
    return q, ref_q


def min_size(sigma, step, n, method):
    T = (I.get_half_kernel_size_opt(sigma, step, n) if method == "optimized_convolution"
         else I.get_half_kernel_size(sigma, step, n))
    return 2 * int(T) + 2


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("dim", [1, 2, 3])
def test_random_shapes_with_edge_samples(dim, precision):
    rng = np.random.default_rng(1000 * dim + (precision == "fp32c"))
    ncase = {1: 12, 2: 16, 3: 6}[dim]
    for case in range(ncase):
        method = "optimized_convolution" if case % 3 else "convolution"
        n = int(rng.integers(1, 7))
        step = [float(rng.choice([0.1, 0.25, 1 / 32, 0.5])) for _ in range(dim)]
        sigma = [float(s * rng.uniform(0.3, 6.0)) for s in step]
        lo = [min_size(sg, st, n, method) for sg, st in zip(sigma, step)]
        hi = {1: 4000, 2: 300, 3: 48}[dim]
        size = [int(rng.integers(l, max(l, hi) + 1)) for l in lo]
        x0 = [float(rng.choice([0.0, -3.25, 7.5])) for _ in range(dim)]
        pts, val = edge_samples(rng, x0, step, size, int(rng.integers(1, 400)))
        if dim == 1:
            pts = pts[:, 0]
        run_case(pts, val, sigma if dim > 1 else sigma[0], x0 if dim > 1 else x0[0],
                 step if dim > 1 else step[0], size if dim > 1 else size[0], n, method, precision)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_upper_edge_ulps(precision):
    """A sample one ulp below x = x0 + (size - 1) step lands in the last cell
    (its weight goes to the last grid point); at and one ulp above that
    point it is skipped, exactly as the reference's xc >= size - 1."""
    x0, step, size = (0.0, 0.0), (0.1, 0.1), (60, 40)
    top_x, top_y = (size[0] - 1) * step[0], (size[1] - 1) * step[1]
    for px in (np.nextafter(top_x, -np.inf), top_x, np.nextafter(top_x, np.inf)):
        pts = np.array([[px, 1.0], [1.5, 1.5], [2.0, np.nextafter(top_y, -np.inf)], [3.0, top_y]])
        val = np.array([100.0, 10.0, 50.0, 70.0])
        run_case(pts, val, 1.0, x0, step, size, 4, "optimized_convolution", precision)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_zero_half_width_in_one_axis(precision):
    """sigma small against the step in x (T = 0: a window of one cell plus
    the tails), ordinary in y."""
    rng = np.random.default_rng(7)
    step, size = (1.0, 0.05), (64, 400)
    sigma = (0.3, 0.8)
    assert I.get_half_kernel_size_opt(sigma[0], step[0], 4) == 0
    pts, val = edge_samples(rng, (0.0, 0.0), step, size, 2000)
    run_case(pts, val, sigma, (0.0, 0.0), step, size, 4, "optimized_convolution", precision)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_one_sample(precision):
    for pts in (np.array([[1.234, 2.5]]), np.array([[0.0, 0.0]]), np.array([[5.9, 3.9]])):
        run_case(pts, np.array([42.0]), 0.5, (0.0, 0.0), (0.1, 0.1), (60, 40), 4, "optimized_convolution",
                 precision)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("method", ["optimized_convolution", "convolution"])
def test_smallest_grids(precision, method):
    """Grids of exactly 2T + 2 cells in every axis."""
    rng = np.random.default_rng(11)
    for sigma, step, n in ((0.5, 0.1, 4), (1.0, 0.05, 3), (0.2, 0.1, 1), (2.0, 0.1, 6)):
        L = min_size(sigma, step, n, method)
        size = (L, L)
        pts, val = edge_samples(rng, (0.0, 0.0), (step, step), size, 200)
        run_case(pts, val, sigma, (0.0, 0.0), step, size, n, method, precision)
        with pytest.raises(RuntimeError):
            I.barnes(pts, val, sigma, (0.0, 0.0), step, (L - 1, L), method=method, num_iter=n,
                     precision=precision)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("n", [1, 2, 4])
def test_long_columns_wide_kernel(precision, n):
    """Columns of 2048 cells with T = 94, 66, 46 (n = 1, 2, 4 at sigma = 1
    deg, step = 75 / 4096 deg): with T > 63 the float32 y launch takes the
    short chunk (a CTA of the long one would need more than eight warps)."""
    rng = np.random.default_rng(40 + n)
    step = (75.0 / 4096, 75.0 / 4096)
    size = (192, 2048)   # at least 2T + 2 cells along x too
    x0 = (-26.0, 34.5)
    assert I.get_half_kernel_size_opt(1.0, step[1], n) == {1: 94, 2: 66, 4: 46}[n]
    pts, val = edge_samples(rng, x0, step, size, 3000)
    run_case(pts, val, 1.0, x0, step, size, n, "optimized_convolution", precision)
