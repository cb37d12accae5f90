"""GPU naive Barnes (method='naive', 'naive_S2', 'radius') against the reference's own
outputs (tests/golden/naive.npz, made by running the reference) and the CPU
oracle at a larger size.

Tolerances: the float64 form within 1e-9 of the reference relative to the
value range (the reference sums with numpy's dot / sum, the GPU sequentially
per thread, and CUDA's exp / cos / acos are not libm's); the float32 form
(Kahan-compensated float32 sums) within 1e-4 of the value range; NaN
positions equal.
"""
import numpy as np
import pytest

from fastbarnes_gb300 import interpolation as I
from fastbarnes_gb300 import interpolationS2 as S2
from oracle import oracle

pytestmark = pytest.mark.gpu


def close(mine, ref, span, tol):
    assert mine.dtype == np.float64
    assert np.array_equal(np.isnan(mine), np.isnan(ref))
    m = ~np.isnan(ref)
    err = float(np.max(np.abs(mine[m] - ref[m]))) if m.any() else 0.0
    assert err <= tol * span, err
    return err


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32c", 1e-4)])
def test_naive_golden(golden, precision, tol):
    g = golden("naive.npz")
    for ci in range(int(g["count"])):
        pts, val, sigma, x0, step, size = (g[f"c{ci}_{k}"] for k in ("pts", "val", "sigma", "x0", "step", "size"))
        size = tuple(int(s) for s in size) if len(size) > 1 else int(size[0])
        mine = I.barnes(pts, val, sigma, x0, step, size, method="naive", precision=precision)
        close(mine, g[f"c{ci}_out"], np.ptp(val), tol)
    mine = S2.barnes_S2(g["s2_pts"], g["s2_val"], float(g["s2_sigma"]), g["s2_x0"], float(g["s2_step"]),
                        tuple(int(s) for s in g["s2_size"]), method="naive_S2", precision=precision)
    close(mine, g["s2_out"], np.ptp(g["s2_val"]), tol)


def test_naive_vs_oracle_subgrid_of_config1():
    """A 256 x 128 window of the 2400 x 1200 European grid, N = 3490."""
    rng = np.random.default_rng(1)
    N = 3490
    lon = rng.uniform(-26, 49, N)
    lat = rng.uniform(34.5, 72, N)
    val = 1000 + 20 * np.sin(lon / 10) * np.cos(lat / 8) + rng.normal(0, 2, N)
    pts = np.c_[lon, lat]
    x0 = np.array([-26.0 + 1000 / 32, 34.5 + 500 / 32])
    args = (pts, val, 1.0, x0, 1 / 32, (256, 128))
    ref = oracle.interpolate_naive(pts, val, (1.0, 1.0), x0, (1 / 32, 1 / 32), (256, 128), nthreads=8)
    close(I.barnes(*args, method="naive"), ref, np.ptp(val), 1e-9)
    close(I.barnes(*args, method="naive", precision="fp32c"), ref, np.ptp(val), 1e-4)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32c", 1e-4)])
def test_radius_golden(golden, precision, tol):
    """method='radius' against the reference's kd-tree form: same masks, sums
    within the tolerances above."""
    g = golden("radius.npz")
    for ci in range(int(g["count"])):
        pts, val = g[f"c{ci}_pts"], g[f"c{ci}_val"]
        mine = I.barnes(pts, val, float(g[f"c{ci}_sigma"]), g[f"c{ci}_x0"], g[f"c{ci}_step"],
                        tuple(int(s) for s in g[f"c{ci}_size"]), method="radius",
                        max_dist=float(g[f"c{ci}_max_dist"]), min_weight=float(g[f"c{ci}_min_weight"]),
                        precision=precision)
        close(mine, g[f"c{ci}_out"], np.ptp(val), tol)


def test_radius_vs_oracle_on_european_grid():
    """A 400 x 200 window of the 2400 x 1200 European grid (1/32 degree), N =
    3490, sigma = 1: the tile skipping must not drop any sample within the
    radius (float64 equal to the oracle's scan to 1e-9); float32 within 1e-4
    with at most 0.1 % of the mask decided differently (weights sums within
    float32 rounding of max_dist_weight)."""
    rng = np.random.default_rng(11)
    N = 3490
    pts = np.c_[rng.uniform(-26, 49, N), rng.uniform(34.5, 72, N)]
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
    x0 = np.array([-26.0 + 800 / 32, 34.5 + 400 / 32])
    for max_dist, min_weight in ((3.5, 0.001), (1.5, 0.05)):
        ref = oracle.interpolate_radius(pts, val, 1.0, x0, (1 / 32, 1 / 32), (400, 200), max_dist=max_dist,
                                        min_weight=min_weight, nthreads=8)
        args = (pts, val, 1.0, x0, 1 / 32, (400, 200))
        mine = I.barnes(*args, method="radius", max_dist=max_dist, min_weight=min_weight)
        close(mine, ref, np.ptp(val), 1e-9)
        m32 = I.barnes(*args, method="radius", max_dist=max_dist, min_weight=min_weight, precision="fp32c")
        mism = np.isnan(m32) != np.isnan(ref)
        assert mism.sum() <= 1e-3 * ref.size
        ok = ~np.isnan(m32) & ~np.isnan(ref)
        assert np.max(np.abs(m32[ok] - ref[ok])) <= 1e-4 * np.ptp(val)
