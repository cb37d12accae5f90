"""GPU naive Barnes (method='naive', 'naive_S2') against the reference's own
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
