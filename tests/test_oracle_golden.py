"""The CPU oracle against the golden fixtures generated from the reference.

The fixtures in tests/golden/ were produced by tests/golden/make_golden.py,
which runs MeteoSwiss/fast-barnes-py itself.  These tests pin the oracle: the
1D/2D/3D paths must agree bit for bit, the sphere path to 1e-12 (the reference
evaluates its trigonometry with NumPy's vectorised functions).
"""
import numpy as np
import pytest

from oracle import oracle


def test_accumulate_vectors(golden):
    g = golden("accumulate.npz")
    for k in range(len(g["kind"])):
        L = int(g["length"][k])
        a = g["inp"][k][:L]
        if g["kind"][k] == 0:
            out = oracle.accumulate_array(a, g["rect"][k], g["n"][k])
        else:
            out = oracle.accumulate_tail_array(a, g["rect"][k], g["n"][k], g["alpha"][k])
        np.testing.assert_array_equal(out, g["out"][k][:L], err_msg=f"case {k}")


def test_accumulate_known_answers():
    """Known answers of the reference's AccumulationTest (tail, 2-fold, alpha 0.5)."""
    a = np.zeros(32)
    a[16] = 1.0
    out = oracle.accumulate_tail_array(a, 7, 2, 0.5)
    assert np.all(out[:8] == 0) and np.all(out[25:] == 0)
    assert out[16] == 7.5 and out[8] == 0.25 and out[24] == 0.25
    # border truncation: impulse at the left border
    a = np.zeros(32)
    a[2] = 1.0
    out = oracle.accumulate_tail_array(a, 7, 2, 0.5)
    assert out[0] == 4.5 and out[3] == 6.5 and out[10] == 0.25 and np.all(out[11:] == 0)


def test_helpers(golden):
    g = golden("helpers.npz")
    for s, st, n, T, A, Tp, Se in zip(g["sigma"], g["step"], g["n"], g["T"], g["alpha"], g["T_plain"],
                                       g["sigma_eff"]):
        assert oracle.half_kernel_size_opt(s, st, n) == T
        assert oracle.tail_value(s, st, n) == A
        assert oracle.half_kernel_size(s, st, n) == Tp
        assert oracle.sigma_effective(s, st, n) == Se


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("tag", ["opt", "conv"])
def test_barnes_bitwise(golden, dim, tag):
    g = golden(f"barnes_{dim}d.npz")
    method = "optimized_convolution" if tag == "opt" else "convolution"
    for c in range(int(g["count"])):
        out, q, _, thr = oracle.interpolate(g[f"c{c}_pts"], g[f"c{c}_val"], g[f"c{c}_sigma"],
                                            g[f"c{c}_x0"], g[f"c{c}_step"], g[f"c{c}_size"],
                                            int(g[f"c{c}_n"]), float(g[f"c{c}_max_dist"]), method)
        # the reference raises (2T+1+2a) to the power n with NumPy's vectorised
        # pow, the oracle (like numba's compiled code) with libm's: the mask
        # level may differ in its last bit
        assert abs(thr - g[f"c{c}_{tag}_thr"]) <= 2.5e-16 * abs(thr)
        np.testing.assert_array_equal(q, g[f"c{c}_{tag}_q64"], err_msg=f"{dim}d case {c}")
        np.testing.assert_array_equal(out, g[f"c{c}_{tag}_out"], err_msg=f"{dim}d case {c}")


def test_barnes_threads_independent(golden):
    g = golden("barnes_2d.npz")
    a = oracle.interpolate(g["c0_pts"], g["c0_val"], g["c0_sigma"], g["c0_x0"], g["c0_step"],
                           g["c0_size"], int(g["c0_n"]), nthreads=1)[1]
    b = oracle.interpolate(g["c0_pts"], g["c0_val"], g["c0_sigma"], g["c0_x0"], g["c0_step"],
                           g["c0_size"], int(g["c0_n"]), nthreads=4)[1]
    np.testing.assert_array_equal(a, b)


def test_s2(golden):
    g = golden("barnes_s2.npz")
    lam = oracle.interpolate_s2(g["pts"], g["val"], float(g["sigma"]), g["x0"], float(g["step"]),
                                g["size"], int(g["n"]), float(g["max_dist"]), resample=False)
    out = oracle.interpolate_s2(g["pts"], g["val"], float(g["sigma"]), g["x0"], float(g["step"]),
                                g["size"], int(g["n"]), float(g["max_dist"]))
    for mine, ref in ((lam, g["lam"]), (out, g["out"])):
        assert np.array_equal(np.isnan(mine), np.isnan(ref))
        m = ~np.isnan(ref)
        np.testing.assert_allclose(mine[m], ref[m], rtol=1e-6, atol=0)
        # float32 results: at most one float32 ulp apart
        assert np.max(np.abs(mine[m] - ref[m]) / np.spacing(np.abs(ref[m]))) <= 1.0


def test_naive_close_to_optimized():
    """Away from the grid borders (where the convolution form truncates and the
    naive form still sees samples outside the grid) the exact Barnes
    interpolation and the optimized convolution agree closely."""
    rng = np.random.default_rng(3)
    N = 2000
    pts = np.c_[rng.uniform(0, 4, N), rng.uniform(0, 3, N)]
    val = np.sin(pts[:, 0]) * np.cos(pts[:, 1]) + rng.normal(0, 0.05, N)
    args = (pts, val, 0.25, (0.0, 0.0), 1 / 32, (128, 96))
    out = oracle.interpolate(*args, num_iter=6)[0]
    nv = oracle.interpolate_naive(*args)
    b = 32  # one sigma-width of cells... four of them
    inner = (slice(b, -b), slice(b, -b))
    err = np.abs(out[inner] - nv[inner])
    assert np.nanmax(err) < 0.02 * np.ptp(val)


def test_oracle_naive_matches_reference(golden):
    """The naive algorithm: the reference sums with numpy's dot / sum, the
    oracle sequentially, so the results agree to rounding (1e-12 relative to
    the value range)."""
    g = golden("naive.npz")
    for ci in range(int(g["count"])):
        args = [g[f"c{ci}_{k}"] for k in ("pts", "val", "sigma", "x0", "step", "size")]
        ref = g[f"c{ci}_out"]
        mine = oracle.interpolate_naive(*args)
        assert np.array_equal(np.isnan(mine), np.isnan(ref))
        m = ~np.isnan(ref)
        assert np.max(np.abs(mine[m] - ref[m])) <= 1e-12 * np.ptp(args[1]), ci
    mine = oracle.interpolate_naive_s2(g["s2_pts"], g["s2_val"], g["s2_sigma"], g["s2_x0"], g["s2_step"],
                                       g["s2_size"])
    ref = g["s2_out"]
    assert np.array_equal(np.isnan(mine), np.isnan(ref))
    m = ~np.isnan(ref)
    assert np.max(np.abs(mine[m] - ref[m])) <= 1e-12 * np.ptp(g["s2_val"])


def test_oracle_quant_matches_reference(golden):
    """demo/quantization.py quant() bit for bit, and the quantised
    'convolution' result of demo/quantinterpolation.py."""
    g = golden("quant.npz")
    for b in (1, 7, 23, 52):
        assert np.array_equal(oracle.quant(g["quant_in"], b), g[f"quant_{b}"])
    size = tuple(int(s) for s in g["size"])
    _, q, _, _ = oracle.interpolate(g["pts"], g["val"], float(g["sigma"]), g["x0"], float(g["step"]), size,
                                    int(g["n"]), method="convolution")
    for b in g["bits"]:
        assert np.array_equal(oracle.quant(q, int(b)), g[f"out_{b}"], equal_nan=True), b


def test_oracle_radius_matches_reference(golden):
    """The oracle's radius form (a scan under the kd-tree's distance test)
    against the reference's barnes(method='radius') on small grids."""
    g = golden("radius.npz")
    for ci in range(int(g["count"])):
        pts, val = g[f"c{ci}_pts"], g[f"c{ci}_val"]
        mine = oracle.interpolate_radius(pts, val, float(g[f"c{ci}_sigma"]), g[f"c{ci}_x0"], g[f"c{ci}_step"],
                                         g[f"c{ci}_size"], max_dist=float(g[f"c{ci}_max_dist"]),
                                         min_weight=float(g[f"c{ci}_min_weight"]))
        ref = g[f"c{ci}_out"]
        assert np.array_equal(np.isnan(mine), np.isnan(ref)), ci
        m = ~np.isnan(ref)
        assert m.any()
        assert np.max(np.abs(mine[m] - ref[m])) <= 1e-12 * np.ptp(val), ci


def test_oracle_rejects_kernel_wider_than_grid():
    """The reference's kernel-size check (interpolation.py:170-184) guards the
    oracle too: a grid of at most 2T + 1 cells along an axis is refused."""
    pts = np.array([[0.5, 0.5]])
    val = np.array([1.0])
    step = (75.0 / 4096, 75.0 / 4096)
    T = oracle.half_kernel_size_opt(1.0, step[0], 1)
    with pytest.raises(RuntimeError):
        oracle.interpolate(pts, val, 1.0, (0.0, 0.0), step, (2 * T + 1, 2048), 1)
    out = oracle.interpolate(pts, val, 1.0, (0.0, 0.0), step, (2 * T + 2, 2 * T + 2), 1)
    assert out[0].shape == (2 * T + 2, 2 * T + 2)
