"""Host-side behaviour that needs no GPU: argument checks and their messages
(fastbarnes/interpolation.py:103-199, interpolationS2.py:84-138), the kernel
size helpers, and the C ABI library's exported symbols."""
import ctypes
import os
import re

import numpy as np
import pytest

from fastbarnes_gb300 import _lib
from fastbarnes_gb300 import interpolation as I
from fastbarnes_gb300 import interpolationS2 as S2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built():
    _lib.build()


def test_exports_every_declared_symbol():
    header = open(os.path.join(ROOT, "include", "fastbarnes_gb300.h")).read()
    names = re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(fb_[a-z_0-9]+)\s*\(", header, re.M)
    assert len(names) >= 15
    L = ctypes.CDLL(_lib.LIB_PATH)
    for n in names:
        assert hasattr(L, n), n


def test_helpers_match_reference(golden):
    g = golden("helpers.npz")
    L = _lib.lib()
    for s, st, n, T, A, Tp, Se in zip(g["sigma"], g["step"], g["n"], g["T"], g["alpha"], g["T_plain"],
                                       g["sigma_eff"]):
        assert I.get_half_kernel_size_opt(s, st, n) == T
        assert I.get_tail_value(s, st, n) == A
        assert I.get_half_kernel_size(s, st, n) == Tp
        assert I.get_sigma_effective(s, st, n) == Se
        assert L.fb_half_kernel_size_opt(s, st, int(n)) == T
        assert L.fb_tail_value(s, st, int(n)) == A
        assert L.fb_half_kernel_size(s, st, int(n)) == Tp
        assert L.fb_sigma_effective(s, st, int(n)) == Se


def test_argument_errors():
    pts = np.zeros((5, 2))
    val = np.zeros(5)
    with pytest.raises(RuntimeError, match="specified pts is not a numpy ndarray"):
        I.barnes([[0, 0]], val, 1.0, 0.0, 0.1, (10, 10))
    with pytest.raises(RuntimeError, match=r"expected pts array of shape \(N, M\) but was: \(5, 2, 1\)"):
        I.barnes(np.zeros((5, 2, 1)), val, 1.0, 0.0, 0.1, (10, 10))
    with pytest.raises(RuntimeError, match="supports only sample points in dimensions 1, 2 or 3"):
        I.barnes(np.zeros((5, 4)), val, 1.0, 0.0, 0.1, (10, 10, 10, 10))
    with pytest.raises(RuntimeError, match="specified val is not a numpy ndarray"):
        I.barnes(pts, [0] * 5, 1.0, 0.0, 0.1, (10, 10))
    with pytest.raises(RuntimeError, match=r"expected val array of shape \(N\) but was: \(5, 1\)"):
        I.barnes(pts, np.zeros((5, 1)), 1.0, 0.0, 0.1, (10, 10))
    with pytest.raises(RuntimeError, match=r"inconsistent shapes: \(5, 2\) vs. \(4,\)"):
        I.barnes(pts, np.zeros(4), 1.0, 0.0, 0.1, (10, 10))
    with pytest.raises(RuntimeError, match="specified sigma with invalid length: 3"):
        I.barnes(pts, val, [1.0, 1.0, 1.0], 0.0, 0.1, (10, 10))
    with pytest.raises(RuntimeError, match="specified x0 with invalid length: 1"):
        I.barnes(pts, val, 1.0, [0.0], 0.1, (10, 10))
    with pytest.raises(RuntimeError, match="specified step with invalid length: 3"):
        I.barnes(pts, val, 1.0, 0.0, (0.1, 0.1, 0.1), (10, 10))
    with pytest.raises(RuntimeError, match="specified size with invalid length: 1"):
        I.barnes(pts, val, 1.0, 0.0, 0.1, (10,))
    with pytest.raises(RuntimeError, match="array size should be array-like of length: 2"):
        I.barnes(pts, val, 1.0, 0.0, 0.1, 10)
    with pytest.raises(RuntimeError, match="encountered invalid Barnes interpolation method: foo"):
        I.barnes(pts, val, 0.01, 0.0, 0.1, (10, 10), method="foo")
    with pytest.raises(RuntimeError, match="radius algorithm works only in 2D but data is: 1D"):
        I.barnes(np.zeros(5), val, 0.01, 0.0, 0.1, 10, method="radius")
    with pytest.raises(ValueError, match="zero-size array"):
        I.barnes(np.zeros((0, 2)), np.zeros(0), 0.5, 0.0, 0.1, (100, 100))


def test_kernel_size_guard():
    """tests/BasicTest.py:105-148 of the reference: size == kernel size
    raises, and the message names the kernel and the grid."""
    sigma, step = 0.5, 1.0 / 32
    pts = np.asarray([0.2, 0.4, 0.7])
    val = np.asarray([18.5, 17.0, 19.25])
    for method, helper in (("optimized_convolution", I.get_half_kernel_size_opt),
                           ("convolution", I.get_half_kernel_size)):
        for n in (3, 4, 6):
            ks = 2 * helper(sigma, step, n) + 1
            with pytest.raises(RuntimeError, match="resulting rectangular kernel size should be smaller"):
                I.barnes(pts, val, sigma, 0.0, step, int(ks), method=method, num_iter=n)


def test_kernel_size_guard_in_c_abi():
    L = _lib.lib()
    need = ctypes.c_size_t(0)
    d = _lib.dvec
    rc = L.fb_workspace_size(0, 0, 1, 3, d([0.5]), d([1 / 32]), d([27], ctypes.c_int64), 4, ctypes.byref(need))
    assert rc == _lib.FB_ERR_KERNEL_SIZE
    assert b"kernel size" in L.fb_last_error()
    rc = L.fb_workspace_size(0, 0, 1, 3, d([0.5]), d([1 / 32]), d([28], ctypes.c_int64), 4, ctypes.byref(need))
    assert rc == 0 and need.value > 0


def test_s2_method_errors():
    pts = np.zeros((3, 2))
    val = np.zeros(3)
    # the reference's default method string is rejected by its own dispatcher
    with pytest.raises(RuntimeError, match="encountered invalid Barnes interpolation method: optimized_convolution"):
        S2.barnes_S2(pts, val, 1.0, (-26, 34.5), 0.25, (300, 150))
    with pytest.raises(RuntimeError, match="specified sigma with invalid length: 3"):
        S2.barnes_S2(pts, val, (1, 1, 1), (-26, 34.5), 0.25, (300, 150), method="optimized_convolution_S2")


def test_workspace_scales_with_plan():
    L = _lib.lib()
    need64, need32 = ctypes.c_size_t(0), ctypes.c_size_t(0)
    d = _lib.dvec
    args = (d([1.0, 1.0]), d([75 / 4096, 37.5 / 2048]), d([4096, 2048], ctypes.c_int64), 4)
    assert L.fb_workspace_size(0, 0, 2, 100000, *args, ctypes.byref(need64)) == 0
    assert L.fb_workspace_size(0, 1, 2, 100000, *args, ctypes.byref(need32)) == 0
    # one intermediate value/weight pair: 2 x 8M points x 8 (or 4) bytes
    assert need64.value >= 2 * 4096 * 2048 * 8
    assert need32.value >= 2 * 4096 * 2048 * 4
    assert need32.value < need64.value


def test_batch_argument_errors_in_c_abi():
    """fb_batch_create rejects bad batches before it touches a device."""
    L = _lib.lib()
    h = ctypes.c_void_p()
    arr = (_lib.Field2D * 2)()
    for F in arr:
        F.pts, F.val, F.out, F.n_pts = 8, 8, 8, 10   # never dereferenced on these paths
        F.sigma[:] = [1.0, 1.0]
        F.x0[:] = [0.0, 0.0]
        F.step[:] = [1 / 32, 1 / 32]
        F.size[:] = [200, 100]
        F.num_iter, F.max_dist_weight, F.method = 4, 0.002, 0
    assert L.fb_batch_create(1, arr, 0, 0, 0, None, ctypes.byref(h)) == _lib.FB_ERR_ARG
    assert b"at least one field" in L.fb_last_error()
    assert L.fb_batch_create(1, arr, 2, 0, 8, None, ctypes.byref(h)) == _lib.FB_ERR_ARG
    kn = _lib.BatchKnobs(5, 0)
    assert L.fb_batch_create(1, arr, 2, 0, 0, ctypes.byref(kn), ctypes.byref(h)) == _lib.FB_ERR_ARG
    assert b"chunk" in L.fb_last_error()
    kn = _lib.BatchKnobs(0, 300)
    assert L.fb_batch_create(1, arr, 2, 0, 0, ctypes.byref(kn), ctypes.byref(h)) == _lib.FB_ERR_ARG
    kn = _lib.BatchKnobs(0, 256, 2)
    assert L.fb_batch_create(1, arr, 2, 0, 0, ctypes.byref(kn), ctypes.byref(h)) == _lib.FB_ERR_ARG
    assert b"mixed" in L.fb_last_error()
    arr[1].size[1] = 20   # 2T+1 = 65 >= 20
    assert L.fb_batch_create(1, arr, 2, 0, 0, None, ctypes.byref(h)) == _lib.FB_ERR_KERNEL_SIZE
    assert L.fb_last_error().startswith(b"field 1:")
    arr[1].size[1] = 100
    arr[0].out = None
    assert L.fb_batch_create(1, arr, 2, 0, 0, None, ctypes.byref(h)) == _lib.FB_ERR_ARG
    assert b"null device pointer" in L.fb_last_error()
    assert h.value is None


def test_resample_noalloc_rejects_grid_beyond_static_scratch():
    """The size check of fb_resample_noalloc runs on the host before any
    device call (the pointers here are never dereferenced)."""
    L = _lib.lib()
    d = _lib.dvec
    proj = d([11.5, 0.7, 1.4, 1.0, 1.0])
    for W, H in ((16385, 16384), (100, 49000), (49153, 1)):
        rc = L.fb_resample_noalloc(8, 640, 440, d([-32.0, -2.0]), d([0.0, 0.0]), d([0.1, 0.1]),
                                   d([W, H], ctypes.c_int64), proj, 8, None)
        assert rc == _lib.FB_ERR_ARG
        assert b"static scratch" in L.fb_last_error()


def test_grad_workspace_holds_cell_fields():
    """The adjoint keeps the forward's final cells and its own: a 1D forward
    plan needs no cell buffer, the gradient plan one of 16 B per cell (fp64)."""
    L = _lib.lib()
    d = _lib.dvec
    fwd, grad = ctypes.c_size_t(0), ctypes.c_size_t(0)
    args = (d([0.3]), d([0.01]), d([5000], ctypes.c_int64), 4)
    assert L.fb_workspace_size(0, 0, 1, 1000, *args, ctypes.byref(fwd)) == 0
    assert L.fb_grad_workspace_size(0, 0, 1, 1000, *args, ctypes.byref(grad)) == 0
    assert grad.value >= fwd.value + 16 * 5000
    args2 = (d([1.0, 1.0]), d([1 / 32, 1 / 32]), d([400, 300], ctypes.c_int64), 4)
    assert L.fb_grad_workspace_size(0, 1, 2, 1000, *args2, ctypes.byref(grad)) == 0
    assert grad.value >= 8 * 400 * 300
    assert L.fb_grad_workspace_size(2, 0, 2, 1000, *args2, ctypes.byref(grad)) == _lib.FB_ERR_UNSUPPORTED


def test_radius_entry_checks_before_device_work():
    """fb_interpolate_radius validates its arguments and workspace on the host
    (the pointers are never dereferenced here); the workspace holds one
    32-byte box per tile of 256 samples."""
    L = _lib.lib()
    d = _lib.dvec
    need = ctypes.c_size_t(0)
    assert L.fb_radius_workspace_size(1000, ctypes.byref(need)) == 0
    assert need.value >= 4 * 32
    assert L.fb_radius_workspace_size(-1, ctypes.byref(need)) == _lib.FB_ERR_ARG
    x0, step, size = d([0.0, 0.0]), d([0.1, 0.1]), d([64, 32], ctypes.c_int64)
    args = (8, 8, 1000, 0.5, x0, step, size, 0.011, 0.001, 8, 1)
    assert L.fb_interpolate_radius(0, *args, 8, 16, None) == _lib.FB_ERR_WORKSPACE
    assert L.fb_interpolate_radius(3, *args, 8, 1 << 20, None) == _lib.FB_ERR_ARG
    bad = (8, 8, 1000, 0.0, x0, step, size, 0.011, 0.001, 8, 1)
    assert L.fb_interpolate_radius(0, *bad, 8, 1 << 20, None) == _lib.FB_ERR_ARG
    assert b"invalid radius arguments" in L.fb_last_error()


def test_kernel_size_guard_agrees_across_layers():
    """The front door, the C ABI and the oracle refuse exactly the same grids
    (interpolation.py:170-184: a grid of at most 2T + 1 cells along an axis),
    over seeded sigma / step / n / sizes (of at least 2 cells) around the
    limit, both methods, 2D."""
    from oracle import oracle
    L = _lib.lib()
    d = _lib.dvec
    rng = np.random.default_rng(5)
    pts = np.asarray([[0.3, 0.4]])
    val = np.asarray([1.0])
    for _ in range(60):
        method = "optimized_convolution" if rng.random() < 0.5 else "convolution"
        helper = I.get_half_kernel_size_opt if method == "optimized_convolution" else I.get_half_kernel_size
        n = int(rng.integers(1, 7))
        step = float(rng.choice([0.1, 1 / 32, 0.05]))
        sigma = float(step * rng.uniform(1.0, 8.0))
        ks = 2 * int(helper(sigma, step, n)) + 1
        size = (max(2, int(ks + rng.integers(-1, 2))), 2 * ks + 2)
        refused = size[0] <= ks
        need = ctypes.c_size_t(0)
        rc = L.fb_workspace_size(0 if method == "optimized_convolution" else 1, 0, 2, 1, d([sigma, sigma]),
                                 d([step, step]), d(list(size), ctypes.c_int64), n, ctypes.byref(need))
        assert (rc == _lib.FB_ERR_KERNEL_SIZE) == refused, (method, n, sigma, step, size, rc)
        try:
            I._kernel_guard((ks, ks), size, 2)
            front = False
        except RuntimeError:
            front = True
        assert front == refused
        try:
            oracle.interpolate(pts, val, sigma, (0.0, 0.0), step, size, n, method=method)
            orc = False
        except RuntimeError:
            orc = True
        assert orc == refused, (method, n, sigma, step, size)
