"""fb_resample_noalloc (static device scratch, no allocation) against
fb_resample (caller scratch) through the C ABI.

Both run the same table and resample kernels, so the results are compared
for exact equality (tolerance 0, NaN positions included), on two calls in a
row.  This file is collected last so that it also runs after every other
test in the session."""
import ctypes

import numpy as np
import pytest

from fastbarnes_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = 0.0


def _setup(torch, W, H, lam_w=640, lam_h=440):
    rng = np.random.default_rng(17)
    L = _lib.lib()
    proj = (ctypes.c_double * 5)()
    L.fb_lambert_create_proj(11.5, 34.5, 42.5, 65.5, proj)
    lam = torch.as_tensor(rng.normal(280.0, 10.0, (lam_h, lam_w)).astype(np.float32), device="cuda")
    lam_x0 = _lib.dvec([-32.0, -2.0])
    x0 = _lib.dvec([-26.0, 34.5])
    step = _lib.dvec([75.0 / W, 37.5 / H])
    size = _lib.dvec([W, H], ctypes.c_int64)
    return L, proj, lam, lam_w, lam_h, lam_x0, x0, step, size


def test_noalloc_resample_matches_workspace_form_twice():
    import torch
    W, H = 600, 300
    L, proj, lam, lam_w, lam_h, lam_x0, x0, step, size = _setup(torch, W, H)
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = torch.empty((H, W), dtype=torch.float32, device="cuda")
    tab = torch.empty(H + 2 * W, dtype=torch.float64, device="cuda")
    _lib.check(L.fb_resample(lam.data_ptr(), lam_w, lam_h, lam_x0, x0, step, size, proj, ref.data_ptr(),
                             tab.data_ptr(), sp), "fb_resample")
    r = ref.cpu().numpy()
    assert np.isfinite(r).any()
    for call in range(2):
        out = torch.full((H, W), -1.0, dtype=torch.float32, device="cuda")
        _lib.check(L.fb_resample_noalloc(lam.data_ptr(), lam_w, lam_h, lam_x0, x0, step, size, proj,
                                         out.data_ptr(), sp), "fb_resample_noalloc")
        o = out.cpu().numpy()
        assert np.array_equal(np.isnan(o), np.isnan(r)), call
        m = ~np.isnan(r)
        assert np.max(np.abs(o[m] - r[m])) <= TOL, call


def test_noalloc_resample_at_the_size_limit():
    """A grid that uses the whole static table array: size[1] + 2 * size[0]
    == 49152 exactly (24000 x 1152), so that an off-by-one near the end of the
    array would show; compared with fb_resample for exact equality, NaN
    positions included, twice."""
    import torch
    W, H = 24000, 1152
    assert H + 2 * W == 49152
    # a Lambert field covering the fixed Lambert domain (64 x 44) at this step
    L, proj, lam, lam_w, lam_h, lam_x0, x0, step, size = _setup(torch, W, H, int(64 * W / 75), int(44 * H / 37.5))
    sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = torch.empty((H, W), dtype=torch.float32, device="cuda")
    tab = torch.empty(H + 2 * W, dtype=torch.float64, device="cuda")
    _lib.check(L.fb_resample(lam.data_ptr(), lam_w, lam_h, lam_x0, x0, step, size, proj, ref.data_ptr(),
                             tab.data_ptr(), sp), "fb_resample")
    r = ref.cpu().numpy()
    assert np.isfinite(r).any()
    for call in range(2):
        out = torch.full((H, W), -1.0, dtype=torch.float32, device="cuda")
        _lib.check(L.fb_resample_noalloc(lam.data_ptr(), lam_w, lam_h, lam_x0, x0, step, size, proj,
                                         out.data_ptr(), sp), "fb_resample_noalloc")
        o = out.cpu().numpy()
        assert np.array_equal(o, r, equal_nan=True), call
    # one more column does not fit and is rejected before any launch
    big = _lib.dvec([W + 1, H], ctypes.c_int64)
    rc = L.fb_resample_noalloc(lam.data_ptr(), lam_w, lam_h, lam_x0, x0, step, big, proj, out.data_ptr(), sp)
    assert rc == _lib.FB_ERR_ARG
