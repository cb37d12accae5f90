"""Gradients of the interpolation (fb_interpolate_grad behind
torch.autograd) against (a) torch autograd through a dense float64 restatement
of the same algorithm (splat as index-add, every axis's n box passes as a dense
band-matrix power, mask, quotient), (b) finite differences, on small problems
and on the full 4096 x 2048 grid with N = 200k, and (c) torch autograd
through the dense naive Barnes (the Gaussian the method approximates; this
bounds approximation error, see its test).

Tolerances: FP64 gradients within 1e-9 of the dense reference relative to the
largest gradient component; finite differences within 1e-6 (values, where f is
linear) and 1e-4 (positions, central differences of h = 1e-5 cells); FP32C
gradients within 1e-4 of the FP64 ones relative to the largest component, and
within 1e-3 for a least-squares loss whose seed changes sign across the grid
(the float32 window sums of the adjoint cancel there).
"""
import math

import numpy as np
import pytest

from fastbarnes_gb300 import autograd as AG
from fastbarnes_gb300 import interpolation as I

pytestmark = pytest.mark.gpu


def band(L, T, alpha, n, torch):
    i = torch.arange(L)
    d = (i[:, None] - i[None, :]).abs()
    B = (d <= T).double() + alpha * (d == T + 1).double()
    return torch.linalg.matrix_power(B, n)


def dense_barnes(pts, val, sigma, x0, step, size, n, max_dist, torch):
    """f = V / W + offset on the grid, NaN where W < thr, from torch ops only
    (pts, val: CPU float64 tensors that may require grad)."""
    dim = pts.shape[1]
    sigma = np.broadcast_to(np.asarray(sigma, float), (dim,))
    step = np.broadcast_to(np.asarray(step, float), (dim,))
    x0 = np.broadcast_to(np.asarray(x0, float), (dim,))
    T = [int(I.get_half_kernel_size_opt(sigma[m], step[m], n)) for m in range(dim)]
    al = [float(I.get_tail_value(sigma[m], step[m], n)) for m in range(dim)]
    thr = 1.0
    for m in range(dim):
        thr *= (2 * T[m] + 1 + 2 * al[m]) ** n / math.sqrt(2 * math.pi) / (sigma[m] / step[m])
    thr *= math.exp(-max_dist ** 2 / 2)
    offset = float((val.detach().min() + val.detach().max()) / 2)
    vp = val - offset
    xc = [(pts[:, m] - x0[m]) / step[m] for m in range(dim)]
    xi = [torch.floor(c.detach()).long() for c in xc]
    keep = torch.ones(len(val), dtype=torch.bool)
    for m in range(dim):
        keep &= (xc[m].detach() >= 0) & (xc[m].detach() < size[m] - 1)
    xw = [xc[m] - xi[m].double() for m in range(dim)]
    shape = tuple(size[::-1])
    V = torch.zeros(int(np.prod(shape)), dtype=torch.float64)
    Wt = torch.zeros_like(V)
    strides = [1, size[0], size[0] * (size[1] if dim > 1 else 1)]
    for corner in range(2 ** dim):
        w = torch.ones(len(val), dtype=torch.float64)
        idx = torch.zeros(len(val), dtype=torch.long)
        for m in range(dim):
            c = (corner >> m) & 1
            w = w * (xw[m] if c else 1 - xw[m])
            idx = idx + (xi[m] + c) * strides[m]
        idx = torch.where(keep, idx, torch.zeros_like(idx))
        w = torch.where(keep, w, torch.zeros_like(w))
        V = V.index_add(0, idx, w * vp)
        Wt = Wt.index_add(0, idx, w)
    V = V.reshape(shape)
    Wt = Wt.reshape(shape)
    for m in range(dim):
        B = band(size[m], T[m], al[m], n, torch)
        ax = dim - 1 - m    # axis of size[m] in the [z][y][x] array
        V = torch.movedim(torch.tensordot(B, torch.movedim(V, ax, 0), dims=1), 0, ax)
        Wt = torch.movedim(torch.tensordot(B, torch.movedim(Wt, ax, 0), dims=1), 0, ax)
    mask = Wt.detach() >= thr
    return torch.where(mask, V / torch.where(mask, Wt, torch.ones_like(Wt)) + offset,
                       torch.full_like(V, float("nan"))), mask


def problem(dim, seed):
    rng = np.random.default_rng(seed)
    if dim == 1:
        size, step, sigma, N = (90,), 0.1, 0.35, 30
    elif dim == 2:
        size, step, sigma, N = (48, 36), 0.1, 0.3, 60
    else:
        size, step, sigma, N = (20, 18, 14), 0.1, 0.22, 80
    x0 = np.zeros(dim)
    hi = np.asarray(size) * step
    pts = rng.uniform(-0.05, 1.0, (N, dim)) * hi
    val = 5 + rng.normal(0, 2, N)
    return pts, val, sigma, x0, step, size


def gpu_grads(pts, val, sigma, x0, step, size, n, precision, c):
    import torch
    tp = torch.tensor(pts, device="cuda", requires_grad=True)
    tv = torch.tensor(val, device="cuda", requires_grad=True)
    f = AG.barnes(tp, tv, sigma, x0, step, size, num_iter=n, precision=precision)
    m = ~torch.isnan(f)
    loss = (torch.where(m, f, torch.zeros_like(f)) * torch.as_tensor(c, device="cuda")).sum()
    loss.backward()
    return f.detach().cpu().numpy(), tv.grad.cpu().numpy(), tp.grad.cpu().numpy()


@pytest.mark.parametrize("dim", [1, 2, 3])
def test_fp64_gradients_match_dense_autograd(dim):
    import torch
    pts, val, sigma, x0, step, size = problem(dim, 30 + dim)
    n = 3
    c = np.random.default_rng(7).normal(0, 1, tuple(size[::-1]))
    f, gv, gp = gpu_grads(pts, val, sigma, x0, step, size, n, "fp64", c)
    tp = torch.tensor(pts, requires_grad=True)
    tv = torch.tensor(val, requires_grad=True)
    fr, mask = dense_barnes(tp, tv, sigma, x0, step, size, n, 3.5, torch)
    assert np.array_equal(np.isnan(f), np.isnan(fr.detach().numpy()))
    ok = ~np.isnan(f)
    assert np.max(np.abs(f[ok] - fr.detach().numpy()[ok])) <= 1e-9 * np.max(np.abs(f[ok]))
    loss = (torch.where(mask, fr, torch.zeros_like(fr)) * torch.as_tensor(c)).sum()
    loss.backward()
    rv, rp = tv.grad.numpy(), tp.grad.numpy()
    assert np.max(np.abs(gv - rv)) <= 1e-9 * np.max(np.abs(rv))
    assert np.max(np.abs(gp - rp)) <= 1e-9 * np.max(np.abs(rp))


def test_fp64_gradients_match_finite_differences():
    pts, val, sigma, x0, step, size = problem(2, 41)
    n = 4
    c = np.random.default_rng(8).normal(0, 1, tuple(size[::-1]))

    def loss(p, v):
        f = I.barnes(p, v, sigma, x0, step, size, num_iter=n, out_dtype=np.float64)
        m = ~np.isnan(f)
        return float(np.sum(f[m] * c[m]))

    _, gv, gp = gpu_grads(pts, val, sigma, x0, step, size, n, "fp64", c)
    rng = np.random.default_rng(9)
    for k in rng.choice(len(val), 8, replace=False):
        h = 1e-3
        v1, v2 = val.copy(), val.copy()
        v1[k] += h
        v2[k] -= h
        # f is linear in val apart from the offset, which cancels; the mask
        # depends on positions only
        fd = (loss(pts, v1) - loss(pts, v2)) / (2 * h)
        assert abs(fd - gv[k]) <= 1e-6 * max(1.0, np.max(np.abs(gv)))
        for m in range(2):
            frac = (pts[k, m] - x0[m]) / step - np.floor((pts[k, m] - x0[m]) / step)
            if frac < 0.01 or frac > 0.99:
                continue   # the bilinear weights bend at cell edges
            hp = 1e-5 * step
            p1, p2 = pts.copy(), pts.copy()
            p1[k, m] += hp
            p2[k, m] -= hp
            fd = (loss(p1, val) - loss(p2, val)) / (2 * hp)
            assert abs(fd - gp[k, m]) <= 1e-4 * max(1.0, np.max(np.abs(gp))), (k, m, fd, gp[k, m])


def test_fp32c_gradients_close_to_fp64():
    pts, val, sigma, x0, step, size = problem(2, 51)
    c = np.random.default_rng(10).normal(0, 1, tuple(size[::-1]))
    _, gv64, gp64 = gpu_grads(pts, val, sigma, x0, step, size, 4, "fp64", c)
    _, gv32, gp32 = gpu_grads(pts, val, sigma, x0, step, size, 4, "fp32c", c)
    assert np.max(np.abs(gv32 - gv64)) <= 1e-4 * np.max(np.abs(gv64))
    assert np.max(np.abs(gp32 - gp64)) <= 1e-4 * np.max(np.abs(gp64))


def test_gradients_at_headline_density():
    """4096 x 2048 at N = 20k: gradients are finite, zero for samples outside
    the grid, and the fp32c ones agree with fp64."""
    import torch
    rng = np.random.default_rng(61)
    N = 20000
    pts = np.c_[rng.uniform(-27, 50, N), rng.uniform(33.5, 73, N)]
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
    args = (2.0, (-26.0, 34.5), (75 / 4096, 37.5 / 2048), (4096, 2048))
    outside = (pts[:, 0] < -26) | (pts[:, 0] >= -26 + 75 * 4095 / 4096) | (pts[:, 1] < 34.5) | \
              (pts[:, 1] >= 34.5 + 37.5 * 2047 / 2048)
    res = {}
    for prec in ("fp64", "fp32c"):
        tp = torch.tensor(pts, device="cuda", requires_grad=True)
        tv = torch.tensor(val, device="cuda", requires_grad=True)
        f = AG.barnes(tp, tv, *args, precision=prec)
        target = torch.full_like(f, 1000.0)
        m = ~torch.isnan(f)
        loss = (torch.where(m, f - target, torch.zeros_like(f)) ** 2).sum()
        loss.backward()
        res[prec] = (tv.grad.cpu().numpy(), tp.grad.cpu().numpy())
        assert np.all(np.isfinite(res[prec][0])) and np.all(np.isfinite(res[prec][1]))
        assert np.all(res[prec][0][outside] == 0) and np.all(res[prec][1][outside] == 0)
    for a, b in zip(res["fp32c"], res["fp64"]):
        assert np.max(np.abs(a - b)) <= 1e-3 * np.max(np.abs(b))


def dense_naive(pts, val, sigma, x0, step, size, torch):
    """The reference's naive Barnes (interpolation.py:861-938) from torch ops:
    f = sum_k w_k v_k / sum_k w_k with w_k = exp(-|x - p_k|^2 / (2 sigma^2))
    over every grid point x; the offset cancels in the quotient."""
    W, H = size
    xs = x0[0] + torch.arange(W, dtype=torch.float64) * step
    ys = x0[1] + torch.arange(H, dtype=torch.float64) * step
    dx = (pts[:, 0][None, None, :] - xs[None, :, None]) ** 2 / (2 * sigma ** 2)
    dy = (pts[:, 1][None, None, :] - ys[:, None, None]) ** 2 / (2 * sigma ** 2)
    w = torch.exp(-(dx + dy))            # [H][W][N]
    return (w * val).sum(-1) / w.sum(-1)


def test_gradients_close_to_dense_naive_autograd():
    """The adjoint against torch autograd through the dense naive Barnes on a
    128 x 64 subproblem (0.25 degree cells, sigma = 2 degrees = 8 cells,
    n = 4, 400 samples).  The optimized convolution approximates the naive
    Gaussian weights, so this bounds approximation error, not rounding (the
    dense restatement of the same algorithm above checks rounding to 1e-9):
    measured 4-5% (values) and 9-13% (positions) relative L2 difference,
    cosine >= 0.99.  Samples and the loss stay 2 sigma inside the grid, where
    the zero-padded box passes do not cut the kernel."""
    import torch
    rng = np.random.default_rng(5)
    size, step, x0, sigma, N = (128, 64), 0.25, (0.0, 0.0), 2.0, 400
    lo = 2 * sigma
    hi = np.array([(size[0] - 1) * step, (size[1] - 1) * step]) - 2 * sigma
    pts = rng.uniform([lo, lo], hi, (N, 2))
    val = 1000 + 20 * np.sin(pts[:, 0] / 3) * np.cos(pts[:, 1] / 2) + rng.normal(0, 2, N)
    gx, gy = np.arange(size[0]) * step, np.arange(size[1]) * step
    inner = (gx[None, :] >= lo) & (gx[None, :] <= hi[0]) & (gy[:, None] >= lo) & (gy[:, None] <= hi[1])
    c = rng.normal(0, 1, (size[1], size[0])) * inner
    f, gv, gp = gpu_grads(pts, val, sigma, x0, step, size, 4, "fp64", c)
    assert not np.isnan(f[inner]).any()
    tp = torch.tensor(pts, requires_grad=True)
    tv = torch.tensor(val, requires_grad=True)
    (dense_naive(tp, tv, sigma, x0, step, size, torch) * torch.as_tensor(c)).sum().backward()
    rv, rp = tv.grad.numpy(), tp.grad.numpy()

    def rel(a, b):
        return np.linalg.norm(a - b) / np.linalg.norm(b)

    def cos(a, b):
        return float(np.dot(a.ravel(), b.ravel()) / np.linalg.norm(a) / np.linalg.norm(b))

    assert rel(gv, rv) <= 0.08 and cos(gv, rv) >= 0.995, (rel(gv, rv), cos(gv, rv))
    assert rel(gp, rp) <= 0.2 and cos(gp, rp) >= 0.98, (rel(gp, rp), cos(gp, rp))


def test_gradients_full_size_finite_differences():
    """The full-size differentiation workload: 4096 x 2048 grid over the
    European domain, N = 200k uniform samples, sigma = 2 degrees, n = 4, loss
    sum over the grid of (f - target)^2 with a seeded smooth target.  FP64
    gradients against central finite differences (h = 1e-3, value units and
    degrees) on 64 random samples, skipping samples within h of a cell edge
    (the bilinear weights bend there); each difference of two losses is
    summed per grid point as (f1 - f2)(f1 + f2 - 2 target), so no two sums of
    8M terms cancel.  FP32C gradients within 1e-3 of the FP64 ones relative to
    the largest component."""
    import torch
    rng = np.random.default_rng(200)
    W, H, N, sigma, n, h = 4096, 2048, 200_000, 2.0, 4, 1e-3
    x0, step = (-26.0, 34.5), (75.0 / W, 37.5 / H)
    pts = np.c_[rng.uniform(-26, 49, N), rng.uniform(34.5, 72, N)]
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
    gx = torch.as_tensor(x0[0] + np.arange(W) * step[0], device="cuda")
    gy = torch.as_tensor(x0[1] + np.arange(H) * step[1], device="cuda")
    ph = rng.uniform(0, 2 * np.pi, 2)
    target = 1000 + 15 * torch.sin(gx[None, :] / 7 + ph[0]) * torch.cos(gy[:, None] / 5 + ph[1])
    args = (sigma, x0, step, (W, H))

    grads = {}
    for prec in ("fp64", "fp32c"):
        tp = torch.tensor(pts, device="cuda", requires_grad=True)
        tv = torch.tensor(val, device="cuda", requires_grad=True)
        f = AG.barnes(tp, tv, *args, num_iter=n, precision=prec)
        m = ~torch.isnan(f)
        (torch.where(m, f - target, torch.zeros_like(f)) ** 2).sum().backward()
        grads[prec] = (tv.grad.cpu().numpy(), tp.grad.cpu().numpy())
    gv, gp = grads["fp64"]
    for a, b in zip(grads["fp32c"], grads["fp64"]):
        assert np.max(np.abs(a - b)) <= 1e-3 * np.max(np.abs(b))

    d_pts = torch.as_tensor(pts, device="cuda")
    d_val = torch.as_tensor(val, device="cuda")

    def field(p, v):
        return I.barnes(p, v, *args, num_iter=n, out_dtype=np.float64)

    def loss_diff(f1, f2):
        ok = ~torch.isnan(f1) & ~torch.isnan(f2)
        d = (f1 - f2) * (f1 + f2 - 2 * target)
        return float(torch.where(ok, d, torch.zeros_like(d)).sum())

    frac = [(pts[:, m] - x0[m]) / step[m] - np.floor((pts[:, m] - x0[m]) / step[m]) for m in range(2)]
    edge = [h / step[m] for m in range(2)]
    inside = (pts[:, 0] >= x0[0]) & (pts[:, 0] < x0[0] + (W - 1) * step[0] - h) & \
             (pts[:, 1] >= x0[1]) & (pts[:, 1] < x0[1] + (H - 1) * step[1] - h)
    ok = inside & (frac[0] > edge[0]) & (frac[0] < 1 - edge[0]) & (frac[1] > edge[1]) & (frac[1] < 1 - edge[1])
    picks = rng.choice(np.flatnonzero(ok), 64, replace=False)
    sv, sp = np.max(np.abs(gv)), np.max(np.abs(gp))
    for k in picks:
        v1, v2 = d_val.clone(), d_val.clone()
        v1[k] += h
        v2[k] -= h
        fd = loss_diff(field(d_pts, v1), field(d_pts, v2)) / (2 * h)
        assert abs(fd - gv[k]) <= 1e-6 * sv, (k, fd, gv[k])
        for m in range(2):
            p1, p2 = d_pts.clone(), d_pts.clone()
            p1[k, m] += h
            p2[k, m] -= h
            fd = loss_diff(field(p1, d_val), field(p2, d_val)) / (2 * h)
            assert abs(fd - gp[k, m]) <= 1e-5 * sp, (k, m, fd, gp[k, m])
