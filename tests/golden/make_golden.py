"""Generate the golden fixtures in tests/golden/ by running the reference itself.

This script imports MeteoSwiss/fast-barnes-py from a source checkout, given
as the FASTBARNES_REF environment variable or the --ref DIR argument (there is
no default location), as plain Python/NumPy: numba is
not installed here, so a stub ``numba`` module whose ``njit`` returns the
function unchanged is put in ``sys.modules`` first.  With ``fastmath`` off (the
numba default the reference uses) the jitted loops are scalar IEEE float64
code, so the pure-Python run computes the same values.

Fixtures written (all small, np.savez_compressed):
  accumulate.npz  - _accumulate_array / _accumulate_tail_array on the impulse
                    inputs of the reference's AccumulationTest plus random lines
  helpers.npz     - T, alpha (optimized) and T, sigma_eff (plain) over a grid
  barnes_{1,2,3}d.npz - end-to-end barnes() cases: inputs, the float32 result,
                    the float64 quotient before the cast, the NaN threshold
  barnes_s2.npz   - barnes_S2 at step 1/4: Lambert field and resampled field
  naive.npz       - barnes(method='naive') in 1D/2D/3D and
                    barnes_S2(method='naive_S2') on small grids
  quant.npz       - demo/quantinterpolation.py barnes() with several
                    quant_bits, and demo/quantization.py quant() on numbers
  radius.npz      - barnes(method='radius') (kd-tree radius search) on small
                    2D grids

Run once in a container that has the reference; the GPU host never runs it.
`python make_golden.py naive` regenerates one group of fixtures only.
"""
import os
import sys
import types
from math import exp

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _reference_dir():
    """The reference checkout: --ref DIR on the command line, else the
    FASTBARNES_REF environment variable; no default."""
    argv = sys.argv[1:]
    if "--ref" in argv:
        i = argv.index("--ref")
        if i + 1 >= len(argv):
            raise SystemExit("--ref needs a directory")
        ref = argv[i + 1]
        del sys.argv[i + 1:i + 3]
        return ref
    ref = os.environ.get("FASTBARNES_REF")
    if not ref:
        raise SystemExit("set FASTBARNES_REF or pass --ref DIR (a MeteoSwiss/fast-barnes-py source checkout)")
    return ref


REF = None


def import_reference():
    global REF
    if REF is None:
        REF = _reference_dir()
    if "numba" not in sys.modules:
        stub = types.ModuleType("numba")

        def njit(*args, **kwargs):
            if len(args) == 1 and callable(args[0]) and not kwargs:
                return args[0]
            return lambda f: f

        stub.njit = njit
        sys.modules["numba"] = stub
    sys.path.insert(0, REF)
    from fastbarnes import interpolation, interpolationS2  # noqa: E402
    return interpolation, interpolationS2


def accumulation_cases(I):
    """The impulse inputs of AccumulationTest plus random lines."""
    cases = []
    size = 32
    for pos in (10, 2, 30, 16):
        a = np.zeros(size)
        a[pos] = 1.0
        for n in (1, 2):
            cases.append(("plain", a, 9, n, 0.0))
            for alpha in (0.25, 0.5):
                cases.append(("tail", a, 7, n, alpha))
    a = np.zeros(size)
    a[3], a[9], a[21], a[30] = 1.0, 2.5, -1.25, 1.0
    cases += [("plain", a, 9, 3, 0.0), ("tail", a, 9, 3, 0.0), ("tail", a, 7, 3, 1.0)]
    rng = np.random.default_rng(7)
    for (L, rect, n, alpha) in ((97, 1, 3, 0.4), (97, 3, 4, 0.3), (64, 21, 2, 0.7),
                                (200, 41, 6, 0.05), (33, 31, 1, 0.9), (50, 11, 10, 0.5)):
        a = rng.normal(0, 1, L) * (rng.random(L) < 0.3)
        cases.append(("tail", a, rect, n, alpha))
        cases.append(("plain", a, rect, n, 0.0))
    kinds, ins, outs, rects, ns, alphas, lens = [], [], [], [], [], [], []
    for kind, a, rect, n, alpha in cases:
        h = np.empty(len(a))
        if kind == "plain":
            o = I._accumulate_array(a.copy(), h, len(a), rect, n)
        else:
            o = I._accumulate_tail_array(a.copy(), h, len(a), rect, n, alpha)
        kinds.append(0 if kind == "plain" else 1)
        ins.append(np.pad(a, (0, 200 - len(a))))
        outs.append(np.pad(np.array(o), (0, 200 - len(a))))
        rects.append(rect), ns.append(n), alphas.append(alpha), lens.append(len(a))
    np.savez_compressed(os.path.join(HERE, "accumulate.npz"), kind=np.array(kinds),
                        inp=np.array(ins), out=np.array(outs), rect=np.array(rects),
                        n=np.array(ns), alpha=np.array(alphas), length=np.array(lens))


def helper_cases(I):
    sig, stp, nit, T, A, Tp, Se = [], [], [], [], [], [], []
    for sigma in (0.05, 0.2, 0.5, 0.6, 1.0, 1.5, 2.0, 4.0):
        for step in (1 / 512, 1 / 64, 1 / 32, 75 / 4096, 1 / 8, 0.25):
            for n in (1, 2, 3, 4, 5, 6, 10):
                sig.append(sigma), stp.append(step), nit.append(n)
                T.append(I.get_half_kernel_size_opt(sigma, step, n))
                A.append(I.get_tail_value(sigma, step, n))
                Tp.append(I.get_half_kernel_size(sigma, step, n))
                Se.append(I.get_sigma_effective(sigma, step, n))
    np.savez_compressed(os.path.join(HERE, "helpers.npz"), sigma=np.array(sig),
                        step=np.array(stp), n=np.array(nit), T=np.array(T), alpha=np.array(A),
                        T_plain=np.array(Tp), sigma_eff=np.array(Se))


def reference_quotient(I, pts, val, sigma, x0, step, size, n, max_dist, method):
    """The reference's float32 result and its float64 quotient before the cast.

    The quotient is obtained by running the reference's own internal steps of
    _interpolate_opt_convol (interpolation.py:328-367) / _interpolate_convol
    (:575-612) and stopping before .astype(np.float32)."""
    dim = pts.shape[1]
    out = I.barnes(pts.copy() if dim > 1 else pts[:, 0].copy(), val.copy(), sigma, x0, step,
                   size, method=method, num_iter=n, max_dist=max_dist)
    sig = np.full(dim, sigma, dtype=np.float64) if np.isscalar(sigma) else np.asarray(sigma, np.float64)
    x0a = np.full(dim, x0, dtype=np.float64) if np.isscalar(x0) else np.asarray(x0, np.float64)
    stp = np.full(dim, step, dtype=np.float64) if np.isscalar(step) else np.asarray(step, np.float64)
    sz = (size,) if np.isscalar(size) else tuple(size)
    v = val.copy()
    offset = I._normalize_values(v)
    vg = np.zeros(sz[::-1])
    wg = np.zeros(sz[::-1])
    [I._inject_data_1d, I._inject_data_2d, I._inject_data_3d][dim - 1](vg, wg, pts, v, x0a, stp, sz)
    mdw = exp(-max_dist ** 2 / 2)
    if method == "optimized_convolution":
        ks = 2 * I._get_half_kernel_size_opt(sig, stp, n) + 1
        tv = I._get_tail_value(sig, stp, n)
        conv = [I._convolve_tail_1d, I._convolve_tail_2d, I._convolve_tail_3d][dim - 1]
        conv(vg, wg, sig, stp, sz, ks, n, tv, mdw)
        thr = np.prod((ks + 2 * tv) ** n / np.sqrt(2 * np.pi) / (sig / stp)) * mdw
    else:
        ks = 2 * I._get_half_kernel_size(sig, stp, n) + 1
        conv = [I._convolve_1d, I._convolve_2d, I._convolve_3d][dim - 1]
        conv(vg, wg, sig, stp, sz, ks, n, mdw)
        thr = np.prod(ks ** n / np.sqrt(2 * np.pi) / (sig / stp)) * mdw
    q = vg / wg + offset
    assert np.array_equal(q.astype(np.float32), out, equal_nan=True)
    return out, q, thr


def barnes_cases(I):
    rng = np.random.default_rng(20240101)
    groups = {1: [], 2: [], 3: []}
    # 1D: points on [0, 3], grid step 1/64, 200 cells
    for sigma in (0.5, 0.2, 0.05, 0.01):
        for n in (1, 3, 4, 6):
            N = 40
            pts = np.sort(rng.uniform(-0.05, 3.2, N))[:, None]
            val = rng.normal(5.0, 2.0, N)
            groups[1].append((pts, val, sigma, 0.0, 1 / 64, 200, n, 3.5))
    # 2D: 96 x 72 grid, step 1/32, some samples outside, some on cell borders
    for sigma, n, step, mdist in ((0.5, 4, 1 / 32, 3.5), (0.2, 2, 1 / 32, 3.5), (0.3, 5, 1 / 32, 2.0),
                                  ((0.4, 0.25), 4, (1 / 32, 1 / 24), 3.5), (0.01, 3, 1 / 32, 3.5),
                                  (0.6, 1, 1 / 32, 3.5), (0.25, 6, 1 / 32, 4.5)):
        N = 150
        pts = np.c_[rng.uniform(-0.2, 3.2, N), rng.uniform(-0.2, 2.4, N)]
        pts[:5] = np.round(pts[:5] * 32) / 32
        val = 1000.0 + 20 * np.sin(pts[:, 0] * 3) * np.cos(pts[:, 1] * 2) + rng.normal(0, 2, N)
        groups[2].append((pts, val, sigma, (0.0, 0.0), step, (96, 72), n, mdist))
    # 3D: 20 x 16 x 12
    for sigma, n in (((0.6, 0.5, 0.5), 3), (0.5, 4), (0.3, 2)):
        N = 120
        pts = np.c_[rng.uniform(0, 2.5, N), rng.uniform(0, 2.0, N), rng.uniform(0, 1.8, N)]
        val = rng.normal(0.0, 1.0, N)
        groups[3].append((pts, val, sigma, (0.0, 0.0, 0.0), (1 / 8, 1 / 8, 1 / 6), (20, 16, 12), n, 3.5))
    for dim, cases in groups.items():
        rec = {}
        for ci, (pts, val, sigma, x0, step, size, n, mdist) in enumerate(cases):
            for method in ("optimized_convolution", "convolution"):
                tag = "opt" if method == "optimized_convolution" else "conv"
                out, q, thr = reference_quotient(I, pts, val, sigma, x0, step, size, n, mdist, method)
                rec[f"c{ci}_{tag}_out"] = out
                rec[f"c{ci}_{tag}_q64"] = q
                rec[f"c{ci}_{tag}_thr"] = np.float64(thr)
            dimn = pts.shape[1]
            rec[f"c{ci}_pts"] = pts
            rec[f"c{ci}_val"] = val
            rec[f"c{ci}_sigma"] = np.broadcast_to(np.asarray(sigma, np.float64), (dimn,)).copy()
            rec[f"c{ci}_x0"] = np.broadcast_to(np.asarray(x0, np.float64), (dimn,)).copy()
            rec[f"c{ci}_step"] = np.broadcast_to(np.asarray(step, np.float64), (dimn,)).copy()
            rec[f"c{ci}_size"] = np.broadcast_to(np.asarray(size, np.int64), (dimn,)).copy()
            rec[f"c{ci}_n"] = np.int64(n)
            rec[f"c{ci}_max_dist"] = np.float64(mdist)
        rec["count"] = np.int64(len(cases))
        np.savez_compressed(os.path.join(HERE, f"barnes_{dim}d.npz"), **rec)


def s2_cases(S2):
    rng = np.random.default_rng(31337)
    step = 1.0 / 4
    x0 = np.asarray([-26.0 + step, 34.5])
    size = (int(75.0 / step), int(37.5 / step))
    N = 300
    pts = np.c_[rng.uniform(-26, 49, N), rng.uniform(34.5, 72, N)]
    val = 1000.0 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, N)
    sigma, n, max_dist = 1.0, 4, 3.5
    # barnes_S2's default method string is not one it accepts, so name it
    m = "optimized_convolution_S2"
    out = S2.barnes_S2(pts, val.copy(), sigma, x0, step, size, method=m, num_iter=n,
                       max_dist=max_dist)
    lam = S2.barnes_S2(pts, val.copy(), sigma, x0, step, size, method=m, num_iter=n,
                       max_dist=max_dist, resample=False)
    np.savez_compressed(os.path.join(HERE, "barnes_s2.npz"), pts=pts, val=val, sigma=sigma,
                        x0=x0, step=step, size=np.array(size), n=n, max_dist=max_dist,
                        out=out, lam=lam)


def naive_cases(I, S2):
    rng = np.random.default_rng(4242)
    rec = {}
    cases = []
    pts = rng.uniform(-0.1, 3.1, (40, 1))
    cases.append((pts, rng.normal(5.0, 2.0, 40), 0.2, 0.0, 1 / 64, 200))
    pts = np.c_[rng.uniform(-0.2, 1.7, 150), rng.uniform(-0.2, 1.3, 150)]
    cases.append((pts, 1000.0 + 20 * np.sin(pts[:, 0] * 3) + rng.normal(0, 2, 150), (0.3, 0.2), (0.0, 0.0),
                  1 / 32, (48, 36)))
    pts = np.c_[rng.uniform(0, 1.5, 60), rng.uniform(0, 1.2, 60), rng.uniform(0, 1.0, 60)]
    cases.append((pts, rng.normal(0.0, 1.0, 60), 0.25, (0.0, 0.0, 0.0), 1 / 8, (12, 10, 8)))
    for ci, (pts, val, sigma, x0, step, size) in enumerate(cases):
        out = I.barnes(pts, val.copy(), sigma, x0, step, size, method="naive")
        dim = pts.shape[1]
        rec[f"c{ci}_pts"] = pts
        rec[f"c{ci}_val"] = val
        rec[f"c{ci}_sigma"] = np.broadcast_to(np.asarray(sigma, np.float64), (dim,)).copy()
        rec[f"c{ci}_x0"] = np.broadcast_to(np.asarray(x0, np.float64), (dim,)).copy()
        rec[f"c{ci}_step"] = np.broadcast_to(np.asarray(step, np.float64), (dim,)).copy()
        rec[f"c{ci}_size"] = np.broadcast_to(np.asarray(size, np.int64), (dim,)).copy()
        rec[f"c{ci}_out"] = out
    rec["count"] = np.int64(len(cases))
    # sphere: 1-degree grid over part of the European domain
    pts = np.c_[rng.uniform(-20, 30, 100), rng.uniform(36, 66, 100)]
    val = 1000.0 + 20 * np.sin(pts[:, 0] / 10) * np.cos(pts[:, 1] / 8) + rng.normal(0, 2, 100)
    x0, step, size, sigma = np.asarray([-20.0, 36.0]), 1.0, (50, 30), 2.0
    rec["s2_pts"], rec["s2_val"], rec["s2_x0"] = pts, val, x0
    rec["s2_step"], rec["s2_size"], rec["s2_sigma"] = np.float64(step), np.array(size), np.float64(sigma)
    rec["s2_out"] = S2.barnes_S2(pts, val.copy(), sigma, x0, step, size, method="naive_S2")
    np.savez_compressed(os.path.join(HERE, "naive.npz"), **rec)


def radius_cases(I):
    """barnes(method='radius') (kd-tree search) on two small 2D grids: the
    default min_weight / max_dist, and a larger min_weight with a tighter
    max_dist so that some grid points are masked."""
    rng = np.random.default_rng(9090)
    rec = {}
    cases = []
    pts = np.c_[rng.uniform(-0.3, 2.8, 120), rng.uniform(-0.3, 1.9, 120)]
    val = 1000.0 + 20 * np.sin(pts[:, 0] * 3) * np.cos(pts[:, 1] * 2) + rng.normal(0, 2, 120)
    cases.append((pts, val, 0.25, (0.0, 0.0), 1 / 16, (40, 28), 3.5, 0.001))
    pts = np.c_[rng.uniform(0, 3.0, 80), rng.uniform(0, 2.0, 80)]
    cases.append((pts, rng.normal(5.0, 1.0, 80), 0.15, (0.1, -0.1), (1 / 12, 1 / 10), (36, 24), 2.0, 0.02))
    for ci, (pts, val, sigma, x0, step, size, max_dist, min_weight) in enumerate(cases):
        out = I.barnes(pts, val.copy(), sigma, x0, step, size, method="radius", max_dist=max_dist,
                       min_weight=min_weight)
        rec[f"c{ci}_pts"] = pts
        rec[f"c{ci}_val"] = val
        rec[f"c{ci}_sigma"] = np.float64(sigma)
        rec[f"c{ci}_x0"] = np.broadcast_to(np.asarray(x0, np.float64), (2,)).copy()
        rec[f"c{ci}_step"] = np.broadcast_to(np.asarray(step, np.float64), (2,)).copy()
        rec[f"c{ci}_size"] = np.asarray(size, np.int64)
        rec[f"c{ci}_max_dist"] = np.float64(max_dist)
        rec[f"c{ci}_min_weight"] = np.float64(min_weight)
        rec[f"c{ci}_out"] = out
    rec["count"] = np.int64(len(cases))
    np.savez_compressed(os.path.join(HERE, "radius.npz"), **rec)


def quant_cases():
    sys.path.insert(0, os.path.join(REF, "demo"))
    import quantinterpolation as QI  # noqa: E402
    from quantization import quant  # noqa: E402
    rng = np.random.default_rng(777)
    N = 200
    pts = np.c_[rng.uniform(-0.2, 3.2, N), rng.uniform(-0.2, 2.4, N)]
    val = 1000.0 + 20 * np.sin(pts[:, 0] * 3) * np.cos(pts[:, 1] * 2) + rng.normal(0, 2, N)
    rec = dict(pts=pts, val=val, sigma=np.float64(0.3), x0=np.zeros(2), step=np.float64(1 / 32),
               size=np.array([96, 72]), n=np.int64(4))
    bits = [0, 8, 24, 40]
    for b in bits:
        rec[f"out_{b}"] = QI.barnes(pts, val.copy(), 0.3, np.zeros(2), 1 / 32, (96, 72), b, num_iter=4)
    x = np.concatenate([rng.normal(0, 1, 64) * 10.0 ** rng.integers(-5, 6, 64), [0.0, -0.0, 1.0, -1.0, 0.5]])
    for b in (1, 7, 23, 52):
        y = x.copy()
        quant(y, b)
        rec[f"quant_in"] = x
        rec[f"quant_{b}"] = y
    rec["bits"] = np.array(bits)
    np.savez_compressed(os.path.join(HERE, "quant.npz"), **rec)


def main():
    I, S2 = import_reference()
    which = sys.argv[1:] or ["accumulate", "helpers", "barnes", "s2", "naive", "quant", "radius"]
    if "accumulate" in which:
        accumulation_cases(I)
    if "helpers" in which:
        helper_cases(I)
    if "barnes" in which:
        barnes_cases(I)
    if "s2" in which:
        s2_cases(S2)
    if "naive" in which:
        naive_cases(I, S2)
    if "quant" in which:
        quant_cases()
    if "radius" in which:
        radius_cases(I)
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
