"""The pipelined column kernel (TMA tile loads, mbarrier ring, persistent
CTAs; csrc/fb_cols.cuh) against the one-CTA-per-column-group kernel it
replaces (k_axis / k_axis_batch in columns layout).

Both run the same pass arithmetic, so every result must be bitwise equal
(NaN positions included).  The knob fb_tune("cols_pipe", 0 | 1) selects the
kernel; 2 (automatic, the default) is restored after every test.  Parity of the
pipelined kernel against the reference itself is covered by every other GPU
parity test that runs on it (float64 column stages by default).
"""
import contextlib
import threading

import numpy as np
import pytest

from fastbarnes_gb300 import _lib
from fastbarnes_gb300 import interpolation as I
from fastbarnes_gb300 import interpolationS2 as S2
from fastbarnes_gb300 import quantinterpolation as Q

pytestmark = pytest.mark.gpu


@contextlib.contextmanager
def pipe(on):
    L = _lib.lib()
    _lib.check(L.fb_tune(b"cols_pipe", 1 if on else 0), "fb_tune")
    try:
        yield
    finally:
        _lib.check(L.fb_tune(b"cols_pipe", 2), "fb_tune")


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(a, b, equal_nan=True)


def field(seed, n, x0, step, size, dim=2):
    rng = np.random.default_rng(seed)
    lo = np.asarray(x0, dtype=np.float64)
    hi = lo + np.asarray(step, dtype=np.float64) * (np.asarray(size) - 1)
    pts = rng.uniform(lo, hi, (n, dim))
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) + rng.normal(0, 2, n)
    return pts, val


CASES = [
    # (name, n, sigma, x0, step, size, num_iter, precision, method)
    ("headline shape fp32c", 100_000, 1.0, (-26.0, 34.5), (75 / 4096, 37.5 / 2048), (4096, 2048), 4, "fp32c",
     "optimized_convolution"),
    ("headline shape fp64", 100_000, 1.0, (-26.0, 34.5), (75 / 4096, 37.5 / 2048), (4096, 2048), 4, "fp64",
     "optimized_convolution"),
    ("example fp32c", 3490, 1.0, (-26.0, 34.5), (1 / 32, 1 / 32), (2400, 1200), 4, "fp32c",
     "optimized_convolution"),
    ("example fp64 n=3", 3490, 1.0, (-26.0, 34.5), (1 / 32, 1 / 32), (2400, 1200), 3, "fp64",
     "optimized_convolution"),
    ("direct sums fp32c", 5000, 0.1, (0.0, 0.0), (0.05, 0.05), (300, 150), 4, "fp32c", "optimized_convolution"),
    ("direct sums fp64", 5000, 0.1, (0.0, 0.0), (0.05, 0.05), (300, 150), 6, "fp64", "optimized_convolution"),
    ("convolution fp64", 20_000, 0.5, (0.0, 0.0), (0.01, 0.01), (1024, 512), 4, "fp64", "convolution"),
    ("ragged column groups fp32c", 20_000, 0.5, (0.0, 0.0), (0.01, 0.01), (1030, 517), 4, "fp32c",
     "optimized_convolution"),
    ("odd width (previous kernel only) fp64", 20_000, 0.5, (0.0, 0.0), (0.01, 0.01), (1023, 511), 4, "fp64",
     "optimized_convolution"),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_2d_pipelined_equals_previous(case):
    name, n, sigma, x0, step, size, num_iter, prec, method = case
    pts, val = field(7, n, x0, step, size)
    outs = {}
    for on in (False, True):
        with pipe(on):
            outs[on] = (I.barnes(pts, val, sigma, x0, step, size, method=method, num_iter=num_iter,
                                 precision=prec, out_dtype=np.float64),
                        I.barnes(pts, val, sigma, x0, step, size, method=method, num_iter=num_iter,
                                 precision=prec))
    assert same(outs[True][0], outs[False][0])
    assert same(outs[True][1], outs[False][1])
    assert np.isfinite(outs[True][0]).any()


@pytest.mark.parametrize("prec", ["fp64", "fp32c"])
def test_3d_pipelined_equals_previous(prec):
    # y lines (axis 1, cells written back) and z lines (axis 2, quotient)
    size = (96, 80, 64)
    x0, step = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    pts, val = field(11, 20_000, x0, step, size, dim=3)
    outs = {}
    for on in (False, True):
        with pipe(on):
            outs[on] = I.barnes(pts, val, 3.0, x0, step, size, num_iter=4, precision=prec, out_dtype=np.float64)
    assert same(outs[True], outs[False])
    assert np.isfinite(outs[True]).any()


def test_s2_and_quantised_pipelined_equal_previous():
    rng = np.random.default_rng(5)
    n = 3000
    pts = np.c_[rng.uniform(-26, 49, n), rng.uniform(34.5, 72, n)]
    val = 1000 + 20 * np.sin(pts[:, 0] / 10) + rng.normal(0, 2, n)
    outs = {}
    for on in (False, True):
        with pipe(on):
            outs[on] = (S2.barnes_S2(pts, val, 1.0, (-26.0, 34.5), 1 / 16, (1200, 600),
                                     method="optimized_convolution_S2"),
                        Q.barnes(pts, val, 1.0, (-26.0, 34.5), 1 / 16, (1200, 600), quant_bits=20))
    assert same(outs[True][0], outs[False][0])
    assert same(outs[True][1], outs[False][1])


@pytest.mark.parametrize("prec", ["fp32c", "fp64"])
def test_batch_pipelined_equals_previous(prec):
    torch = _lib.torch_cuda()
    from fastbarnes_gb300.batched import BatchPlan
    dev = torch.device("cuda", 0)
    flds = []
    for f in range(3):
        pts, val = field(100 + f, 30_000, (-26.0, 34.5), (75 / 2048, 37.5 / 1024), (2048, 1024))
        flds.append(dict(pts=torch.as_tensor(pts, device=dev), val=torch.as_tensor(val, device=dev), sigma=1.0,
                         x0=(-26.0, 34.5), step=(75 / 2048, 37.5 / 1024), size=(2048, 1024)))
    outs = {}
    for on in (False, True):
        with pipe(on):
            plan = BatchPlan(flds, precision=prec, graph=True, knobs=(0, 0, 0, 1 if on else 2), device=dev)
            plan.run()
            plan.run()
            torch.cuda.synchronize()
            outs[on] = [o.cpu().numpy() for o in plan.outs]
            plan.close()
    for a, b in zip(outs[True], outs[False]):
        assert same(a, b)


def test_two_streams_two_threads_match_sequential():
    """The drop-in on two host threads, each on its own torch stream, gives
    the same results as sequential calls (per-call workspace)."""
    torch = _lib.torch_cuda()
    dev = torch.device("cuda", 0)
    inputs = []
    for s in range(2):
        pts, val = field(200 + s, 50_000, (-26.0, 34.5), (75 / 2048, 37.5 / 1024), (2048, 1024))
        inputs.append((torch.as_tensor(pts, device=dev), torch.as_tensor(val, device=dev)))
    args = (1.0, (-26.0, 34.5), (75 / 2048, 37.5 / 1024), (2048, 1024))
    seq = [I.barnes(p, v, *args, precision="fp32c").cpu().numpy() for p, v in inputs]
    results = [None, None]
    errors = []
    streams = [torch.cuda.Stream(dev), torch.cuda.Stream(dev)]
    start = threading.Barrier(2)

    def work(i):
        try:
            torch.cuda.set_device(dev)
            start.wait()
            with torch.cuda.stream(streams[i]):
                outs = [I.barnes(inputs[i][0], inputs[i][1], *args, precision="fp32c") for _ in range(4)]
                streams[i].synchronize()
            results[i] = [o.cpu().numpy() for o in outs]
        except Exception as e:  # reported by the main thread
            errors.append(e)

    th = [threading.Thread(target=work, args=(i,)) for i in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    assert not errors, errors
    for i in range(2):
        for r in results[i]:
            assert same(r, seq[i])
