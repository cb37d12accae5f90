"""Quantised interpolation (fastbarnes_gb300.quantinterpolation, the fused
epilogue of fb_interpolate_quant) against the reference's demo outputs
(tests/golden/quant.npz) and against the oracle's quant() of the GPU's own
float64 result.

Tolerances: the quantisation of the GPU's float64 quotient is reproduced bit
for bit; against the reference the quantised values agree except where the
unquantised values (1e-14-level apart) fall on different sides of a rounding
boundary, i.e. within one unit of the kept last bit.
"""
import numpy as np
import pytest

from fastbarnes_gb300 import interpolation as I
from fastbarnes_gb300 import quantinterpolation as QI
from oracle import oracle

pytestmark = pytest.mark.gpu


def test_quantised_matches_reference_and_epilogue(golden):
    g = golden("quant.npz")
    size = tuple(int(s) for s in g["size"])
    args = (g["pts"], g["val"], float(g["sigma"]), g["x0"], float(g["step"]), size)
    plain = I.barnes(*args, method="convolution", num_iter=int(g["n"]), out_dtype=np.float64)
    for b in g["bits"]:
        b = int(b)
        mine = QI.barnes(*args, b, num_iter=int(g["n"]))
        assert mine.dtype == np.float64
        assert np.array_equal(mine, oracle.quant(plain, b), equal_nan=True), b
        ref = g[f"out_{b}"]
        assert np.array_equal(np.isnan(mine), np.isnan(ref))
        m = ~np.isnan(ref)
        ulp = np.ldexp(1.0, np.frexp(np.abs(ref[m]))[1] - (53 - b))
        assert np.all(np.abs(mine[m] - ref[m]) <= ulp), b
