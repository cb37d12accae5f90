"""fastbarnes_gb300: the optimized-convolution Barnes interpolation of
MeteoSwiss/fast-barnes-py, rebuilt as sm_103a CUDA kernels for one GB300.

Modules mirror the reference package:
  fastbarnes_gb300.interpolation    -> fastbarnes.interpolation (barnes, helpers)
  fastbarnes_gb300.interpolationS2  -> fastbarnes.interpolationS2 (barnes_S2)
  fastbarnes_gb300.util.lambert_conformal -> fastbarnes.util.lambert_conformal
plus fastbarnes_gb300.batched (many fields per launch) and
fastbarnes_gb300.autograd (gradients through the interpolation).
"""
from ._lib import FastBarnesError, build, version  # noqa: F401

__all__ = ["FastBarnesError", "build", "version"]
