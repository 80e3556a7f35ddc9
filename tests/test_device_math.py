"""Host checks of constants the kernels use (no GPU): the polynomial for
(1 - e^-x)/x on [0, 0.5] (Gaussian and lattice profiles), evaluated in FP32
Horner form as the device does, against the function in FP64."""
import os
import re

import numpy as np

SRC = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                   "worldline-flux-tube-lattice_gb300", "csrc", "wl_device.cuh")


def test_small_x_polynomial_of_gaussian_integrand():
    src = open(SRC).read()
    body = src[src.index("one_minus_expneg_over_x(float x) {"):]
    body = body[:body.index("return p;")]
    # the Horner chain from c5 down to c0, as the device evaluates it
    c = np.array([float(v) for v in re.findall(r"(-?\d\.\d+(?:e-?\d+)?)f", body)][::-1],
                 np.float32)
    assert len(c) == 6
    x = np.linspace(0.0, 0.5, 200001).astype(np.float32)
    p = np.full_like(x, c[5])
    for k in (4, 3, 2, 1, 0):  # fmaf: one rounding per step
        p = (p.astype(np.float64) * x.astype(np.float64) + np.float64(c[k])).astype(np.float32)
    xd = x.astype(np.float64)
    ref = np.where(xd > 0, -np.expm1(-xd) / np.where(xd > 0, xd, 1.0), 1.0)
    assert np.max(np.abs(p - ref) / ref) < 5.5e-8
