"""Host checks of constants the kernels use (no GPU): the polynomial for
(1 - e^-x)/x on [0, 0.5] (Gaussian and lattice profiles), evaluated in FP32
Horner form as the device does, against the function in FP64; and the
FP32-pipe reciprocal of the smooth profile's many-interval segments."""
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


def fma32(a, b, c):
    """fmaf on float32 arrays: the float64 product of two floats is exact, so
    one float64 add and the rounding to float32 give fmaf except in rare
    double-rounding ties (well below the bound checked here)."""
    return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(np.float32)


def test_newton_reciprocal_within_one_ulp():
    src = open(SRC).read()
    body = src[src.index("float rcp_newton(float d) {"):]
    body = body[:body.index("\n}")]
    K = int(re.search(r"0x([0-9a-f]+) - __float_as_int", body).group(1), 16)
    rng = np.random.default_rng(11)
    d = np.concatenate([np.exp(rng.uniform(np.log(1e-30), np.log(1e30), 1_000_000)),
                        np.linspace(1.0, 4.0, 300001)]).astype(np.float32)
    x = newton_reciprocal(d, K, seed_only=True)
    assert np.max(np.abs(x.astype(np.float64) * d.astype(np.float64) - 1.0)) < 0.051
    x = newton_reciprocal(d, K)
    exact = 1.0 / d.astype(np.float64)
    ulp = np.spacing(exact.astype(np.float32)).astype(np.float64)
    assert np.max(np.abs(x.astype(np.float64) - exact) / ulp) < 0.8
    with np.errstate(invalid="ignore"):
        assert np.isnan(newton_reciprocal(np.float32([np.nan]), K)[0])


def newton_reciprocal(d, K, seed_only=False):
    """rcp_newton of the device, step for step in FP32."""
    x = (K - d.view(np.int32).astype(np.int64)).astype(np.int32).view(np.float32)
    if seed_only:
        return x
    one = np.ones_like(d)
    e = fma32(-d, x, one)            # Newton-Raphson step
    x = fma32(x, e, x)
    e = fma32(-d, x, one)            # third-order step
    return fma32(x, fma32(e, e, e), x)
