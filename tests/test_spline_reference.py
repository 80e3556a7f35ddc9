"""The spline profile's table (no GPU) against the reference's own table
builder: getspline of periodic.c:113-164, compiled from the reference's
source with the GSL ODE stand-in of oracle/refshim/ (its rk8pd step on the
profile's y-independent right-hand side restated as a quadrature of the
step), in tests/golden/spline_ref.npz (tests/golden/make_spline_golden.py).

The library's table (wl_spline_table, the one the kernels interpolate) has
the reference's knots bit for bit, its values f to the last FP32 bit, and
its spline coefficients to within two FP32 ulps (the reference's double
values of f come from GSL's stepper, the library's from its own quadrature:
a last-bit difference in f can move a coefficient by an ulp); the oracle's
independently built table matches to its FP32 rounding."""
import os
import sys

import numpy as np

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "worldline-flux-tube-lattice_gb300"))
GOLD = os.path.join(ROOT, "tests", "golden", "spline_ref.npz")


def interp64(rho2, knots, coef):
    """interp (intEV.cu:64-107) on a table, in FP64."""
    out = np.zeros_like(rho2)
    inside = (rho2 < knots[-1]) & (rho2 > knots[0])
    j = np.searchsorted(knots, rho2[inside], side="right") - 1
    d = rho2[inside] - knots[j].astype(np.float64)
    c = coef[j].astype(np.float64)
    out[inside] = c[:, 0] + d * (c[:, 1] + d * (c[:, 2] + d * c[:, 3]))
    return out


def test_library_table_is_the_references():
    import wltube

    z = np.load(GOLD)
    rng = np.random.default_rng(3)
    for (l2, a), rk, rc in zip(z["cases"], z["knots"], z["coefs"]):
        knots, coef = wltube.spline_table(float(l2), float(a), len(rk))
        assert np.array_equal(knots, rk), (l2, a)
        ulp = np.spacing(np.abs(rc[:-1]).astype(np.float32))
        diff = np.abs(coef[:-1].astype(np.float64) - rc[:-1])
        assert np.all(diff[:, 0] <= ulp[:, 0]), (l2, a)          # f: the last bit at most
        assert np.all(diff[:, 1:] <= 2 * ulp[:, 1:]), (l2, a)    # b, c, d: two ulps
        assert np.array_equal(coef[-1, [0, 2]], rc[-1, [0, 2]])
        # the interpolants agree to FP32 rounding of the profile
        r2 = np.concatenate([rng.uniform(0, float(rk[-1]), 5000), rng.uniform(0, 1, 1000)])
        lib, ref = interp64(r2, knots, coef), interp64(r2, rk, rc)
        assert np.abs(lib - ref).max() <= 1e-7 * np.abs(rc[:, 0]).max(), (l2, a)


def test_oracle_table_matches_the_reference():
    z = np.load(GOLD)
    for (l2, a), rk, rc in zip(z["cases"], z["knots"], z["coefs"]):
        x, f = O.spline_table(float(l2), float(a), len(rk))
        assert np.array_equal(x, rk.astype(np.float64)), (l2, a)
        np.testing.assert_allclose(f, rc[:, 0], rtol=2e-7, atol=1e-12)
