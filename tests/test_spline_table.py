"""The spline profile's table (no GPU): the library's host builder
(wl_spline_table: Gauss-Legendre per knot interval, clamped cubic spline in
rho^2) against the oracle's independent restatement (composite Simpson,
second-derivative spline form).  Both against the reference's own table
builder (periodic.c:113-164 with a GSL stand-in): test_spline_reference.py."""
import os
import sys

import numpy as np
import pytest

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "worldline-flux-tube-lattice_gb300"))


def library_interp(rho2, knots, coef):
    """interp (intEV.cu:64-107) on the library's table, in FP64."""
    out = np.zeros_like(rho2)
    inside = (rho2 < knots[-1]) & (rho2 > knots[0])
    j = np.searchsorted(knots, rho2[inside], side="right") - 1
    d = rho2[inside] - knots[j].astype(np.float64)
    c = coef[j].astype(np.float64)
    out[inside] = c[:, 0] + d * (c[:, 1] + d * (c[:, 2] + d * c[:, 3]))
    return out


@pytest.mark.parametrize("l2,a", [(1.0, 1.0), (0.25, 2.0), (2.0, 5.0)])
def test_library_table_matches_oracle(l2, a):
    import wltube

    knots, coef = wltube.spline_table(l2, a)
    ox, of = O.spline_table(l2, a)
    assert np.array_equal(knots.astype(np.float64), ox)          # float(rho_i^2)
    np.testing.assert_allclose(coef[:, 0], of, rtol=2e-7, atol=1e-9)
    # the interpolant between the knots
    rng = np.random.default_rng(0)
    r2 = np.concatenate([rng.uniform(0, 400, 4000), rng.uniform(0, 2, 1000), [0.0, 1e-4, 401.0]])
    fld = O.field("spline", lambda2=l2, tubedist=a)
    ref = np.array([O.spline_eval(x, fld) for x in r2])
    lib = library_interp(r2, knots, coef)
    scale = np.abs(of).max()
    assert np.abs(lib - ref).max() <= 2e-6 * scale
    # outside the table interp gives 0 (intEV.cu:82-101)
    assert lib[-3] == 0.0 and ref[-3] == 0.0 and lib[-1] == 0.0


def test_table_is_the_profile_integral():
    """f(rho) at the knots against the integral of the right-hand side done
    independently (fine trapezoid), and f' = df/drho^2 matching the
    right-hand side / (2 rho)."""
    import wltube

    l2, a = 0.5, 1.0
    knots, coef = wltube.spline_table(l2, a)
    r = np.linspace(0.0, 20.0, 2_000_001)
    g = 2.0 / l2 * r * np.exp(-np.sin(np.pi * r / a) ** 2 / l2)
    F = np.concatenate([[0.0], np.cumsum(0.5 * (g[1:] + g[:-1]) * np.diff(r))])
    idx = np.arange(1, 1001) * 2000
    np.testing.assert_allclose(coef[:, 0], F[idx], rtol=1e-6, atol=1e-9)
    # the spline slope b at interior knots approximates df/drho^2
    rho = np.sqrt(knots[100:900].astype(np.float64))
    fp = np.exp(-np.sin(np.pi * rho / a) ** 2 / l2) / l2
    assert np.abs(coef[100:900, 1] - fp).max() < 1e-3 * fp.max()
