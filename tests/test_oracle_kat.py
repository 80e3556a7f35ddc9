"""Known-answer tests of the oracle (CPU): physics limits and invariants the
reference's formulas must satisfy, independent of the golden vectors."""
import math

import numpy as np

from oracle import oracle as O


def test_philox_known_answers():
    # Random123 kat_vectors, philox4x32_10
    assert O.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert O.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E,
                                                             0xA20BC7C6, 0x6D5451FD]
    assert O.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344],
                    [0xA4093822, 0x299F31D0]) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_vloops_are_closed_unit_bridges():
    L = O.vloops(5, 512, 256).astype(np.float64)
    assert np.abs(L.mean(axis=1)).max() < 1e-6          # centre of mass at the origin
    d = np.diff(np.concatenate([L, L[:, :1]], axis=1), axis=1)
    # per-component step variance 2/N (kinetic weight exp(-1/4 int xdot^2))
    v = (d ** 2).mean() * 256 / 2.0
    assert abs(v - 1.0) < 0.02
    # different seeds / loop offsets give different loops; same give the same
    assert not np.array_equal(O.vloops(5, 4, 64), O.vloops(6, 4, 64))
    np.testing.assert_array_equal(O.vloops(5, 4, 64, first=2)[0], O.vloops(5, 6, 64)[2])


def test_zero_flux_gives_unit_wilson_loop():
    L = O.vloops(1, 256, 64)
    for prof in ("smooth", "gaussian", "step"):
        for fe in (0, 1):
            w = O.eval_groups(L, [0.3, 1.5], [0.0, 0.2], [0.1, 2.0], [0.0], O.field(prof, fermion=fe))
            np.testing.assert_allclose(w, 1.0, atol=1e-14)


def test_phases_are_linear_in_flux():
    L = O.vloops(2, 128, 64)
    fld = O.field("smooth", fermion=1, nint=4)
    s1, f1 = O.loops_phases(L, 0.7, 0.1, 0.5, 1.0, fld)
    s3, f3 = O.loops_phases(L, 0.7, 0.1, 0.5, 3.0, fld)
    np.testing.assert_allclose(s3, 3 * s1, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(f3, 3 * f1, rtol=1e-13, atol=1e-15)


def test_richardson_combination():
    s = np.array([0.3, 0.1, 0.2])
    f = np.array([0.5, 0.2, 0.1])
    w = O.wfactors(s, f, 1)
    nb4, nb4f = 0.3, 0.3
    assert math.isclose(w[0], math.cos(0.15 + 0.25 * nb4) * math.cosh(0.25 + 0.25 * nb4f))
    assert math.isclose(w[1], math.cos(0.3) * math.cosh(0.5))
    assert math.isclose(w[2], math.cos(0.5 * nb4) * math.cosh(0.5 * nb4f))
    ev = O.evmean(np.tile(s, (4, 1)), np.tile(f, (4, 1)), [0, 1, 2, 3], 1)
    assert math.isclose(ev, 8 / 3 * w[0] - 2 * w[1] + w[2] / 3)


def test_spin_sentinel_truncates_like_c_abs():
    # Integrand.c:371: abs() of a double truncates to int -> fires from 601 on
    w = O.wfactors([0, 0, 0], [600.9, 0, 0], 1)
    assert np.isfinite(w).all() and w[1] > 1e200
    w = O.wfactors([0, 0, 0], [601.0, 0, 0], 1)
    np.testing.assert_allclose(w, 1e10)


def test_constant_field_limit():
    """Inside a wide step tube (rho^2 < lambda^2) the field is constant, eB =
    2F/lambda^2 (Integrand.c:106-112 with B = 2F/e f'): the Monte Carlo <W>
    approaches e B T / sinh(e B T) (scalar) and e B T / tanh(e B T) (spinor),
    Integrand.c:20-37, within the Monte Carlo error.  The reference's
    sub-loop Richardson estimate carries an O(1/N) bias (+0.008 at N = 128,
    below the Monte Carlo error from N ~ 512 on), hence 512 points."""
    Nl, ppl = 2048, 512
    L = O.vloops(7, Nl, ppl)
    l2, F, T = 400.0, 200.0, 0.5      # eBT = 2 F T / l2 = 0.5; loops stay far inside
    x = 2 * F * T / l2
    for fe, exact in ((0, x / math.sinh(x)), (1, x / math.tanh(x))):
        g = O.eval_groups(L, 0.0, 0.0, T, F, O.field("step", fermion=fe, lambda2=l2, nint=4),
                          group=128)[0, 0]
        mean, sem = g.mean(), g.std(ddof=1) / math.sqrt(len(g))
        assert abs(mean - exact) < 4 * sem + 2e-3, (fe, mean, exact, sem)


def test_tfunc_regimes_follow_reference_thresholds():
    fld = O.field("smooth", fermion=0, lambda2=1.0)
    # smallT = (l2 + rho^2)/2 = 0.5 at rho = 0
    assert O.tfunc_regime(0.001, 0.0, 0.0, 1.0, fld)[0] == 0   # T < 0.1 and < 0.01 smallT
    assert O.tfunc_regime(0.5, 0.0, 0.0, 1.0, fld)[0] == 3     # Monte Carlo
    assert O.tfunc_regime(60.0, 0.0, 0.0, 1.0, fld)[0] == 2    # large T
    fld2 = O.field("smooth", fermion=0, lambda2=100.0)
    assert O.tfunc_regime(0.2, 0.0, 0.0, 1.0, fld2)[0] == 1    # const field (T >= 0.1)


def test_lattice_image_selection_matches_full_sum():
    """Skipping the images farther than sqrt(18) lambda from the loop's
    bounding box (pure gauge in FP32, winding 0) leaves the per-loop phases
    and spin exponents of the full image sum (|R| <= 12 a) unchanged to the
    Simpson discretisation error of those pure-gauge images, which 50
    intervals make negligible."""
    L = O.vloops(3, 24, 128)
    try:
        for a, T in ((2.0, 0.05), (2.0, 3.0), (5.0, 10.0)):
            fld = O.field("lattice", fermion=1, nint=50, mode=1, lambda2=1.0, tubedist=a)
            O.set_lattice_rcut(O.LATTICE_RCUT_L)
            s_cut, f_cut = O.loops_phases(L, 0.3 * a, 0.6 * a, T, 1.0, fld)
            O.set_lattice_rcut(0.0)
            s_all, f_all = O.loops_phases(L, 0.3 * a, 0.6 * a, T, 1.0, fld)
            scale = np.abs(s_all).max()
            assert np.abs(s_cut - s_all).max() < 1e-6 * max(scale, 1.0), (a, T)
            assert np.abs(f_cut - f_all).max() < 1e-6 * max(np.abs(f_all).max(), 1.0), (a, T)
    finally:
        O.set_lattice_rcut(O.LATTICE_RCUT_L)


def circle_loops(n_points, radius, windings):
    """Closed polygons on a circle about the origin (float4 points, z = w = 0)."""
    k = np.arange(n_points)
    ang = 2.0 * np.pi * windings * k / n_points
    L = np.zeros((1, n_points, 4), np.float32)
    L[0, :, 0] = radius * np.cos(ang)
    L[0, :, 1] = radius * np.sin(ang)
    return L


def test_pure_gauge_winding_phase():
    """Outside a step tube f = 1: A is pure gauge and every closed sub-loop
    that winds n times around the tube picks up the phase 2 pi F n (the
    scope table's winding known answer) -- in exact mode.  The reference's
    clamp b >= 1e-8 (intEV.cu:420) replaces the negative b of every chord of
    a circle about the origin, so in ref-compat mode the phase falls short
    (2 pi (1 - 7.5e-5) for the N/2 loop of 1024 points)."""
    for windings in (1, 2, -1):
        L = circle_loops(1024, 3.0, windings)
        for F in (0.3, 1.0):
            s, _ = O.loops_phases(L, 0.0, 0.0, 1.0, F,
                                  O.field("step", lambda2=1.0, nint=8, mode=1))
            np.testing.assert_allclose(s[0], 2 * np.pi * F * windings, rtol=1e-9)
    s, _ = O.loops_phases(circle_loops(1024, 3.0, 1), 0.0, 0.0, 1.0, 1.0,
                          O.field("step", lambda2=1.0, nint=8, mode=0))
    assert 1e-5 < 1 - s[0, 0] / (2 * np.pi) < 1e-4
