"""The CPU oracle against the reference's own outputs (golden vectors).

tests/golden/golden_ref.npz was produced by tests/golden/make_golden.py,
which runs the reference's own intEV.cu / intEVff.cu / Integrand.c / Tint.c
(compiled for the CPU by oracle/build_ref.sh) on a seeded 256 x 64 ensemble.
The reference computes in FP32 (kernel) and FP64 (host), the oracle in FP64;
tolerances are set by the reference's FP32 rounding.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_ref.npz")


@pytest.fixture(scope="module")
def gold():
    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]).decode())
    return z, meta


def test_fixture_shapes(gold):
    z, meta = gold
    assert z["loops"].shape == (meta["NL"], meta["PPL"], 4)
    assert z["loop_out"].shape == (len(meta["LOOP_CASES"]), meta["NL"], 8)


def test_per_loop_phases_match_reference(gold):
    z, meta = gold
    loops = z["loops"]
    for case, ref in zip(meta["LOOP_CASES"], z["loop_out"]):
        _d, prof, ffv, fe, l2, cx, cy, T, F, a = case
        fld = O.field(prof, fermion=fe, nint=50, lambda2=l2, tubedist=a, ff_variant=ffv)
        s, f = O.loops_phases(loops, cx, cy, T, F, fld)
        scale = max(np.abs(s).max(), 1e-30)
        # FP32 reference: relative to the largest phase of the case
        assert np.abs(ref[:, :3] - s).max() / scale < 3e-6, case
        if fe:
            fscale = max(np.abs(f).max(), 1e-30)
            assert np.abs(ref[:, 4:7] - f).max() / fscale < 3e-6, case


def test_ev_matches_reference(gold):
    z, meta = gold
    loops = z["loops"]
    for case, ref in zip(meta["EV_CASES"], z["ev_out"]):
        d, fe, l2, cx, T, F = case
        fld = O.field(d, fermion=fe, nint=50, lambda2=l2)
        o = O.eval_groups(loops, cx, 0.0, T, F, fld, group=128)[0, 0]
        np.testing.assert_allclose(o, ref, rtol=2e-6, err_msg=str(case))


def test_tfunc_matches_reference(gold):
    z, meta = gold
    loops = z["loops"]
    for case, ref in zip(meta["TF_CASES"], z["tf_out"]):
        d, fe, l2, cx, T, F = case
        fld = O.field(d, fermion=fe, nint=50, lambda2=l2)
        reg, an = O.tfunc_regime(T, cx, 0.0, F, fld)
        if reg == 3:
            ev = O.eval_groups(loops, cx, 0.0, T, F, fld)[0, 0]
            o = np.array([O.tfunc_mc(T, e, cx, 0.0, F, fld) for e in ev])
        else:
            o = np.full(len(ref), an)
        np.testing.assert_allclose(o, ref, rtol=1e-6, atol=1e-12, err_msg=str(case))


def test_integrateT_matches_reference(gold):
    z, meta = gold
    loops = z["loops"]
    for case, ref in zip(meta["IT_CASES"], z["it_out"]):
        d, fe, l2, cx, n, F = case
        fld = O.field(d, fermion=fe, nint=50, lambda2=l2)
        val, leff, sem = O.integrateT(loops, n, cx, 0.0, F, fld)
        np.testing.assert_allclose(val, ref, rtol=1e-6, err_msg=str(case))
        # Tintout (Tint.c:51-73)
        avg = val.mean()
        assert np.isclose(leff, avg / (4 * np.pi) if fe else avg / (-2 * np.pi))


def test_profile_and_field_functions_match_reference(gold):
    z, meta = gold
    pairs = z["fn_pairs"]
    for case, ref in zip(meta["FN_CASES"], z["fn_out"]):
        d, l2, F, fe, a = case
        fld = O.field(d, fermion=fe, lambda2=l2, tubedist=a)
        L = O.lib()
        fl = np.array([L.wlo64_flambda(p[0], fld) for p in pairs])
        fpl = np.array([L.wlo64_fplambda(p[0], fld) for p in pairs])
        B = np.array([O.magfield(p[0], F, fld) for p in pairs])
        # f_lambda, f'_lambda: FP32 in the reference kernel
        np.testing.assert_allclose(fl, ref[:, 0], rtol=2e-6, atol=1e-6, err_msg=d)
        np.testing.assert_allclose(fpl, ref[:, 1], rtol=2e-6, atol=1e-6, err_msg=d)
        # host FP64 functions
        np.testing.assert_allclose(B, ref[:, 2], rtol=1e-12, err_msg=d)
        ex = np.array([O.exact(p[1], b, fe) for p, b in zip(pairs, B)])
        # TB/sinh(TB) - 1 + TB^2/6 cancels: B differences of 1e-16 grow to ~1e-9
        np.testing.assert_allclose(ex, ref[:, 3], rtol=1e-6, atol=1e-300, err_msg=d)
        s1 = np.array([O.smT(b, p[1], 0) for p, b in zip(pairs, B)])
        s2 = np.array([O.smT(b, p[1], 1) for p, b in zip(pairs, B)])
        np.testing.assert_allclose(s1, ref[:, 4], rtol=1e-12, atol=1e-300, err_msg=d)
        np.testing.assert_allclose(s2, ref[:, 5], rtol=1e-12, atol=1e-300, err_msg=d)
