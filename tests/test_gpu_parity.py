"""GPU parity: libwlgpu.so through its C ABI against the FP64 oracle and the
reference's own outputs.

Tolerances (stated once, used throughout):
  PHASE_TOL  per-loop phases / spin exponents, relative to the largest value
             of the case: FP32 kernel vs FP64 oracle (the reference kernel
             itself is FP32 with approximate divides).
  W_TOL      <W> per group: |W - W64| / max(|W64|, W_FLOOR * S) <= 1e-5, the
             spec tolerance.  S = 8/3 <|w_N|> + 2 <|w_N/2|> + 1/3 <|w_N/4|>
             is the magnitude of the terms of the Richardson sum (S <= 5 for
             scalar QED; with the spin factor each term carries a cosh): the
             floor keeps the metric meaningful when <W> is small because loop
             averages of cos * cosh and the 8/3, -2, 1/3 combination cancel.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

PHASE_TOL = 2e-5
W_TOL = 1e-5
W_FLOOR = 1e-2
GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_ref.npz")


@pytest.fixture(scope="module")
def wl():
    import wltube

    wltube.lib()
    return wltube


@pytest.fixture(scope="module")
def ctx(wl):
    c = wl.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def gold():
    z = np.load(GOLD)
    return z, json.loads(bytes(z["meta"]).decode())


def werr(w, ref, scale=None):
    floor = W_FLOOR * (scale if scale is not None else 1.0)
    return np.max(np.abs(w - ref) / np.maximum(np.abs(ref), floor))


def test_generator_matches_oracle(ctx):
    h = ctx.generate(seed=3, Nl=64, ppl=256, first=5)
    dev = ctx.download(h)
    ctx.release(h)
    host = O.vloops(3, 64, 256, first=5)
    assert np.abs(dev - host).max() < 2e-6
    # closed bridge with the centre of mass at the origin
    assert np.abs(dev.mean(axis=1)).max() < 1e-5


def test_per_loop_phases_match_reference_golden(ctx, wl, gold):
    z, meta = gold
    h = ctx.upload(z["loops"])
    try:
        for case, ref in zip(meta["LOOP_CASES"], z["loop_out"]):
            _d, prof, ffv, fe, l2, cx, cy, T, F, a = case
            fld = wl.field(prof, fermion=fe, nint=50, lambda2=l2, tubedist=a, ff_variant=ffv)
            s, f = ctx.loops(h, fld, cx, cy, T, F)
            scale = max(np.abs(ref[:, :3]).max(), 1e-30)
            assert np.abs(s[:, :3] - ref[:, :3]).max() / scale < PHASE_TOL, case
            if fe:
                fscale = max(np.abs(ref[:, 4:7]).max(), 1e-30)
                assert np.abs(f[:, :3] - ref[:, 4:7]).max() / fscale < PHASE_TOL, case
    finally:
        ctx.release(h)


@pytest.mark.parametrize("nint", [4, 50, 8])
@pytest.mark.parametrize("mode", [0, 1])
def test_per_loop_phases_match_oracle(ctx, wl, nint, mode):
    loops = O.vloops(21, 128, 128)
    h = ctx.upload(loops)
    try:
        for prof, fe, l2, cx, T, F in [("smooth", 1, 1.0, 0.5, 1.0, 1.0),
                                       ("gaussian", 1, 0.5, 1.2, 0.3, 2.0),
                                       ("step", 0, 2.0, 0.2, 0.7, 1.0),
                                       ("quadratic", 1, 1.5, 0.0, 0.2, 1.0)]:
            fld = wl.field(prof, fermion=fe, nint=nint, mode=mode, lambda2=l2)
            s, f = ctx.loops(h, fld, cx, 0.0, T, F)
            os_, of = O.loops_phases(loops, cx, 0.0, T, F,
                                     O.field(prof, fermion=fe, nint=nint, mode=mode, lambda2=l2))
            assert np.abs(s[:, :3] - os_).max() / np.abs(os_).max() < PHASE_TOL, (prof, nint)
            if fe:
                assert np.abs(f[:, :3] - of).max() / np.abs(of).max() < PHASE_TOL, (prof, nint)
    finally:
        ctx.release(h)


def f32_exact(cx, cy, T):
    """Instances the FP32 kernel represents exactly: it evaluates
    (float(cx), float(cy), T' = float(sqrt(T))^2), so the FP64 oracle is given
    the same values and the comparison measures arithmetic error only."""
    rt = np.sqrt(np.asarray(T, dtype=np.float64)).astype(np.float32).astype(np.float64)
    return (np.asarray(cx, np.float32).astype(np.float64),
            np.asarray(cy, np.float32).astype(np.float64), rt * rt)


def _instances(n, rho_max, Tlo, Thi, seed):
    rng = np.random.default_rng(seed)
    cx = rng.uniform(0.0, rho_max, n)
    cy = rng.uniform(-0.2, 0.2, n)
    T = np.exp(rng.uniform(np.log(Tlo), np.log(Thi), n))
    return f32_exact(cx, cy, T)


@pytest.mark.parametrize("prof,fe,nint,l2,tol", [
    ("smooth", 0, 4, 1.0, W_TOL), ("smooth", 1, 4, 1.0, W_TOL), ("smooth", 1, 50, 1.0, W_TOL),
    ("gaussian", 1, 4, 1.0, W_TOL), ("gaussian", 0, 50, 0.25, W_TOL),
    ("quadratic", 1, 8, 1.0, W_TOL), ("step", 0, 4, 2.0, W_TOL),
    ("smooth", 0, 50, 0.01, W_TOL), ("gaussian", 1, 50, 1.0, W_TOL),
    ("quadratic", 0, 50, 1.0, W_TOL), ("quadratic", 1, 50, 1.0, W_TOL),
    ("step", 0, 50, 2.0, W_TOL),
    # the step profile's f' jumps from 1/lambda^2 to 0 at rho^2 = lambda^2: a
    # Simpson node within FP32 rounding of the edge lands on either side in the
    # FP32 kernel and the FP64 oracle, which moves that loop's spin exponent by
    # a finite amount -- the spinor result is discontinuous in its inputs
    ("step", 1, 4, 2.0, 1e-3)])
def test_batched_eval_matches_oracle(ctx, wl, prof, fe, nint, l2, tol):
    # T <= 4 and F <= 1.5 keep F T' <= 6: beyond F T' ~ 10 the FP32 rounding
    # of each segment's phase contribution (summed over loops whose segment
    # contributions cancel) gives phase errors that the 1e-2 S floor turns
    # into more than 1e-5 -- see test_strong_field_error_is_fp32_limited
    loops = O.vloops(2, 256, 256)
    cx, cy, T = _instances(160, 3.0, 0.01, 4.0, 7)
    F = [0.1, 1.0, 1.5]
    h = ctx.upload(loops)
    try:
        g, mean, sem = ctx.eval(h, wl.field(prof, fermion=fe, nint=nint, lambda2=l2),
                                cx, cy, T, F, group=128)
        assert ctx.last_launches()[1] == "instance-parallel"
    finally:
        ctx.release(h)
    ref, S = O.eval_groups(loops, cx, cy, T, F, O.field(prof, fermion=fe, nint=nint, lambda2=l2),
                           return_scale=True)
    assert werr(g, ref, S) < tol
    # the mean over groups inherits the per-group error budget
    budget = tol * np.maximum(np.abs(ref), W_FLOOR * S).mean(axis=2)
    assert np.all(np.abs(mean - ref.mean(axis=2)) <= budget)


def test_strong_field_error_is_fp32_limited(ctx, wl):
    """With F T' up to 30 (spin exponents up to ~60) the error against FP64
    grows with the field: |dW| <= 1e-5 max(|W|, 1e-2 S) (1 + 2 F T'/25).
    The FP32 segment phases set it (their absolute error, ~1e-7 of the sum of
    the segment contributions' magnitudes, is amplified 100-fold by the floor
    wherever the cosines of the dominant loops are small); the spin exponents'
    FP32 error contributes an order of magnitude less."""
    loops = O.vloops(2, 256, 256)
    cx, cy, T = _instances(96, 1.0, 1.0, 10.0, 9)
    F = [1.0, 3.0]
    fld = wl.field("smooth", fermion=1, nint=4)
    h = ctx.upload(loops)
    try:
        g, _, _ = ctx.eval(h, fld, cx, cy, T, F)
    finally:
        ctx.release(h)
    ofld = O.field("smooth", fermion=1, nint=4)
    ref, S = O.eval_groups(loops, cx, cy, T, F, ofld, return_scale=True)
    # 2 F T' (the largest spin exponent, 2 F T' f'(0) with lambda = 1)
    psi = 2.0 * np.asarray(F)[None, :, None] * T[:, None, None]
    err = np.abs(g - ref) / np.maximum(np.abs(ref), W_FLOOR * S)
    assert np.all(err <= W_TOL * (1.0 + psi / 25.0))


def test_cosh_sentinel_regime_matches_oracle(ctx, wl):
    """The reference's large-cosh sentinel (Integrand.c:371-377): a loop whose
    int-truncated N/2 spin exponent or N/4 sum exceeds 600 gets its three W
    factors multiplied by 1e10 instead of by cosh.  A wide smooth tube
    (lambda^2 = 100) at F = 50, rho = 0, T = 2000 (eB = 1 at the axis, as
    testT.c:20 sets it) gives ten such loops among 256 beside loops with
    cosh arguments up to ~350.  Per loop (EV() over a list of one loop
    repeated, the W factors of the loop-parallel kernel) the result equals
    the oracle's EVMean of that loop: 1e10 times the Richardson sum of its
    cosines for the sentinel loops, the cos * cosh sum for the others; and
    the group <W> of the instance-parallel sweep matches the oracle."""
    torch = pytest.importorskip("torch")
    loops = O.vloops(8, 256, 256)
    Nl, ppl = loops.shape[:2]
    l2, F = 100.0, 50.0
    cx, cy, T = f32_exact([0.0], [0.0], [2000.0])
    ofld = O.field("smooth", fermion=1, nint=4, lambda2=l2)
    s64, f64 = O.loops_phases(loops, cx[0], cy[0], T[0], F, ofld)
    nb4 = f64[:, 1] + f64[:, 2]
    sent = (np.trunc(np.abs(nb4)) > 600) | (np.trunc(np.abs(f64[:, 0])) > 600)
    assert 3 <= sent.sum() <= 40
    # no loop within reach of the truncation edge (FP32 exponent error ~1e-4)
    assert np.min(np.abs(np.abs(np.concatenate([nb4, f64[:, 0]])) - 601.0)) > 1e-2
    args = np.stack([0.5 * f64[:, 0] + 0.25 * nb4, f64[:, 0], 0.5 * nb4], 1)
    order = np.argsort(-np.abs(args).max(axis=1) * ~sent)
    check = list(np.flatnonzero(sent)[:4]) + list(order[:4])
    dev = torch.from_numpy(loops.reshape(-1)).cuda()
    scal_d = torch.zeros(Nl * 4, device="cuda")
    ferm_d = torch.zeros(Nl * 4, device="cuda")
    p = wl.Wparams()
    p.Nl, p.Nppl, p.F, p.l2, p.fermion, p.ng = Nl, ppl, F, l2, 1, Nl // 128
    p.xcm.x, p.xcm.y = float(cx[0]), float(cy[0])
    p.worldlines, p.Wsscal_d, p.Wsferm_d = dev.data_ptr(), scal_d.data_ptr(), ferm_d.data_ptr()
    try:
        wl.legacy_configure("smooth", nint=4)
        for l in check:
            got = wl.EV(float(T[0]), p, np.full(128, l))
            w = O.wfactors(s64[l], f64[l], 1)
            ref = 8 / 3 * w[0] - 2 * w[1] + 1 / 3 * w[2]
            # each factor's size without its cosine (1e10, or cosh of its
            # argument); the kernel's phases are good to ~1e-5 rad and its
            # spin exponents to ~1e-7 relative: tolerance 1e-4 rad and 1e-6
            # of the argument
            size = np.full(3, 1e10) if sent[l] else np.cosh(args[l])
            err_k = 1e-4 + (0.0 if sent[l] else 1e-6 * np.abs(args[l]))
            tol = np.dot([8 / 3, 2.0, 1 / 3], size * err_k)
            assert abs(got - ref) <= tol, (int(l), bool(sent[l]), got, ref)
            if sent[l]:
                assert abs(got) <= 5.1e10  # 1e10 times cosines: the sentinel fired
            else:
                assert abs(got) > 1e20     # cosh of an argument above 50
    finally:
        wl.legacy_configure("smooth")
    h = ctx.upload(loops)
    try:
        g, _, _ = ctx.eval(h, wl.field("smooth", fermion=1, nint=4, lambda2=l2), cx, cy, T, [F])
    finally:
        ctx.release(h)
    ref, S = O.eval_groups(loops, cx, cy, T, [F], ofld, return_scale=True)
    assert np.all(np.isfinite(g))
    assert werr(g, ref, S) <= 1e-2


def test_loop_parallel_eval_matches_oracle(ctx, wl):
    loops = O.vloops(4, 512, 64)
    cx, cy, T = _instances(5, 2.0, 0.05, 5.0, 11)
    fld = wl.field("smooth", fermion=1, nint=4)
    h = ctx.upload(loops)
    try:
        g, mean, sem = ctx.eval(h, fld, cx, cy, T, [1.0], group=128)
        assert ctx.last_launches()[1] == "loop-parallel"
    finally:
        ctx.release(h)
    ref, S = O.eval_groups(loops, cx, cy, T, [1.0], O.field("smooth", fermion=1, nint=4),
                           return_scale=True)
    assert werr(g, ref, S) < W_TOL
    assert np.all(sem >= 0)


def test_same_alone_and_in_the_mix(ctx, wl):
    """An instance's <W> does not depend on the batch it is evaluated in."""
    loops = O.vloops(5, 256, 128)
    cx, cy, T = _instances(300, 2.5, 0.02, 8.0, 3)
    fld = wl.field("smooth", fermion=1, nint=4)
    h = ctx.upload(loops)
    try:
        g_all, _, _ = ctx.eval(h, fld, cx, cy, T, [1.0, 2.0])
        g_sub, _, _ = ctx.eval(h, fld, cx[:40], cy[:40], T[:40], [1.0, 2.0])
        g_one, _, _ = ctx.eval(h, fld, cx[7:8], cy[7:8], T[7:8], [1.0, 2.0])
    finally:
        ctx.release(h)
    # same sweep kernel, batch-independent loop partition: bit for bit
    assert np.array_equal(g_sub, g_all[:40])
    # alone, a single instance runs on the loop-parallel kernel
    assert werr(g_one, g_all[7:8]) < W_TOL


def test_legacy_EV_matches_reference_golden(wl, gold):
    torch = pytest.importorskip("torch")
    z, meta = gold
    loops = z["loops"]
    Nl, ppl = loops.shape[:2]
    dev = torch.from_numpy(loops.reshape(-1)).cuda()
    scal_d = torch.zeros(Nl * 4, device="cuda")
    ferm_d = torch.zeros(Nl * 4, device="cuda")
    scal_h = np.zeros((Nl, 4), dtype=np.float32)
    ferm_h = np.zeros((Nl, 4), dtype=np.float32)
    for case, ref in zip(meta["EV_CASES"], z["ev_out"]):
        d, fe, l2, cx, T, F = case
        wl.legacy_configure(d, nint=50)
        p = wl.Wparams()
        p.Nl, p.Nppl, p.F, p.l2, p.fermion, p.ng = Nl, ppl, F, l2, fe, Nl // 128
        p.xcm.x, p.xcm.y = cx, 0.0
        p.worldlines = dev.data_ptr()
        p.Wsscal_d, p.Wsferm_d = scal_d.data_ptr(), ferm_d.data_ptr()
        p.Wsscal_h = scal_h.ctypes.data
        p.Wsferm_h = ferm_h.ctypes.data
        got = np.array([wl.EV(T, p, np.arange(g * 128, (g + 1) * 128)) for g in range(Nl // 128)])
        np.testing.assert_allclose(got, ref, rtol=W_TOL, err_msg=str(case))
        # any other index list goes through the list kernel: a group in
        # another order (FP64 sums in another order), and one loop repeated
        # against its phases (Integrand.c:325-407's W factors, scalar QED)
        rot = wl.EV(T, p, np.roll(np.arange(128, 256), 5))
        assert abs(rot - got[1]) <= 1e-12 * max(abs(got[1]), 1.0)
        if not fe:
            sx, sy, sz = (float(v) for v in scal_h[7, :3])
            one = (8 / 3 * np.cos(0.5 * sx + 0.25 * (sy + sz)) - 2 * np.cos(sx)
                   + 1 / 3 * np.cos(0.5 * (sy + sz)))
            # the phases in Wsscal_h are rounded to float: a few ulp of |phase|
            tol = 20 * 2.0 ** -24 * max(abs(sx), abs(sy), abs(sz), 1.0)
            assert abs(wl.EV(T, p, np.full(128, 7)) - one) <= tol, case
        # the reference's side effect: per-loop phases copied to Wsscal_h
        s64, f64 = O.loops_phases(loops, cx, 0.0, T, F, O.field(d, fermion=fe, lambda2=l2))
        assert np.abs(scal_h[:, :3] - s64).max() / np.abs(s64).max() < PHASE_TOL
    wl.legacy_configure("smooth")


def test_legacy_EV_selects_the_intEVff_variant(ctx, wl):
    """EV() for the fixflux profile with intEVff.cu's fits (the reference
    links intEVff.o instead of intEV.o): every group's <W> equals wl_eval's
    with ff_variant 1, and differs from the intEV.cu variant's."""
    torch = pytest.importorskip("torch")
    loops = O.vloops(14, 256, 128)
    Nl, ppl = loops.shape[:2]
    dev = torch.from_numpy(loops.reshape(-1)).cuda()
    scal_d = torch.zeros(Nl * 4, device="cuda")
    p = wl.Wparams()
    p.Nl, p.Nppl, p.F, p.l2, p.fermion, p.ng = Nl, ppl, 1.0, 0.5, 0, Nl // 128
    p.xcm.x, p.xcm.y = 1.1, 0.0
    p.worldlines, p.Wsscal_d = dev.data_ptr(), scal_d.data_ptr()
    T = 0.7
    try:
        res = {}
        for name, ffv in (("fixflux-ff", 1), ("fixflux", 0)):
            wl.legacy_configure(name, tubedist=2.0, nint=8)
            res[ffv] = np.array([wl.EV(T, p, np.arange(g * 128, (g + 1) * 128))
                                 for g in range(Nl // 128)])
            h = ctx.upload(loops)
            g, _, _ = ctx.eval(h, wl.field("fixflux", nint=8, lambda2=0.5, tubedist=2.0,
                                           ff_variant=ffv), [1.1], [0.0], [T], [1.0])
            ctx.release(h)
            assert werr(res[ffv], g[0, 0]) < W_TOL, name
        assert np.max(np.abs(res[1] - res[0])) > 1e-6
    finally:
        wl.legacy_configure("smooth")


def test_legacy_EV_sees_an_ensemble_rewritten_in_place(wl):
    """EV() caches the sweep of its last (T, x_cm, ...) key; a caller that
    rewrites the loops in place and calls again at the same key gets the new
    loops' <W>: the first group's call compares the ensemble's fingerprint,
    and wl_legacy_invalidate() drops the cache for the other groups."""
    torch = pytest.importorskip("torch")
    a = O.vloops(31, 256, 128)
    b = O.vloops(32, 256, 128)
    Nl, ppl = a.shape[:2]
    dev = torch.from_numpy(a.reshape(-1).copy()).cuda()
    scal_d = torch.zeros(Nl * 4, device="cuda")
    p = wl.Wparams()
    p.Nl, p.Nppl, p.F, p.l2, p.fermion, p.ng = Nl, ppl, 1.0, 1.0, 0, Nl // 128
    p.xcm.x, p.xcm.y = 0.4, 0.0
    p.worldlines, p.Wsscal_d = dev.data_ptr(), scal_d.data_ptr()
    T = 1.3
    g0, g1 = np.arange(128), np.arange(128, 256)
    fld = O.field("smooth", fermion=0, nint=50)
    cx, _, Tp = f32_exact([0.4], [0.0], [T])
    ref_a = O.eval_groups(a, cx, 0.0, Tp, [1.0], fld)[0, 0]
    ref_b = O.eval_groups(b, cx, 0.0, Tp, [1.0], fld)[0, 0]
    try:
        wl.legacy_configure("smooth", nint=50)
        got_a = [wl.EV(T, p, g0), wl.EV(T, p, g1)]
        np.testing.assert_allclose(got_a, ref_a, rtol=W_TOL)
        # rewrite in place, same key: the first group's call notices
        dev.copy_(torch.from_numpy(b.reshape(-1).copy()).cuda())
        torch.cuda.synchronize()
        got_b0 = wl.EV(T, p, g0)
        np.testing.assert_allclose(got_b0, ref_b[0], rtol=W_TOL)
        np.testing.assert_allclose(wl.EV(T, p, g1), ref_b[1], rtol=W_TOL)
        # rewrite back, then ask for the second group first: invalidate
        dev.copy_(torch.from_numpy(a.reshape(-1).copy()).cuda())
        torch.cuda.synchronize()
        wl.legacy_invalidate()
        np.testing.assert_allclose(wl.EV(T, p, g1), ref_a[1], rtol=W_TOL)
        # any non-consecutive list also checks the fingerprint
        dev.copy_(torch.from_numpy(b.reshape(-1).copy()).cuda())
        torch.cuda.synchronize()
        rot = wl.EV(T, p, np.roll(g1, 3))
        np.testing.assert_allclose(rot, ref_b[1], rtol=W_TOL)
    finally:
        wl.legacy_configure("smooth")


def test_legacy_EV_rejects_host_pointers(wl):
    p = wl.Wparams()
    loops = np.zeros((128, 8, 4), dtype=np.float32)
    p.Nl, p.Nppl, p.F, p.l2 = 128, 8, 1.0, 1.0
    p.worldlines = loops.ctypes.data  # host memory: must be refused, not dereferenced
    assert np.isnan(wl.EV(1.0, p, np.arange(128)))


def test_invalid_arguments_return_status(ctx, wl):
    loops = O.vloops(1, 128, 16)
    h = ctx.upload(loops)
    try:
        with pytest.raises(wl.WlError) as e:
            ctx.eval(h, wl.field("smooth", nint=3), [0.0], [0.0], [1.0], [1.0])
        assert e.value.status == -1
        with pytest.raises(wl.WlError):
            ctx.eval(h, wl.field("smooth"), [0.0], [0.0], [-1.0], [1.0])
        with pytest.raises(wl.WlError):
            ctx.eval(h, wl.field("smooth"), [0.0], [0.0], [1.0], [1.0], group=100)
        with pytest.raises(wl.WlError) as e:
            ctx.eval(h + 1000, wl.field("smooth"), [0.0], [0.0], [1.0], [1.0])
        assert e.value.status == -5
        with pytest.raises(wl.WlError):
            ctx.upload(np.zeros((4, 6, 4), dtype=np.float32))  # ppl not a multiple of 4
    finally:
        ctx.release(h)


@pytest.mark.parametrize("a,l2,fe", [(2.0, 1.0, 1), (5.0, 1.0, 0), (2.0, 0.25, 0),
                                     (10.0, 1.0, 1), (10.0, 1.0, 0)])
def test_lattice_matches_oracle(ctx, wl, a, l2, fe):
    """Square lattice of Gaussian tubes (image sum to |R| <= 12a) against the
    FP64 oracle's image sum on a 4 x 4 grid of centres over one unit cell."""
    loops = O.vloops(3, 128, 128)
    g1 = (np.arange(4) + 0.5) * a / 4
    cx0, cy0 = [v.ravel() for v in np.meshgrid(g1, g1)]
    T0 = np.array([0.05, 0.5, 2.0, 6.0])
    cx, cy, T = f32_exact(np.repeat(cx0, 4), np.repeat(cy0, 4), np.tile(T0, 16))
    fld = wl.field("lattice", fermion=fe, nint=4, lambda2=l2, tubedist=a)
    ofld = O.field("lattice", fermion=fe, nint=4, mode=1, lambda2=l2, tubedist=a)
    # the per-loop phase check takes the instance with the largest phases (at
    # a = 10 lambda most centres are far from every tube: phases ~1e-5)
    k = int(np.argmax([np.abs(O.loops_phases(loops, x, y, t, 1.0, ofld)[0]).max()
                       for x, y, t in zip(cx, cy, T)]))
    h = ctx.upload(loops)
    try:
        g, _, _ = ctx.eval(h, fld, cx, cy, T, [1.0])
        # a different set of launch-mates (other thread partners and warps):
        # the same bits for every instance
        sub = np.array([i for i in range(len(T)) if i % 3])  # >= 32: the same kernel
        g_sub, _, _ = ctx.eval(h, fld, cx[sub], cy[sub], T[sub], [1.0])
        assert np.array_equal(g_sub, g[sub])
        s, f = ctx.loops(h, fld, float(cx[k]), float(cy[k]), float(T[k]), 1.0)
    finally:
        ctx.release(h)
    ref, S = O.eval_groups(loops, cx, cy, T, [1.0], ofld, return_scale=True)
    # the FP32 limit of test_strong_field_error_is_fp32_limited
    psi = np.array([np.abs(O.loops_phases(loops, x, y, t, 1.0, ofld)[1]).max() if fe else 0.0
                    for x, y, t in zip(cx, cy, T)])
    err = np.abs(g - ref) / np.maximum(np.abs(ref), W_FLOOR * S)
    assert np.all(err[:, 0, :] <= W_TOL * (1.0 + psi[:, None] / 25.0))
    os_, of = O.loops_phases(loops, cx[k], cy[k], T[k], 1.0, ofld)
    assert np.abs(os_).max() > 0.1
    assert np.abs(s[:, :3] - os_).max() / np.abs(os_).max() < PHASE_TOL


@pytest.mark.parametrize("mode,fe,a", [(0, 0, 1.0), (0, 1, 1.0), (1, 1, 2.0), (1, 0, 2.0)])
def test_spline_profile_matches_oracle(ctx, wl, mode, fe, a):
    """The tabulated profile of periodic.c (the library's table against the
    oracle's independently built one), per-loop phases and <W> per group."""
    loops = O.vloops(6, 256, 256)
    cx, cy, T = _instances(96, 2.0 * a, 0.01, 4.0, 13)
    F = [0.5, 1.0]
    fld = wl.field("spline", fermion=fe, nint=8, mode=mode, lambda2=0.5, tubedist=a)
    ofld = O.field("spline", fermion=fe, nint=8, mode=mode, lambda2=0.5, tubedist=a)
    h = ctx.upload(loops)
    try:
        g, _, _ = ctx.eval(h, fld, cx, cy, T, F)
        s, f = ctx.loops(h, fld, float(cx[5]), float(cy[5]), float(T[5]), 1.0)
    finally:
        ctx.release(h)
    ref, S = O.eval_groups(loops, cx, cy, T, F, ofld, return_scale=True)
    assert werr(g, ref, S) < W_TOL
    rs, rf = O.loops_phases(loops, float(cx[5]), float(cy[5]), float(T[5]), 1.0, ofld)
    assert np.abs(s[:, :3] - rs).max() / max(np.abs(rs).max(), 1e-30) < PHASE_TOL
    if fe:
        assert np.abs(f[:, :3] - rf).max() / max(np.abs(rf).max(), 1e-30) < PHASE_TOL
