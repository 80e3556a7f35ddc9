"""Edge cases of the sweep through the C ABI: instance counts around the tile
sizes (32 = loop-parallel threshold, 128 one-instance tiles, 256 pair
tiles) at 4 and 50 intervals, loops whose point count is not a multiple of
the 256-point staging chunk, the smallest loops (4 points), one group, the
largest flux-value count, extreme proper times, argument limits, and the
bounded device wait."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

W_TOL, W_FLOOR = 1e-5, 1e-2


def werr(w, ref, scale):
    return np.max(np.abs(w - ref) / np.maximum(np.abs(ref), W_FLOOR * scale))


def f32_exact(cx, cy, T):
    rt = np.sqrt(np.asarray(T, np.float64)).astype(np.float32).astype(np.float64)
    return (np.asarray(cx, np.float32).astype(np.float64),
            np.asarray(cy, np.float32).astype(np.float64), rt * rt)


@pytest.fixture(scope="module")
def ctx():
    import wltube

    c = wltube.Context(0)
    yield c
    c.close()


def instances(n, seed):
    rng = np.random.default_rng(seed)
    return f32_exact(rng.uniform(0, 2.0, n), rng.uniform(-0.3, 0.3, n),
                     np.exp(rng.uniform(np.log(0.02), np.log(3.0), n)))


@pytest.mark.parametrize("nint", [4, 50])
@pytest.mark.parametrize("n", [31, 32, 33, 127, 128, 129, 255, 256, 257, 513])
def test_instance_counts_around_tile_sizes(ctx, n, nint):
    import wltube

    loops = O.vloops(31, 256, 64)
    cx, cy, T = instances(600, 17)
    fld = wltube.field("smooth", fermion=1, nint=nint)
    h = ctx.upload(loops)
    try:
        g_all, _, _ = ctx.eval(h, fld, cx, cy, T, [1.0, 2.0])
        g, _, _ = ctx.eval(h, fld, cx[:n], cy[:n], T[:n], [1.0, 2.0])
    finally:
        ctx.release(h)
    if n >= 32:  # the same instance-parallel kernel: bit for bit
        assert np.array_equal(g, g_all[:n])
    idx = [0, n // 2, n - 1]
    ref, S = O.eval_groups(loops, cx[idx], cy[idx], T[idx], [1.0, 2.0],
                           O.field("smooth", fermion=1, nint=nint), return_scale=True)
    assert werr(g[idx], ref, S) < W_TOL


@pytest.mark.parametrize("ppl", [4, 8, 260, 516, 1028])
def test_points_per_loop_not_a_multiple_of_the_staging_chunk(ctx, ppl):
    import wltube

    loops = O.vloops(32, 256, ppl)
    cx, cy, T = instances(64, 3)
    for prof, fe, nint in (("smooth", 1, 4), ("gaussian", 0, 4), ("smooth", 0, 50),
                           ("gaussian", 1, 50)):
        fld = wltube.field(prof, fermion=fe, nint=nint)
        h = ctx.upload(loops)
        try:
            g, _, _ = ctx.eval(h, fld, cx, cy, T, [1.0])
        finally:
            ctx.release(h)
        ref, S = O.eval_groups(loops, cx, cy, T, [1.0], O.field(prof, fermion=fe, nint=nint),
                               return_scale=True)
        assert werr(g, ref, S) < W_TOL, (prof, ppl, nint)


def test_one_group_four_flux_values_extreme_proper_times(ctx):
    import wltube

    loops = O.vloops(33, 128, 64)
    cx, cy, T = f32_exact(np.linspace(0, 3, 40), np.zeros(40), np.geomspace(1e-8, 1e4, 40))
    F = [0.0, 0.01, 1.0, 5.0]
    fld = wltube.field("smooth", fermion=1, nint=4)
    h = ctx.upload(loops)
    try:
        g, mean, sem = ctx.eval(h, fld, cx, cy, T, F, group=128)
    finally:
        ctx.release(h)
    assert g.shape == (40, 4, 1)
    assert np.all(sem == 0.0)                 # one group: no spread
    assert np.all(g[:, 0, 0] == 1.0)          # F = 0
    assert np.all(np.isfinite(g))
    small = T < 1e-5                          # tiny loops: W within 1e-6 of 1
    assert small.sum() >= 10
    assert np.all(np.abs(g[small, 1:, 0] - 1.0) < 1e-6)


def test_argument_limits(ctx):
    import wltube

    loops = O.vloops(34, 128, 64)
    fld = wltube.field("smooth", fermion=0, nint=4)
    h = ctx.upload(loops)
    try:
        with pytest.raises(wltube.WlError):   # more than 4 flux values
            ctx.eval(h, fld, [0.1], [0.0], [1.0], [1, 2, 3, 4, 5])
        with pytest.raises(wltube.WlError):   # odd interval count
            ctx.eval(h, wltube.field("smooth", nint=5), [0.1], [0.0], [1.0], [1.0])
        with pytest.raises(wltube.WlError):   # non-finite centre
            ctx.eval(h, fld, [np.nan], [0.0], [1.0], [1.0])
        with pytest.raises(wltube.WlError):   # group larger than Nl
            ctx.eval(h, fld, [0.1], [0.0], [1.0], [1.0], group=256)
        with pytest.raises(wltube.WlError):   # ppl not a multiple of 4
            ctx.upload(O.vloops(34, 8, 64)[:, :30])
    finally:
        ctx.release(h)


def test_pure_gauge_winding_phase_on_the_gpu(ctx):
    """Circles about a step tube (f = 1 on them): every sub-loop's phase is
    2 pi F n for n windings (exact mode; see the oracle's known answer)."""
    import wltube

    for windings in (1, 2, -1):
        k = np.arange(1024)
        ang = 2.0 * np.pi * windings * k / 1024
        L = np.zeros((8, 1024, 4), np.float32)
        L[:, :, 0] = 3.0 * np.cos(ang)
        L[:, :, 1] = 3.0 * np.sin(ang)
        h = ctx.upload(L)
        try:
            s, _ = ctx.loops(h, wltube.field("step", nint=8, mode=1, lambda2=1.0), 0.0, 0.0, 1.0,
                             0.7)
        finally:
            ctx.release(h)
        np.testing.assert_allclose(s[:, :3], 2 * np.pi * 0.7 * windings, rtol=2e-6)


def test_nan_loop_poisons_only_its_group(ctx):
    """A loop with a NaN point (an injected bad input the library does not
    scan for on the device, as the reference does not) makes its group's <W>
    NaN; the other groups, the status and later calls are unaffected."""
    import wltube

    loops = O.vloops(35, 512, 64)
    loops[300, 17, 0] = np.nan          # loop 300: group 2 of 128-loop groups
    cx, cy, T = f32_exact(np.linspace(0, 2, 48), np.zeros(48), np.geomspace(0.05, 2.0, 48))
    fld = wltube.field("smooth", fermion=1, nint=4)
    h = ctx.upload(loops)
    try:
        g, mean, sem = ctx.eval(h, fld, cx, cy, T, [1.0])
        assert np.all(np.isnan(g[:, 0, 2]))
        assert np.all(np.isfinite(g[:, 0, [0, 1, 3]]))
        assert np.all(np.isnan(mean))
        clean = O.vloops(35, 512, 64)
        h2 = ctx.upload(clean)
        g2, _, _ = ctx.eval(h2, fld, cx, cy, T, [1.0])
        ctx.release(h2)
        assert np.all(np.isfinite(g2))
        np.testing.assert_array_equal(g2[:, 0, [0, 1, 3]], g[:, 0, [0, 1, 3]])
    finally:
        ctx.release(h)


def test_bounded_wait_gives_up_with_a_status(ctx):
    """The bounded mbarrier wait that guards every staged copy, on a barrier
    nothing arrives at: the kernel gives up, the call returns the timeout
    status, and the context stays usable (no fault, no hang)."""
    import wltube

    ctx.selftest_wait(True)
    for tries in (1, 16, 64):
        with pytest.raises(wltube.WlError) as e:
            ctx.selftest_wait(False, tries)
        assert e.value.status == -4
        assert ctx.last_launches() == (1, "wait-selftest")
    ctx.selftest_wait(True, 64)
    loops = O.vloops(36, 128, 64)
    cx, cy, T = instances(40, 5)
    h = ctx.upload(loops)
    try:
        g, _, _ = ctx.eval(h, wltube.field("smooth", fermion=0, nint=4), cx, cy, T, [1.0])
    finally:
        ctx.release(h)
    assert np.all(np.isfinite(g))
