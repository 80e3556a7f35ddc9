"""The FP64 proper-time integral (wl_tint) against the same integral built
from the FP64 oracle: Tfunc's regimes and counterterms (Integrand.c:195-316),
Simpson over ln T, Tintout's normalisation (Tint.c:69-72) and a jackknife
over bins of loop groups."""
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def log_simpson_weights(T):
    n = len(T)
    du = np.log(T[1]) - np.log(T[0])
    w = np.zeros(n)
    m = n - 1
    m13 = m if m % 2 == 0 else m - 3
    for k in range(0, m13, 2):
        w[k:k + 3] += np.array([1, 4, 1]) * du / 3
    if m13 < m:
        w[m13:m13 + 4] += np.array([3, 9, 9, 3]) * du / 8
    return w * T


def oracle_tint(loops, rho, T, F, fld, nbins):
    cx = np.repeat(rho, len(T))
    TT = np.tile(T, len(rho))
    g = O.eval_groups(loops, cx, 0 * cx, TT, F, fld)          # [inst][F][ng]
    ng = g.shape[2]
    ig = np.zeros((len(rho), len(F), len(T), ng))
    for r, x in enumerate(rho):
        for j, f in enumerate(F):
            for k, t in enumerate(T):
                reg, an = O.tfunc_regime(t, x, 0.0, f, fld)
                if reg == 3:
                    ig[r, j, k] = [O.tfunc_mc(t, W, x, 0.0, f, fld) for W in g[r * len(T) + k, j]]
                else:
                    ig[r, j, k] = an
    I = np.einsum("rjkg,k->rjg", ig, log_simpson_weights(T))
    per = ng // nbins
    mean = I.mean(axis=2)
    binsum = I.reshape(len(rho), len(F), nbins, per).sum(axis=3)
    loo = (I.sum(axis=2)[..., None] - binsum) / (ng - per)
    jk = np.sqrt((nbins - 1) / nbins * ((loo - mean[..., None]) ** 2).sum(axis=2))
    norm = 1 / (4 * np.pi) if fld.fermion else -1 / (2 * np.pi)
    return mean * norm, jk * abs(norm), ig


@pytest.mark.parametrize("fermion", [0, 1])
def test_tint_matches_oracle_within_error_bars(fermion):
    import wltube

    loops = O.vloops(8, 512, 128)
    rho = np.array([0.0, 0.5, 1.5], dtype=np.float32).astype(np.float64)
    rt = np.sqrt(np.geomspace(1e-3, 1e2, 33)).astype(np.float32).astype(np.float64)
    T = rt * rt
    T = np.exp(np.linspace(np.log(T[0]), np.log(T[-1]), len(T)))  # exactly log-spaced
    F = [0.5, 1.0]
    with wltube.Context(0) as ctx:
        h = ctx.upload(loops)
        leff, err, ig = ctx.tint(h, wltube.field("smooth", fermion=fermion, nint=4), rho, T, F,
                                 group=128, nbins=4, want_igrand=True)
        ctx.release(h)
    # the oracle at the instances the FP32 kernel represents exactly
    rtf = np.sqrt(T).astype(np.float32).astype(np.float64)
    ref_leff, ref_err, ref_ig = oracle_tint(loops, rho, rtf * rtf, F,
                                            O.field("smooth", fermion=fermion, nint=4), 4)
    assert np.all(np.isfinite(leff)) and np.all(err > 0)
    # numerical difference far inside the Monte Carlo error bars
    assert np.all(np.abs(leff - ref_leff) <= 0.05 * ref_err + 1e-12)
    np.testing.assert_allclose(err, ref_err, rtol=0.05, atol=1e-12)


def test_tint_rejects_non_log_grid():
    import wltube

    loops = O.vloops(8, 256, 16)
    with wltube.Context(0) as ctx:
        h = ctx.upload(loops)
        with pytest.raises(wltube.WlError):
            ctx.tint(h, wltube.field("smooth"), [0.0], [0.1, 0.2, 0.4, 0.5], [1.0], nbins=2)
        ctx.release(h)


def rho_rule(profile_cell, nrho, a, ref):
    """Nodes and weights of the radial integral of rho I(rho) as
    wl_effective_action documents them (EffAct.c:83-210)."""
    if profile_cell:
        n = 2 * nrho
        h = a / (2.0 * n)
        rho = h * np.arange(n + 1)
        if ref:
            w = np.array([1.0] + [2.0 if (k - 1) % 2 == 0 else 4.0 for k in range(1, n + 1)])
            w[n] += 1.0
        else:
            w = np.array([1.0] + [4.0 if k % 2 else 2.0 for k in range(1, n)] + [1.0])
        return rho, w * h / 3.0
    h = 1.0 / nrho
    wt = np.zeros(2 * nrho + 1)
    for i in range(nrho):
        if ref:
            wt[2 * i + 2] += 2 * h / 6
        else:
            wt[2 * i] += h / 6
            wt[2 * i + 2] += h / 6
        wt[2 * i + 1] += 4 * h / 6
    t = 0.5 * h * np.arange(1, 2 * nrho + 1)
    return (1 - t) / t, wt[1:] / t ** 2


@pytest.mark.parametrize("prof,fermion,mode", [("smooth", 1, 0), ("smooth", 0, 1),
                                               ("fixflux", 0, 0)])
def test_effective_action_matches_oracle(prof, fermion, mode):
    import wltube

    loops = O.vloops(9, 512, 128)
    T = np.exp(np.linspace(np.log(1e-2), np.log(30.0), 17))
    a, nrho, F = 2.0, 3, 1.0
    fld = wltube.field(prof, fermion=fermion, nint=4, mode=mode, tubedist=a, lambda2=0.5)
    with wltube.Context(0) as ctx:
        h = ctx.upload(loops)
        act, err, ca, groups = ctx.effective_action(h, fld, F, T, group=128, nrho=nrho)
        assert ctx.last_launches()[0] >= 3
        ctx.release(h)
    rho, w = rho_rule(prof == "fixflux", nrho, a, mode == 0)
    rho = rho.astype(np.float32).astype(np.float64)  # the kernel's float centre
    rtf = np.sqrt(T).astype(np.float32).astype(np.float64)
    ofld = O.field(prof, fermion=fermion, nint=4, mode=mode, tubedist=a, lambda2=0.5)
    _, _, ig = oracle_tint(loops, rho, rtf * rtf, [F], ofld, 2)
    I = np.einsum("rjkg,k->rg", ig, log_simpson_weights(T))         # [rho][group]
    norm = 1 / (4 * np.pi) if fermion else -1 / (2 * np.pi)
    ref_g = norm * np.einsum("r,r,rg->g", w, rho, np.where(np.isinf(I), 0.0, I))
    ref = ref_g.mean()
    ref_se = ref_g.std(ddof=1) / np.sqrt(len(ref_g))
    assert np.isfinite(act) and err > 0
    assert abs(act - ref) <= 0.05 * ref_se + 1e-12
    np.testing.assert_allclose(groups, ref_g, rtol=0, atol=0.05 * ref_se + 1e-12)
    if prof == "smooth":
        e = 0.30282212
        assert np.isclose(ca, -2 * np.pi * F * F / (3 * 0.5 * e * e))


@pytest.mark.parametrize("prof,fermion", [("smooth", 1), ("gaussian", 0)])
def test_effective_action_with_the_reference_T_rule(prof, fermion):
    """The proper-time integral by integrateT's own rule (T = (1 - t)/t, the
    reference's 40 panels in rhogrand) under the radial integral, against the
    oracle's integrateT (pinned to the reference's Tint.c by the golden
    vectors) at every radial node."""
    import wltube

    loops = O.vloops(10, 512, 128)
    nrho, F = 2, 1.0
    fld = wltube.field(prof, fermion=fermion, nint=4, lambda2=0.5)
    with wltube.Context(0) as ctx:
        h = ctx.upload(loops)
        act, err, ca, groups = ctx.effective_action(h, fld, F, None, group=128, nrho=nrho,
                                                    t_panels=40)
        ctx.release(h)
    rho, w = rho_rule(False, nrho, 0.0, True)
    ofld = O.field(prof, fermion=fermion, nint=4, lambda2=0.5)
    I = np.array([O.integrateT(loops, 40, float(r), 0.0, F, ofld)[0] for r in rho])  # [rho][g]
    norm = 1 / (4 * np.pi) if fermion else -1 / (2 * np.pi)
    ref_g = norm * np.einsum("r,r,rg->g", w, rho, np.where(np.isinf(I), 0.0, I))
    ref_se = ref_g.std(ddof=1) / np.sqrt(len(ref_g))
    assert np.isfinite(act) and err > 0
    # the kernel evaluates W at T' = float(sqrt(T))^2, the oracle at T: both
    # far inside the Monte Carlo error
    assert abs(act - ref_g.mean()) <= 0.05 * ref_se + 1e-12
    np.testing.assert_allclose(groups, ref_g, rtol=0, atol=0.05 * ref_se + 1e-12)


def test_legacy_integrateT_through_the_host_layer(capfd):
    """The reference's own caller chain, unchanged: integrateT (Tint.c:100-175)
    -> Tfunc (Integrand.c:195-316) -> EV (intEV.cu:111-148) through
    libwlhost.so and libwlgpu.so with a struct Wparams of device buffers, as
    EffAct.c:368-413 sets them up; per-group integrals against the oracle's
    integrateT, and the Leffvsrho line the reference prints."""
    import ctypes

    torch = pytest.importorskip("torch")
    import wltube

    loops = O.vloops(12, 512, 128)
    Nl, ppl = loops.shape[:2]
    rho, F, l2 = 0.7, 1.0, 0.5
    wltube.legacy_configure("smooth", nint=4)
    try:
        dev = torch.from_numpy(loops.reshape(-1)).cuda()
        scal_d = torch.zeros(Nl * 4, device="cuda")
        ferm_d = torch.zeros(Nl * 4, device="cuda")
        scal_h = np.zeros((Nl, 4), dtype=np.float32)
        ferm_h = np.zeros((Nl, 4), dtype=np.float32)
        for fermion in (0, 1):
            p = wltube.Wparams()
            p.Nl, p.Nppl, p.F, p.l2, p.fermion, p.ng = Nl, ppl, F, l2, fermion, Nl // 128
            p.xcm.x, p.xcm.y = rho, 0.0
            p.worldlines = dev.data_ptr()
            p.Wsscal_d, p.Wsferm_d = scal_d.data_ptr(), ferm_d.data_ptr()
            p.Wsscal_h, p.Wsferm_h = scal_h.ctypes.data, ferm_h.ctypes.data
            got = wltube.integrateT(40, p)
            ref, _, _ = O.integrateT(loops, 40, rho, 0.0, F,
                                  O.field("smooth", fermion=fermion, nint=4, lambda2=l2))
            se = ref.std(ddof=1) / np.sqrt(len(ref))
            # EV evaluates W at T' = float(sqrt(T))^2, the oracle at T
            np.testing.assert_allclose(got, ref, rtol=0, atol=0.05 * se + 1e-12)
            ctypes.CDLL(None).fflush(None)  # the C library's stdout buffer
            out = capfd.readouterr().out.strip().splitlines()
            tag = [line for line in out if line.startswith("Leffvsrho:")]
            assert len(tag) == 1
            x, leff, err = map(float, tag[0].split()[1:])
            norm = 4 * np.pi if fermion else -2 * np.pi
            assert abs(x - rho) < 1e-6 and np.isclose(leff, got.mean() / norm, rtol=1e-5)
    finally:
        wltube.legacy_configure("smooth")


def test_c_driver_in_the_reference_style(tmp_path):
    """A C program built the way the reference's drivers are (intT.h first,
    then the library's headers; getwl, cudaMalloc/cudaMemcpy, struct Wparams,
    integrateT) and linked with libwlhost.so + libwlgpu.so: its per-group
    integrals against the oracle's integrateT, its Leffvsrho line against
    their mean."""
    import shutil
    import subprocess

    import wltube

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    libdir = os.path.join(root, "worldline-flux-tube-lattice_gb300", "lib")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cuda = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    exe = str(tmp_path / "legacy_driver")
    subprocess.check_call(
        ["gcc", "-O2", "-Wall", "-I" + os.path.join(root, "include"), "-I" + cuda + "/include",
         os.path.join(root, "tests", "c", "legacy_driver.c"), "-o", exe, "-L" + libdir,
         "-lwlhost", "-lwlgpu", "-L" + cuda + "/lib64", "-lcudart", "-lm",
         "-Wl,-rpath," + libdir + ":" + cuda + "/lib64"])
    loops = O.vloops(13, 256, 128)
    txt = str(tmp_path / "loops.txt")
    wltube.save_text_ensemble(txt, loops)
    rho, F, l2 = 0.4, 1.0, 0.5
    out = subprocess.check_output([exe, txt, "256", "128", str(rho), str(F), str(l2), "0", "4",
                                   "40"], text=True).splitlines()
    got = np.array([float(line.split()[2]) for line in out if line.startswith("I ")])
    ref, _, _ = O.integrateT(loops, 40, rho, 0.0, F, O.field("smooth", fermion=0, nint=4,
                                                              lambda2=l2))
    se = ref.std(ddof=1) / np.sqrt(len(ref))
    np.testing.assert_allclose(got, ref, rtol=0, atol=0.05 * se + 1e-12)
    tag = [line for line in out if line.startswith("Leffvsrho:")]
    assert len(tag) == 1
    assert np.isclose(float(tag[0].split()[2]), got.mean() / (-2 * np.pi), rtol=1e-5)
