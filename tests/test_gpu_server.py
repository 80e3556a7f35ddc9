"""The request server (wl_server): served results against the same request
evaluated alone (bit for bit) and against the FP64 oracle, effective action
density requests against wl_tint, continuous batching (a small request that
arrives behind a large one finishes first), admission by HBM footprint with
eviction of idle ensembles, and argument checks."""
import time

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

W_TOL, W_FLOOR = 1e-5, 1e-2


def werr(w, ref, scale=1.0):
    return np.max(np.abs(w - ref) / np.maximum(np.abs(ref), W_FLOOR * scale))


def done(srv, ticket, timeout_ms=120000.0):
    """The request's outputs; a request still open after timeout_ms fails the test."""
    out = srv.wait(ticket, timeout_ms)
    assert out is not None, "request %d still open after %.0f ms" % (ticket, timeout_ms)
    return out


def f32_exact(cx, cy, T):
    rt = np.sqrt(np.asarray(T, np.float64)).astype(np.float32).astype(np.float64)
    return (np.asarray(cx, np.float32).astype(np.float64),
            np.asarray(cy, np.float32).astype(np.float64), rt * rt)


# (profile, fermion, lambda2, seed, Nl, ppl, instances, F, extra field args)
SPECS = [("smooth", 1, 1.0, 11, 512, 256, 300, [0.5, 1.0], {}),
         ("gaussian", 0, 0.5, 12, 256, 512, 70, [2.0], {}),
         ("step", 1, 3.0, 11, 512, 256, 9, [1.0], {}),
         ("quadratic", 1, 1.5, 13, 256, 128, 200, [0.7, 0.2, 1.3], {}),
         ("lattice", 0, 1.0, 14, 256, 256, 8, [1.0], {"tubedist": 5.0})]


def make_requests(wltube, rng):
    reqs = []
    for prof, fe, l2, seed, Nl, ppl, n, F, kw in SPECS:
        cx, cy, T = f32_exact(rng.uniform(0, 2.5, n), rng.uniform(-0.2, 0.2, n),
                              np.exp(rng.uniform(np.log(0.02), np.log(2.0), n)))
        fld = wltube.field(prof, fermion=fe, nint=4, lambda2=l2, **kw)
        reqs.append(dict(prof=prof, seed=seed, Nl=Nl, ppl=ppl, fld=fld, cx=cx, cy=cy, T=T,
                         F=F, fe=fe, l2=l2, kw=kw))
    return reqs


def test_served_equals_alone_and_oracle():
    import wltube

    rng = np.random.default_rng(5)
    reqs = make_requests(wltube, rng)
    with wltube.Server(0, quantum_ms=2.0) as srv:
        tickets = [srv.submit_w(r["seed"], r["Nl"], r["ppl"], r["fld"], r["cx"], r["cy"], r["T"],
                                r["F"], group=128, want_groups=True) for r in reqs]
        served = [done(srv, t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["rejected"] == 0
    assert st["launches"] >= 1 and 0 < st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert st["resident_ensembles"] == 4
    with wltube.Context(0) as ctx:
        for r, (g, m, s) in zip(reqs, served):
            h = ctx.generate(r["seed"], r["Nl"], r["ppl"])
            job = {"handle": h, "field": r["fld"], "cx": r["cx"], "cy": r["cy"], "T": r["T"],
                   "F": r["F"], "group": 128}
            (g1, m1, s1), = ctx.batch_eval([job], graph=False)
            # the same request alone: bit for bit
            assert np.array_equal(g, g1) and np.array_equal(m, m1) and np.array_equal(s, s1), \
                r["prof"]
            # and the FP64 oracle on a few instances
            loops = ctx.download(h)
            idx = np.arange(0, len(r["T"]), max(1, len(r["T"]) // 4))
            of = O.field(r["prof"], fermion=r["fe"], nint=4, lambda2=r["l2"],
                         **({"tubedist": r["kw"]["tubedist"], "mode": 1, "rimage": 60.0}
                            if r["prof"] == "lattice" else {}))
            ref, S = O.eval_groups(loops, r["cx"][idx], r["cy"][idx], r["T"][idx], r["F"], of,
                                   return_scale=True)
            tol = 2e-5 if (r["prof"] == "lattice" and r["fe"]) else W_TOL
            assert werr(g[idx], ref, S) < tol, r["prof"]
            ctx.release(h)


def test_served_leff_matches_tint():
    import wltube

    rho = np.linspace(0.0, 3.0, 5)
    T = np.geomspace(1e-2, 10.0, 9)
    F = [0.5, 2.0]
    fld = wltube.field("smooth", fermion=1, nint=4, lambda2=1.0)
    with wltube.Server(0) as srv:
        t = srv.submit_leff(21, 1280, 2048, fld, rho, T, F, group=128, nbins=5)
        le, er = done(srv, t)
    with wltube.Context(0) as ctx:
        h = ctx.generate(21, 1280, 2048)
        le1, er1, _ = ctx.tint(h, fld, rho, T, F, group=128, nbins=5)
    # the same loops per chunk (8 of 2048 points) on both paths; the FP64
    # reductions may differ in summation order only
    assert np.all(np.abs(le - le1) <= 1e-7 * np.abs(le1) + 1e-4 * er1)
    np.testing.assert_allclose(er, er1, rtol=1e-3, atol=1e-14)
    assert np.all(np.isfinite(le)) and np.all(er >= 0)


def test_small_request_overtakes_large():
    """Continuous batching: a request submitted while a large one is on the
    GPU shares the next launches and completes first."""
    import wltube

    fld = wltube.field("smooth", fermion=1, nint=4, lambda2=1.0)
    n_big = 12000                       # about 0.3 s of device work
    rng = np.random.default_rng(9)
    cx, T = rng.uniform(0, 3, n_big), np.exp(rng.uniform(np.log(0.01), np.log(5.0), n_big))
    with wltube.Server(0, quantum_ms=10.0) as srv:
        # warm the ensembles so that generation time is not part of the race
        done(srv, srv.submit_w(31, 8192, 2048, fld, [0.1], [0.0], [0.5], [1.0]))
        done(srv, srv.submit_w(32, 1024, 512, fld, [0.1], [0.0], [0.5], [1.0]))
        big = srv.submit_w(31, 8192, 2048, fld, cx, np.zeros(n_big), T, [1.0])
        time.sleep(0.02)
        small = srv.submit_w(32, 1024, 512, fld, [0.3, 0.6], [0.0, 0.0], [0.2, 1.0], [1.0])
        m_small = done(srv, small)[1]
        big_pending = srv.wait(big, timeout_ms=0.0) is None
        m_big = done(srv, big)[1]
        st = srv.stats()
    assert big_pending, "the small request did not overtake the large one"
    assert st["launches"] >= 3
    assert np.all(np.isfinite(m_small)) and np.all(np.isfinite(m_big))


def test_admission_budget_and_eviction():
    import wltube

    fld = wltube.field("smooth", fermion=0, nint=4, lambda2=1.0)
    # ensembles of 1024 x 1024 points = 16 MiB; the budget holds one of them
    budget = 24 * 2 ** 20
    with wltube.Server(0, hbm_budget_bytes=budget) as srv:
        too_big = srv.submit_w(41, 4096, 1024, fld, [0.1], [0.0], [0.5], [1.0])  # 64 MiB
        a = srv.submit_w(42, 1024, 1024, fld, [0.1, 0.2], [0.0, 0.0], [0.5, 0.5], [1.0])
        b = srv.submit_w(43, 1024, 1024, fld, [0.1, 0.2], [0.0, 0.0], [0.5, 0.5], [1.0])
        c = srv.submit_w(42, 1024, 1024, fld, [0.1, 0.2], [0.0, 0.0], [0.5, 0.5], [1.0])
        with pytest.raises(wltube.WlError) as ei:
            srv.wait(too_big, 120000.0)
        assert ei.value.status == -6
        ra, rb, rc = done(srv, a), done(srv, b), done(srv, c)
        st = srv.stats()
    assert np.array_equal(ra[1], rc[1])          # same ensemble (regenerated): same result
    assert not np.array_equal(ra[1], rb[1])
    assert st["rejected"] == 1 and st["completed"] == 3
    assert st["resident_ensembles"] == 1
    assert st["hbm_bytes_in_use"] <= budget


def test_invalid_requests_are_refused_at_submit():
    import wltube

    fld = wltube.field("smooth", fermion=0, nint=4)
    with wltube.Server(0) as srv:
        with pytest.raises(wltube.WlError):        # group does not divide Nl
            srv.submit_w(1, 1000, 64, fld, [0.1], [0.0], [0.5], [1.0], group=128)
        with pytest.raises(wltube.WlError):        # T <= 0
            srv.submit_w(1, 256, 64, fld, [0.1], [0.0], [0.0], [1.0])
        with pytest.raises(wltube.WlError):        # odd interval count
            srv.submit_w(1, 256, 64, wltube.field("periodic", nint=5), [0.1], [0.0], [0.5],
                         [1.0])
        with pytest.raises(wltube.WlError):        # T grid not log-spaced
            srv.submit_leff(1, 256, 64, fld, [0.0], [0.1, 0.2, 0.4, 0.5], [1.0], nbins=2)
        st = srv.stats()
    assert st["submitted"] == 0


def test_many_concurrent_requests_equal_alone():
    """Forty small requests submitted from two host threads while earlier ones
    run: each result equals the request evaluated alone, bit for bit."""
    import threading

    import wltube

    rng = np.random.default_rng(77)
    profs = ["smooth", "gaussian", "step", "quadratic"]
    reqs = []
    for i in range(40):
        prof = profs[i % 4]
        Nl = int(rng.choice([256, 512]))
        ppl = int(rng.choice([64, 128, 256]))
        n = int(rng.integers(1, 300))
        cx, cy, T = f32_exact(rng.uniform(0, 2, n), rng.uniform(-0.2, 0.2, n),
                              np.exp(rng.uniform(np.log(0.05), np.log(2.0), n)))
        reqs.append(dict(seed=int(rng.integers(60, 64)), Nl=Nl, ppl=ppl, cx=cx, cy=cy, T=T,
                         F=[float(rng.uniform(0.2, 1.5))],
                         fld=wltube.field(prof, fermion=i % 2, nint=4, lambda2=1.0)))
    tickets = [None] * len(reqs)
    with wltube.Server(0, quantum_ms=1.0, max_requests=8) as srv:
        def submit(part):
            for i in part:
                r = reqs[i]
                tickets[i] = srv.submit_w(r["seed"], r["Nl"], r["ppl"], r["fld"], r["cx"], r["cy"],
                                          r["T"], r["F"], want_groups=True)
        th = [threading.Thread(target=submit, args=(range(k, 40, 2),)) for k in (0, 1)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        served = [done(srv, t) for t in tickets]
        st = srv.stats()
    assert st["completed"] == 40 and st["failed"] == 0
    with wltube.Context(0) as ctx:
        handles = {}
        for r, (g, m, s) in zip(reqs, served):
            key = (r["seed"], r["Nl"], r["ppl"])
            if key not in handles:
                handles[key] = ctx.generate(*key)
            (g1, m1, s1), = ctx.batch_eval([{"handle": handles[key], "field": r["fld"],
                                             "cx": r["cx"], "cy": r["cy"], "T": r["T"],
                                             "F": r["F"], "group": 128}], graph=False)
            assert np.array_equal(g, g1) and np.array_equal(m, m1) and np.array_equal(s, s1)
        for h in handles.values():
            ctx.release(h)


def test_served_heavy_profiles_equal_alone():
    """Periodic, spline and fixflux requests (not in the persistent kernel:
    chunk ranges of their own sweep per quantum) beside a smooth one: each
    result equals the request alone in a batch, bit for bit, and L_eff of a
    spline request equals wl_tint."""
    import wltube

    rng = np.random.default_rng(23)
    specs = [("periodic", 1, 0, 1.0, 40), ("spline", 0, 0, 2.0, 150), ("fixflux", 0, 0, 2.0, 20),
             ("fixflux", 1, 1, 2.0, 9), ("smooth", 1, 0, 1.0, 300)]
    reqs = []
    for prof, fe, ffv, a, n in specs:
        cx, cy, T = f32_exact(rng.uniform(0, 2 * a, n), rng.uniform(-0.2, 0.2, n),
                              np.exp(rng.uniform(np.log(0.02), np.log(2.0), n)))
        fld = wltube.field(prof, fermion=fe, nint=8, lambda2=0.5, tubedist=a, ff_variant=ffv)
        reqs.append((prof, fld, cx, cy, T))
    rho, Tg, F = np.linspace(0.0, 2.0, 3), np.geomspace(1e-2, 2.0, 5), [1.0]
    spl = wltube.field("spline", fermion=0, nint=8, lambda2=0.5, tubedist=2.0)
    # 64 loop chunks per request (16384 points per tile, the batch default)
    # and one persistent CTA per SM: ~500 tiles, several quanta, so the heavy
    # requests run as sweeps over chunk ranges that start past chunk 0
    with wltube.Server(0, quantum_ms=0.5, ctas_per_sm=1) as srv:
        tickets = [srv.submit_w(31, 8192, 128, fld, cx, cy, T, [0.5, 1.0], group=128,
                                want_groups=True) for _, fld, cx, cy, T in reqs]
        tl = srv.submit_leff(31, 8192, 128, spl, rho, Tg, F, group=128, nbins=2)
        served = [done(srv, t) for t in tickets]
        le, er = done(srv, tl)
        st = srv.stats()
    assert st["completed"] == len(reqs) + 1 and st["failed"] == 0
    assert st["launches"] >= 3
    with wltube.Context(0) as ctx:
        h = ctx.generate(31, 8192, 128)
        for (prof, fld, cx, cy, T), (g, m, s) in zip(reqs, served):
            job = {"handle": h, "field": fld, "cx": cx, "cy": cy, "T": T, "F": [0.5, 1.0],
                   "group": 128}
            (g1, m1, s1), = ctx.batch_eval([job], graph=False)
            assert np.array_equal(g, g1) and np.array_equal(m, m1), prof
        le1, er1, _ = ctx.tint(h, spl, rho, Tg, F, group=128, nbins=2)
        ctx.release(h)
    assert np.all(np.abs(le - le1) <= 1e-7 * np.abs(le1) + 1e-4 * er1)
