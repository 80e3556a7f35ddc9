"""wl_eval_noalloc, the entry point for callers that cannot let the library
allocate device memory (their framework's allocator owns the device, or
cudaMalloc is not permitted or would synchronise where they call), checked
against wl_eval_device on the same device buffers, twice in a row.

This file is collected last on purpose: if it fails, a run that stops at the
first failure has already run every other test.  It passes alone in a fresh
process and after the other tests.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

W_TOL = 1e-5      # the <W> tolerance of the other GPU tests
W_FLOOR = 1e-2


def _werr(w, ref):
    return np.max(np.abs(w - ref) / np.maximum(np.abs(ref), W_FLOOR))


@pytest.mark.parametrize("ninst", [96, 7])  # instance-parallel and loop-parallel kernels
def test_noalloc_matches_existing_entry_point_twice(ninst):
    torch = pytest.importorskip("torch")
    import wltube

    rng = np.random.default_rng(42 + ninst)
    Nl, ppl, group, F = 256, 128, 128, [0.5, 1.0]
    loops = O.vloops(13, Nl, ppl)
    rt = np.sqrt(np.exp(rng.uniform(np.log(0.02), np.log(3.0), ninst))).astype(np.float32)
    cx = rng.uniform(0.0, 2.0, ninst).astype(np.float32).astype(np.float64)
    cy = rng.uniform(-0.3, 0.3, ninst).astype(np.float32).astype(np.float64)
    T = rt.astype(np.float64) ** 2
    fld = wltube.field("smooth", fermion=1, nint=4)
    ng, nF = Nl // group, len(F)

    dev = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    dloops = torch.from_numpy(loops.reshape(-1)).cuda()
    dcx, dcy, dT = dev(cx), dev(cy), dev(T)
    outs = [[torch.full((n,), np.nan, dtype=torch.float64, device="cuda")
             for n in (ninst * nF * ng, ninst * nF, ninst * nF)] for _ in range(3)]

    # the existing entry point (context, library-allocated scratch)
    with wltube.Context(0) as ctx:
        h = ctx.wrap(dloops.data_ptr(), Nl, ppl)
        ctx.eval_device(h, fld, ninst, dcx.data_ptr(), dcy.data_ptr(), dT.data_ptr(), F, group,
                        *[t.data_ptr() for t in outs[0]])
        ctx.synchronize()
        ctx.release(h)
    torch.cuda.synchronize()
    # two calls in a row of the allocation-free entry point
    for k in (1, 2):
        wltube.eval_noalloc(dloops.data_ptr(), Nl, ppl, fld, ninst, dcx.data_ptr(),
                            dcy.data_ptr(), dT.data_ptr(), F, group,
                            *[t.data_ptr() for t in outs[k]])
    torch.cuda.synchronize()
    ref = [t.cpu().numpy() for t in outs[0]]
    assert np.all(np.isfinite(ref[0]))
    for k in (1, 2):
        got = [t.cpu().numpy() for t in outs[k]]
        assert _werr(got[0], ref[0]) <= W_TOL   # per-group <W>
        assert _werr(got[1], ref[1]) <= W_TOL   # mean over groups
        np.testing.assert_allclose(got[2], ref[2], rtol=1e-6, atol=1e-12)  # SEM


def test_noalloc_rejects_requests_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    import wltube

    Nl, ppl, ninst = 4096, 4, 2048  # 512 chunks x 4 F x 3 x 2048 x 8 B = 100 MiB > 32 MiB
    dloops = torch.zeros(Nl * ppl * 4, dtype=torch.float32, device="cuda")
    d = torch.ones(ninst, dtype=torch.float64, device="cuda")
    out = torch.zeros(ninst * 4, dtype=torch.float64, device="cuda")
    with pytest.raises(wltube.WlError) as e:
        wltube.eval_noalloc(dloops.data_ptr(), Nl, ppl, wltube.field("smooth", nint=4), ninst,
                            d.data_ptr(), d.data_ptr(), d.data_ptr(), [1.0, 1.0, 1.0, 1.0],
                            128, 0, out.data_ptr(), 0)
    assert e.value.status == -1


def test_noalloc_matches_the_oracle():
    """The allocation-free entry point against the FP64 oracle directly, at
    the tolerance of the other GPU tests, for a scalar and a spinor field."""
    torch = pytest.importorskip("torch")
    import wltube

    rng = np.random.default_rng(7)
    Nl, ppl, group, ninst = 256, 256, 128, 64
    loops = O.vloops(17, Nl, ppl)
    rt = np.sqrt(np.exp(rng.uniform(np.log(0.01), np.log(4.0), ninst))).astype(np.float32)
    cx = rng.uniform(0.0, 3.0, ninst).astype(np.float32).astype(np.float64)
    cy = rng.uniform(-0.2, 0.2, ninst).astype(np.float32).astype(np.float64)
    T = rt.astype(np.float64) ** 2
    F = [0.1, 1.0]
    dev = lambda a: torch.tensor(a, dtype=torch.float64, device="cuda")  # noqa: E731
    dloops = torch.from_numpy(loops.reshape(-1)).cuda()
    dcx, dcy, dT = dev(cx), dev(cy), dev(T)
    ng = Nl // group
    for prof, fe in (("smooth", 1), ("gaussian", 0)):
        out = torch.full((ninst * len(F) * ng,), np.nan, dtype=torch.float64, device="cuda")
        wltube.eval_noalloc(dloops.data_ptr(), Nl, ppl, wltube.field(prof, fermion=fe, nint=4),
                            ninst, dcx.data_ptr(), dcy.data_ptr(), dT.data_ptr(), F, group,
                            out.data_ptr(), 0, 0)
        torch.cuda.synchronize()
        got = out.cpu().numpy().reshape(ninst, len(F), ng)
        ref, S = O.eval_groups(loops, cx, cy, T, F, O.field(prof, fermion=fe, nint=4),
                               return_scale=True)
        assert O.werr(got, ref, S, floor=W_FLOOR) <= W_TOL, prof


@pytest.mark.parametrize("prof", ["lattice", "spline"])
def test_noalloc_refuses_fields_that_need_library_memory(prof):
    """The lattice profile needs per-loop bounding boxes and the spline
    profile a table, both of which the library would allocate: refused with
    WL_ERR_INVALID before any launch, leaving the outputs untouched."""
    torch = pytest.importorskip("torch")
    import wltube

    Nl, ppl, ninst = 128, 16, 4
    dloops = torch.zeros(Nl * ppl * 4, dtype=torch.float32, device="cuda")
    d = torch.ones(ninst, dtype=torch.float64, device="cuda")
    out = torch.full((ninst,), 7.0, dtype=torch.float64, device="cuda")
    with pytest.raises(wltube.WlError) as e:
        wltube.eval_noalloc(dloops.data_ptr(), Nl, ppl,
                            wltube.field(prof, nint=4, tubedist=2.0), ninst,
                            d.data_ptr(), d.data_ptr(), d.data_ptr(), [1.0], 128, 0,
                            out.data_ptr(), 0)
    assert e.value.status == -1
    assert torch.all(out == 7.0)
