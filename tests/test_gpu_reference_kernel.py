"""Parity with the reference's own CUDA kernel on the GB300.

oracle/build_ref.sh compiles the reference's intEV.cu / intEVff.cu (its own
-prec-div=false -prec-sqrt=false, 50 Simpson intervals) to sm_103a cubins;
oracle/ref_gpu.cu launches ExpectValue exactly as EV() does (intEV.cu:123).
Both kernels run on the golden ensemble; the library must match the
reference kernel within PHASE_TOL of the largest per-loop value.
"""
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

PHASE_TOL = 2e-5
GOLD = os.path.join(os.path.dirname(__file__), "golden", "golden_ref.npz")
# golden driver -> (cubin, threads per block as EffAct.c:313-353 sets them)
CUBINS = {("smooth", 1.0): ("ref_smooth", 512), ("step", 1.0): ("ref_step", 512),
          ("quadratic", 1.0): ("ref_quadratic", 512), ("gaussian", 1.0): ("ref_gaussian", 512),
          ("periodic", 1.0): ("ref_periodic_a1", 256), ("periodic", 2.0): ("ref_periodic_a2", 256),
          ("fixflux", 2.0): ("ref_fixflux_a2", 128), ("ff", 2.0): ("ref_ff_a2", 128)}


@pytest.fixture(scope="module")
def refgpu():
    import ctypes as C

    path = O.build_ref_gpu()
    if path is None or not any(os.path.exists(os.path.join(O.REF_DIR, c + ".cubin"))
                               for c, _ in CUBINS.values()):
        pytest.skip("reference cubins not built (oracle/build_ref.sh needs the reference tree)")
    L = C.CDLL(path)
    L.refgpu_load.argtypes = [C.c_char_p, C.c_int]
    L.refgpu_run.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_float, C.c_float,
                             C.c_float, C.c_float, C.c_float, C.c_int, C.c_int, C.c_int, C.c_int,
                             C.c_longlong, C.POINTER(C.c_float)]
    return L


def run_reference_kernel(L, torch, cubin, nthreads, loops, cx, cy, T, F, l2, fermion, ff):
    import ctypes as C

    h = L.refgpu_load(os.path.join(O.REF_DIR, cubin + ".cubin").encode(), int(ff))
    assert h >= 0, "cannot load %s (%d)" % (cubin, h)
    Nl, ppl = loops.shape[:2]
    padded = -(-Nl // nthreads) * nthreads          # EffAct.c:368-369
    wl = torch.zeros((padded, ppl, 4), dtype=torch.float32, device="cuda")
    wl[:Nl] = torch.from_numpy(loops).cuda()
    scal = torch.zeros((padded, 4), dtype=torch.float32, device="cuda")
    ferm = torch.zeros((padded, 4), dtype=torch.float32, device="cuda")
    ms = C.c_float()
    rtT = float(np.float32(np.sqrt(T)))
    rc = L.refgpu_run(h, scal.data_ptr(), ferm.data_ptr(), wl.data_ptr(), cx, cy, F, l2, rtT,
                      Nl, ppl, int(fermion), nthreads, padded, C.byref(ms))
    assert rc == 0, rc
    return scal[:Nl].cpu().numpy(), ferm[:Nl].cpu().numpy()


def test_library_matches_reference_kernel_per_loop(refgpu):
    torch = pytest.importorskip("torch")
    import wltube

    z = np.load(GOLD)
    meta = json.loads(bytes(z["meta"]).decode())
    loops = z["loops"]
    ran = 0
    with wltube.Context(0) as ctx:
        h = ctx.upload(loops)
        for case, gold in zip(meta["LOOP_CASES"], z["loop_out"]):
            d, prof, ffv, fe, l2, cx, cy, T, F, a = case
            key = (d, a if d in ("periodic", "fixflux", "ff") else 1.0)
            if key not in CUBINS or not os.path.exists(
                    os.path.join(O.REF_DIR, CUBINS[key][0] + ".cubin")):
                continue
            cub, nthr = CUBINS[key]
            rs, rf = run_reference_kernel(refgpu, torch, cub, nthr, loops, cx, cy, T, F, l2,
                                          fe, d == "ff")
            s, f = ctx.loops(h, wltube.field(prof, fermion=fe, nint=50, lambda2=l2, tubedist=a,
                                             ff_variant=ffv), cx, cy, T, F)
            scale = max(np.abs(rs[:, :3]).max(), 1e-30)
            # the reference GPU kernel against its own code on the CPU (fast-math only)
            assert np.abs(rs[:, :3] - gold[:, :3]).max() / scale < PHASE_TOL, case
            # the library against the reference GPU kernel
            assert np.abs(s[:, :3] - rs[:, :3]).max() / scale < PHASE_TOL, case
            if fe:
                fscale = max(np.abs(rf[:, :3]).max(), 1e-30)
                assert np.abs(f[:, :3] - rf[:, :3]).max() / fscale < PHASE_TOL, case
            ran += 1
        ctx.release(h)
    assert ran >= 8


def test_reference_kernel_throughput_vs_library(refgpu, capsys):
    """The reference's own kernel (smooth, spinor, its 50 Simpson intervals,
    512 threads per block as EffAct.c sets them, one launch per instance as
    EV() makes them) against the library's sweep at the same 50 intervals, on
    the spinor benchmark ensemble (Nl 5120 x ppl 2048, seed 2).  Both are
    timed with CUDA events around their launches only."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    import wltube

    cub = os.path.join(O.REF_DIR, "ref_smooth.cubin")
    if not os.path.exists(cub):
        pytest.skip("reference smooth cubin not built")
    Nl, ppl, F = 5120, 2048, 1.0
    with wltube.Context(0) as ctx:
        h = ctx.generate(2, Nl, ppl)
        wl = torch.from_numpy(ctx.download(h)).cuda()          # 5120 = 10 blocks of 512
        scal = torch.zeros((Nl, 4), dtype=torch.float32, device="cuda")
        ferm = torch.zeros((Nl, 4), dtype=torch.float32, device="cuda")
        kh = refgpu.refgpu_load(cub.encode(), 0)
        assert kh >= 0
        sample = [(r, t) for r in (0.0, 2.0, 4.0, 8.0) for t in (0.01, 1.0)]
        ms = C.c_float()
        r, t = sample[0]                                         # warm-up launch
        assert refgpu.refgpu_run(kh, scal.data_ptr(), ferm.data_ptr(), wl.data_ptr(), r, 0.0, F,
                                 1.0, float(np.float32(np.sqrt(t))), Nl, ppl, 1, 512, Nl,
                                 C.byref(ms)) == 0
        ref_ms = 0.0
        for r, t in sample:
            rc = refgpu.refgpu_run(kh, scal.data_ptr(), ferm.data_ptr(), wl.data_ptr(), r, 0.0,
                                   F, 1.0, float(np.float32(np.sqrt(t))), Nl, ppl, 1, 512, Nl,
                                   C.byref(ms))
            assert rc == 0, rc
            ref_ms += ms.value
        ref_rate = len(sample) * Nl * ppl / (ref_ms * 1e-3)

        n = 512
        rho = np.repeat(np.linspace(0.0, 8.0, 16), n // 16)
        T = np.tile(np.geomspace(1e-3, 1e3, n // 16), 16)
        fld = wltube.field("smooth", fermion=1, nint=50)
        dcx = torch.tensor(rho, dtype=torch.float64, device="cuda")
        dcy = torch.zeros(n, dtype=torch.float64, device="cuda")
        dT = torch.tensor(T, dtype=torch.float64, device="cuda")
        dm = torch.empty(n, dtype=torch.float64, device="cuda")
        ds = torch.empty(n, dtype=torch.float64, device="cuda")
        stream = torch.cuda.ExternalStream(ctx.stream())
        args = (h, fld, n, dcx.data_ptr(), dcy.data_ptr(), dT.data_ptr(), [F], 128, 0,
                dm.data_ptr(), ds.data_ptr())
        ctx.eval_device(*args)
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.eval_device(*args)
        e1.record(stream)
        ctx.synchronize()
        torch.cuda.synchronize()
        lib_rate = n * Nl * ppl / (e0.elapsed_time(e1) * 1e-3)
        ctx.release(h)
    with capsys.disabled():
        print(json.dumps({"reference_kernel_segments_per_s": ref_rate,
                          "library_segments_per_s": lib_rate, "speedup": lib_rate / ref_rate,
                          "simpson_intervals": 50, "reference_sample_instances": len(sample),
                          "library_instances": n}))
    assert lib_rate > 10 * ref_rate
