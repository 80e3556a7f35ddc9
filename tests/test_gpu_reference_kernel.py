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
