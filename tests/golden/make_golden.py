"""Generate the golden vectors of the Wilson-loop path from the reference itself.

Runs the reference's own code (intEV.cu / intEVff.cu device functions,
Integrand.c, Tint.c), compiled for the CPU by oracle/build_ref.sh from the
reference tree, on a small seeded loop ensemble and stores inputs and outputs
in tests/golden/golden_ref.npz.  The tests compare the CPU oracle (and, on a
GPU, the CUDA library) against this file; nothing at test time needs the
reference tree.

    python tests/golden/make_golden.py [REFERENCE_DIR]

The loops are stored in the fixture (float32 [256][64][4], seed 11) so the
fixture does not depend on the generator's last-ulp behaviour.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

NL, PPL, SEED = 256, 64, 11

# per-loop cases: (driver, profile, ff_variant, fermion, lambda2, cx, cy, T, F, a)
LOOP_CASES = [
    ("smooth", "smooth", 0, 0, 1.0, 0.0, 0.0, 0.1, 1.0, 1.0),
    ("smooth", "smooth", 0, 0, 1.0, 0.5, 0.0, 1.0, 1.0, 1.0),
    ("smooth", "smooth", 0, 1, 1.0, 0.5, 0.0, 1.0, 1.0, 1.0),
    ("smooth", "smooth", 0, 1, 1.0, 2.0, 0.0, 5.0, 0.1, 1.0),
    ("smooth", "smooth", 0, 1, 1.0, 0.3, 0.4, 0.05, 10.0, 1.0),
    ("smooth", "smooth", 0, 1, 0.01, 0.05, 0.0, 0.02, 1.0, 1.0),
    ("step", "step", 0, 1, 2.0, 0.3, 0.0, 0.5, 0.7, 1.0),
    ("quadratic", "quadratic", 0, 1, 2.0, 0.3, 0.0, 0.5, 0.7, 1.0),
    ("gaussian", "gaussian", 0, 1, 1.0, 1.0, 0.0, 2.0, 1.0, 1.0),
    ("gaussian", "gaussian", 0, 0, 0.25, 0.2, 0.1, 0.3, 1.0, 1.0),
    ("periodic", "periodic", 0, 1, 0.04, 3.0, 0.0, 0.5, 1.0, 1.0),
    ("periodic", "periodic", 0, 1, 0.25, 2.2, 0.0, 0.3, 1.0, 2.0),
    ("fixflux", "fixflux", 0, 1, 0.09, 1.3, 0.0, 0.4, 1.0, 2.0),
    ("ff", "fixflux", 1, 1, 0.09, 1.3, 0.0, 0.4, 1.0, 2.0),
    ("ff", "fixflux", 1, 1, 0.16, 0.3, 0.0, 0.1, 1.0, 2.0),
]

# EV() cases (two identity-ordered groups of 128): (driver, fermion, l2, cx, T, F)
EV_CASES = [
    ("smooth", 0, 1.0, 0.5, 0.05, 1.0),
    ("smooth", 0, 1.0, 0.5, 3.0, 1.0),
    ("smooth", 1, 1.0, 0.5, 0.5, 1.0),
    ("smooth", 1, 1.0, 0.0, 3.0, 1.0),
    ("gaussian", 1, 1.0, 1.0, 1.0, 1.0),
]

# Tfunc(T) cases covering the four regimes: (driver, fermion, l2, cx, T, F)
TF_CASES = [(d, fe, 1.0, 0.5, T, 1.0) for d in ("smooth",) for fe in (0, 1)
            for T in (0.001, 0.004, 0.5, 3.0, 60.0)]

# integrateT(n) cases: (driver, fermion, l2, cx, n, F)
IT_CASES = [("smooth", 1, 1.0, 0.5, 4, 1.0), ("smooth", 0, 1.0, 0.5, 3, 1.0)]

# profile / field / analytic-function tables: (driver, l2, F, fermion, a)
FN_CASES = [("step", 2.0, 1.0, 0, 1.0), ("smooth", 1.0, 1.0, 1, 1.0),
            ("quadratic", 2.0, 1.0, 0, 1.0), ("gaussian", 1.0, 1.0, 1, 1.0),
            ("periodic", 0.04, 1.0, 1, 1.0), ("fixflux", 0.09, 1.0, 1, 2.0)]


def run(exe, args, tmp):
    subprocess.run([exe] + [str(a) for a in args], check=True, cwd=tmp,
                   stdout=subprocess.DEVNULL)


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    subprocess.check_call([os.path.join(ROOT, "oracle", "build_ref.sh"), ref])
    drv = lambda name: os.path.join(ROOT, "oracle", "_ref", "ref_driver_" + name)  # noqa
    loops = O.vloops(SEED, NL, PPL)
    out = {"loops": loops}
    with tempfile.TemporaryDirectory() as tmp:
        lp = os.path.join(tmp, "loops.bin")
        op = os.path.join(tmp, "out.bin")
        loops.tofile(lp)
        res = []
        for (d, _p, _v, fe, l2, cx, cy, T, F, a) in LOOP_CASES:
            run(drv(d), ["loops", NL, PPL, cx, cy, T, F, l2, fe, a, lp, op], tmp)
            res.append(np.fromfile(op, dtype=np.float32).reshape(NL, 8))
        out["loop_out"] = np.stack(res)
        res = []
        for (d, fe, l2, cx, T, F) in EV_CASES:
            run(drv(d), ["ev", NL, PPL, cx, 0.0, T, F, l2, fe, 1.0, lp, op], tmp)
            res.append(np.fromfile(op))
        out["ev_out"] = np.stack(res)
        res = []
        for (d, fe, l2, cx, T, F) in TF_CASES:
            run(drv(d), ["tfunc", NL, PPL, cx, 0.0, T, F, l2, fe, 1.0, lp, op], tmp)
            res.append(np.fromfile(op))
        out["tf_out"] = np.stack(res)
        res = []
        for (d, fe, l2, cx, n, F) in IT_CASES:
            run(drv(d), ["intT", NL, PPL, cx, 0.0, n, F, l2, fe, 1.0, lp, op], tmp)
            res.append(np.fromfile(op))
        out["it_out"] = np.stack(res)
        rho2 = np.concatenate([np.linspace(0.0, 1.0, 23)[1:], np.linspace(1.0, 30.0, 17)])
        Ts = np.geomspace(1e-3, 40.0, len(rho2))
        pairs = np.stack([rho2, Ts], axis=1).astype(np.float64)
        ip = os.path.join(tmp, "in.bin")
        pairs.tofile(ip)
        res = []
        for (d, l2, F, fe, a) in FN_CASES:
            run(drv(d), ["funcs", l2, F, fe, a, ip, op], tmp)
            res.append(np.fromfile(op).reshape(-1, 6))
        out["fn_pairs"] = pairs
        out["fn_out"] = np.stack(res)
    meta = {"NL": NL, "PPL": PPL, "SEED": SEED, "LOOP_CASES": LOOP_CASES,
            "EV_CASES": EV_CASES, "TF_CASES": TF_CASES, "IT_CASES": IT_CASES,
            "FN_CASES": FN_CASES}
    out["meta"] = np.frombuffer(json.dumps(meta).encode(), dtype=np.uint8)
    np.savez_compressed(os.path.join(HERE, "golden_ref.npz"), **out)
    print("wrote", os.path.join(HERE, "golden_ref.npz"))


if __name__ == "__main__":
    main()
