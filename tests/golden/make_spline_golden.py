"""Generate the spline-profile tables from the reference's own table builder.

Runs getspline (periodic.c:113-164) compiled from the reference's source by
oracle/build_ref.sh (oracle/_ref/ref_spline), with the GSL ODE stand-in of
oracle/refshim/ (GSL is not installed: its rk8pd step on periodic.c's
y-independent right-hand side is a quadrature of the step, restated as
10-point Gauss-Legendre), for a few (lambda^2, a) at the reference's
Nspline = 1000 knots, and stores knots and coefficients in
tests/golden/spline_ref.npz.  Nothing at test time needs the reference tree.

    oracle/build_ref.sh && python tests/golden/make_spline_golden.py
"""
from __future__ import annotations

import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
EXE = os.path.join(ROOT, "oracle", "_ref", "ref_spline")
CASES = [(1.0, 1.0), (0.25, 2.0), (2.0, 5.0), (0.5, 1.0)]
N = 1000


def main() -> None:
    knots, coefs = [], []
    for l2, a in CASES:
        out = subprocess.run([EXE, repr(l2), repr(a), str(N)], check=True,
                             capture_output=True).stdout
        assert len(out) == 20 * N
        knots.append(np.frombuffer(out[:4 * N], np.float32))
        coefs.append(np.frombuffer(out[4 * N:], np.float32).reshape(N, 4))
    np.savez_compressed(os.path.join(HERE, "spline_ref.npz"), cases=np.array(CASES),
                        knots=np.stack(knots), coefs=np.stack(coefs))


if __name__ == "__main__":
    main()
