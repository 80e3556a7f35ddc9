"""The reference's own host files link against the library unchanged.

The reference's effective-action program is EffAct.c (main, EAction, the
radial integral) + Tint.c (integrateT) + Integrand.c (Tfunc, EVMean) +
getwl.c, linked with intEV.o, whose only host entry point they call is
EV(T, p, WLlist) (Integrand.c:297-301; Makefile:27-28).  These tests compile
those four files (and testT.c, the reference's second driver) from the
reference tree as they are, against this repository's include/intT.h (the
reconstructed configuration header) and the two-name GSL stand-in Tint.c
needs (oracle/refshim/gsl; GSL is not installed), with -fcommon for their
tentative definitions (EffAct.c:7 and Integrand.c:12-14 both define e, m2),
and link them against libwlgpu.so in place of intEV.o with --no-undefined:
every symbol they use resolves, EV from libwlgpu.so.

The linked programs need the reference's loop file and a GPU to run, so they
are only linked here (CPU); the same call chain in this repository's C
restatement (host/wl_host.c, libwlhost.so) runs on the GPU in
tests/test_gpu_tint.py.  Skipped when the reference tree is absent.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "worldline-flux-tube-lattice_gb300")
INC = os.path.join(ROOT, "include")
GSL_SHIM = os.path.join(ROOT, "oracle", "refshim")
REF = "/root/reference"
CUDA = "/usr/local/cuda"

pytestmark = pytest.mark.skipif(not os.path.isfile(os.path.join(REF, "EffAct.c")),
                                reason="reference tree not present")


@pytest.fixture(scope="module")
def libdir():
    import sys

    sys.path.insert(0, PKG)
    import build as pkg_build

    pkg_build.build()
    return os.path.dirname(pkg_build.LIB)


def _compile(tmp, name, profile="smooth"):
    obj = os.path.join(tmp, name + ".o")
    cmd = ["gcc", "-c", "-O2", "-fcommon", "-D_GNU_SOURCE", "-w", "-Dprofile=" + profile,
           "-I" + INC, "-I" + GSL_SHIM, "-I" + os.path.join(CUDA, "include"),
           os.path.join(REF, name + ".c"), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return obj


def _link(tmp, exe, objs, libdir):
    out = os.path.join(tmp, exe)
    cmd = ["gcc", "-o", out] + objs + [
        "-L" + libdir, "-lwlgpu", "-Wl,-rpath," + libdir,
        "-L" + os.path.join(CUDA, "lib64"), "-lcudart", "-lm", "-Wl,--no-undefined"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def _undefined(obj):
    r = subprocess.run(["nm", "-u", obj], capture_output=True, text=True, check=True)
    return {ln.split()[-1] for ln in r.stdout.splitlines() if ln.strip()}


def _defined(path, dynamic=False):
    cmd = ["nm", "-D", "--defined-only", path] if dynamic else ["nm", "--defined-only", path]
    r = subprocess.run(cmd, capture_output=True, text=True, check=True)
    return {ln.split()[-1] for ln in r.stdout.splitlines() if len(ln.split()) >= 3}


@pytest.mark.skipif(shutil.which("nm") is None, reason="binutils absent")
@pytest.mark.parametrize("profile", ["smooth", "gaussian", "step", "quadratic"])
def test_effact_links_against_the_library(tmp_path, libdir, profile):
    """EffAct.c + Tint.c + Integrand.c + getwl.c, unmodified, link with
    libwlgpu.so in place of intEV.o; EV is the only kernel-side symbol they
    need and the library exports it."""
    tmp = str(tmp_path)
    objs = [_compile(tmp, n, profile) for n in ("EffAct", "Tint", "Integrand", "getwl")]
    need = set().union(*(_undefined(o) for o in objs))
    have = set().union(*(_defined(o) for o in objs))
    lib_syms = _defined(os.path.join(libdir, "libwlgpu.so"), dynamic=True)
    # what the reference's host files take from the kernel file intEV.cu
    from_kernel = {s for s in need - have if not s.startswith(("cuda", "__"))
                   and s in lib_syms}
    assert from_kernel == {"EV"}, from_kernel
    exe = _link(tmp, "EffAct", objs, libdir)
    # EV is resolved through libwlgpu.so, not defined in the program
    assert "EV" not in _defined(exe)
    r = subprocess.run(["readelf", "-d", exe], capture_output=True, text=True, check=True)
    assert "libwlgpu.so" in r.stdout


@pytest.mark.skipif(shutil.which("nm") is None, reason="binutils absent")
def test_testT_links_against_the_library(tmp_path, libdir):
    """The reference's second driver (testT.c: integrateT at rho = 0, eB = 1,
    spinor) with Tint.c + Integrand.c + getwl.c links the same way."""
    if not os.path.isfile(os.path.join(REF, "testT.c")):
        pytest.skip("testT.c absent")
    tmp = str(tmp_path)
    objs = [_compile(tmp, n) for n in ("testT", "Tint", "Integrand", "getwl")]
    exe = _link(tmp, "testT", objs, libdir)
    assert "EV" not in _defined(exe)
