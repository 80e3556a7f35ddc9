"""The C-ABI library loads without a GPU and exports every declared symbol.

Every function declared in include/wlgpu.h and include/wl_legacy.h must be
exported by libwlgpu.so (wl_legacy.h's Tfunc / integrateT / getwl by the C
host library libwlhost.so, which links libwlgpu.so).  No compute call is made.
"""
import ctypes
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "worldline-flux-tube-lattice_gb300")
INC = os.path.join(ROOT, "include")


def declared(header):
    txt = open(os.path.join(INC, header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\(", txt, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "while", "return", "sizeof")))


@pytest.fixture(scope="module")
def libs():
    sys.path.insert(0, PKG)
    import build as pkg_build

    pkg_build.build()
    return {"wlgpu": ctypes.CDLL(pkg_build.LIB), "wlhost": ctypes.CDLL(pkg_build.HOST_LIB)}


def test_wlgpu_exports_declared_symbols(libs):
    names = declared("wlgpu.h")
    assert "wl_eval" in names and "wl_ctx_create" in names
    for n in names:
        assert hasattr(libs["wlgpu"], n), n


def test_legacy_symbols_exported(libs):
    names = declared("wl_legacy.h")
    assert set(names) == {"EV", "Tfunc", "integrateT", "getwl"}
    assert hasattr(libs["wlgpu"], "EV")
    for n in ("Tfunc", "integrateT", "getwl"):
        assert hasattr(libs["wlhost"], n), n


def test_host_file_symbols_exported(libs):
    names = declared("wl_host.h")
    assert set(names) == {"wlh_putwl", "wlh_write_ensemble", "wlh_ensemble_file_info",
                          "wlh_read_ensemble"}
    for n in names:
        assert hasattr(libs["wlhost"], n), n


def test_version_string_without_gpu(libs):
    f = libs["wlgpu"].wl_version
    f.restype = ctypes.c_char_p
    assert b"sm_103a" in f()


def test_built_for_sm_103a_only():
    src = open(os.path.join(PKG, "build.py")).read()
    assert "arch=compute_103a,code=sm_103a" in src
    assert "sm_100" not in src and "sm_90" not in src


@pytest.mark.parametrize("compiler", ["gcc", "g++"])
def test_headers_compile_after_intT_h(tmp_path, compiler):
    """A reference source includes intT.h first, whose profile names and
    constants (smooth, profile, tubedist, lmin, ...) are object-like macros;
    the library's headers must still compile after it, as C and as C++, and
    leave those macros as intT.h defined them."""
    src = tmp_path / "order.c"
    src.write_text(
        '#include "intT.h"\n#include "wlgpu.h"\n#include "wl_host.h"\n'
        "int main(void) {\n"
        "  double c = pi * q1 * q2 + tubedist + lmin;\n"
        "  int p = profile;\n"
        "  (void)c;\n"
        "  return p == smooth && WL_PROFILE_FIXFLUX_FF == 7 ? 0 : 1;\n"
        "}\n")
    cuda_inc = "/usr/local/cuda/include"
    cmd = [compiler, "-Wall", "-Werror", "-fsyntax-only", "-I" + INC, "-I" + cuda_inc]
    if compiler == "g++":
        cmd += ["-x", "c++"]
    r = subprocess.run(cmd + [str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
