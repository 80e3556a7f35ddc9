"""Ensemble files of the C host layer (no GPU): the binary format round trip
and its checks, and the text format that getwl reads (getwl.c:6-40) written
by wlh_putwl and read back by getwl."""
import ctypes as C
import os
import struct

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "worldline-flux-tube-lattice_gb300")


@pytest.fixture(scope="module")
def host():
    import sys

    sys.path.insert(0, PKG)
    import build as pkg_build

    pkg_build.build()
    C.CDLL(pkg_build.LIB, mode=C.RTLD_GLOBAL)
    L = C.CDLL(pkg_build.HOST_LIB)
    vp, ip = C.c_void_p, C.POINTER(C.c_int)
    L.wlh_write_ensemble.argtypes = [C.c_char_p, vp, C.c_int, C.c_int, C.c_uint64]
    L.wlh_ensemble_file_info.argtypes = [C.c_char_p, ip, ip, C.POINTER(C.c_uint64)]
    L.wlh_read_ensemble.argtypes = [C.c_char_p, vp, C.c_int, C.c_int]
    L.wlh_putwl.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.c_int]
    L.getwl.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.c_int]
    return L


def test_binary_round_trip(host, tmp_path):
    rng = np.random.default_rng(1)
    loops = rng.standard_normal((7, 12, 4)).astype(np.float32)
    p = str(tmp_path / "e.wlens").encode()
    assert host.wlh_write_ensemble(p, loops.ctypes.data, 7, 12, 0x1234567890ABCDEF) == 0
    nl, ppl, seed = C.c_int(), C.c_int(), C.c_uint64()
    assert host.wlh_ensemble_file_info(p, C.byref(nl), C.byref(ppl), C.byref(seed)) == 0
    assert (nl.value, ppl.value, seed.value) == (7, 12, 0x1234567890ABCDEF)
    back = np.zeros_like(loops)
    assert host.wlh_read_ensemble(p, back.ctypes.data, 7, 12) == 0
    assert np.array_equal(back, loops)
    raw = open(p, "rb").read()
    assert raw[:8] == b"WLENSv1\x00" and struct.unpack("<IIQI", raw[8:28]) == (
        7, 12, 0x1234567890ABCDEF, 4)
    assert len(raw) == 32 + loops.nbytes


def test_binary_checks(host, tmp_path):
    loops = np.zeros((2, 8, 4), np.float32)
    p = str(tmp_path / "e.wlens").encode()
    assert host.wlh_write_ensemble(p, loops.ctypes.data, 2, 8, 0) == 0
    back = np.zeros((2, 8, 4), np.float32)
    assert host.wlh_read_ensemble(p, back.ctypes.data, 2, 4) == -1     # other shape
    raw = open(p, "rb").read()
    short = str(tmp_path / "short.wlens").encode()
    open(short, "wb").write(raw[:-16])
    assert host.wlh_read_ensemble(short, back.ctypes.data, 2, 8) == -1  # short file
    bad = str(tmp_path / "bad.wlens").encode()
    open(bad, "wb").write(b"XXXXXXXX" + raw[8:])
    assert host.wlh_ensemble_file_info(bad, None, None, None) == -1     # not an ensemble
    assert host.wlh_ensemble_file_info(str(tmp_path / "none").encode(), None, None, None) == -1


def test_text_format_round_trip(host, tmp_path):
    rng = np.random.default_rng(2)
    loops = rng.standard_normal((3, 5, 4)).astype(np.float32)
    loops[..., 3] = 0.0
    p = str(tmp_path / "wl.dat").encode()
    assert host.wlh_putwl(loops.ctypes.data, p, 3, 5, 3) == 0
    back = np.zeros_like(loops)
    assert host.getwl(back.ctypes.data, p, 3, 5, 3) == 0
    assert np.array_equal(back[..., :3], loops[..., :3])


def test_python_helpers_round_trip(tmp_path):
    import sys

    sys.path.insert(0, PKG)
    import wltube

    loops = np.random.default_rng(3).standard_normal((4, 8, 4)).astype(np.float32)
    p = str(tmp_path / "x.wlens")
    wltube.save_ensemble(p, loops, seed=5)
    back, seed = wltube.load_ensemble(p)
    assert seed == 5 and np.array_equal(back, loops)
    # the text format through the Python helper, read back by getwl (x, y)
    t = str(tmp_path / "x.txt")
    wltube.save_text_ensemble(t, loops)
    back2 = np.zeros_like(loops)
    assert wltube.host_lib().getwl(back2.ctypes.data, t.encode(), 4, 8, 2) == 0
    assert np.array_equal(back2[..., :2], loops[..., :2]) and not back2[..., 2:].any()
