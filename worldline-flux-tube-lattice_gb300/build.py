"""Build recipe of libwlgpu.so (CUDA kernels + C-ABI runtime) for sm_103a.

    python build.py            # from anywhere; output lib/libwlgpu.so

Compiles every translation unit of csrc/ in parallel with nvcc
(-gencode arch=compute_103a,code=sm_103a) and links one shared library with
the CUDA runtime linked statically, so the library needs only the driver.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libwlgpu.so")
HOST_LIB = os.path.join(LIBDIR, "libwlhost.so")
HOST_SRC = os.path.join(HERE, "host", "wl_host.c")
BUILD = os.path.join(HERE, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                  "-Xcompiler", "-fvisibility=hidden", "--expt-relaxed-constexpr"]
# The periodic and fixflux profiles divide and take square roots at every
# node, inside Lentz's continued fraction too: their translation units are
# compiled as the reference compiles intEV.cu / intEVff.cu, with approximate
# single-precision division and square root (measured 1.5-1.8x faster for
# periodic, 2.2-2.8x for fixflux).  FP64 arithmetic (the epilogue, the sums)
# is not affected by these options.  The spline profile keeps IEEE division
# and square root (with the approximate ones a spinor case moved to 1.05e-5
# of the FP64 oracle, above the 1e-5 tolerance, for a 1.2x gain).
# The spline table is built on the host in FP64 with every operation rounded
# on its own (no fused multiply-add, which Arm hosts would otherwise contract
# and x86 hosts not), so that it is the same table on every host.
EXTRA_FLAGS = {"wl_sweep_periodic.cu": ["-prec-div=false", "-prec-sqrt=false"],
               "wl_sweep_fixflux.cu": ["-prec-div=false", "-prec-sqrt=false"],
               "wl_spline.cpp": ["-Xcompiler", "-ffp-contract=off"]}
SOURCES = ["wl_sweep_smooth.cu", "wl_sweep_simple.cu", "wl_sweep_periodic.cu",
           "wl_sweep_lattice.cu", "wl_sweep_spline.cu",
           "wl_sweep_fixflux.cu", "wl_misc.cu", "wl_api.cpp", "wl_noalloc.cu",
           "wl_tint.cu", "wl_batch.cu", "wl_server.cpp", "wl_spline.cpp"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _deps_mtime() -> float:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files += [os.path.join(HERE, "..", "include", f)
              for f in os.listdir(os.path.join(HERE, "..", "include"))]
    files.append(os.path.abspath(__file__))
    files.append(HOST_SRC)
    return max(os.path.getmtime(f) for f in files)


def cuda_include() -> str:
    return os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "include")


def build_host() -> str:
    """libwlhost.so: the C host layer (Tfunc, integrateT, getwl) on libwlgpu.so."""
    tmp = HOST_LIB + ".tmp%d" % os.getpid()
    cc = shutil.which("gcc") or "cc"
    cmd = [cc, "-O2", "-fPIC", "-shared", "-fvisibility=hidden", "-I" + cuda_include(),
           HOST_SRC, "-o", tmp, "-L" + LIBDIR, "-lwlgpu", "-Wl,-rpath,$ORIGIN", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host library build failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, HOST_LIB)
    return HOST_LIB


def build(force: bool = False, verbose: bool = False) -> str:
    if (not force and os.path.exists(LIB) and os.path.exists(HOST_LIB)
            and min(os.path.getmtime(LIB), os.path.getmtime(HOST_LIB)) >= _deps_mtime()):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nv = nvcc()

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [nv] + NVFLAGS + EXTRA_FLAGS.get(src, []) + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose:
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nv] + ARCH + ["-shared", "-o", tmp] + objs + ["-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    build_host()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
