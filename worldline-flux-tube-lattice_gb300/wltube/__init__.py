"""Python host binding of libwlgpu.so, the GB300 Wilson-loop library.

A thin ctypes layer over the C ABI of include/wlgpu.h and include/wl_legacy.h.
It mirrors the reference's host interface for the path: ``Wparams`` and
``EV(T, params, WLlist)`` (intEV.cu:111-148) plus the batched API.  There is
no CPU fallback: importing raises if the CUDA library is missing, and every
call raises ``WlError`` on a non-zero status.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libwlgpu.so")

PROFILES = {"step": 0, "smooth": 1, "quadratic": 2, "gaussian": 3, "periodic": 4,
            "spline": 5, "fixflux": 6, "lattice": 8}
MODE_REFCOMPAT, MODE_EXACT = 0, 1
STATUS = {0: "ok", -1: "invalid argument", -2: "CUDA error", -3: "out of memory",
          -4: "device wait timed out", -5: "unknown handle", -6: "admission rejected"}


class WlError(RuntimeError):
    def __init__(self, status, msg=""):
        super().__init__("%s (%d)%s" % (STATUS.get(status, "error"), status,
                                        (": " + msg) if msg else ""))
        self.status = status


class Field(C.Structure):
    """wl_field of wlgpu.h."""
    _fields_ = [("profile", C.c_int), ("fermion", C.c_int), ("nint", C.c_int),
                ("mode", C.c_int), ("ff_variant", C.c_int), ("reserved", C.c_int),
                ("lambda2", C.c_double), ("tubedist", C.c_double), ("lmin", C.c_double),
                ("rimage", C.c_double)]


def field(profile="smooth", fermion=0, nint=50, mode=None, lambda2=1.0,
          tubedist=1.0, lmin=None, ff_variant=0, rimage=None) -> Field:
    """wl_field; the lattice profile defaults to exact mode and images within
    12 lattice spacings, the others to the reference's clamps."""
    if isinstance(profile, str):
        profile = PROFILES[profile]
    if mode is None:
        mode = MODE_EXACT if profile == PROFILES["lattice"] else MODE_REFCOMPAT
    if lmin is None:
        lmin = 0.1 * tubedist
    if rimage is None:
        rimage = 12.0 * tubedist
    return Field(profile, int(fermion), int(nint), int(mode), int(ff_variant), 0,
                 float(lambda2), float(tubedist), float(lmin), float(rimage))


class Job(C.Structure):
    """wl_job of wlgpu.h."""
    _fields_ = [("handle", C.c_int), ("field", Field), ("ninst", C.c_int),
                ("cx", C.POINTER(C.c_double)), ("cy", C.POINTER(C.c_double)),
                ("T", C.POINTER(C.c_double)), ("nF", C.c_int), ("F", C.c_double * 4),
                ("group", C.c_int), ("out_group", C.POINTER(C.c_double)),
                ("out_mean", C.POINTER(C.c_double)), ("out_sem", C.POINTER(C.c_double))]


class Request(C.Structure):
    """wl_request of wlgpu.h."""
    _fields_ = [("seed", C.c_uint64), ("Nl", C.c_int), ("ppl", C.c_int), ("field", Field),
                ("kind", C.c_int), ("ninst", C.c_int),
                ("cx", C.POINTER(C.c_double)), ("cy", C.POINTER(C.c_double)),
                ("T", C.POINTER(C.c_double)), ("nrho", C.c_int), ("nT", C.c_int),
                ("nbins", C.c_int), ("rho", C.POINTER(C.c_double)),
                ("Tgrid", C.POINTER(C.c_double)), ("nF", C.c_int), ("F", C.c_double * 4),
                ("group", C.c_int), ("out_group", C.POINTER(C.c_double)),
                ("out_mean", C.POINTER(C.c_double)), ("out_sem", C.POINTER(C.c_double)),
                ("out_leff", C.POINTER(C.c_double)), ("out_err", C.POINTER(C.c_double))]


class ServerConfig(C.Structure):
    """wl_server_config of wlgpu.h."""
    _fields_ = [("device", C.c_int), ("hbm_budget_bytes", C.c_double),
                ("quantum_ms", C.c_double), ("points_per_tile", C.c_int),
                ("ctas_per_sm", C.c_int), ("max_requests", C.c_int)]


class ServerStats(C.Structure):
    """wl_server_stats of wlgpu.h."""
    _fields_ = [("submitted", C.c_longlong), ("completed", C.c_longlong),
                ("rejected", C.c_longlong), ("failed", C.c_longlong),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("p999_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double), ("wall_s", C.c_double),
                ("segments", C.c_double), ("launches", C.c_longlong),
                ("resident_ensembles", C.c_int), ("hbm_bytes_in_use", C.c_double),
                ("device_busy_s", C.c_double), ("device_span_s", C.c_double)]


REQ_W, REQ_LEFF = 0, 1
TRULE_LOG, TRULE_SUBST = 0, 1


class Float4(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float), ("w", C.c_float)]


class Wparams(C.Structure):
    """struct Wparams of wl_legacy.h (the reference's intT.h).  CUDA's float4
    is 16-byte aligned, so xcm sits at offset 32 and the struct is 128 bytes;
    ctypes has no alignment attribute, hence the explicit padding."""
    _fields_ = [("Nl", C.c_int), ("Nppl", C.c_int), ("F", C.c_double), ("l2", C.c_double),
                ("_pad_xcm", C.c_char * 8),
                ("xcm", Float4), ("Wsscal_h", C.c_void_p), ("Wsscal_d", C.c_void_p),
                ("Wsferm_h", C.c_void_p), ("Wsferm_d", C.c_void_p),
                ("worldlines", C.c_void_p), ("SE", C.c_double), ("nBlocks", C.c_int),
                ("nThreads", C.c_int), ("ng", C.c_int), ("fermion", C.c_int),
                ("flcoefs", C.c_void_p), ("rho2sp", C.c_void_p)]


_lib = None


def lib():
    """The loaded libwlgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libwlgpu.so is not built (%s); run build.py" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        vp, ip, dp, fp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), \
            C.POINTER(C.c_float)
        L.wl_version.restype = C.c_char_p
        L.wl_status_string.restype = C.c_char_p
        L.wl_status_string.argtypes = [C.c_int]
        L.wl_ctx_create.argtypes = [C.c_int, C.POINTER(vp)]
        L.wl_ctx_destroy.argtypes = [vp]
        L.wl_last_error.argtypes = [vp, C.c_char_p, C.c_int]
        L.wl_ctx_synchronize.argtypes = [vp]
        L.wl_ensemble_upload.argtypes = [vp, fp, C.c_int, C.c_int, ip]
        L.wl_ensemble_wrap.argtypes = [vp, vp, C.c_int, C.c_int, ip]
        L.wl_ensemble_generate.argtypes = [vp, C.c_uint64, C.c_int, C.c_int, C.c_int, ip]
        L.wl_ensemble_download.argtypes = [vp, C.c_int, fp]
        L.wl_ensemble_release.argtypes = [vp, C.c_int]
        L.wl_ensemble_info.argtypes = [vp, C.c_int, C.POINTER(vp), ip, ip]
        L.wl_eval.argtypes = [vp, C.c_int, C.POINTER(Field), C.c_int, dp, dp, dp, C.c_int,
                              dp, C.c_int, dp, dp, dp]
        L.wl_eval_device.argtypes = [vp, C.c_int, C.POINTER(Field), C.c_int, vp, vp, vp,
                                     C.c_int, dp, C.c_int, vp, vp, vp]
        L.wl_ctx_stream.argtypes = [vp, C.POINTER(vp)]
        L.wl_tint.argtypes = [vp, C.c_int, C.POINTER(Field), C.c_int, dp, C.c_int, dp, C.c_int, dp,
                              C.c_int, C.c_int, dp, dp, dp]
        L.wl_peak_probe.argtypes = [vp, C.c_int, dp]
        L.wl_selftest_wait.argtypes = [vp, C.c_int, C.c_int, dp]
        L.wl_spline_table.argtypes = [C.c_double, C.c_double, C.c_int, fp, fp]
        L.wl_effective_action.argtypes = [vp, C.c_int, C.POINTER(Field), C.c_double, C.c_int,
                                          C.c_int, dp, C.c_int, C.c_int, dp, dp, dp, dp]
        L.wl_batch_eval.argtypes = [vp, C.c_int, C.POINTER(Job), C.c_int]
        L.wl_batch_autotune.argtypes = [vp, C.c_int, C.POINTER(Job), ip, ip]
        L.wl_batch_stats.argtypes = [vp, dp, ip, ip, ip]
        L.wl_eval_plain.argtypes = [vp, C.c_int, C.POINTER(Field), C.c_int, dp, dp, dp, C.c_int,
                                    dp, C.c_int, dp, dp, dp, dp]
        L.wl_eval_noalloc.argtypes = [vp, C.c_int, C.c_int, C.POINTER(Field), C.c_int, vp, vp,
                                      vp, C.c_int, dp, C.c_int, vp, vp, vp, vp]
        L.wl_loops.argtypes = [vp, C.c_int, C.POINTER(Field), C.c_double, C.c_double,
                               C.c_double, C.c_double, fp, fp]
        L.wl_last_launches.argtypes = [vp, ip, C.POINTER(C.c_char_p)]
        L.wl_legacy_configure.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_int]
        L.wl_legacy_invalidate.argtypes = []
        L.wl_server_create.argtypes = [C.POINTER(ServerConfig), C.POINTER(vp)]
        L.wl_server_submit.argtypes = [vp, C.POINTER(Request), C.POINTER(C.c_longlong)]
        L.wl_server_wait.argtypes = [vp, C.c_longlong, C.c_double]
        L.wl_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
        L.wl_server_last_error.argtypes = [vp, C.c_char_p, C.c_int]
        L.wl_server_reset_stats.argtypes = [vp]
        L.wl_server_destroy.argtypes = [vp]
        L.EV.restype = C.c_double
        L.EV.argtypes = [C.c_double, C.c_void_p, ip]
        _lib = L
    return _lib


_host = None


def host_lib():
    """The loaded libwlhost.so (the C host layer and the ensemble files)."""
    global _host
    if _host is None:
        lib()
        H = C.CDLL(os.path.join(PKG, "lib", "libwlhost.so"))
        vp, ip = C.c_void_p, C.POINTER(C.c_int)
        H.wlh_write_ensemble.argtypes = [C.c_char_p, vp, C.c_int, C.c_int, C.c_uint64]
        H.wlh_ensemble_file_info.argtypes = [C.c_char_p, ip, ip, C.POINTER(C.c_uint64)]
        H.wlh_read_ensemble.argtypes = [C.c_char_p, vp, C.c_int, C.c_int]
        H.integrateT.argtypes = [C.c_int, vp]
        H.integrateT.restype = C.POINTER(C.c_double)
        H.Tfunc.argtypes = [C.c_double, vp, ip]
        H.Tfunc.restype = C.POINTER(C.c_double)
        H.wlh_putwl.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.c_int]
        H.getwl.argtypes = [vp, C.c_char_p, C.c_int, C.c_int, C.c_int]
        _host = H
    return _host


_libc = None


def _free(ptr):
    """free() of the C library for the host layer's malloc'd results."""
    global _libc
    if _libc is None:
        _libc = C.CDLL(None)
        _libc.free.argtypes = [C.c_void_p]
    _libc.free(C.cast(ptr, C.c_void_p))


def integrateT(n: int, params: "Wparams") -> np.ndarray:
    """The reference's integrateT(n, p) (Tint.c:100-175) through the C host
    layer: the proper-time integral of every loop group, Simpson with n
    panels in t, T = (1 - t)/t, each Tfunc evaluated through EV() on the
    device.  Like the reference it prints the Leffvsrho line to stdout."""
    ptr = host_lib().integrateT(int(n), C.cast(C.pointer(params), C.c_void_p))
    if not ptr:
        raise WlError(-1, "integrateT")
    try:
        return np.ctypeslib.as_array(ptr, shape=(params.ng,)).copy()
    finally:
        _free(ptr)


def save_ensemble(path: str, loops: np.ndarray, seed: int = 0):
    """Write a [Nl][ppl][4] float32 ensemble as a binary ensemble file."""
    loops = np.ascontiguousarray(loops, dtype=np.float32)
    Nl, ppl = loops.shape[:2]
    if host_lib().wlh_write_ensemble(path.encode(), loops.ctypes.data, Nl, ppl, seed) != 0:
        raise OSError("cannot write ensemble file %s" % path)


def save_text_ensemble(path: str, loops: np.ndarray, dim: int = 2):
    """Write loops in the text format getwl reads (getwl.c:6-40): per loop
    ppl x values, then ppl y values (and z for dim 3)."""
    loops = np.ascontiguousarray(loops, dtype=np.float32)
    Nl, ppl = loops.shape[:2]
    if host_lib().wlh_putwl(loops.ctypes.data, path.encode(), Nl, ppl, dim) != 0:
        raise OSError("cannot write %s" % path)


def load_ensemble(path: str):
    """(loops [Nl][ppl][4] float32, seed) of a binary ensemble file."""
    nl, ppl, seed = C.c_int(), C.c_int(), C.c_uint64()
    H = host_lib()
    if H.wlh_ensemble_file_info(path.encode(), C.byref(nl), C.byref(ppl), C.byref(seed)):
        raise OSError("not an ensemble file: %s" % path)
    out = np.empty((nl.value, ppl.value, 4), dtype=np.float32)
    if H.wlh_read_ensemble(path.encode(), out.ctypes.data, nl.value, ppl.value):
        raise OSError("cannot read ensemble file %s" % path)
    return out, seed.value


def _d(a):
    return np.ascontiguousarray(np.atleast_1d(a), dtype=np.float64)


def _p(a, t):
    return a.ctypes.data_as(C.POINTER(t))


class Context:
    """One device and one stream (wl_ctx)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        st = lib().wl_ctx_create(device, C.byref(self._h))
        if st != 0:
            raise WlError(st, "wl_ctx_create(%d)" % device)

    def close(self):
        if self._h:
            lib().wl_ctx_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def _check(self, st):
        if st != 0:
            buf = C.create_string_buffer(512)
            lib().wl_last_error(self._h, buf, 512)
            raise WlError(st, buf.value.decode())

    def upload(self, loops: np.ndarray) -> int:
        loops = np.ascontiguousarray(loops, dtype=np.float32)
        Nl, ppl = loops.shape[:2]
        h = C.c_int()
        self._check(lib().wl_ensemble_upload(self._h, _p(loops, C.c_float), Nl, ppl,
                                             C.byref(h)))
        return h.value

    def wrap(self, dev_ptr: int, Nl: int, ppl: int) -> int:
        h = C.c_int()
        self._check(lib().wl_ensemble_wrap(self._h, C.c_void_p(dev_ptr), Nl, ppl, C.byref(h)))
        return h.value

    def generate(self, seed: int, Nl: int, ppl: int, first: int = 0) -> int:
        h = C.c_int()
        self._check(lib().wl_ensemble_generate(self._h, seed, first, Nl, ppl, C.byref(h)))
        return h.value

    def device_pointer(self, handle: int) -> int:
        """The ensemble's device address (float4 [Nl][ppl]), e.g. for the
        worldlines field of a struct Wparams."""
        ptr = C.c_void_p()
        self._check(lib().wl_ensemble_info(self._h, handle, C.byref(ptr), None, None))
        return ptr.value

    def download(self, handle: int) -> np.ndarray:
        Nl, ppl = C.c_int(), C.c_int()
        self._check(lib().wl_ensemble_info(self._h, handle, None, C.byref(Nl), C.byref(ppl)))
        out = np.empty((Nl.value, ppl.value, 4), dtype=np.float32)
        self._check(lib().wl_ensemble_download(self._h, handle, _p(out, C.c_float)))
        return out

    def release(self, handle: int):
        self._check(lib().wl_ensemble_release(self._h, handle))

    def eval(self, handle: int, fld: Field, cx, cy, T, F, group: int = 128,
             want_groups: bool = True):
        """<W> per group, mean and SEM: arrays [ninst][nF][ng], [ninst][nF] x2."""
        cx, cy, T, F = _d(cx), _d(cy), _d(T), _d(F)
        n = len(T)
        Nl = C.c_int()
        self._check(lib().wl_ensemble_info(self._h, handle, None, C.byref(Nl), None))
        ng = Nl.value // group if group > 0 else 0
        groups = np.empty((n, len(F), max(ng, 1))) if want_groups else None
        mean = np.empty((n, len(F)))
        sem = np.empty((n, len(F)))
        self._check(lib().wl_eval(
            self._h, handle, C.byref(fld), n, _p(cx, C.c_double), _p(cy, C.c_double),
            _p(T, C.c_double), len(F), _p(F, C.c_double), group,
            _p(groups, C.c_double) if want_groups else None, _p(mean, C.c_double),
            _p(sem, C.c_double)))
        return groups, mean, sem

    def eval_device(self, handle: int, fld: Field, ninst: int, dev_cx: int, dev_cy: int,
                    dev_T: int, F, group: int = 128, dev_out_group: int = 0,
                    dev_out_mean: int = 0, dev_out_sem: int = 0):
        """Asynchronous evaluation on device-resident instance arrays (FP64
        device pointers given as integers); call synchronize() for the status."""
        F = _d(F)
        self._check(lib().wl_eval_device(
            self._h, handle, C.byref(fld), ninst, C.c_void_p(dev_cx), C.c_void_p(dev_cy),
            C.c_void_p(dev_T), len(F), _p(F, C.c_double), group,
            C.c_void_p(dev_out_group or None), C.c_void_p(dev_out_mean or None),
            C.c_void_p(dev_out_sem or None)))

    def tint(self, handle: int, fld: Field, rho, T, F, group: int = 128, nbins: int = 20,
             want_igrand: bool = False):
        """Effective action density per radius (wl_tint): L_eff[nrho][nF], its
        jackknife error, and optionally the integrand [nrho][nF][nT][ng]."""
        rho, T, F = _d(rho), _d(T), _d(F)
        Nl = C.c_int()
        self._check(lib().wl_ensemble_info(self._h, handle, None, C.byref(Nl), None))
        ng = Nl.value // group
        leff = np.empty((len(rho), len(F)))
        err = np.empty((len(rho), len(F)))
        ig = np.empty((len(rho), len(F), len(T), ng)) if want_igrand else None
        self._check(lib().wl_tint(self._h, handle, C.byref(fld), len(rho), _p(rho, C.c_double),
                                  len(T), _p(T, C.c_double), len(F), _p(F, C.c_double), group,
                                  nbins, _p(leff, C.c_double), _p(err, C.c_double),
                                  _p(ig, C.c_double) if want_igrand else None))
        return leff, err, ig

    def effective_action(self, handle: int, fld: Field, F: float, T=None, group: int = 128,
                         nrho: int = 20, t_panels: int = 40):
        """wl_effective_action: (mean, standard error, classical action,
        per-group values) of the effective action per unit length.  T: a
        log-spaced grid (Simpson in ln T); None: integrateT's t-substitution
        with t_panels panels, as the reference's rhogrand (40)."""
        Nl = C.c_int()
        self._check(lib().wl_ensemble_info(self._h, handle, None, C.byref(Nl), None))
        groups = np.empty(Nl.value // group)
        a, e, ca = C.c_double(), C.c_double(), C.c_double()
        if T is None:
            rule, n, Tp = TRULE_SUBST, t_panels, None
        else:
            T = _d(T)
            rule, n, Tp = TRULE_LOG, len(T), _p(T, C.c_double)
        self._check(lib().wl_effective_action(self._h, handle, C.byref(fld), float(F), rule, n,
                                              Tp, group, nrho, C.byref(a), C.byref(e),
                                              C.byref(ca), _p(groups, C.c_double)))
        return a.value, e.value, ca.value, groups

    def _jobs(self, jobs):
        """Pack job dicts (handle, field, cx, cy, T, F, group) into wl_job
        structs with freshly allocated outputs; returns (array, outputs, keep)."""
        arr = (Job * len(jobs))()
        outs, keep = [], []
        for i, j in enumerate(jobs):
            cx, cy, T, F = _d(j["cx"]), _d(j["cy"]), _d(j["T"]), _d(j["F"])
            group = j.get("group", 128)
            Nl = C.c_int()
            self._check(lib().wl_ensemble_info(self._h, j["handle"], None, C.byref(Nl), None))
            ng = Nl.value // group
            g = np.empty((len(T), len(F), max(ng, 1)))
            m = np.empty((len(T), len(F)))
            se = np.empty((len(T), len(F)))
            a = arr[i]
            a.handle, a.field, a.ninst = j["handle"], j["field"], len(T)
            a.cx, a.cy, a.T = _p(cx, C.c_double), _p(cy, C.c_double), _p(T, C.c_double)
            a.nF = len(F)
            for k, f in enumerate(F):
                a.F[k] = f
            a.group = group
            a.out_group, a.out_mean, a.out_sem = (_p(g, C.c_double), _p(m, C.c_double),
                                                  _p(se, C.c_double))
            outs.append((g, m, se))
            keep += [cx, cy, T, F]
        return arr, outs, keep

    def batch_eval(self, jobs, graph: bool = True):
        """Evaluate a list of job dicts in one persistent launch (wl_batch_eval);
        returns [(groups, mean, sem)] per job."""
        arr, outs, keep = self._jobs(jobs)
        self._check(lib().wl_batch_eval(self._h, len(jobs), arr, 1 if graph else 0))
        return outs

    def batch_autotune(self, jobs):
        arr, _, keep = self._jobs(jobs)
        p, c = C.c_int(), C.c_int()
        self._check(lib().wl_batch_autotune(self._h, len(jobs), arr, C.byref(p), C.byref(c)))
        return p.value, c.value

    def batch_stats(self):
        ms, nt, g, p = C.c_double(), C.c_int(), C.c_int(), C.c_int()
        self._check(lib().wl_batch_stats(self._h, C.byref(ms), C.byref(nt), C.byref(g),
                                         C.byref(p)))
        return {"device_ms": ms.value, "tiles": nt.value, "grid": g.value,
                "points_per_tile": p.value}

    def eval_plain(self, handle: int, fld: Field, cx, cy, T, F, group: int = 128):
        """The plain per-instance kernel (one launch per instance); returns
        (groups, mean, sem, device_ms)."""
        cx, cy, T, F = _d(cx), _d(cy), _d(T), _d(F)
        Nl = C.c_int()
        self._check(lib().wl_ensemble_info(self._h, handle, None, C.byref(Nl), None))
        ng = Nl.value // group
        g = np.empty((len(T), len(F), ng))
        m = np.empty((len(T), len(F)))
        se = np.empty((len(T), len(F)))
        ms = C.c_double()
        self._check(lib().wl_eval_plain(self._h, handle, C.byref(fld), len(T), _p(cx, C.c_double),
                                        _p(cy, C.c_double), _p(T, C.c_double), len(F),
                                        _p(F, C.c_double), group, _p(g, C.c_double),
                                        _p(m, C.c_double), _p(se, C.c_double), C.byref(ms)))
        return g, m, se, ms.value

    def peak_probe(self, kind: int) -> float:
        """Lane operations per second of the FP32 FMA (0) or MUFU rcp (1) pipe."""
        v = C.c_double()
        self._check(lib().wl_peak_probe(self._h, kind, C.byref(v)))
        return v.value

    def selftest_wait(self, arrive: bool, max_tries: int = 64) -> float:
        """The device's bounded mbarrier wait on a barrier that gets its
        arrival (returns the kernel's ms) or never does (raises WlError,
        status -4)."""
        ms = C.c_double()
        self._check(lib().wl_selftest_wait(self._h, int(bool(arrive)), int(max_tries),
                                           C.byref(ms)))
        return ms.value

    def stream(self) -> int:
        """The context's cudaStream_t as an integer."""
        s = C.c_void_p()
        self._check(lib().wl_ctx_stream(self._h, C.byref(s)))
        return s.value or 0

    def loops(self, handle: int, fld: Field, cx: float, cy: float, T: float, F: float):
        """Per-loop Wsscal / Wsferm of one instance: two float32 arrays [Nl][4]."""
        Nl = C.c_int()
        self._check(lib().wl_ensemble_info(self._h, handle, None, C.byref(Nl), None))
        s = np.empty((Nl.value, 4), dtype=np.float32)
        f = np.empty((Nl.value, 4), dtype=np.float32)
        self._check(lib().wl_loops(self._h, handle, C.byref(fld), cx, cy, T, F,
                                   _p(s, C.c_float), _p(f, C.c_float)))
        return s, f

    def last_launches(self):
        n, k = C.c_int(), C.c_char_p()
        self._check(lib().wl_last_launches(self._h, C.byref(n), C.byref(k)))
        return n.value, k.value.decode()

    def synchronize(self):
        self._check(lib().wl_ctx_synchronize(self._h))


class Server:
    """Continuously batched request server (wl_server): ensembles named by
    (seed, Nl, ppl) are generated on the device at first use and stay
    resident; requests are admitted by HBM footprint and their tiles share
    the persistent kernel's launches with every other admitted request."""

    def __init__(self, device: int = 0, hbm_budget_bytes: float = 0.0,
                 quantum_ms: float = 0.0, points_per_tile: int = 0, ctas_per_sm: int = 0,
                 max_requests: int = 0):
        cfg = ServerConfig(device, float(hbm_budget_bytes), float(quantum_ms),
                           int(points_per_tile), int(ctas_per_sm), int(max_requests))
        self._h = C.c_void_p()
        st = lib().wl_server_create(C.byref(cfg), C.byref(self._h))
        if st != 0:
            raise WlError(st, "wl_server_create")
        self._open = {}  # ticket -> (outputs, kept inputs)

    def close(self):
        if self._h:
            lib().wl_server_destroy(self._h)
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _error(self, st):
        buf = C.create_string_buffer(512)
        lib().wl_server_last_error(self._h, buf, 512)
        return WlError(st, buf.value.decode())

    def _submit(self, q, outs, keep):
        t = C.c_longlong()
        st = lib().wl_server_submit(self._h, C.byref(q), C.byref(t))
        if st != 0:
            raise self._error(st)
        self._open[t.value] = (outs, keep)
        return t.value

    @staticmethod
    def _base(seed, Nl, ppl, fld, F, group, kind):
        F = _d(F)
        q = Request()
        q.seed, q.Nl, q.ppl, q.field, q.kind = seed, Nl, ppl, fld, kind
        q.nF = len(F)
        for k, f in enumerate(F[:4]):
            q.F[k] = f
        q.group = group
        return q, F

    def submit_w(self, seed: int, Nl: int, ppl: int, fld: Field, cx, cy, T, F,
                 group: int = 128, want_groups: bool = False) -> int:
        """<W> request; wait() returns (groups or None, mean, sem)."""
        q, F = self._base(seed, Nl, ppl, fld, F, group, REQ_W)
        cx, cy, T = _d(cx), _d(cy), _d(T)
        n = len(T)
        q.ninst = n
        q.cx, q.cy, q.T = _p(cx, C.c_double), _p(cy, C.c_double), _p(T, C.c_double)
        g = np.empty((n, len(F), max(Nl // max(group, 1), 1))) if want_groups else None
        m, se = np.empty((n, len(F))), np.empty((n, len(F)))
        if want_groups:
            q.out_group = _p(g, C.c_double)
        q.out_mean, q.out_sem = _p(m, C.c_double), _p(se, C.c_double)
        return self._submit(q, (g, m, se), [cx, cy, T, F])

    def submit_leff(self, seed: int, Nl: int, ppl: int, fld: Field, rho, T, F,
                    group: int = 128, nbins: int = 20) -> int:
        """Effective-action-density request; wait() returns (leff, err)."""
        q, F = self._base(seed, Nl, ppl, fld, F, group, REQ_LEFF)
        rho, T = _d(rho), _d(T)
        q.nrho, q.nT, q.nbins = len(rho), len(T), nbins
        q.rho, q.Tgrid = _p(rho, C.c_double), _p(T, C.c_double)
        le, er = np.empty((len(rho), len(F))), np.empty((len(rho), len(F)))
        q.out_leff, q.out_err = _p(le, C.c_double), _p(er, C.c_double)
        return self._submit(q, (le, er), [rho, T, F])

    def wait(self, ticket: int, timeout_ms: float = -1.0):
        """The request's outputs, or None if it is not done within timeout_ms."""
        st = lib().wl_server_wait(self._h, ticket, float(timeout_ms))
        if st == 1:  # WL_PENDING
            return None
        outs, _ = self._open.pop(ticket, (None, None))
        if st != 0:
            raise self._error(st)
        return outs

    def reset_stats(self):
        lib().wl_server_reset_stats(self._h)

    def stats(self) -> dict:
        s = ServerStats()
        lib().wl_server_get_stats(self._h, C.byref(s))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}


def spline_table(lambda2: float, tubedist: float, n: int = 1000):
    """The spline profile's table: knots rho^2 [n] and coefficients [n][4]."""
    rho2 = np.empty(n, dtype=np.float32)
    coef = np.empty((n, 4), dtype=np.float32)
    st = lib().wl_spline_table(float(lambda2), float(tubedist), int(n), _p(rho2, C.c_float),
                               _p(coef, C.c_float))
    if st != 0:
        raise WlError(st, "wl_spline_table")
    return rho2, coef


def eval_noalloc(dev_loops: int, Nl: int, ppl: int, fld: Field, ninst: int, dev_cx: int,
                 dev_cy: int, dev_T: int, F, group: int = 128, dev_out_group: int = 0,
                 dev_out_mean: int = 0, dev_out_sem: int = 0, stream: int = 0):
    """wl_eval_noalloc: the batched evaluation for callers that cannot let the
    library allocate device memory (all buffers are the caller's device
    pointers, given as integers; scratch is a fixed 32 MiB array in the
    library).  Raises WlError on a non-zero status."""
    F = _d(F)
    st = lib().wl_eval_noalloc(C.c_void_p(dev_loops), Nl, ppl, C.byref(fld), ninst,
                               C.c_void_p(dev_cx), C.c_void_p(dev_cy), C.c_void_p(dev_T), len(F),
                               _p(F, C.c_double), group, C.c_void_p(dev_out_group or None),
                               C.c_void_p(dev_out_mean or None), C.c_void_p(dev_out_sem or None),
                               C.c_void_p(stream or None))
    if st != 0:
        raise WlError(st, "wl_eval_noalloc")


def legacy_configure(profile="smooth", tubedist=1.0, lmin=None, nint=50,
                     mode=MODE_REFCOMPAT):
    """wl_legacy_configure: the profile EV() evaluates ("fixflux-ff": the
    fixflux profile with intEVff.cu's fits)."""
    if isinstance(profile, str):
        profile = 7 if profile == "fixflux-ff" else PROFILES[profile]
    if lmin is None:
        lmin = 0.1 * tubedist
    st = lib().wl_legacy_configure(profile, tubedist, lmin, nint, mode)
    if st != 0:
        raise WlError(st, "wl_legacy_configure")


def legacy_invalidate():
    """wl_legacy_invalidate: the next EV() call recomputes its sweep."""
    st = lib().wl_legacy_invalidate()
    if st != 0:
        raise WlError(st, "wl_legacy_invalidate")


def EV(T: float, params: Wparams, WLlist) -> float:
    """The reference's EV(T, p, WLlist) through the C ABI."""
    wl = np.ascontiguousarray(WLlist, dtype=np.int32)
    return lib().EV(T, C.cast(C.pointer(params), C.c_void_p), _p(wl, C.c_int))


def version() -> str:
    return lib().wl_version().decode()
