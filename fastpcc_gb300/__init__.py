"""fastpcc_gb300 — GB300-native interstation correlations behind a C ABI.

The compute path is the native library ``libfastpcc_gb300.so`` (sm_103a CUDA
kernels + C ABI, see include/fastpcc_gb300.h).  This module is the host-side
mirror of the reference's method layer (FastPCC src/FFTapps.c): the ``*_set``
functions take the same arguments as the reference's ``pcc2_set``, ``pcc1_set``,
``pcc_set``, ``ccgn_set``, ``cc1b_set`` — windows of station 1 and station 2 and a
lag window — with numpy arrays in place of row-pointer arrays, and raise
``FpccError`` with the library's message where the reference returns a negative
code.  There is no CPU fallback: without the native library every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfastpcc_gb300.so")

# methods (enum fpcc_method)
PCC2, GNCC, CC1B, CC1B_POPCOUNT, PCC1, PCCV, WPCC = 0, 1, 2, 3, 4, 5, 6
# amplitude-normalisation rules (enum fpcc_amp_rule)
AMP_F_REG, AMP_D_REG, AMP_PURE, AMP_THRESH, AMP_SUMTHR = 0, 1, 2, 3, 4
F32, F16, I16 = 0, 1, 2
SIGN_GE, SIGN_GT = 0, 1
NZ_TUNED, NZ_REFERENCE, NZ_FAST = -1, 0, 1
ANALYTIC_F32, ANALYTIC_AUTO, ANALYTIC_F64 = 0, 1, 2
STACK_LINEAR, STACK_PWS, STACK_TSPWS = 0, 1, 2

_lock = threading.Lock()
_lib = None


class Request(C.Structure):
    """fpcc_request of include/fastpcc_gb300.h."""
    _fields_ = [("method", C.c_int), ("sta1", C.c_int32), ("sta2", C.c_int32), ("window", C.c_int32),
                ("Lag1", C.c_int), ("Lag2", C.c_int), ("v", C.c_float), ("y", C.c_void_p), ("num", C.c_void_p)]


class PairDesc(C.Structure):
    """fpcc_pair_desc: one correlation of a packed pair stage (device addresses)."""
    _fields_ = [("a", C.c_void_p), ("b", C.c_void_p), ("ea", C.c_void_p), ("eb", C.c_void_p), ("y", C.c_void_p),
                ("N", C.c_int32), ("lag0", C.c_int32), ("L", C.c_int32), ("scale", C.c_float)]


class ServerStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("batches", C.c_int64), ("station_rows", C.c_int64),
                ("hbm_used", C.c_int64), ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double),
                ("pair_stages", C.c_int64), ("worker_ms", C.c_double), ("deliver_ms", C.c_double)]


class FpccError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"fastpcc_gb300 error {code}: {msg}")
        self.code = code


def build(force: bool = False) -> str:
    from . import native_build
    return native_build.build(force=force)


def lib():
    """The loaded native library (raises if it has not been built)."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise FpccError(-4, f"native library missing: {LIB_PATH} (run fastpcc_gb300.build)")
            L = C.CDLL(LIB_PATH)
            i, u, f, i64, vp = C.c_int, C.c_uint, C.c_float, C.c_int64, C.c_void_p
            fpp = C.POINTER(C.POINTER(C.c_float))
            L.fpcc_create.argtypes = [C.POINTER(vp), i]
            L.fpcc_destroy.argtypes = [vp]
            L.fpcc_set_stream.argtypes = [vp, vp]
            L.fpcc_get_stream.argtypes = [vp]
            L.fpcc_get_stream.restype = vp
            L.fpcc_sync.argtypes = [vp]
            L.fpcc_last_error.restype = C.c_char_p
            L.fpcc_version.restype = C.c_char_p
            L.fpcc_launch_count.restype = i64
            L.fpcc_choose_nz.argtypes = [i, i, i, i]
            L.fpcc_max_block_len.restype = i
            L.fpcc_station_row_elems.argtypes = [i, i, i]
            L.fpcc_station_row_elems.restype = i64
            L.fpcc_station_row_bytes.argtypes = [i, i, i, i]
            L.fpcc_station_row_bytes.restype = i64
            L.fpcc_station_stage.argtypes = [vp, i, vp, i64, i, i, i, i, i, vp, i64]
            L.fpcc_station_stage_ex.argtypes = [vp, i, vp, i64, i, i, i, i, i, vp, i64, vp, i]
            L.fpcc_set_analytic_precision.argtypes = [vp, i]
            L.fpcc_energy_stage.argtypes = [vp, vp, i64, i, i, vp, i64]
            L.fpcc_pair_stage.argtypes = [vp, i, vp, i64, i, vp, i, i, i, i, i, f, vp, i64, vp, i64, vp]
            L.fpcc_host_batched.argtypes = [i, fpp, fpp, fpp, u, u, i, i, f, i, i]
            L.fpcc_host_plain.argtypes = [i, fpp, fpp, fpp, u, u, i, i, f, i, i]
            L.fpcc_allpairs_host.argtypes = [vp, i, vp, i, i, vp, i, i, i, f, i, i, vp]
            for name in ("pcc2_highlevel", "ccgn_highlevel", "cc1b_highlevel"):
                getattr(L, name).argtypes = [fpp, fpp, fpp, u, u, i, i]
            d = C.c_double
            L.fpcc_wpcc_host.argtypes = [fpp, fpp, fpp, u, u, i, i, d, d, u, i, d, i, i]
            L.fpcc_wpcc_plan_create.argtypes = [vp, C.POINTER(vp), u, i, i, d, d, u, i, d, i, i]
            L.fpcc_wpcc_plan_info.argtypes = [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i)]
            L.fpcc_wpcc_plan_destroy.argtypes = [vp]
            L.fpcc_wpcc_plan_set_band.argtypes = [vp, i, i]
            L.fpcc_wpcc_station_stage.argtypes = [vp, vp, vp, i64, i, vp, i]
            L.fpcc_wpcc_pair_stage.argtypes = [vp, vp, vp, i, vp, i, vp, i64]
            L.fpcc_wpcc_plan_set_lags.argtypes = [vp, i, i]
            L.fpcc_pair_stage_packed.argtypes = [vp, i, i, i, vp, i, i, f, i]
            L.fpcc_clip_rows.argtypes = [vp, vp, i64, i, i]
            L.fpcc_whiten_rows.argtypes = [vp, vp, i64, i, i, d, d, d]
            L.fpcc_prep_last_error.restype = C.c_char_p
            L.fpcc_stack.argtypes = [vp, i, vp, i64, i64, i, i, i, d, d, d, i, i, d, vp, i64]
            L.fpcc_station_stage_multi.argtypes = [vp, i, vp, i, i, i, vp, i64]
            L.fpcc_server_create.argtypes = [C.POINTER(vp), i, C.c_size_t, i]
            L.fpcc_server_set_format.argtypes = [vp, i]
            L.fpcc_server_set_nz_mode.argtypes = [vp, i]
            L.fpcc_autotune.argtypes = [vp, i, i, C.c_double, C.c_char_p]
            L.fpcc_autotune_load.argtypes = [C.c_char_p]
            L.fpcc_pair_form.argtypes = [i, i]
            L.fpcc_server_set_wavelet.argtypes = [vp, d, d, u, i, d, i]
            L.fpcc_server_destroy.argtypes = [vp]
            L.fpcc_server_register_output.argtypes = [vp, vp, C.c_size_t]
            L.fpcc_server_unregister_output.argtypes = [vp, vp]
            L.fpcc_put_station_window.argtypes = [vp, C.c_int32, C.c_int32, vp, i]
            L.fpcc_submit.argtypes = [vp, C.POINTER(Request)]
            L.fpcc_submit.restype = i64
            L.fpcc_submit_many.argtypes = [vp, C.POINTER(Request), i, C.POINTER(i64)]
            L.fpcc_server_offer_poisson.argtypes = [vp, C.POINTER(Request), i, C.c_double, C.c_uint64,
                                                    C.POINTER(i64)]
            L.fpcc_poll.argtypes = [vp, i64]
            L.fpcc_wait.argtypes = [vp, i64, C.c_double]
            L.fpcc_server_drain.argtypes = [vp]
            L.fpcc_server_get_stats.argtypes = [vp, C.POINTER(ServerStats)]
            L.fpcc_server_reset_stats.argtypes = [vp]
            L.cc1b_popcount_highlevel.argtypes = [C.POINTER(C.POINTER(C.c_int64)), fpp, fpp, u, u, i, i]
            _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != 0:
        raise FpccError(rc, lib().fpcc_last_error().decode(errors="replace"))


def launch_count() -> int:
    return int(lib().fpcc_launch_count())


def choose_nz(N: int, Lag1: int, Lag2: int, mode: int = NZ_FAST) -> int:
    nz = lib().fpcc_choose_nz(N, Lag1, Lag2, mode)
    if nz <= 0:
        raise FpccError(-4, f"no supported correlation length for N={N}, lags [{Lag1},{Lag2}]")
    return nz


PAIR_BLOCK, PAIR_TILED = 1, 2


def pair_form(Nz: int, form: int = 0) -> int:
    """Pair kernel used at padded length Nz (fpcc_pair_form); form > 0 selects it."""
    r = lib().fpcc_pair_form(Nz, form)
    if r < 0:
        raise FpccError(r, f"pair form {form} does not run Nz={Nz}")
    return r


def load_tuning(path: str) -> dict:
    """Loads an autotuner table into the library (fpcc_autotune_load) and returns it."""
    import json
    check(lib().fpcc_autotune_load(path.encode()))
    with open(path) as f:
        d = json.load(f)
    return {int(k): tuple(v) for k, v in d["lengths"].items()}


def lag_count(Lag1: int, Lag2: int) -> int:
    return abs(Lag2 - Lag1) + 1


def _rows(a, ctype=C.c_float):
    rows = (C.POINTER(ctype) * a.shape[0])()
    for k in range(a.shape[0]):
        rows[k] = a[k].ctypes.data_as(C.POINTER(ctype))
    return rows


def _windows(x1, x2):
    x1 = np.ascontiguousarray(np.atleast_2d(x1), dtype=np.float32)
    x2 = np.ascontiguousarray(np.atleast_2d(x2), dtype=np.float32)
    if x1.shape != x2.shape:
        raise ValueError("x1 and x2 must have the same shape (Tr, N)")
    return x1, x2, x1.shape[0], x1.shape[1]


def correlate(method, x1, x2, Lag1, Lag2, v=2.0, plain=False, nz_mode=NZ_FAST, fmt=F32):
    """Correlate same-index windows of two stations on the GPU (host arrays in and out)."""
    x1, x2, Tr, N = _windows(x1, x2)
    L = lag_count(Lag1, Lag2)
    y = np.zeros((Tr, L), np.float32)
    fn = lib().fpcc_host_plain if plain else lib().fpcc_host_batched
    check(fn(method, _rows(y), _rows(x1), _rows(x2), N, Tr, Lag1, Lag2, float(v), nz_mode, fmt))
    return y


# --- mirror of the reference method layer (src/FFTapps.c) -----------------------
def pcc2_set(x1, x2, Lag1, Lag2, **kw):
    """PCC at power 2 (reference pcc2_set, src/FFTapps.c:785)."""
    return correlate(PCC2, x1, x2, Lag1, Lag2, **kw)


def pcc1_set(x1, x2, Lag1, Lag2, **kw):
    """PCC at power 1 by direct lag sums (reference pcc1_set, src/FFTapps.c:611)."""
    return correlate(PCC1, x1, x2, Lag1, Lag2, v=1.0, **kw)


def pcc_set(x1, x2, v, Lag1, Lag2, **kw):
    """PCC at power v by direct lag sums, GPU normalisation 2(N-|lag|) (src/ccs_cuda.cu:452)."""
    return correlate(PCCV, x1, x2, Lag1, Lag2, v=v, **kw)


def ccgn_set(x1, x2, Lag1, Lag2, **kw):
    """Geometrically normalised cross-correlation (reference ccgn_set, src/FFTapps.c:883)."""
    return correlate(GNCC, x1, x2, Lag1, Lag2, v=0.0, **kw)


def cc1b_set(x1, x2, Lag1, Lag2, popcount=False, **kw):
    """1-bit GNCC (reference cc1b_set, src/FFTapps.c:980); popcount=True uses exact
    integer numerators from packed sign bits."""
    return correlate(CC1B_POPCOUNT if popcount else CC1B, x1, x2, Lag1, Lag2, v=0.0, **kw)


def wpcc_set(x1, x2, Lag1, Lag2, pmin, pmax, V=2, type=-3, op1=0.0, rule=AMP_D_REG, nz_mode=NZ_FAST):
    """Wavelet PCC (reference tspcc2_set, src/FFTapps.c:1076): pmin/pmax in samples,
    V voices per octave, type -1 Morlet / -2 complete Morlet / -3 complex Mexican hat."""
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.zeros((Tr, lag_count(Lag1, Lag2)), np.float32)
    check(lib().fpcc_wpcc_host(_rows(y), _rows(x1), _rows(x2), N, Tr, Lag1, Lag2, float(pmin), float(pmax),
                               V, type, float(op1), rule, nz_mode))
    return y


def cc1b_numerators(x1, x2, Lag1, Lag2):
    """Exact int64 numerators sum_n s1[n] s2[n+lag] of 1-bit GNCC."""
    x1, x2, Tr, N = _windows(x1, x2)
    num = np.zeros((Tr, lag_count(Lag1, Lag2)), np.int64)
    check(lib().cc1b_popcount_highlevel(_rows(num, C.c_int64), _rows(x1), _rows(x2), N, Tr, Lag1, Lag2))
    return num


def pcc2_highlevel(x1, x2, Lag1, Lag2):
    """The plain per-pair drop-in (one launch sequence per window) through its C symbol."""
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.zeros((Tr, lag_count(Lag1, Lag2)), np.float32)
    check(lib().pcc2_highlevel(_rows(y), _rows(x1), _rows(x2), N, Tr, Lag1, Lag2))
    return y


class Context:
    """A device context: its own CUDA stream and workspace (device pointers as ints)."""

    def __init__(self, device: int = 0):
        self._h = C.c_void_p()
        check(lib().fpcc_create(C.byref(self._h), device))

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().fpcc_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int | None):
        check(lib().fpcc_set_stream(self._h, C.c_void_p(stream_ptr or 0)))

    def stream(self) -> int:
        return int(lib().fpcc_get_stream(self._h) or 0)

    def sync(self):
        check(lib().fpcc_sync(self._h))

    def set_analytic_precision(self, mode):
        """ANALYTIC_F32, ANALYTIC_AUTO (FP64 for windows with zero runs) or ANALYTIC_F64."""
        check(lib().fpcc_set_analytic_precision(self._h, mode))

    def station_stage(self, method, d_x, ldx, nrows, N, Nz, fmt, rule, d_out, ldo):
        check(lib().fpcc_station_stage(self._h, method, C.c_void_p(d_x), ldx, nrows, N, Nz, fmt, rule,
                                       C.c_void_p(d_out), ldo))

    def stack(self, mode, d_y, ldy, K, L, ngroups, d_out, ldo, nu=2.0, pmin=0.0, pmax=0.0, V=4, type=-1,
              op1=0.0, ldg=None, ldj=None):
        """Stacks of ngroups groups of K traces into rows of d_out: STACK_LINEAR,
        STACK_PWS (phase-weighted) or STACK_TSPWS (time-scale phase-weighted;
        pmin/pmax in samples, V voices, wavelet type).  Trace j of group g starts
        at d_y + g*ldg + j*ldj floats (default: rows g*K + j of stride ldy)."""
        ldj = ldy if ldj is None else ldj
        ldg = K * ldy if ldg is None else ldg
        check(lib().fpcc_stack(self._h, mode, C.c_void_p(d_y), ldg, ldj, K, L, ngroups, float(nu), float(pmin),
                               float(pmax), V, type, float(op1), C.c_void_p(d_out), ldo))

    def station_stage_multi(self, method, rows, fmt, rule, d_out, ldo):
        """Station stage of windows of different lengths in shared launches:
        rows = [(d_x, N, Nz, f64)] ordered by (N, Nz); row r is written at
        d_out + r * ldo elements of the format."""
        class _Row(C.Structure):
            _fields_ = [("d_x", C.c_void_p), ("N", C.c_int32), ("Nz", C.c_int32), ("f64", C.c_int32),
                        ("pad", C.c_int32)]
        arr = (_Row * len(rows))(*[_Row(int(x), int(n), int(nz), int(f), 0) for (x, n, nz, f) in rows])
        check(lib().fpcc_station_stage_multi(self._h, method, C.addressof(arr), len(rows), fmt, rule,
                                             C.c_void_p(d_out), ldo))

    def energy_stage(self, d_x, ldx, nrows, N, d_E, ldE):
        check(lib().fpcc_energy_stage(self._h, C.c_void_p(d_x), ldx, nrows, N, C.c_void_p(d_E), ldE))

    def pair_stage(self, method, d_station, lds, fmt, d_pairs, npairs, N, Nz, Lag1, Lag2, v=0.0,
                   d_E=0, ldE=0, d_y=0, ldy=0, d_num=0):
        check(lib().fpcc_pair_stage(self._h, method, C.c_void_p(d_station), lds, fmt, C.c_void_p(d_pairs),
                                    npairs, N, Nz, Lag1, Lag2, float(v), C.c_void_p(d_E or 0), ldE,
                                    C.c_void_p(d_y or 0), ldy, C.c_void_p(d_num or 0)))

    def autotune(self, min_nz=512, max_nz=1 << 19, reuse=8.0, path=None) -> dict:
        """Times every usable padded length on this GPU, and both pair kernels where
        two run a length (fpcc_autotune); the table then drives NZ_TUNED and the
        faster kernel is selected.  Returns {Nz: (pair ns per correlation,
        station ns per window, kernel form or 0)}."""
        check(lib().fpcc_autotune(self._h, min_nz, max_nz, float(reuse), path.encode() if path else None))
        return load_tuning(path) if path else {}

    def pair_stage_packed(self, method, fmt, Nz, d_desc, npairs, maxL, v=0.0, numerators=False):
        """d_desc: device array of npairs PairDesc (lengths and lags per correlation)."""
        check(lib().fpcc_pair_stage_packed(self._h, method, fmt, Nz, C.c_void_p(d_desc), npairs, maxL, float(v),
                                           1 if numerators else 0))

    def allpairs_host(self, method, x, pairs, Lag1, Lag2, y, v=0.0, nz_mode=NZ_FAST, fmt=F32):
        """x: (nsta, N) float32 host array (pinned or pageable); pairs (npairs, 2) int32;
        y: (npairs, L) float32 host output."""
        assert x.dtype == np.float32 and x.flags.c_contiguous
        assert pairs.dtype == np.int32 and pairs.flags.c_contiguous
        assert y.dtype == np.float32 and y.flags.c_contiguous
        check(lib().fpcc_allpairs_host(self._h, method, C.c_void_p(x.ctypes.data), x.shape[0], x.shape[1],
                                       C.c_void_p(pairs.ctypes.data), pairs.shape[0], Lag1, Lag2, float(v),
                                       nz_mode, fmt, C.c_void_p(y.ctypes.data)))


class Server:
    """Continuous-batching correlation server (fpcc_server_* of the C ABI).

    Outputs are written into numpy arrays owned by the caller; keep them alive
    until the request completes (``wait``/``drain``)."""

    def __init__(self, device: int = 0, hbm_budget: int = 150 << 30, max_batch: int = 4096, fmt: int = F32,
                 wavelet: dict = None, nz_mode: int = NZ_FAST):
        """fmt: storage of cached phase spectra / phase signals (F32 or F16).
        wavelet: family of WPCC requests, keys pmin, pmax, V, type, op1, rule
        (as WpccPlan)."""
        self._h = C.c_void_p()
        check(lib().fpcc_server_create(C.byref(self._h), device, hbm_budget, max_batch))
        self._keep = {}
        try:
            if fmt != F32:
                check(lib().fpcc_server_set_format(self._h, fmt))
            if nz_mode != NZ_FAST:
                check(lib().fpcc_server_set_nz_mode(self._h, nz_mode))
            if wavelet is not None:
                w = dict(V=2, type=-3, op1=0.0, rule=AMP_D_REG)
                w.update(wavelet)
                check(lib().fpcc_server_set_wavelet(self._h, float(w["pmin"]), float(w["pmax"]), int(w["V"]),
                                                    int(w["type"]), float(w["op1"]), int(w["rule"])))
        except Exception:
            self.close()
            raise

    def close(self):
        if self._h:
            lib().fpcc_server_destroy(self._h)
            self._h = C.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def register_output(self, arr):
        """Lets results land in `arr` (a C-contiguous numpy array holding the
        requests' output rows) straight from the device (fpcc_server_register_output);
        keep `arr` alive until unregister_output or close."""
        assert arr.flags.c_contiguous
        check(lib().fpcc_server_register_output(self._h, arr.ctypes.data, arr.nbytes))
        self._keep[("out", arr.ctypes.data)] = arr

    def unregister_output(self, arr):
        check(lib().fpcc_server_unregister_output(self._h, arr.ctypes.data))
        self._keep.pop(("out", arr.ctypes.data), None)

    def put(self, sta: int, window: int, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        check(lib().fpcc_put_station_window(self._h, sta, window, x.ctypes.data, x.shape[0]))

    @staticmethod
    def request(method, sta1, sta2, window, Lag1, Lag2, out, v=0.0):
        r = Request(method, sta1, sta2, window, Lag1, Lag2, float(v), None, None)
        if method == CC1B_POPCOUNT:
            r.num = out.ctypes.data
        else:
            r.y = out.ctypes.data
        return r

    def submit(self, method, sta1, sta2, window, Lag1, Lag2, out, v=0.0) -> int:
        r = self.request(method, sta1, sta2, window, Lag1, Lag2, out, v)
        rid = int(lib().fpcc_submit(self._h, C.byref(r)))
        if rid < 0:
            check(rid)
        self._keep[rid] = out
        return rid

    @staticmethod
    def request_array(reqs):
        """A ctypes array of Request for submit_many (build once, submit many times)."""
        return (Request * len(reqs))(*reqs)

    def submit_many(self, reqs, outs=None, poisson_rate=None, seed=1, count=None):
        arr = reqs if isinstance(reqs, C.Array) else self.request_array(reqs)
        n = len(arr) if count is None else int(count)
        ids = np.zeros(n, np.int64)
        idp = ids.ctypes.data_as(C.POINTER(C.c_int64))
        if poisson_rate:
            rc = lib().fpcc_server_offer_poisson(self._h, arr, n, float(poisson_rate), seed, idp)
        else:
            rc = lib().fpcc_submit_many(self._h, arr, n, idp)
        check(rc)
        return ids

    def wait(self, rid: int, timeout: float = 0.0) -> int:
        st = lib().fpcc_wait(self._h, rid, float(timeout))
        if st < 0:
            check(st)
        self._keep.pop(rid, None)
        return st

    def drain(self):
        check(lib().fpcc_server_drain(self._h))
        self._keep = {k: v for k, v in self._keep.items() if isinstance(k, tuple)}   # registered outputs stay

    def stats(self) -> dict:
        s = ServerStats()
        check(lib().fpcc_server_get_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def reset_stats(self):
        check(lib().fpcc_server_reset_stats(self._h))


class WpccPlan:
    """Device-resident wavelet PCC plan (fpcc_wpcc_plan_* of the C ABI)."""

    def __init__(self, ctx, N, Lag1, Lag2, pmin, pmax, V=2, type=-3, op1=0.0, rule=AMP_D_REG, nz_mode=NZ_FAST):
        self._h = C.c_void_p()
        self.ctx = ctx
        check(lib().fpcc_wpcc_plan_create(ctx.handle, C.byref(self._h), N, Lag1, Lag2, float(pmin), float(pmax),
                                          V, type, float(op1), rule, nz_mode))
        nz, S, L = C.c_int(), C.c_int(), C.c_int()
        check(lib().fpcc_wpcc_plan_info(self._h, C.byref(nz), C.byref(S), C.byref(L)))
        self.Nz, self.S, self.L, self.N = nz.value, S.value, L.value, N

    def set_band(self, s_lo, s_hi):
        check(lib().fpcc_wpcc_plan_set_band(self._h, s_lo, s_hi))

    def set_lags(self, Lag1, Lag2):
        check(lib().fpcc_wpcc_plan_set_lags(self._h, Lag1, Lag2))
        self.L = lag_count(Lag1, Lag2)

    def station_stage(self, d_x, ldx, nrows, d_P, fmt=F32):
        check(lib().fpcc_wpcc_station_stage(self.ctx.handle, self._h, C.c_void_p(d_x), ldx, nrows,
                                            C.c_void_p(d_P), fmt))

    def pair_stage(self, d_P, d_pairs, npairs, d_y, ldy, fmt=F32):
        check(lib().fpcc_wpcc_pair_stage(self.ctx.handle, self._h, C.c_void_p(d_P), fmt, C.c_void_p(d_pairs),
                                         npairs, C.c_void_p(d_y), ldy))

    def close(self):
        if self._h:
            lib().fpcc_wpcc_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
