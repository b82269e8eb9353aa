"""ctypes front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` as the checker.  The product package never imports
this module.

Two libraries are wrapped:

* ``liboracle64.so`` — the FP64 restatement of the reference's methods
  (oracle64.c, each function citing the reference lines it follows) on an FP64
  DFT (fft64.c).  Built by ``make`` in this folder on any machine.
* ``_ref/libref_fastpcc.so`` — the reference's own CPU method layer
  (src/FFTapps.c and the src/FWTa wavelet files), compiled unmodified against the
  project's FFTW-API shim.  Built only where the reference sources are present;
  it pins the restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
AMP_F_REG, AMP_D_REG, AMP_PURE, AMP_THRESH, AMP_SUMTHR = 0, 1, 2, 3, 4

_lock = threading.Lock()
_lib = None
_ref = None

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_c128p = np.ctypeslib.ndpointer(np.complex128, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")


def reference_sources() -> str:
    """Folder holding the reference's src/: FPCC_REFSRC, else the REFSRC default of
    this folder's Makefile (the one place that names it)."""
    env = os.environ.get("FPCC_REFSRC")
    if env:
        return env
    with open(os.path.join(HERE, "Makefile")) as f:
        for line in f:
            if line.startswith("REFSRC") and "?=" in line:
                return line.split("?=", 1)[1].strip()
    return ""


def make_vars() -> list:
    """REFSRC for make when FPCC_REFSRC overrides the Makefile's default."""
    return [f"REFSRC={os.environ['FPCC_REFSRC']}"] if os.environ.get("FPCC_REFSRC") else []


def build(ref: bool = False) -> None:
    """Compile the oracle (and, when asked and present, the reference CPU path)."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle64.so", "libcpuref.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, *make_vars(), "ref"], check=True)


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = os.path.join(HERE, "liboracle64.so")
            if not os.path.exists(path):
                build()
            L = C.CDLL(path)
            u, i, d = C.c_uint, C.c_int, C.c_double
            L.orc_nz_rule.argtypes = [u, i, i]
            L.orc_nz_rule.restype = u
            L.orc_phase.argtypes = [_c128p, _f32p, u, i]
            L.orc_analytic.argtypes = [_c128p, _f32p, u]
            L.orc_pcc2_set.argtypes = [_f64p, _f32p, _f32p, u, u, i, i, u, i]
            L.orc_pccv_set.argtypes = [_f64p, _f32p, _f32p, u, u, d, i, i, i, i]
            L.orc_pccv_phase.argtypes = [_f64p, _c128p, _c128p, u, d, i, i, i]
            L.orc_gncc_set.argtypes = [_f64p, _f32p, _f32p, u, u, i, i]
            L.orc_cc1b_set.argtypes = [_f64p, _f32p, _f32p, u, u, i, i]
            L.orc_cc1b_num.argtypes = [_i64p, _f32p, _f32p, u, u, i, i]
            L.orc_wpcc_set.argtypes = [_f64p, _f32p, _f32p, u, u, i, i, d, d, u, i, d, i]
            L.orc_wpcc_band.argtypes = [_f64p, _f32p, _f32p, u, u, i, i, d, d, u, i, d, i, u, u]
            L.orc_wpcc_setup.argtypes = [u, i, i, d, d, u, i, d, C.POINTER(u), C.POINTER(d),
                                         C.POINTER(d), C.POINTER(u)]
            L.orc_wpcc_setup.restype = u
            L.orc_wavelet_family.argtypes = [i, u, u, u, d, d, _f64p,
                                             np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS"),
                                             np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS"),
                                             C.c_void_p]
            L.orc_wavelet_family.restype = u
            L.orc_stack.argtypes = [_f64p, _f32p, u, u, i, d, d, d, u, i, d]
            L.orc_stack_family.argtypes = [u, d, d, u, i, d, C.POINTER(d), C.POINTER(d), C.POINTER(u)]
            L.orc_stack_family.restype = u
            L.orc_cpsi.argtypes = [i, d]
            L.orc_cpsi.restype = d
            L.orc_cwt.argtypes = [_c128p, _f64p, u, u, np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS"),
                                  np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS"), _c128p]
            L.orc_icwt.argtypes = [_f64p, _c128p, u, u, u, d, _f64p,
                                   np.ctypeslib.ndpointer(np.uint32, flags="C_CONTIGUOUS"),
                                   np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS"), _c128p]
            _lib = L
    return _lib


def _windows(x1, x2):
    x1 = np.ascontiguousarray(np.atleast_2d(x1), dtype=np.float32)
    x2 = np.ascontiguousarray(np.atleast_2d(x2), dtype=np.float32)
    if x1.shape != x2.shape:
        raise ValueError("x1 and x2 must have the same shape (Tr, N)")
    return x1, x2, x1.shape[0], x1.shape[1]


def lag_count(Lag1: int, Lag2: int) -> int:
    return abs(Lag2 - Lag1) + 1


def nz_rule(N: int, Lag1: int, Lag2: int) -> int:
    return int(lib().orc_nz_rule(N, Lag1, Lag2))


def phase(x, rule=AMP_F_REG):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.shape[0], np.complex128)
    lib().orc_phase(y, x, x.shape[0], rule)
    return y


def analytic(x):
    x = np.ascontiguousarray(x, dtype=np.float32)
    y = np.empty(x.shape[0], np.complex128)
    lib().orc_analytic(y, x, x.shape[0])
    return y


def _check(rc, name):
    if rc != 0:
        raise RuntimeError(f"{name} returned {rc}")


def pcc2(x1, x2, Lag1, Lag2, Nz=0, rule=AMP_F_REG):
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.empty((Tr, lag_count(Lag1, Lag2)), np.float64)
    _check(lib().orc_pcc2_set(y, x1, x2, N, Tr, Lag1, Lag2, Nz, rule), "orc_pcc2_set")
    return y


def pccv(x1, x2, v, Lag1, Lag2, rule=AMP_F_REG, norm_gpu=False):
    if Lag1 > Lag2:
        raise ValueError("direct lag sums take Lag1 <= Lag2")
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.zeros((Tr, Lag2 - Lag1 + 1), np.float64)
    _check(lib().orc_pccv_set(y, x1, x2, N, Tr, float(v), Lag1, Lag2, rule, int(norm_gpu)), "orc_pccv_set")
    return y


def pcc1(x1, x2, Lag1, Lag2, rule=AMP_F_REG):
    """PCC at power 1 as src/FFTapps.c:611-783 computes it (divides by 2*(N-|lag|))."""
    return pccv(x1, x2, 1.0, Lag1, Lag2, rule=rule, norm_gpu=True)


def pccv_phase(p1, p2, v, Lag1, Lag2, norm_gpu=True):
    p1 = np.ascontiguousarray(p1, np.complex128)
    p2 = np.ascontiguousarray(p2, np.complex128)
    y = np.zeros(Lag2 - Lag1 + 1, np.float64)
    lib().orc_pccv_phase(y, p1, p2, p1.shape[0], float(v), Lag1, Lag2, int(norm_gpu))
    return y


def gncc(x1, x2, Lag1, Lag2):
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.empty((Tr, lag_count(Lag1, Lag2)), np.float64)
    _check(lib().orc_gncc_set(y, x1, x2, N, Tr, Lag1, Lag2), "orc_gncc_set")
    return y


def cc1b(x1, x2, Lag1, Lag2):
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.empty((Tr, lag_count(Lag1, Lag2)), np.float64)
    _check(lib().orc_cc1b_set(y, x1, x2, N, Tr, Lag1, Lag2), "orc_cc1b_set")
    return y


def cc1b_num(x1, x2, Lag1, Lag2):
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.empty((Tr, lag_count(Lag1, Lag2)), np.int64)
    _check(lib().orc_cc1b_num(y, x1, x2, N, Tr, Lag1, Lag2), "orc_cc1b_num")
    return y


def wpcc_setup(N, Lag1, Lag2, pmin, pmax, V, wtype, op1=0.0):
    Nz, J = C.c_uint(0), C.c_uint(0)
    s0, op = C.c_double(0), C.c_double(0)
    S = lib().orc_wpcc_setup(N, Lag1, Lag2, pmin, pmax, V, wtype, op1, C.byref(Nz), C.byref(s0),
                             C.byref(op), C.byref(J))
    if S == 0:
        raise ValueError("invalid WPCC parameters")
    return dict(S=int(S), Nz=int(Nz.value), s0=float(s0.value), op1=float(op.value), J=int(J.value))


def wavelet_family(wtype, J, V, Nz, s0, op1):
    S = J * V
    scale = np.empty(S, np.float64)
    Ls = np.empty(S, np.uint32)
    center = np.empty(S, np.int32)
    n = lib().orc_wavelet_family(wtype, J, V, Nz, s0, op1, scale, Ls, center, None)
    taps = np.empty(n, np.complex128)
    lib().orc_wavelet_family(wtype, J, V, Nz, s0, op1, scale, Ls, center, taps.ctypes.data)
    return scale, Ls, center, taps


def wpcc(x1, x2, Lag1, Lag2, pmin, pmax, V=2, wtype=-3, op1=0.0, rule=AMP_D_REG):
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.empty((Tr, abs(Lag2 - Lag1 + 1)), np.float64)
    _check(lib().orc_wpcc_set(y, x1, x2, N, Tr, Lag1, Lag2, pmin, pmax, V, wtype, op1, rule), "orc_wpcc_set")
    return y


def wpcc_band(x1, x2, Lag1, Lag2, pmin, pmax, s_lo, s_hi, V=2, wtype=-3, op1=0.0, rule=AMP_D_REG):
    """WPCC accumulating only scales s_lo <= s < s_hi (per-band error diagnostics)."""
    x1, x2, Tr, N = _windows(x1, x2)
    y = np.empty((Tr, abs(Lag2 - Lag1 + 1)), np.float64)
    _check(lib().orc_wpcc_band(y, x1, x2, N, Tr, Lag1, Lag2, pmin, pmax, V, wtype, op1, rule, s_lo, s_hi),
           "orc_wpcc_band")
    return y


STACK_LINEAR, STACK_PWS, STACK_TSPWS = 0, 1, 2


def stack(y, mode, nu=2.0, pmin=0.0, pmax=0.0, V=4, wtype=-1, op1=0.0):
    """Stack of the rows of y (K, L): linear mean, time-domain phase-weighted, or
    time-scale phase-weighted (oracle64.c orc_stack).  Returns float64 (L,)."""
    y = np.ascontiguousarray(y, np.float32)
    K, L = y.shape
    out = np.empty(L, np.float64)
    _check(lib().orc_stack(out, y, K, L, mode, nu, pmin, pmax, V, wtype, op1), "orc_stack")
    return out


def stack_family(L, pmin, pmax, V, wtype, op1=0.0):
    """(S, J, s0, op1, scale, Ls, center, taps, cpsi) of a ts-PWS stack over L samples."""
    s0, op, J = C.c_double(0), C.c_double(0), C.c_uint(0)
    S = lib().orc_stack_family(L, pmin, pmax, V, wtype, op1, C.byref(s0), C.byref(op), C.byref(J))
    if S == 0:
        raise ValueError("invalid stack parameters")
    scale, Ls, center, taps = wavelet_family(wtype, J.value, V, L, s0.value, op.value)
    return dict(S=int(S), J=int(J.value), s0=float(s0.value), op1=float(op.value), scale=scale, Ls=Ls,
                center=center, taps=taps, cpsi=float(lib().orc_cpsi(wtype, op.value)))


def cwt(x, fam):
    """CWT rows (S, L) of a real trace with a stack_family family."""
    x = np.ascontiguousarray(x, np.float64)
    W = np.empty((fam["S"], x.size), np.complex128)
    lib().orc_cwt(W, x, x.size, fam["S"], fam["Ls"], fam["center"], fam["taps"])
    return W


def icwt(W, fam, V):
    W = np.ascontiguousarray(W, np.complex128)
    L = W.shape[1]
    x = np.empty(L, np.float64)
    lib().orc_icwt(x, W, L, fam["S"], V, fam["cpsi"], fam["scale"], fam["Ls"], fam["center"], fam["taps"])
    return x


# ---------------------------------------------------------------------------
# The reference's own CPU path (oracle/_ref), where it was built.

def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libref_fastpcc.so"))


def ref():
    global _ref
    with _lock:
        if _ref is None:
            L = C.CDLL(os.path.join(HERE, "_ref", "libref_fastpcc.so"))
            fpp = C.POINTER(C.POINTER(C.c_float))
            u, i, d = C.c_uint, C.c_int, C.c_double
            for name in ("pcc2_set", "ccgn_set", "cc1b_set"):
                getattr(L, name).argtypes = [fpp, fpp, fpp, u, u, i, i]
            L.pcc1_set.argtypes = [fpp, fpp, fpp, i, u, i, i]
            L.pcc_set.argtypes = [fpp, fpp, fpp, i, u, d, i, i]
            L.tspcc2_set.argtypes = [fpp, fpp, fpp, u, u, i, i, d, d, u, i, d]
            _ref = L
    return _ref


def _rows(a):
    rows = (C.POINTER(C.c_float) * a.shape[0])()
    for k in range(a.shape[0]):
        rows[k] = a[k].ctypes.data_as(C.POINTER(C.c_float))
    return rows


def ref_call(method, x1, x2, Lag1, Lag2, **kw):
    """Run one of the reference's ``*_set`` functions on float32 windows.

    method: 'pcc2' | 'pcc1' | 'pcc' (kw v=) | 'ccgn' | 'cc1b' | 'wpcc'
    (kw pmin, pmax, V, wtype, op1).  Returns float32 (Tr, L)."""
    x1, x2, Tr, N = _windows(x1, x2)
    x1 = x1.copy()
    x2 = x2.copy()
    L = abs(Lag2 - Lag1) + 1
    # The reference's lag copy loops run to -min(Lag1,Lag2) even when that exceeds L
    # (src/FFTapps.c:351,368,855,1223 with Lag2 < 0), so its rows get slack here.
    slack = max(0, -min(Lag1, Lag2))
    y = np.zeros((Tr, L + slack), np.float32)
    R = ref()
    args = (_rows(y), _rows(x1), _rows(x2))
    if method == "pcc2":
        rc = R.pcc2_set(*args, N, Tr, Lag1, Lag2)
    elif method == "pcc1":
        rc = R.pcc1_set(*args, N, Tr, Lag1, Lag2)
    elif method == "pcc":
        rc = R.pcc_set(*args, N, Tr, float(kw["v"]), Lag1, Lag2)
    elif method == "ccgn":
        rc = R.ccgn_set(*args, N, Tr, Lag1, Lag2)
    elif method == "cc1b":
        rc = R.cc1b_set(*args, N, Tr, Lag1, Lag2)
    elif method == "wpcc":
        rc = R.tspcc2_set(*args, N, Tr, Lag1, Lag2, kw["pmin"], kw["pmax"], kw.get("V", 2),
                          kw.get("wtype", -3), kw.get("op1", 0.0))
    else:
        raise ValueError(method)
    if rc != 0:
        raise RuntimeError(f"reference {method}_set returned {rc}")
    return np.ascontiguousarray(y[:, :L])


def relerr(y, y64):
    """max_l |y - y64| / max_l |y64| per row (the error metric of the parity tests)."""
    y = np.atleast_2d(np.asarray(y, np.float64))
    y64 = np.atleast_2d(np.asarray(y64, np.float64))
    return np.max(np.abs(y - y64), axis=1) / np.max(np.abs(y64), axis=1)
