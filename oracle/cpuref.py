"""CPU restatement of the reference's method layer in the reference's own
precision, for the timed CPU baseline.

TEST INFRASTRUCTURE ONLY: the CPU legs of ``bench.py`` (``cpu_baseline`` and
``--impl reference``) time it, and tests/test_cpuref.py checks it against the
FP64 oracle.  The product never imports it.

The reference computes every correlation per pair and window on the host with
FFTW and OpenMP.  This module follows its steps and precisions, with scipy's
FFT (pocketfft, all host threads) in place of FFTW; the reference's own sources
do not travel to the machine that runs the benchmark, so this is a port:

* ``pcc2_set``  src/FFTapps.c:785-881: single precision.  Per window and
  station: r2c DFT_N, analytic mask with 1/N (:104-124), c2c inverse DFT_N,
  AmpNormf (:178-205), zero pad to Nz = 2^ceil(log2(N+M)), DFT_Nz; then
  conj(X1) X2, inverse DFT_Nz, real part times 1/(Nz N) at the lags: seven
  transforms per correlation.
* ``ccgn_set``  :883-978 with cc_lowlevel :338-353 and gn_lowlevel :372-399:
  double precision; r2c DFT_Nz of both traces, c2r of conj(X1) X2 over Nz, each
  lag divided by sqrt(E1 E2) of the overlap energies (prefix sums here, the
  reference's running sums there).
* ``cc1b_set``  :980-1073: single precision; signs x1 >= 0 and x2 > 0 (:1037,
  :1042), r2c / c2r DFT_Nz, each lag divided by its overlap count.
* ``pcc1_set``  :611-783 (CPU branch): single-precision analytic signals and
  AmpNormf, then pcc1f_lowlevel (:251-278) with the station-2 phase first:
  float square roots, double sums (cpuref.c, OpenMP over windows and lags).
"""
from __future__ import annotations

import ctypes as C
import math
import os
import threading

import numpy as np
import scipy.fft as sfft

HERE = os.path.dirname(os.path.abspath(__file__))
_lock = threading.Lock()
_lib = None


def threads() -> int:
    return os.cpu_count() or 1


def cpu_model() -> str:
    """CPU model string of this host (first 'model name' / 'CPU part' style line)."""
    try:
        with open("/proc/cpuinfo") as f:
            text = f.read()
    except OSError:
        return "unknown"
    for key in ("model name", "Model Name", "Hardware"):
        for line in text.splitlines():
            if line.startswith(key):
                return line.split(":", 1)[1].strip()
    parts = sorted({line.split(":", 1)[1].strip() for line in text.splitlines() if line.startswith("CPU part")})
    impl = sorted({line.split(":", 1)[1].strip() for line in text.splitlines() if line.startswith("CPU implementer")})
    if parts:
        return f"CPU implementer {','.join(impl)} part {','.join(parts)}"
    return "unknown"


def _cpulib():
    global _lib
    with _lock:
        if _lib is None:
            path = os.path.join(HERE, "libcpuref.so")
            if not os.path.exists(path):
                from oracle import oracle as O
                O.build()
            L = C.CDLL(path)
            f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
            L.cpu_pcc1f_set.argtypes = [f32p, f32p, f32p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int64]
            L.cpu_pcc1f_set.restype = None
            _lib = L
    return _lib


def _lags(Lag1, Lag2):
    return (Lag1, Lag2 - Lag1 + 1) if Lag2 >= Lag1 else (Lag2, Lag1 - Lag2 + 1)


def nz_rule(N, Lag1, Lag2):
    """Nz = 2^ceil(log2(N + M)) (src/FFTapps.c:805)."""
    M = max(abs(Lag1), abs(Lag2))
    if M >= N:
        raise ValueError("lags must be below N")
    return 1 << math.ceil(math.log2(N + M))


def _pick(out, Nz, Lag1, Lag2):
    """Lags lag0 .. lag0+L-1 of circular correlation rows (index lag mod Nz)."""
    lag0, L = _lags(Lag1, Lag2)
    idx = (lag0 + np.arange(L)) % Nz
    return out[:, idx]


def analytic_f32(x, workers=None):
    """AnalyticSignal_plan_float (:104-124) in single precision: (Tr, N) -> complex64."""
    workers = workers or threads()
    Tr, N = x.shape
    X = sfft.rfft(x.astype(np.float32, copy=False), axis=1, workers=workers)
    full = np.zeros((Tr, N), np.complex64)
    h = (N + 1) >> 1
    full[:, 0] = X[:, 0]
    full[:, 1:h] = 2.0 * X[:, 1:h]
    if N % 2 == 0:
        full[:, N // 2] = X[:, N // 2]
    return sfft.ifft(full, axis=1, workers=workers)   # the 1/N of the mask


def ampnormf(a):
    """AmpNormf (:178-205): x / (|x| + 1e-6 max|x|), zero where that factor is not normal."""
    m = np.abs(a)
    eps = (1e-6 * np.sqrt(np.max(m * m, axis=1, keepdims=True).astype(np.float64))).astype(np.float32)
    with np.errstate(divide="ignore", over="ignore", invalid="ignore"):
        f = (np.float32(1.0) / (m + eps)).astype(np.float32)
    ok = np.isfinite(f) & (f >= np.finfo(np.float32).tiny)
    return np.where(ok, a * f, np.complex64(0)).astype(np.complex64)


def pcc2_set(x1, x2, Lag1, Lag2, workers=None):
    workers = workers or threads()
    Tr, N = x1.shape
    Nz = nz_rule(N, Lag1, Lag2)

    def spectrum(x):
        a = ampnormf(analytic_f32(x, workers))
        z = np.zeros((Tr, Nz), np.complex64)
        z[:, :N] = a
        return sfft.fft(z, axis=1, workers=workers)

    X1, X2 = spectrum(x1), spectrum(x2)
    out = sfft.ifft(np.conj(X1) * X2, axis=1, workers=workers)   # carries 1/Nz
    return (_pick(out.real, Nz, Lag1, Lag2) * np.float32(1.0 / N)).astype(np.float32)


def _overlap_norms(x1, x2, lags):
    """sqrt(E1 E2) over the overlap of every lag (double): E from prefix sums."""
    N = x1.shape[1]
    c1 = np.concatenate([np.zeros((x1.shape[0], 1)), np.cumsum(x1 * x1, axis=1)], axis=1)
    c2 = np.concatenate([np.zeros((x2.shape[0], 1)), np.cumsum(x2 * x2, axis=1)], axis=1)
    pos = lags > 0
    n1lo = np.where(pos, 0, -lags)
    n1hi = np.where(pos, N - lags, N)
    n2lo = np.where(pos, lags, 0)
    n2hi = np.where(pos, N, N + lags)
    e1 = c1[:, n1hi] - c1[:, n1lo]
    e2 = c2[:, n2hi] - c2[:, n2lo]
    return np.sqrt(e1 * e2)


def ccgn_set(x1, x2, Lag1, Lag2, workers=None):
    workers = workers or threads()
    Tr, N = x1.shape
    Nz = nz_rule(N, Lag1, Lag2)
    a = x1.astype(np.float64)
    b = x2.astype(np.float64)
    F1 = sfft.rfft(a, n=Nz, axis=1, workers=workers)
    F2 = sfft.rfft(b, n=Nz, axis=1, workers=workers)
    out = sfft.irfft(np.conj(F1) * F2, n=Nz, axis=1, workers=workers)   # carries 1/Nz
    lag0, L = _lags(Lag1, Lag2)
    y = _pick(out, Nz, Lag1, Lag2) / _overlap_norms(a, b, lag0 + np.arange(L))
    return y.astype(np.float32)


def cc1b_set(x1, x2, Lag1, Lag2, workers=None):
    workers = workers or threads()
    Tr, N = x1.shape
    Nz = nz_rule(N, Lag1, Lag2)
    s1 = np.where(x1 >= 0, np.float32(1), np.float32(-1))
    s2 = np.where(x2 > 0, np.float32(1), np.float32(-1))
    F1 = sfft.rfft(s1, n=Nz, axis=1, workers=workers)
    F2 = sfft.rfft(s2, n=Nz, axis=1, workers=workers)
    out = sfft.irfft(np.conj(F1) * F2, n=Nz, axis=1, workers=workers)
    lag0, L = _lags(Lag1, Lag2)
    cnt = (N - np.abs(lag0 + np.arange(L))).astype(np.float64)
    return (_pick(out, Nz, Lag1, Lag2) / cnt).astype(np.float32)


def pcc1_set(x1, x2, Lag1, Lag2, workers=None):
    if Lag1 > Lag2:
        raise ValueError("direct lag sums take Lag1 <= Lag2")
    workers = workers or threads()
    Tr, N = x1.shape
    p1 = np.ascontiguousarray(ampnormf(analytic_f32(x1, workers))).view(np.float32)
    p2 = np.ascontiguousarray(ampnormf(analytic_f32(x2, workers))).view(np.float32)
    L = Lag2 - Lag1 + 1
    y = np.zeros((Tr, L), np.float32)
    _cpulib().cpu_pcc1f_set(y, p1.reshape(-1), p2.reshape(-1), N, Tr, Lag1, Lag2, L)
    return y


METHODS = {"pcc2": pcc2_set, "gncc": ccgn_set, "cc1b": cc1b_set, "pcc1": pcc1_set}
