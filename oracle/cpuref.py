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
* ``wpcc_set``  tspcc2_set :1076-1255 (CPU branch): double precision, 4S+3
  transforms of the padded length per correlation; the wavelet family comes
  from the oracle's restatement of CreateWaveletFamily.

Windows are spread over the host threads, each with single-threaded FFTs, as
the reference's OpenMP loops over windows.
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
    arm = {"0xd4f": "Arm Neoverse V2", "0xd40": "Arm Neoverse V1", "0xd0c": "Arm Neoverse N1",
           "0xd49": "Arm Neoverse N2", "0xd8e": "Arm Neoverse N3", "0xd84": "Arm Neoverse V3"}
    if parts:
        names = [arm.get(p, f"part {p}") for p in parts] if impl == ["0x41"] else [f"part {p}" for p in parts]
        return f"{', '.join(names)} (CPU implementer {','.join(impl)})"
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


_pool = None


def _rows_in_parallel(fn, x1, x2, Lag1, Lag2):
    """fn over row blocks of (x1, x2) on all host threads, one block per thread with
    single-threaded FFTs (the reference's OpenMP loop over windows); numpy and
    scipy release the GIL inside their kernels."""
    global _pool
    n = threads()
    Tr = x1.shape[0]
    if n == 1 or Tr < 2:
        return fn(x1, x2, Lag1, Lag2, 1)
    import concurrent.futures as cf
    with _lock:
        if _pool is None:
            _pool = cf.ThreadPoolExecutor(max_workers=n)
    cuts = np.linspace(0, Tr, min(n, Tr) + 1).astype(int)
    futs = [_pool.submit(fn, x1[lo:hi], x2[lo:hi], Lag1, Lag2, 1) for lo, hi in zip(cuts[:-1], cuts[1:]) if hi > lo]
    return np.concatenate([f.result() for f in futs])


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
    if workers is None:
        return _rows_in_parallel(pcc2_set, x1, x2, Lag1, Lag2)
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
    if workers is None:
        return _rows_in_parallel(ccgn_set, x1, x2, Lag1, Lag2)
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
    if workers is None:
        return _rows_in_parallel(cc1b_set, x1, x2, Lag1, Lag2)
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


_family = {}


def _wavelet_spectra(N, Lag1, Lag2, pmin, pmax, V, wtype, op1):
    """Padded length, scales, Ls0, C and the S wavelet spectra (FP64) of
    src/FFTapps.c:1087-1147, from the oracle's restatement of the family."""
    key = (N, Lag1, Lag2, pmin, pmax, V, wtype, op1)
    with _lock:
        if key in _family:
            return _family[key]
    from oracle import oracle as O
    st = O.wpcc_setup(N, Lag1, Lag2, pmin, pmax, V, wtype, op1)
    M = max(abs(Lag1), abs(Lag2))
    Nz0 = 1 << math.ceil(math.log2(N + M))
    scale, Ls, center, taps = O.wavelet_family(wtype, st["J"], V, Nz0, st["s0"], st["op1"])
    Nz, S = st["Nz"], st["S"]
    fw = np.zeros((S, Nz), np.complex128)
    off = 0
    for k in range(S):
        c, l = int(center[k]), int(Ls[k])
        t = taps[off:off + l]
        fw[k, :l - c] = t[c:]
        if c:
            fw[k, Nz - c:] = t[:c]
        off += l
    fw = sfft.fft(fw, axis=1, workers=threads())
    C = 1.0 / (float(np.sum(1.0 / scale)) * N)
    fam = (Nz, scale, int(Ls[-1]), C, fw)
    with _lock:
        _family[key] = fam
    return fam


def _ampnorm(a):
    """AmpNorm (src/FFTapps.c:147-175): x / sqrt(|x|^2 + 1e-6 max|x|^2), double."""
    m2 = a.real * a.real + a.imag * a.imag
    eps = 1e-6 * np.max(m2, axis=-1, keepdims=True)
    with np.errstate(divide="ignore", invalid="ignore"):
        f = 1.0 / np.sqrt(m2 + eps)
    return np.where(np.isfinite(f), a * f, 0)


def wpcc_set(x1, x2, Lag1, Lag2, pmin, pmax, V=2, wtype=-3, op1=0.0, workers=None):
    """tspcc2_set (src/FFTapps.c:1076-1255), CPU path, double precision: traces at
    offset Ls0 scaled by 1/Nz, DFT; per scale the band IDFT(X W_s), AmpNorm, DFT;
    sum_s conj(P1_s) P2_s / (scale_s Nz), IDFT; C Re(.) at the lags."""
    if workers is None:
        return _rows_in_parallel(lambda a, b, l1, l2, w: wpcc_set(a, b, l1, l2, pmin, pmax, V, wtype, op1, w),
                                 x1, x2, Lag1, Lag2)
    Tr, N = x1.shape
    Nz, scale, Ls0, Cc, fw = _wavelet_spectra(N, Lag1, Lag2, pmin, pmax, V, wtype, op1)
    S = fw.shape[0]
    lag0, L = _lags(Lag1, Lag2)
    L = abs(Lag2 - Lag1 + 1)   # :1084
    y = np.zeros((Tr, L), np.float32)
    idx = (lag0 + np.arange(L)) % Nz
    for tr in range(Tr):
        X = []
        for x in (x1[tr], x2[tr]):
            z = np.zeros(Nz, np.complex128)
            z[Ls0:Ls0 + N] = x.astype(np.float64) / Nz
            X.append(sfft.fft(z, workers=workers))
        acc = np.zeros(Nz, np.complex128)
        for s0 in range(0, S, 8):
            fs = fw[s0:s0 + 8]
            P1 = sfft.fft(_ampnorm(sfft.ifft(X[0][None] * fs, axis=1, workers=workers)), axis=1, workers=workers)
            P2 = sfft.fft(_ampnorm(sfft.ifft(X[1][None] * fs, axis=1, workers=workers)), axis=1, workers=workers)
            w = 1.0 / (scale[s0:s0 + 8] * Nz)
            acc += np.sum(w[:, None] * np.conj(P1) * P2, axis=0)
        out = sfft.ifft(acc, workers=workers) * Nz
        y[tr] = (Cc * out.real[idx]).astype(np.float32)
    return y


METHODS = {"pcc2": pcc2_set, "gncc": ccgn_set, "cc1b": cc1b_set, "pcc1": pcc1_set}
