"""Seeded synthetic station windows for the benchmark and parity workloads.

The reference benchmarks on real GEOSCOPE records; the workloads here are seeded
synthetic stand-ins with the same shapes: each station window is white Gaussian
noise (sigma = 1) plus a shared component — independent Gaussian noise through a
4-pole (order-2 band-pass) Butterworth filter, run causally after a 4096-sample
burn-in and scaled to a standard deviation of ``snr`` — that reaches each station
with its own delay.  Every window draws from its own PCG64 stream seeded by
(workload tag, station, window), so any subset regenerates bit-identically.
"""
from __future__ import annotations

import hashlib

import numpy as np

BURN_IN = 4096


def _seed(*parts) -> int:
    h = hashlib.sha256("/".join(str(p) for p in parts).encode()).digest()
    return int.from_bytes(h[:8], "little")


def _shared(tag, window, n_total, fs, band, snr):
    from scipy import signal

    rng = np.random.Generator(np.random.PCG64(_seed(tag, "shared", window)))
    sos = signal.butter(2, band, btype="bandpass", fs=fs, output="sos")
    s = signal.sosfilt(sos, rng.standard_normal(n_total + BURN_IN))[BURN_IN:]
    return s * (snr / s.std())


def stations(tag: str, n_stations: int, n_windows: int, N: int, delays, fs: float,
             band=(0.05, 2.0), snr: float = 0.3) -> np.ndarray:
    """Return float32 array (n_stations, n_windows, N).

    ``delays[k]`` is station k's delay in samples (x_k[n] = noise + s[n - d_k])."""
    delays = np.asarray(delays, dtype=np.int64)
    assert delays.shape == (n_stations,)
    dmax = int(np.abs(delays).max()) if n_stations else 0
    out = np.empty((n_stations, n_windows, N), np.float32)
    for w in range(n_windows):
        s = _shared(tag, w, N + 2 * dmax, fs, band, snr)
        for k in range(n_stations):
            rng = np.random.Generator(np.random.PCG64(_seed(tag, "noise", k, w)))
            d = int(delays[k])
            out[k, w] = (rng.standard_normal(N) + s[dmax - d: dmax - d + N]).astype(np.float32)
    return out


def plain_pair(N=36000, n_windows=24, delay=150, fs=10.0, band=(0.05, 2.0), snr=0.3,
               tag="plain-pair"):
    """Stations A and B; B carries the shared component delayed by ``delay``.

    Default sizes: 24 windows of 36,000 samples (1 h at 10 Hz), lags +-3000."""
    x = stations(tag, 2, n_windows, N, [0, delay], fs, band, snr)
    return x[0], x[1]


def all_pairs(n_stations=64, n_windows=48, N=18000, max_delay=750, fs=10.0,
              band=(0.05, 2.0), snr=0.3, tag="all-pairs"):
    """64 stations x 48 windows x 18,000 samples; station delays U[-750, 750] so pair
    delays fall within +-1500 samples."""
    rng = np.random.Generator(np.random.PCG64(_seed(tag, "delays")))
    delays = rng.integers(-max_delay, max_delay + 1, size=n_stations)
    return stations(tag, n_stations, n_windows, N, delays, fs, band, snr), delays


def wavelet_pairs(n_pairs=16, n_windows=24, N=65536, fs=20.0, band=(0.02, 5.0), snr=0.3,
                  max_delay=1500, tag="wavelet-pairs"):
    """16 disjoint station pairs x 24 windows of 65,536 samples at 20 Hz."""
    rng = np.random.Generator(np.random.PCG64(_seed(tag, "delays")))
    d = rng.integers(-max_delay, max_delay + 1, size=n_pairs)
    a = np.empty((n_pairs, n_windows, N), np.float32)
    b = np.empty((n_pairs, n_windows, N), np.float32)
    for p in range(n_pairs):
        x = stations(f"{tag}/{p}", 2, n_windows, N, [0, int(d[p])], fs, band, snr)
        a[p], b[p] = x[0], x[1]
    return a, b, d


def gaps(x: np.ndarray, frac=0.05, lo=50, hi=2000, seed_tag="gaps") -> np.ndarray:
    """Zero about ``frac`` of the samples of a 1-D trace in gaps of U[lo, hi] samples."""
    x = x.copy()
    N = x.shape[0]
    rng = np.random.Generator(np.random.PCG64(_seed(seed_tag, N)))
    target = int(frac * N)
    zeroed = 0
    while zeroed < target:
        g = int(rng.integers(lo, hi + 1))
        g = min(g, target - zeroed) if target - zeroed >= lo else target - zeroed
        s = int(rng.integers(0, max(1, N - g)))
        x[s:s + g] = 0
        zeroed += g
    return x


def uneven_windows(lengths, n_stations, fs=10.0, band=(0.05, 2.0), snr=0.3, max_delay=1500, gap_frac=0.0,
                   tag="uneven"):
    """One window per entry of ``lengths`` shared by all stations: a list of
    float32 arrays (n_stations, lengths[w]); with ``gap_frac`` > 0 each trace has
    that fraction of its samples zeroed in gaps of 50-2000 samples."""
    rng = np.random.Generator(np.random.PCG64(_seed(tag, "delays")))
    delays = rng.integers(-max_delay, max_delay + 1, size=n_stations)
    out = []
    for w, N in enumerate(lengths):
        N = int(N)
        d = np.clip(delays, -(N // 4), N // 4)
        x = stations(f"{tag}/{w}", n_stations, 1, N, d, fs, band, snr)[:, 0]
        if gap_frac > 0:
            for k in range(n_stations):
                x[k] = gaps(x[k], frac=gap_frac, seed_tag=f"{tag}/gaps/{w}/{k}")
        out.append(x)
    return out


def mixed_requests(n_req, n_stations, lengths, mix, seed, lag_lo=0.01, lag_hi=0.10):
    """Requests (method, station 1, station 2, window, Lag1, Lag2): a random
    station pair, a window drawn uniformly, symmetric lags of half-width
    U[lag_lo, lag_hi] x the window length, and the method drawn from ``mix``
    ({method: probability})."""
    rng = np.random.Generator(np.random.PCG64(_seed("mixed-requests", seed)))
    methods = list(mix)
    p = np.asarray([mix[m] for m in methods], np.float64)
    p /= p.sum()
    out = []
    for _ in range(n_req):
        w = int(rng.integers(0, len(lengths)))
        N = int(lengths[w])
        s1, s2 = rng.choice(n_stations, 2, replace=False)
        M = max(1, min(N - 1, int(rng.uniform(lag_lo, lag_hi) * N)))
        out.append((int(methods[rng.choice(len(methods), p=p)]), int(s1), int(s2), w, -M, M))
    return out
