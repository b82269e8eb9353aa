"""Golden fixture of the stacking consumer: ts-PWS computed on the reference's
own wavelet library, and its CWT / inverse CWT of one trace.

Run in a container that holds the reference: ``make -C oracle wt`` builds
oracle/_ref/libref_wt.so from src/FWTa (CreateWaveletFamily,
complex_1D_wavelet_dec, Re_complex_1D_wavelet_rec, unmodified) with the harness
oracle/ref_wt.c; the stacks' inputs are seeded synthetic correlation traces
(a band-limited pulse at a causal and an acausal lag with per-trace amplitude
and jitter, plus noise), stored with the outputs as ``golden_stack.npz``.

    python tests/golden/make_stack_golden.py
"""
import ctypes as C
import os
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

# (L, K, wavelet type, V, pmin, pmax, nu) - pmin/pmax in samples
CASES = [(1001, 24, -1, 4, 8.0, 200.0, 2.0),
         (800, 16, -3, 2, 10.0, 120.0, 1.0),
         (1501, 20, -2, 3, 12.0, 300.0, 2.0)]


def traces(L, K, seed):
    rng = np.random.default_rng(seed)
    t = np.arange(L) - L // 2
    out = np.empty((K, L), np.float32)
    for j in range(K):
        y = 0.6 * rng.standard_normal(L)
        for lag, amp in ((L // 5, 1.0), (-L // 5, 0.7)):
            d = t - lag - rng.integers(-2, 3)
            y += amp * (0.5 + rng.random()) * np.exp(-0.5 * (d / 12.0) ** 2) * np.cos(2 * np.pi * d / 40.0)
        out[j] = y
    return out


def main():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), *O.make_vars(), "wt"], check=True)
    R = C.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_wt.so"))
    R.ref_wt_pair.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint, C.c_int, C.c_uint, C.c_uint,
                              C.c_double, C.c_double]
    R.ref_wt_tspws.argtypes = [C.c_void_p, C.c_void_p, C.c_uint, C.c_uint, C.c_double, C.c_int, C.c_uint,
                               C.c_uint, C.c_double, C.c_double]
    rec = {"cases": np.array(CASES, np.float64)}
    for i, (L, K, wt, V, pmin, pmax, nu) in enumerate(CASES):
        c = traces(L, K, 100 + i)
        fam = O.stack_family(L, pmin, pmax, V, wt)
        out = np.empty(L, np.float64)
        rc = R.ref_wt_tspws(out.ctypes.data, c.ctypes.data, K, L, nu, wt, fam["J"], V, fam["s0"], fam["op1"])
        assert rc == 0, rc
        x = c[0].astype(np.float64)
        W = np.empty((fam["S"], L), np.complex128)
        xr = np.empty(L, np.float64)
        rc = R.ref_wt_pair(W.ctypes.data, xr.ctypes.data, x.ctypes.data, L, wt, fam["J"], V, fam["s0"], fam["op1"])
        assert rc == 0, rc
        rec[f"c{i}"] = c
        rec[f"tspws{i}"] = out
        if i == 0:   # one CWT is enough for the pin; float32 keeps the fixture small (relative 1e-7)
            rec["cwt0"] = W.astype(np.complex64)
        rec[f"icwt{i}"] = xr
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden_stack.npz")
    np.savez_compressed(path, **rec)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
