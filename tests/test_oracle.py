"""The FP64 oracle against the reference's golden vectors and known answers.

The golden fixtures were produced by the reference's own CPU method layer
(src/FFTapps.c, compiled unmodified against the oracle's FFTW-API shim, see
tests/golden/make_golden.py).  The reference rounds its outputs to float32, so
the tolerance is a few float32 ulps of the correlation peak.
"""
import glob
import os

import numpy as np
import pytest

from fastpcc_gb300 import synth

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "golden_n*.npz")))
TOL_REF = 1e-6   # reference output is float32


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[7:-4] for p in GOLDEN])
def test_oracle_matches_reference_golden(orc, path):
    g = np.load(path)
    x1, x2, l1, l2 = g["x1"], g["x2"], int(g["Lag1"]), int(g["Lag2"])
    lo, hi = min(l1, l2), max(l1, l2)
    assert orc.relerr(g["pcc2"], orc.pcc2(x1, x2, l1, l2)).max() < TOL_REF
    assert orc.relerr(g["cc1b"], orc.cc1b(x1, x2, l1, l2)).max() < TOL_REF
    if "ccgn" in g:
        assert orc.relerr(g["ccgn"], orc.gncc(x1, x2, l1, l2)).max() < TOL_REF
    assert orc.relerr(g["pcc1"], orc.pcc1(x1, x2, lo, hi)).max() < TOL_REF
    assert orc.relerr(g["pcc_v1.5"], orc.pccv(x1, x2, 1.5, lo, hi)).max() < TOL_REF


def test_oracle_matches_reference_golden_wpcc(orc):
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_wpcc_n3000.npz"))
    x1, x2 = g["x1"], g["x2"]
    for key, wt in (("wpcc_mexhat", -3), ("wpcc_morlet", -1)):
        y = orc.wpcc(x1, x2, int(g["Lag1"]), int(g["Lag2"]), float(g["pmin"]), float(g["pmax"]),
                     V=int(g["V"]), wtype=wt)
        assert orc.relerr(g[key], y).max() < TOL_REF, key


def test_oracle_matches_reference_cli_on_example_records(orc):
    """The reference CLI's own outputs on three days of its GEOSCOPE example
    records (N = 21600, lags +-3000); its phase methods run in float, hence the
    looser bound for PCC2 / PCC1."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden_cli_geoscope.npz"))
    x1, x2, l1, l2 = g["x1"], g["x2"], int(g["Lag1"]), int(g["Lag2"])
    assert orc.relerr(g["pcc2"], orc.pcc2(x1, x2, l1, l2)).max() < 2e-5
    assert orc.relerr(g["pcc1"], orc.pcc1(x1, x2, l1, l2)).max() < 2e-5
    assert orc.relerr(g["ccgn"], orc.gncc(x1, x2, l1, l2)).max() < TOL_REF
    assert orc.relerr(g["cc1b"], orc.cc1b(x1, x2, l1, l2)).max() < TOL_REF
    y = orc.wpcc(x1, x2, l1, l2, float(g["pmin"]), float(g["pmax"]), V=2, wtype=-3)
    assert orc.relerr(g["wpcc2"], y).max() < TOL_REF


@pytest.mark.parametrize("N", [64, 97, 1000, 1024, 18000 // 8, 4099])
def test_analytic_signal_matches_numpy(orc, N):
    x = np.random.default_rng(N).standard_normal(N).astype(np.float32)
    X = np.fft.fft(x.astype(np.float64))
    h = np.zeros(N)
    h[0] = 1
    h[1:(N + 1) // 2] = 2
    if N % 2 == 0:
        h[N // 2] = 1
    ref = np.fft.ifft(X * h) * N / N
    # the reference's IDFT is unnormalised and its mask carries the 1/N
    assert np.max(np.abs(orc.analytic(x) - ref)) < 1e-12 * np.max(np.abs(ref)) * 10


def test_cosine_phase_is_unit_modulus(orc):
    N = 4000
    n = np.arange(N)
    x = np.cos(2 * np.pi * 37 * n / N).astype(np.float32)
    p = orc.phase(x)
    assert np.allclose(np.abs(p), 1.0, atol=1e-5)
    assert np.allclose(p, np.exp(2j * np.pi * 37 * n / N), atol=1e-5)


def test_identity_lag0_is_one(orc):
    a, _ = synth.plain_pair(N=2000, n_windows=2, tag="identity")
    lag = 50
    for f in (orc.gncc, orc.cc1b):
        y = f(a, a, -lag, lag)
        assert np.allclose(y[:, lag], 1.0, atol=1e-9), f.__name__
    # AmpNormf's x/(|x| + 1e-6 max|x|) leaves |p| a hair below 1
    y = orc.pcc2(a, a, -lag, lag)
    assert np.allclose(y[:, lag], 1.0, atol=1e-4)
    y = orc.pcc1(a, a, -lag, lag)
    assert np.allclose(y[:, lag], 1.0, atol=1e-4)


def test_pure_shift_peaks_at_delay(orc):
    d = 37
    a, b = synth.plain_pair(N=3000, n_windows=1, delay=d, snr=3.0, tag="shift")
    for f in (orc.pcc2, orc.gncc, orc.cc1b):
        y = f(a, b, -200, 200)[0]
        assert int(np.argmax(y)) - 200 == d, f.__name__
    y = orc.pcc1(a, b, -200, 200)[0]
    assert int(np.argmax(y)) - 200 == d


def test_cc1b_zero_sample_asymmetry(orc):
    # x1 = 0 counts as +1, x2 = 0 counts as -1 (src/FFTapps.c:1037,1042)
    x = np.zeros((1, 64), np.float32)
    num = orc.cc1b_num(x, x, 0, 0)
    assert num[0, 0] == -64


def test_cc1b_numerator_is_integer_of_fft_path(orc):
    a, b = synth.plain_pair(N=1500, n_windows=2, tag="cc1b-int")
    num = orc.cc1b_num(a, b, -300, 300)
    y = orc.cc1b(a, b, -300, 300)
    lags = np.arange(-300, 301)
    assert np.allclose(y, num / (1500 - np.abs(lags)), atol=0)


def test_lag_windows_conventions(orc):
    a, b = synth.plain_pair(N=1000, n_windows=1, tag="lagwin")
    full = orc.pcc2(a, b, -300, 300)[0]
    assert np.allclose(orc.pcc2(a, b, 20, 90)[0], full[320:391], atol=1e-12)
    assert np.allclose(orc.pcc2(a, b, -90, -20)[0], full[210:281], atol=1e-12)
    assert np.allclose(orc.pcc2(a, b, 90, -90)[0], full[210:391], atol=1e-12)


def test_nz_independence(orc):
    """Linear correlation: any padded length >= N + M gives the same lags."""
    a, b = synth.plain_pair(N=1800, n_windows=1, tag="nz")
    y0 = orc.pcc2(a, b, -200, 200)
    for nz in (2000, 2048, 2250, 4096):
        assert np.max(np.abs(orc.pcc2(a, b, -200, 200, Nz=nz) - y0)) < 1e-12


def test_reference_live_if_present(orc):
    """Where the reference sources exist, the restatement equals them on fresh inputs."""
    if not os.path.isdir(orc.reference_sources()):
        pytest.skip("reference sources absent")
    orc.build(ref=True)
    a, b = synth.plain_pair(N=1500, n_windows=2, tag="live")
    assert orc.relerr(orc.ref_call("pcc2", a, b, -150, 150), orc.pcc2(a, b, -150, 150)).max() < TOL_REF
